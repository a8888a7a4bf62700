"""A TTNO from one dense operator tensor (``TTNO.from_tensor``, ``ttno/ttno_class.py:163-298``).

The operator tensor has legs (out_1 .. out_n, in_1 .. in_n); ``leg_dict``
maps each node to its out leg. The legs are first ordered node by node: a
node's (out, in) pair, then the blocks of its children's subtrees with the
last child's block first. Starting at the root, the tensor is split once per
child, in the children's order: the child's whole block (the trailing legs)
becomes the columns of a matrix whose rows are all other legs, in the node's
current leg order (parent bond, the children bonds made so far, out, in, the
blocks still attached). The row factor stays at the node with the new bond
appended after the earlier children bonds; the column factor, with the bond
as its first leg, is split the same way below the child. That leg
bookkeeping and row order are the reference's, so the reduced QR (Householder
on the device, LAPACK's sign conventions) gives the reference's tensors up to
rounding. The SVD modes factor the same matrices as U (S V^H) through a
device QR and a Jacobi SVD of the small triangular factor: the same operator,
with singular vectors whose phases may differ from LAPACK's.
"""
from __future__ import annotations

from enum import Enum

import numpy as np
import torch

from . import engine as E
from .engine import CDT


class Decomposition(Enum):
    SVD = "SVD"
    QR = "QR"
    tSVD = "tSVD"


def _subtree_size(tree, nid) -> int:
    return 1 + sum(_subtree_size(tree, c) for c in tree.nodes[nid].children)


def _leg_order(tree, legs: dict, nid, acc: list) -> list:
    """``_get_qr_decomposition_shape``: the node's pair, then its children's
    blocks, the last child's first."""
    for c in tree.nodes[nid].children:
        acc = _leg_order(tree, legs, c, acc)
    return legs[nid] + acc


def _svd_factors(M: torch.Tensor, truncate: bool):
    """M = U (S V^H) with U isometric, from a device QR and a k x k Jacobi SVD."""
    from .bug import small_svd
    from .svd_truncation import qr_split
    from .truncation import SVDParameters, truncate_singular_values
    m, K = M.shape
    if m >= K:
        Q, R = qr_split(M, 1, reduced=True)                    # M = Q R, R K x K
        Ut, Vt, s = small_svd(R)
        left, right_t = Q @ Ut.transpose(0, 1), Vt            # R = (Ut^T) diag(s) (Vt^T)^H
    else:
        Q2, R2 = qr_split(M.conj().transpose(0, 1).contiguous(), 1, reduced=True)   # M^H = Q2 R2
        Ut, Vt, s = small_svd(R2.conj().transpose(0, 1).contiguous())               # R2^H = U S W^H
        left, right_t = Ut.transpose(0, 1), Vt @ Q2.transpose(0, 1)                 # conj rows: (Q2 W)^H
    keep = len(s)
    if truncate:
        keep = len(truncate_singular_values(s, SVDParameters(max_bond_dim=float("inf"), rel_tol=1e-10,
                                                              total_tol=1e-15))[0])
    S = torch.from_numpy(np.ascontiguousarray(s[:keep])).to(M.device, CDT)
    U = left[:, :keep].contiguous()
    R = (S[:, None] * right_t[:keep].conj()).contiguous()
    return U, R


def ttno_from_tensor(reference_tree, tensor, leg_dict: dict, mode: Decomposition = Decomposition.QR):
    """The TTNO of ``tensor`` on ``reference_tree``'s structure (node ids and
    children order of the tree)."""
    from .svd_truncation import qr_split
    from .ttn import TreeTensorNetworkOperator
    if isinstance(mode, str):
        mode = Decomposition(mode)
    tensor = np.asarray(tensor)
    if tensor.ndim % 2 != 0:
        raise ValueError("an operator tensor has an even number of legs")
    half = tensor.ndim // 2
    tree = reference_tree
    if half != len(tree.nodes):
        raise ValueError(f"{half} output legs for {len(tree.nodes)} nodes")
    legs = {nid: [int(leg_dict[nid]), half + int(leg_dict[nid])] for nid in leg_dict}
    order = _leg_order(tree, legs, tree.root_id, [])
    T = torch.from_numpy(np.ascontiguousarray(np.transpose(np.asarray(tensor, dtype=np.complex128), order)))
    T = T.to(E.DEFAULT_DEVICE)
    final: dict = {}

    def split(nid, T, has_parent: bool):
        nbonds = 0
        for child in tree.nodes[nid].children:
            ncols = 2 * _subtree_size(tree, child)
            q = T.dim() - ncols
            rows, cols = T.shape[:q], T.shape[q:]
            M = T.reshape(int(np.prod(rows)), int(np.prod(cols))).contiguous()
            if mode is Decomposition.QR:
                Q, R = qr_split(M, 1, reduced=True)
            else:
                Q, R = _svd_factors(M, truncate=mode is Decomposition.tSVD)
            k = Q.shape[1]
            Qt = Q.reshape(tuple(rows) + (k,))
            pre = (1 if has_parent else 0) + nbonds
            perm = list(range(pre)) + [Qt.dim() - 1] + list(range(pre, Qt.dim() - 1))
            T = Qt.permute(perm).contiguous()
            nbonds += 1
            split(child, R.reshape((k,) + tuple(cols)).contiguous(), True)
        final[nid] = T.cpu().numpy()

    split(tree.root_id, T, False)
    ttno = TreeTensorNetworkOperator()
    ttno.add_root(tree.root_id, final[tree.root_id])
    frontier = [tree.root_id]
    while frontier:
        nxt = []
        for nid in frontier:
            offset = 0 if nid == tree.root_id else 1
            for i, child in enumerate(tree.nodes[nid].children):
                ttno.add_child_to_parent(child, final[child], 0, nid, offset + i)
                nxt.append(child)
        frontier = nxt
    return ttno
