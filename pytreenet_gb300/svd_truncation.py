"""SVD truncation of a whole TTNS on the device (``core/truncation/svd_truncation.py``).

Along the leaf-to-leaf path the orthogonality centre moves (REDUCED QR hops)
to every non-root node and the bond to its parent is cut by a truncated SVD:
the node's tensor is factored with its parent leg as the column index
(Householder QR, then the Jacobi SVD of the k x k R), U stays at the node and
S V^H goes into the parent, with the rule of ``truncate_singular_values``.
Used by the rank-adaptive BUG and by ``apply_and_truncate``.
"""
from __future__ import annotations

from enum import Enum

import numpy as np
import torch

from .adjoint import absorb, qr_keep_raw
from .truncation import truncate_singular_values


class SplitMode(Enum):
    """``util/tensor_splitting.py:23-50``: REDUCED shrinks a bond to the row
    count of a wide split, KEEP keeps it (zero-padded Q); FULL is not provided."""
    FULL = "full"
    REDUCED = "reduced"
    KEEP = "keep"


class TruncationMethod(Enum):
    """``core/truncation/truncating.py:14-60`` (SVD and NONE run here)."""
    RECURSIVE = "recursive"
    SVD = "svd"
    SVD2SITE = "svd_2site"
    VARIATIONAL = "variational"
    DENSITYMATRIX = "density matrix"
    NONE = "none"


class TreeOps:
    """Leg bookkeeping of a TTNS whose tensors are held in a dict in the
    physical layout (parent, children in insertion order, physical)."""

    def __init__(self, ttns):
        ttns._finalise()
        self.tree = ttns
        self.root = ttns.root_id
        self.nbrs = {n: ttns.nodes[n].phys_neighbours() for n in ttns._order}
        self.parent = {n: ttns.nodes[n].parent for n in ttns._order}
        self.children = {n: list(ttns.nodes[n].phys_children) for n in ttns._order}

    def ax(self, u, v):
        return self.nbrs[u].index(v)


def qr_split(A, ax, reduced: bool):
    """QR with leg ``ax`` as the column index; ``reduced`` (SplitMode.REDUCED)
    shrinks that leg to the row count when A is wide, else it is kept."""
    Q, R = qr_keep_raw(A, ax)
    k = A.shape[ax]
    m = A.numel() // k
    if reduced and m < k:
        Q = Q.narrow(ax, 0, m).contiguous()
        R = R[:m].contiguous()
    return Q, R


def move_center(ops: TreeOps, A: dict, center: str, target: str, reduced: bool) -> str:
    path = ops.tree.path_from_to(center, target)
    for a, b in zip(path[:-1], path[1:]):
        Q, R = qr_split(A[a], ops.ax(a, b), reduced=reduced)
        A[a] = Q
        A[b] = absorb(R, A[b], ops.ax(b, a))
    return target


def canonical_form(ops: TreeOps, A: dict, center: str, reduced: bool = True) -> str:
    """``canonical_form`` (``core/canonical_form.py:162-208``): farthest nodes
    first, each split toward its neighbour closest to the centre."""
    dist = ops.tree.distance_to_node(center)
    for d in range(max(dist.values(), default=0), 0, -1):
        for nid in [n for n in dist if dist[n] == d]:
            target = min(ops.tree.nodes[nid].neighbouring_nodes(), key=lambda x: dist[x])
            move_center(ops, A, nid, target, reduced)
    return center


def compress_parent_leg(ops: TreeOps, A: dict, nid: str, params) -> str:
    """``compress_parent_leg``: truncated SVD of the bond between nid and its parent."""
    from .bug import small_svd
    T = A[nid]
    Q, R = qr_keep_raw(T, 0)
    Ut, Vt, s = small_svd(R)
    new_s, _ = truncate_singular_values(s, params)
    r = len(new_s)
    A[nid] = absorb(Ut[:r].contiguous(), Q, 0)
    p = ops.parent[nid]
    svh = new_s[:, None] * Vt[:r].cpu().numpy().conj()
    A[p] = absorb(torch.from_numpy(np.ascontiguousarray(svh)).to(T.device), A[p], ops.ax(p, nid))
    return p


def truncate_tensors(ops: TreeOps, A: dict, center: str, params) -> str:
    """The sweep of ``svd_truncation`` starting from a state whose centre is
    ``center``; returns the final centre."""
    from .tdvp import leaf_to_leaf_update_path
    path = leaf_to_leaf_update_path(ops.tree)
    center = move_center(ops, A, center, path[0], True)
    for nid in path:
        if nid == ops.root:
            continue
        center = move_center(ops, A, center, nid, True)
        center = compress_parent_leg(ops, A, nid, params)
    return center


def svd_truncation(ttns, params):
    """``svd_truncation(tree, params)``: canonical form at the start of the
    leaf-to-leaf path (REDUCED QRs), then the truncation sweep; the TTNS's
    tensors are replaced by device tensors and its centre recorded."""
    from .tdvp import leaf_to_leaf_update_path
    from .application import _device_tensor
    from . import engine as E
    if not torch.cuda.is_available():
        raise RuntimeError("pytreenet_gb300 needs a CUDA device (no CPU fallback)")
    dev = torch.device(E.DEFAULT_DEVICE)
    ops = TreeOps(ttns)
    with torch.no_grad():
        A = {n: _device_tensor(ttns.phys(n), dev) for n in ttns._order}
        start = leaf_to_leaf_update_path(ttns)[0]
        if ttns.orthogonality_center_id is None:
            center = canonical_form(ops, A, start)
        else:
            center = move_center(ops, A, ttns.orthogonality_center_id, start, True)
        center = truncate_tensors(ops, A, center, params)
    for n, t in A.items():
        ttns._phys[n] = t
        ttns.nodes[n].shape = tuple(t.shape)
    ttns.orthogonality_center_id = center
    return ttns


def apply_and_truncate(ttns, ttno, app_method=None, trunc_method: TruncationMethod = TruncationMethod.SVD,
                       app_args: tuple = (), app_kwargs: dict | None = None, trunc_args: tuple = (),
                       trunc_kwargs: dict | None = None):
    """``apply_and_truncate`` (``ttns_ttno/application.py:186-228``): the TTNO
    applied (DIRECT), then the result truncated (SVD with ``trunc_args[0]`` or
    ``trunc_kwargs['params']`` as SVDParameters, or NONE)."""
    from .application import ApplicationMethod, apply_ttno_to_ttns
    from .truncation import SVDParameters
    out = apply_ttno_to_ttns(ttns, ttno, app_method or ApplicationMethod.DIRECT, *app_args, **(app_kwargs or {}))
    if trunc_method is TruncationMethod.NONE:
        return out
    if trunc_method is not TruncationMethod.SVD:
        raise NotImplementedError(f"truncation method {trunc_method} is not provided (SVD, NONE)")
    kw = dict(trunc_kwargs or {})
    params = trunc_args[0] if trunc_args else kw.pop("params", kw.pop("svd_params", SVDParameters()))
    return svd_truncation(out, params)
