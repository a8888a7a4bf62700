"""TTNO application to a TTNS on the device (``ttns/ttns_ttno/application.py``,
``direct_application.py:21-142``).

The direct method contracts every state tensor with its TTNO tensor over the
physical leg and merges each pair of bond legs into one (state index slow,
operator index fast), in one ``ptn_zcontract`` per node whose output strides
write the merged layout directly. The result is a new TTNS whose bond
dimensions are the products chi * w; compression (zip-up, variational,
density-matrix methods) is not provided.
"""
from __future__ import annotations

from enum import Enum

import numpy as np
import torch

from .adjoint import _raw_contract, qr_keep_raw
from . import engine as E
from .engine import CDT, ttno_site_tensors
from .ttn import Node, TreeTensorNetworkState


class ApplicationMethod(Enum):
    """``ttns_ttno/application.py:23-98`` (DIRECT, ZIPUP, DIRECT_TRUNCATE and
    DIRECT_TRUNCATE_RANDOM run)."""
    DIRECT = "direct"
    DENSITY_MATRIX = "density_matrix"
    HALF_DENSITY_MATRIX = "half_density_matrix"
    SRC = "src"
    ZIPUP = "zipup"
    ZIPUP_CANONICAL = "zipup_canonical"
    VARIATIONAL = "variational"
    ZIPUP_VARIATIONAL = "zipup_variational"
    HALF_DENSITY_MATRIX_VARIATIONAL = "half_density_matrix_variational"
    DIRECT_TRUNCATE = "direct_truncate"
    DIRECT_TRUNCATE_RANDOM = "direct_truncate_random"


def _device_tensor(t, device):
    if isinstance(t, torch.Tensor):
        return t.to(device, CDT).contiguous()
    return torch.from_numpy(np.ascontiguousarray(t, dtype=np.complex128)).to(device)


def apply_ttno_to_ttns(ttns: TreeTensorNetworkState, ttno, method: ApplicationMethod = ApplicationMethod.DIRECT,
                       *args, device=None, **kwargs) -> TreeTensorNetworkState:
    """H|psi> as a new TTNS (``apply_ttno_to_ttns``, ``application.py:164-184``):
    DIRECT, or ZIPUP with ``svd_params`` (positional or keyword)."""
    if method is ApplicationMethod.ZIPUP:
        return zipup(ttno, ttns, *args, device=device, **kwargs)
    if method in (ApplicationMethod.DIRECT_TRUNCATE, ApplicationMethod.DIRECT_TRUNCATE_RANDOM):
        # ``application.py:67-85``: DIRECT followed by the SVD truncation; the
        # random variant sets ``params.random`` (the engine's rank rule for it)
        from .svd_truncation import TruncationMethod, apply_and_truncate
        if method is ApplicationMethod.DIRECT_TRUNCATE_RANDOM:
            from .truncation import SVDParameters
            kwargs = dict(kwargs)
            params = kwargs.get("params", SVDParameters())
            params.random = True
            kwargs["params"] = params
        return apply_and_truncate(ttns, ttno, ApplicationMethod.DIRECT, TruncationMethod.SVD,
                                  trunc_args=args, trunc_kwargs=kwargs)
    if method is not ApplicationMethod.DIRECT:
        raise NotImplementedError(f"TTNO application method {method} is not provided "
                                  "(DIRECT, ZIPUP, DIRECT_TRUNCATE, DIRECT_TRUNCATE_RANDOM)")
    if not torch.cuda.is_available():
        raise RuntimeError("pytreenet_gb300 needs a CUDA device (no CPU fallback)")
    dev = torch.device(device or E.DEFAULT_DEVICE)
    ttns._finalise()
    W = ttno_site_tensors(ttns, ttno)
    out = TreeTensorNetworkState()
    for nid in ttns._order:
        A = _device_tensor(ttns.phys(nid), dev)
        Wn = torch.from_numpy(W[nid]).to(dev)
        n = A.dim() - 1
        la = [f"a{k}" for k in range(n)] + ["s"]
        lw = [f"b{k}" for k in range(n)] + ["t", "s"]
        lc = [x for k in range(n) for x in (f"a{k}", f"b{k}")] + ["t"]
        C = _raw_contract(A, la, Wn, lw, lc, ["s"])
        shape = [A.shape[k] * Wn.shape[k] for k in range(n)] + [Wn.shape[n]]
        node = Node(nid)
        src = ttns.nodes[nid]
        node.parent = src.parent
        node.children = list(src.phys_children)
        node.phys_children = list(src.phys_children)
        node.shape = tuple(shape)
        out.nodes[nid] = node
        out._order.append(nid)
        out._phys[nid] = C.view(shape)
    out.root_id = ttns.root_id
    return out


def apply_operator_in_place(ttns: TreeTensorNetworkState, operator, device=None):
    """``TTNS.apply_operator`` (``ttns/ttns.py:329-337``): every one-site operator
    of the tensor product absorbed into its node's physical leg."""
    if not torch.cuda.is_available():
        raise RuntimeError("pytreenet_gb300 needs a CUDA device (no CPU fallback)")
    dev = torch.device(device or E.DEFAULT_DEVICE)
    ttns._finalise()
    for nid, op in operator.items():
        A = _device_tensor(ttns.phys(nid), dev)
        O = _device_tensor(op, dev)
        n = A.dim() - 1
        la = [f"a{k}" for k in range(n)] + ["s"]
        ttns._phys[nid] = _raw_contract(A, la, O, ["t", "s"], [f"a{k}" for k in range(n)] + ["t"], ["s"])


def zipup(operator, state: TreeTensorNetworkState, svd_params=None, id_trafo=None, canonicalize: bool = False,
          device=None) -> TreeTensorNetworkState:
    """Non-canonical zip-up (``ttns/ttns_ttno/zipup.py:22-105,191-253``): from the
    leaves up, a node's state tensor, TTNO tensor and its children's blocks are
    contracted on the device, and a truncated SVD of the result (rows: the new
    child bonds and the physical leg; columns: the state and operator bonds
    toward the parent) leaves U at the node and sends S V^H, with legs (state
    bond, operator bond, new bond), to the parent; the root keeps the rest.
    The SVD is a Householder QR followed by the Jacobi SVD of the k x k R."""
    from .bug import small_svd
    from .truncation import SVDParameters, truncate_singular_values
    if canonicalize:
        raise NotImplementedError("the canonical zip-up is not provided")
    if id_trafo is not None:
        raise NotImplementedError("identifier transformations are not provided")
    if not torch.cuda.is_available():
        raise RuntimeError("pytreenet_gb300 needs a CUDA device (no CPU fallback)")
    params = svd_params if svd_params is not None else SVDParameters()
    dev = torch.device(device or E.DEFAULT_DEVICE)
    state._finalise()
    W = ttno_site_tensors(state, operator)
    cache, new = {}, {}

    def post(nid):
        out = []
        for c in state.nodes[nid].phys_children:
            out += post(c)
        return out + [nid]
    for v in post(state.root_id):
        node = state.nodes[v]
        nb = node.phys_neighbours()
        n = len(nb)
        kids = [k for k, x in enumerate(nb) if x != node.parent]
        A = _device_tensor(state.phys(v), dev)
        Wv = torch.from_numpy(W[v]).to(dev)
        la = [f"a{k}" for k in range(n)] + ["s"]
        lw = [f"b{k}" for k in range(n)] + ["t", "s"]
        final = [f"n{k}" for k in kids] + (["t", "a0", "b0"] if node.parent is not None else ["t"])
        cur = [f"a{k}" for k in range(n)] + [f"b{k}" for k in range(n)] + ["t"]
        T = _raw_contract(A, la, Wv, lw, final if not kids else cur, ["s"])
        if kids:
            cur = list(cur)
        for i, k in enumerate(kids):
            R = cache.pop(nb[k])
            nxt = [l for l in cur if l not in (f"a{k}", f"b{k}")] + [f"n{k}"]
            out_l = final if i == len(kids) - 1 else nxt
            T = _raw_contract(T, cur, R, [f"a{k}", f"b{k}", f"n{k}"], out_l, [f"a{k}", f"b{k}"])
            cur = out_l
        if node.parent is None:
            new[v] = T
            continue
        rows = list(T.shape[:-2])
        cp, wp = T.shape[-2], T.shape[-1]
        K = cp * wp
        Tm = T.reshape(rows + [K])
        Q, Rm = qr_keep_raw(Tm, len(rows))
        Ut, Vt, sv = small_svd(Rm)
        new_s, _ = truncate_singular_values(sv, params)
        r = len(new_s)
        lq = [f"r{i}" for i in range(len(rows))] + ["col"]
        new[v] = _raw_contract(Q, lq, Ut[:r].contiguous(), ["new", "col"], ["new"] + lq[:-1], ["col"])
        svh = (new_s[:, None] * Vt[:r].cpu().numpy().conj()).reshape(r, cp, wp)
        cache[v] = torch.from_numpy(np.ascontiguousarray(np.transpose(svh, (1, 2, 0)))).to(dev)
    out = TreeTensorNetworkState()
    for nid in state._order:
        node = Node(nid)
        src = state.nodes[nid]
        node.parent = src.parent
        node.children = list(src.phys_children)
        node.phys_children = list(src.phys_children)
        node.shape = tuple(new[nid].shape)
        out.nodes[nid] = node
        out._order.append(nid)
        out._phys[nid] = new[nid]
    out.root_id = state.root_id
    return out
