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

from .adjoint import _raw_contract
from . import engine as E
from .engine import CDT, ttno_site_tensors
from .ttn import Node, TreeTensorNetworkState


class ApplicationMethod(Enum):
    """``ttns_ttno/application.py:23-98`` (only DIRECT runs)."""
    DIRECT = "direct"
    ZIPUP = "zipup"
    ZIPUP_VARIATIONAL = "zipup_variational"
    HALF_DENSITY_MATRIX = "half_density_matrix"
    DENSITY_MATRIX = "density_matrix"
    SRC = "src"


def _device_tensor(t, device):
    if isinstance(t, torch.Tensor):
        return t.to(device, CDT).contiguous()
    return torch.from_numpy(np.ascontiguousarray(t, dtype=np.complex128)).to(device)


def apply_ttno_to_ttns(ttns: TreeTensorNetworkState, ttno, method: ApplicationMethod = ApplicationMethod.DIRECT,
                       device=None) -> TreeTensorNetworkState:
    """H|psi> as a new TTNS (``apply_ttno_to_ttns``, ``application.py:164-184``)."""
    if method is not ApplicationMethod.DIRECT:
        raise NotImplementedError(f"TTNO application method {method} is not provided (DIRECT only)")
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
