"""Nearest-neighbour Hamiltonians on trees as TTNOs.

PyTreeNet compiles a symbolic Hamiltonian into a TTNO through a state
diagram (``ttno/ttno_class.py:60-97``, ``ttno/state_diagram.py``). That
compiler is set-up code, not part of the time-evolution path; for the sums of
one-site and nearest-neighbour two-site terms used by TDVP workloads this
module builds an equivalent TTNO directly from a finite-state description.
Each bond (parent p, child v) carries 2 + K states seen from p:
  0      nothing placed in v's subtree yet (identity),
  1      one complete term lies in v's subtree,
  2 + a  v holds B_a, the child end of coupling channel a; A_a goes on p.
The TTNO bond dimension is 2 + K (3 for the transverse-field Ising model,
5 for Heisenberg/XXZ). Any TTNO for the same operator gives the same TDVP
evolution; this one need not match the reference's tensors entry by entry.
"""
from __future__ import annotations

import numpy as np

from .ttn import Node, TreeTensorNetworkOperator, TreeTensorNetworkState

X = np.array([[0, 1], [1, 0]], dtype=complex)
Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
Z = np.diag([1.0, -1.0]).astype(complex)
I2 = np.eye(2, dtype=complex)


def nearest_neighbour_ttno(state: TreeTensorNetworkState, onsite: dict, edge_terms: dict,
                           phys_dim: int = 2) -> TreeTensorNetworkOperator:
    """TTNO of H = sum_v onsite[v] + sum_(p,v) sum_a c_a A_a(p) B_a(v).

    ``edge_terms[(parent, child)]`` is a list of (c_a, A_a, B_a) with A_a acting
    on the parent and B_a on the child. Tensor legs follow the state's physical
    neighbour order: (parent, children..., out, in)."""
    state._finalise()
    d = phys_dim
    eye = np.eye(d, dtype=complex)
    K = {}
    for nid in state._order:
        p = state.nodes[nid].parent
        if p is not None:
            K[(p, nid)] = len(edge_terms.get((p, nid), []))
    ttno = TreeTensorNetworkOperator()
    for nid in state._order:
        snode = state.nodes[nid]
        node = Node(nid)
        node.parent = snode.parent
        node.children = list(snode.phys_children)
        node.phys_children = list(snode.phys_children)
        kids = list(snode.phys_children)
        wp = None if snode.parent is None else 2 + K[(snode.parent, nid)]
        wc = [2 + K[(nid, c)] for c in kids]
        shape = ([wp] if wp is not None else []) + wc + [d, d]
        W = np.zeros(shape, dtype=complex)

        def put(bp, bc, op):
            idx = ([bp] if wp is not None else []) + list(bc) + [slice(None), slice(None)]
            W[tuple(idx)] += op
        zero = [0] * len(kids)
        h = onsite.get(nid)
        # parent state 0: identity everywhere below
        if wp is not None:
            put(0, zero, eye)
        # parent state 1 (or the root's only component): one complete term
        put(1, zero, h if h is not None else np.zeros((d, d), dtype=complex))
        for i, c in enumerate(kids):
            bc = list(zero)
            bc[i] = 1
            put(1, bc, eye)
            for a, (coef, A, _B) in enumerate(edge_terms.get((nid, c), [])):
                bc = list(zero)
                bc[i] = 2 + a
                put(1, bc, coef * np.asarray(A, dtype=complex))
        if wp is not None:
            for a, (_coef, _A, B) in enumerate(edge_terms.get((snode.parent, nid), [])):
                put(2 + a, zero, np.asarray(B, dtype=complex))
        node.shape = W.shape
        ttno.nodes[nid] = node
        ttno._order.append(nid)
        ttno._phys[nid] = W
    ttno.root_id = state.root_id
    return ttno


def _edges(state):
    return [(state.nodes[nid].parent, nid) for nid in state._order if state.nodes[nid].parent is not None]


def tfim_ttno(state: TreeTensorNetworkState, J: float = 1.0, g=0.5) -> TreeTensorNetworkOperator:
    """H = -J sum_<ij> Z_i Z_j - sum_i g_i X_i (g scalar or dict node -> g_i)."""
    state._finalise()
    gd = g if isinstance(g, dict) else {nid: g for nid in state._order}
    onsite = {nid: -gd[nid] * X for nid in state._order}
    edges = {e: [(-J, Z, Z)] for e in _edges(state)}
    return nearest_neighbour_ttno(state, onsite, edges)


def heisenberg_ttno(state: TreeTensorNetworkState, fields=None, jxy=None, jz=None) -> TreeTensorNetworkOperator:
    """H = sum_<ij> (Jxy (X X + Y Y) + Jz Z Z) + sum_i h_i Z_i; per-edge couplings
    are dicts keyed by (parent, child), defaults 1."""
    state._finalise()
    onsite = {}
    if fields is not None:
        onsite = {nid: fields[nid] * Z for nid in state._order}
    edges = {}
    for e in _edges(state):
        cxy = 1.0 if jxy is None else jxy[e]
        cz = 1.0 if jz is None else jz[e]
        edges[e] = [(cxy, X, X), (cxy, Y, Y), (cz, Z, Z)]
    return nearest_neighbour_ttno(state, onsite, edges)
