"""Seeded synthetic workloads in the shapes of the benchmark configurations.

* T-tree: root with three arms of ``arm_len`` sites (61 sites for arm_len=20),
  every bond of dimension ``chi``, Gaussian complex entries (each tensor scaled
  to unit Frobenius norm so the contraction of 61 tensors stays in range),
  Heisenberg couplings plus random fields h_i ~ U[-1, 1] (TTNO bond 5).
* binary tree: heap-ordered (node i has children 2i+1, 2i+2), transverse-field
  Ising H = -J sum Z_i Z_j - g sum X_i, product state on the Bloch sphere
  zero-padded to ``chi`` (TTNO bond 3).
"""
from __future__ import annotations

import numpy as np

from .operators import heisenberg_ttno, tfim_ttno
from .ttn import TreeTensorNetworkState


def _build(spec, tensors) -> TreeTensorNetworkState:
    st = TreeTensorNetworkState()
    parent = dict(spec)
    slot = {nid: 0 for nid, _ in spec}
    for nid, p in spec:
        if p is None:
            st.add_root(nid, tensors[nid])
        else:
            off = 1 if parent[p] is not None else 0
            st.add_child_to_parent(nid, tensors[nid], 0, p, off + slot[p])
            slot[p] += 1
    st._finalise()
    return st


def t_tree_spec(arm_len: int):
    spec = [("root", None)]
    for a in range(3):
        prev = "root"
        for k in range(arm_len):
            nid = f"a{a}_{k}"
            spec.append((nid, prev))
            prev = nid
    return spec


def t_tree_state(arm_len: int = 20, chi: int = 256, seed: int = 0, dtype=np.complex128):
    """Returns (TTNS, spec, tensors in physical layout)."""
    rng = np.random.default_rng(seed)
    spec = t_tree_spec(arm_len)
    nkids = {nid: 0 for nid, _ in spec}
    for nid, p in spec:
        if p is not None:
            nkids[p] += 1
    tensors = {}
    for nid, p in spec:
        nv = nkids[nid] + (0 if p is None else 1)
        shape = [chi] * nv + [2]
        t = (rng.standard_normal(size=shape, dtype=np.float64)
             + 1j * rng.standard_normal(size=shape, dtype=np.float64)).astype(dtype)
        t /= np.linalg.norm(t)
        tensors[nid] = t
    return _build(spec, tensors), spec, tensors


def t_tree_heisenberg(state: TreeTensorNetworkState, seed: int = 1):
    """Heisenberg + random fields on the state's tree; returns (TTNO, W in physical layout)."""
    rng = np.random.default_rng(seed)
    fields = {nid: rng.uniform(-1.0, 1.0) for nid in state._order}
    H = heisenberg_ttno(state, fields)
    return H, {nid: H.phys(nid) for nid in state._order}


def binary_tree_spec(n: int):
    return [(f"s{i}", None if i == 0 else f"s{(i - 1) // 2}") for i in range(n)]


def binary_tfim_product_state(n: int = 15, chi: int = 8, seed: int = 0, J: float = 1.0, g: float = 0.5):
    rng = np.random.default_rng(seed)
    spec = binary_tree_spec(n)
    nkids = {nid: 0 for nid, _ in spec}
    for nid, p in spec:
        if p is not None:
            nkids[p] += 1
    tensors = {}
    for nid, p in spec:
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        th, ph = np.arccos(v[2]), np.arctan2(v[1], v[0])
        site = np.array([np.cos(th / 2), np.exp(1j * ph) * np.sin(th / 2)], dtype=complex)
        nv = nkids[nid] + (0 if p is None else 1)
        t = np.zeros([chi] * nv + [2], dtype=complex)
        t[(0,) * nv] = site
        tensors[nid] = t
    st = _build(spec, tensors)
    H = tfim_ttno(st, J=J, g=g)
    return st, H, spec, tensors


def binary_tfim_random_state(n: int = 31, chi: int = 64, seed: int = 0, g_low: float = 0.3,
                             g_high: float = 0.7, J: float = 1.0):
    """Gradient workload: heap-ordered binary tree of ``n`` sites, Gaussian complex
    tensors (unit Frobenius norm each) with the bond to a subtree of s sites of
    dimension min(chi, 2^s, 2^(n-s)), so every QR split of a one-site sweep is
    tall and of full rank; transverse fields g_i ~ U[g_low, g_high], coupling J.
    Returns (TTNS, spec, tensors in physical layout, g dict, J)."""
    rng = np.random.default_rng(seed)
    spec = binary_tree_spec(n)
    kids = {nid: [] for nid, _ in spec}
    for nid, p in spec:
        if p is not None:
            kids[p].append(nid)
    size = {}
    for nid, _ in reversed(spec):
        size[nid] = 1 + sum(size[c] for c in kids[nid])

    def bond(c):
        s = size[c]
        return int(min(chi, 2 ** min(s, 60), 2 ** min(n - s, 60)))
    tensors = {}
    for nid, p in spec:
        shape = ([bond(nid)] if p is not None else []) + [bond(c) for c in kids[nid]] + [2]
        t = rng.standard_normal(size=shape) + 1j * rng.standard_normal(size=shape)
        tensors[nid] = t / np.linalg.norm(t)
    g = {nid: float(rng.uniform(g_low, g_high)) for nid, _ in spec}
    return _build(spec, tensors), spec, tensors, g, J


def ternary_spec(depth: int):
    """Complete ternary tree: t0 at the root, three children per internal node
    (1 + 3 + 9 + 27 = 40 sites for depth 3)."""
    spec = [("t0", None)]
    frontier, idx = ["t0"], 1
    for _ in range(depth):
        nxt = []
        for p in frontier:
            for _ in range(3):
                nid = f"t{idx}"
                idx += 1
                spec.append((nid, p))
                nxt.append(nid)
        frontier = nxt
    return spec


def ternary_state(depth: int = 2, chi: int = 4, seed: int = 0):
    """Random ternary-tree TTNS (unit-norm Gaussian tensors, every bond ``chi``).
    Returns (TTNS, spec, tensors in physical layout)."""
    rng = np.random.default_rng(seed)
    spec = ternary_spec(depth)
    nkids = {nid: 0 for nid, _ in spec}
    for nid, p in spec:
        if p is not None:
            nkids[p] += 1
    tensors = {}
    for nid, p in spec:
        shape = [chi] * (nkids[nid] + (0 if p is None else 1)) + [2]
        t = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        tensors[nid] = t / np.linalg.norm(t)
    return _build(spec, tensors), spec, tensors


def ternary_neel_state(depth: int = 3):
    """Neel product state by depth parity (up on even depths), every bond of
    dimension 1. Returns (TTNS, spec, tensors)."""
    spec = ternary_spec(depth)
    nkids = {nid: 0 for nid, _ in spec}
    depth_of = {}
    for nid, p in spec:
        depth_of[nid] = 0 if p is None else depth_of[p] + 1
        if p is not None:
            nkids[p] += 1
    tensors = {}
    for nid, p in spec:
        v = np.array([1, 0], dtype=complex) if depth_of[nid] % 2 == 0 else np.array([0, 1], dtype=complex)
        tensors[nid] = v.reshape([1] * (nkids[nid] + (0 if p is None else 1)) + [2])
    return _build(spec, tensors), spec, tensors


def ternary_xxz(state: TreeTensorNetworkState, seed: int = 7):
    """XXZ with per-edge couplings Jxy, Jz ~ U[0.5, 1.5]; returns (TTNO, W in physical layout)."""
    rng = np.random.default_rng(seed)
    edges = [(state.nodes[nid].parent, nid) for nid in state._order if state.nodes[nid].parent is not None]
    jxy = {e: rng.uniform(0.5, 1.5) for e in edges}
    jz = {e: rng.uniform(0.5, 1.5) for e in edges}
    H = heisenberg_ttno(state, None, jxy, jz)
    return H, {nid: H.phys(nid) for nid in state._order}


def ternary_saturated_state(depth: int = 3, chi: int = 64, seed: int = 0):
    """Random ternary-tree TTNS whose bonds are as large as a two-site TDVP run
    with max_bond_dim ``chi`` makes them: min(chi, 2^(sites below the bond),
    2^(sites above it)). Returns (TTNS, spec, tensors)."""
    rng = np.random.default_rng(seed)
    spec = ternary_spec(depth)
    kids = {nid: [] for nid, _ in spec}
    for nid, p in spec:
        if p is not None:
            kids[p].append(nid)
    below = {}

    def count(nid):
        below[nid] = 1 + sum(count(c) for c in kids[nid])
        return below[nid]
    total = count(spec[0][0])

    def bond(child):
        b = min(below[child], total - below[child])
        return int(min(chi, 2 ** min(b, 30)))
    tensors = {}
    for nid, p in spec:
        shape = ([bond(nid)] if p is not None else []) + [bond(c) for c in kids[nid]] + [2]
        t = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        tensors[nid] = t / np.linalg.norm(t)
    return _build(spec, tensors), spec, tensors


def binary_neel_random_field(n: int = 31, seed: int = 0, h: float = 2.0):
    """Heap-ordered binary tree of ``n`` sites, Neel product state by depth
    parity (every bond of dimension 1), Heisenberg couplings (Jxy = Jz = 1) and
    random fields h_i ~ U[-h, h]. Returns (TTNS, TTNO, spec, tensors, W)."""
    rng = np.random.default_rng(seed)
    spec = binary_tree_spec(n)
    nkids = {nid: 0 for nid, _ in spec}
    depth = {}
    for nid, p in spec:
        depth[nid] = 0 if p is None else depth[p] + 1
        if p is not None:
            nkids[p] += 1
    tensors = {}
    for nid, p in spec:
        v = np.array([1, 0], dtype=complex) if depth[nid] % 2 == 0 else np.array([0, 1], dtype=complex)
        tensors[nid] = v.reshape([1] * (nkids[nid] + (0 if p is None else 1)) + [2])
    st = _build(spec, tensors)
    fields = {nid: rng.uniform(-h, h) for nid, _ in spec}
    H = heisenberg_ttno(st, fields)
    return st, H, spec, tensors, {nid: H.phys(nid) for nid in st._order}


def disorder_realisation(i: int, caps=(8, 16, 32, 64), precision: str = "mixed", n: int = 31, h: float = 2.0,
                         dt: float = 0.05, cutoff: float = 1e-9):
    """Realisation i of the disorder average: ``binary_neel_random_field``
    (seed i) under second-order two-site TDVP with max_bond_dim
    caps[i mod len(caps)] and rel_tol = total_tol = cutoff. Module-level, so
    worker processes can build it (``run_realisations(..., processes=P)``)."""
    from .tdvp import SecondOrderTwoSiteTDVP, TimeEvoMode, TwoSiteTDVPConfig
    st, H, _, _, _ = binary_neel_random_field(n=n, seed=i, h=h)
    cfg = TwoSiteTDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV, max_bond_dim=caps[i % len(caps)],
                            rel_tol=cutoff, total_tol=cutoff)
    return SecondOrderTwoSiteTDVP(st, H, dt, 1000 * dt, {}, config=cfg, solver_options={"krylov_tol": 1e-10},
                                  precision=precision)


def realisation_bond_dims(i: int, algo) -> dict:
    """The bond dimensions of a finished realisation (a picklable result)."""
    return dict(algo.state.bond_dims())
