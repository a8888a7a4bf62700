"""NumPy restatement of PyTreeNet's TDVP (one-site, two-site) and TEBD hot path (oracle, test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use this module; the GPU engine never imports it.

Every function cites the reference function whose algorithm it restates
(paths are relative to the PyTreeNet project root). The data model differs
from the reference on purpose: each node tensor keeps ONE physical leg layout
(parent, children in insertion order, physical), while the reference's
*logical* children order -- which the reference reshuffles during QR splits
and contractions (``core/ttn.py:1235-1313``, ``contractions/node_contraction.py:88-138``)
-- is tracked separately and used only where it changes numbers: the row order
of every QR matricisation (``util/tensor_splitting.py:60-107``) and the
processing order of ``canonical_form`` (``core/canonical_form.py:162-208``).
On rank-deficient (zero-padded) tensors the Householder complement chosen by
LAPACK depends on that row order, and one-site TDVP's result depends on the
complement, so the order has to match for 1e-10 parity.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "OTree", "OState", "init_cache_but_one", "heff_apply", "bond_apply",
    "env_update", "krylov_exp_action", "qr_keep_split", "canonical_form",
    "leaf_to_root_path", "orthogonalisation_paths", "FirstOrderOneSiteTDVPOracle",
    "SecondOrderOneSiteTDVPOracle", "state_vector", "expect_product",
    "scalar_product", "SVDParams", "truncate_singular_values", "two_site_merge",
    "two_site_heff_apply", "two_site_split", "SecondOrderTwoSiteTDVPOracle",
    "FirstOrderTwoSiteTDVPOracle", "tebd_apply_gate", "TEBDOracle", "ttno_expectation",
    "fixed_bug_step", "adaptive_bug_step", "svd_truncation", "leaf_to_leaf_path", "dense_exp_action",
    "zipup_apply",
]


# ----------------------------------------------------------------------------
# tree structure
# ----------------------------------------------------------------------------
class OTree:
    """Rooted tree; physical children order is fixed, logical order evolves."""

    def __init__(self):
        self.parent: dict[str, str | None] = {}
        self.children: dict[str, list[str]] = {}
        self.lchildren: dict[str, list[str]] = {}
        self.root: str | None = None
        self.nodes: list[str] = []

    def copy(self) -> "OTree":
        t = OTree()
        t.parent = dict(self.parent)
        t.children = {k: list(v) for k, v in self.children.items()}
        t.lchildren = {k: list(v) for k, v in self.lchildren.items()}
        t.root = self.root
        t.nodes = list(self.nodes)
        return t

    def add_root(self, nid: str):
        assert self.root is None
        self.root = nid
        self.parent[nid] = None
        self.children[nid] = []
        self.lchildren[nid] = []
        self.nodes.append(nid)

    def add_child(self, nid: str, pid: str):
        self.parent[nid] = pid
        self.children[nid] = []
        self.lchildren[nid] = []
        self.children[pid].append(nid)
        self.lchildren[pid].append(nid)
        self.nodes.append(nid)

    def is_leaf(self, nid):
        return len(self.children[nid]) == 0

    def neighbours(self, nid):
        """Physical order: parent first, then children in insertion order."""
        p = self.parent[nid]
        return ([p] if p is not None else []) + list(self.children[nid])

    def lneighbours(self, nid):
        """Reference order (``core/graph_node.py:340-355``)."""
        p = self.parent[nid]
        return ([p] if p is not None else []) + list(self.lchildren[nid])

    def axis(self, nid, nbr):
        """Physical tensor axis of ``nid`` that points to neighbour ``nbr``."""
        return self.neighbours(nid).index(nbr)

    def path_to_root(self, nid):
        """``core/tree_structure.py:609-624``."""
        path = [nid]
        while self.parent[nid] is not None:
            nid = self.parent[nid]
            path.append(nid)
        return path

    def path_from_to(self, a, b):
        """Unique tree path a -> b (``core/tree_structure.py:626-651``)."""
        if a == b:
            return [a]
        pa = self.path_to_root(a)
        pb = self.path_to_root(b)
        sb = set(pb)
        lca = next(x for x in pa if x in sb)
        up = pa[:pa.index(lca) + 1]
        down = pb[:pb.index(lca)]
        return up + list(reversed(down))

    def distance_to_node(self, center):
        """Pre-order DFS over logical neighbours (``core/tree_structure.py:225-271``)."""
        out = {center: 0}

        def rec(nid, last, d):
            out[nid] = d
            for nb in self.lneighbours(nid):
                if nb != last:
                    rec(nb, nid, d + 1)
        for nb in self.lneighbours(center):
            rec(nb, center, 1)
        return out


class OState:
    """A TTNS on an :class:`OTree`: one tensor per node in physical layout."""

    def __init__(self, tree: OTree, tensors: dict[str, np.ndarray]):
        self.tree = tree
        self.tensors = {k: np.asarray(v) for k, v in tensors.items()}
        self.orth_center: str | None = None

    def copy(self) -> "OState":
        s = OState(self.tree.copy(), {k: v.copy() for k, v in self.tensors.items()})
        s.orth_center = self.orth_center
        return s


# ----------------------------------------------------------------------------
# QR split with KEEP padding, in the reference's row order
# ----------------------------------------------------------------------------
def qr_keep_split(state: OState, nid: str, nbr: str):
    """Split ``nid`` toward neighbour ``nbr``: tensor[nid] <- Q, return R.

    Restates ``tensor_qr_decomposition(mode=KEEP)`` (``util/tensor_splitting.py:60-107``)
    as called by ``OneSiteTDVP._split_updated_site`` (``time_evolution/tdvp_algorithms/onesitetdvp.py:69-101``)
    and ``split_qr_contract_r_to_neighbour`` (``core/canonical_form.py:76-120``).
    Rows are matricised in the reference's logical order: (parent, logical
    children without ``nbr``, physical) when ``nbr`` is a child, (logical
    children, physical) when ``nbr`` is the parent. R has legs
    (new bond on the Q side, bond on the ``nbr`` side).
    Logical order afterwards: a split toward child X puts X first in
    ``nid``'s children (``core/ttn.py:1409-1440``).
    """
    tree = state.tree
    A = state.tensors[nid]
    if tree.parent[nid] == nbr:
        row_nbrs = list(tree.lchildren[nid])
    else:
        p = tree.parent[nid]
        row_nbrs = ([p] if p is not None else []) + [c for c in tree.lchildren[nid] if c != nbr]
    row_axes = [tree.axis(nid, x) for x in row_nbrs] + [A.ndim - 1]
    col_axis = tree.axis(nid, nbr)
    k = A.shape[col_axis]
    mat = np.transpose(A, row_axes + [col_axis]).reshape(-1, k)
    q, r = np.linalg.qr(mat, mode="reduced")
    if q.shape[1] < k:
        diff = k - q.shape[1]
        q = np.pad(q, [(0, 0), (0, diff)])
        r = np.pad(r, [(0, diff), (0, 0)])
    qt = q.reshape([A.shape[a] for a in row_axes] + [k])
    perm_to_phys = np.argsort(row_axes + [col_axis])
    state.tensors[nid] = np.ascontiguousarray(np.transpose(qt, perm_to_phys))
    if tree.parent[nid] != nbr:
        tree.lchildren[nid] = [nbr] + [c for c in tree.lchildren[nid] if c != nbr]
    return r


def absorb_r(state: OState, r: np.ndarray, src: str, dst: str, link_variant: bool):
    """Contract R (legs: src-side, dst-side) into ``dst``'s leg toward ``src``.

    Logical order when ``dst`` is the parent of ``src``: the move-orthogonality
    variant (``contract_nodes(neighbour, r)``, ``core/canonical_form.py:113-114``)
    puts ``src`` LAST among ``dst``'s children, the link-update variant
    (``contract_nodes(link, next)``, ``onesitetdvp.py:125-126``) puts it FIRST
    (``contractions/node_contraction.py:120-131``).
    """
    tree = state.tree
    T = state.tensors[dst]
    ax = tree.axis(dst, src)
    out = np.tensordot(r, T, axes=([1], [ax]))          # new leg first
    out = np.moveaxis(out, 0, ax)
    state.tensors[dst] = out
    if tree.parent[src] == dst:
        others = [c for c in tree.lchildren[dst] if c != src]
        tree.lchildren[dst] = ([src] + others) if link_variant else (others + [src])


def move_orth_one_hop(state: OState, a: str, b: str):
    """``split_qr_contract_r_to_neighbour(a -> b)`` with KEEP (``core/canonical_form.py:76-120``)."""
    r = qr_keep_split(state, a, b)
    absorb_r(state, r, a, b, link_variant=False)


def move_orth_center(state: OState, new_center: str):
    """``TreeTensorNetwork.move_orthogonalization_center`` (``core/ttn.py:1530-1552``)."""
    assert state.orth_center is not None
    path = state.tree.path_from_to(state.orth_center, new_center)
    for a, b in zip(path[:-1], path[1:]):
        move_orth_one_hop(state, a, b)
    state.orth_center = new_center


def canonical_form(state: OState, center: str):
    """``canonical_form`` (``core/canonical_form.py:162-208``): farthest nodes first,
    each split toward its neighbour closest to the centre, within one distance
    in pre-order DFS order."""
    dist = state.tree.distance_to_node(center)
    maxd = max(dist.values()) if dist else 0
    for d in range(maxd, 0, -1):
        for nid in [n for n in dist if dist[n] == d]:
            nbrs = state.tree.lneighbours(nid)
            target = min(nbrs, key=lambda x: dist[x])
            move_orth_one_hop(state, nid, target)
    state.orth_center = center


# ----------------------------------------------------------------------------
# contractions
# ----------------------------------------------------------------------------
class _L:
    """A tensor with one label per leg; contractions go through np.tensordot."""
    __slots__ = ("t", "legs")

    def __init__(self, t, legs):
        self.t, self.legs = t, list(legs)

    def dot(self, other: "_L", labels):
        ia = [self.legs.index(x) for x in labels]
        ib = [other.legs.index(x) for x in labels]
        t = np.tensordot(self.t, other.t, axes=(ia, ib))
        legs = [x for x in self.legs if x not in labels] + [x for x in other.legs if x not in labels]
        return _L(t, legs)

    def out(self, order):
        return np.transpose(self.t, [self.legs.index(x) for x in order])


def _site_chain(x, W, nbrs, envs_of, open_k=None):
    """Apply the environments and W to a site tensor in the interleaved order:
    the first half of the environments, then W, then the rest (the cheapest
    order for degree >= 2; the reference contracts all environments first).
    ``open_k`` leaves neighbour k's bond (ket leg and ham leg) open.
    Returns a labelled tensor with legs a'_k (bra), s', and for ``open_k``
    also a_k, b_k."""
    n = len(nbrs)
    T = _L(x, [f"a{k}" for k in range(n)] + ["s"])
    ks = [k for k in range(n) if k != open_k]
    half = len(ks) // 2
    for k in ks[:half]:
        T = T.dot(_L(envs_of(nbrs[k]), [f"a{k}", f"b{k}", f"c{k}"]), [f"a{k}"])
    Wl = _L(W, [f"b{k}" for k in range(n)] + ["t", "s"])
    T = T.dot(Wl, [f"b{k}" for k in ks[:half]] + ["s"])
    for k in ks[half:]:
        T = T.dot(_L(envs_of(nbrs[k]), [f"a{k}", f"b{k}", f"c{k}"]), [f"a{k}", f"b{k}"])
    return T


def heff_apply(x, tree: OTree, nid: str, W, envs):
    """y = H_eff x for one site (``contract_ket_ham_with_envs``,
    ``contractions/state_operator_contraction.py:227-273``).

    x legs (physical neighbours..., s); env for neighbour k is the cache entry
    (k -> nid) with legs (ket, ham, bra); W legs (neighbours..., out, in).
    y[a'..., s'] = sum E_k[a_k, b_k, a'_k] W[b..., s', s] x[a..., s].
    """
    nbrs = tree.neighbours(nid)
    T = _site_chain(x, W, nbrs, lambda nb: envs[(nb, nid)])
    return T.out([f"c{k}" for k in range(len(nbrs))] + ["t"])


def env_update(tree: OTree, nid: str, nxt: str, A, W, envs):
    """Environment E(nid -> nxt), legs (ket, ham, bra)
    (``contract_any``/``contract_leaf``/``contract_subtrees_using_dictionary``,
    ``contractions/state_operator_contraction.py:407-694``)."""
    nbrs = tree.neighbours(nid)
    k = nbrs.index(nxt)
    T = _site_chain(A, W, nbrs, lambda nb: envs[(nb, nid)], open_k=k)
    B = _L(A.conj(), [f"c{j}" if j != k else "z" for j in range(len(nbrs))] + ["t"])
    E = T.dot(B, [f"c{j}" for j in range(len(nbrs)) if j != k] + ["t"])
    return E.out([f"a{k}", f"b{k}", "z"])


def bond_apply(r, e_q, e_n):
    """Bond H_eff matvec (``contract_bond_tensor``,
    ``contractions/state_operator_contraction.py:984-1040``):
    y[a', c'] = sum E_q[a, b, a'] r[a, c] E_n[c, b, c']."""
    t = np.tensordot(e_q, r, axes=([0], [0]))          # (b, a', c)
    return np.tensordot(t, e_n, axes=([0, 2], [1, 0]))


def init_cache_but_one(state: OState, W: dict, left_out: str) -> dict:
    """All environments pointing toward ``left_out``
    (``SandwichCache.init_cache_but_one``, ``contractions/sandwich_caching.py:97-126``)."""
    tree = state.tree
    envs = {}

    def rec(nid, toward):
        for nb in tree.neighbours(nid):
            if nb != toward:
                rec(nb, nid)
        if toward is not None:
            envs[(nid, toward)] = env_update(tree, nid, toward, state.tensors[nid], W[nid], envs)
    rec(left_out, None)
    return envs


# ----------------------------------------------------------------------------
# Krylov exponential
# ----------------------------------------------------------------------------
def _small_propagator(T, dt, exp_factor, hermitian=True):
    """First column of exp(exp_factor dt T) (``_krylov_small_propagator``,
    ``time_evolution/time_evolution.py:696-718``)."""
    if hermitian:
        H = 0.5 * (T + T.conj().T)
        ev, V = np.linalg.eigh(H)
        return V @ (np.exp(exp_factor * dt * ev) * V[0].conj())
    import scipy.linalg
    return scipy.linalg.expm(exp_factor * dt * T)[:, 0]


def krylov_exp_action(psi, action, dt, exp_factor, krylov_tol=1e-10,
                      max_krylov_dim=None, hermitian=True, stats=None):
    """exp(exp_factor dt A) psi by Arnoldi with two Gram-Schmidt passes
    (``krylov_exp_action``, ``time_evolution/time_evolution.py:721-821``)."""
    shape = psi.shape
    v0 = np.asarray(psi, dtype=complex).reshape(-1)
    n = v0.size
    beta0 = float(np.linalg.norm(v0))
    if beta0 == 0.0:
        return v0.copy().reshape(shape)
    max_steps = n if max_krylov_dim is None else min(n, int(max_krylov_dim))
    floor_abs = np.finfo(float).eps * max(n, 1)
    Q = [v0 / beta0]
    T = np.zeros((min(max_steps, 32) + 1,) * 2, dtype=complex)
    m = 0
    for j in range(max_steps):
        if j + 2 > T.shape[0]:
            T2 = np.zeros((2 * T.shape[0],) * 2, dtype=complex)
            T2[:T.shape[0], :T.shape[0]] = T
            T = T2
        w = np.asarray(action(Q[j].reshape(shape)), dtype=complex).reshape(-1)
        w0 = float(np.linalg.norm(w))
        for _ in range(2):
            for i in range(j + 1):
                h = np.vdot(Q[i], w)
                T[i, j] += h
                w = w - h * Q[i]
        beta = float(np.linalg.norm(w))
        T[j + 1, j] = beta
        m = j + 1
        if beta <= max(floor_abs, 1e-12 * w0):
            break
        if krylov_tol > 0.0:
            col = _small_propagator(T[:m, :m], dt, exp_factor, hermitian)
            if beta0 * beta * abs(col[m - 1]) < krylov_tol:
                break
        Q.append(w / beta)
    if stats is not None:
        stats.append(m)
    c = beta0 * _small_propagator(T[:m, :m], dt, exp_factor, hermitian)
    out = np.zeros(n, dtype=complex)
    for i in range(m):
        out += c[i] * Q[i]
    return out.reshape(shape)


# ----------------------------------------------------------------------------
# update paths
# ----------------------------------------------------------------------------
def dense_exp_action(psi, action, dt, exp_factor):
    """exp(exp_factor dt H) psi with H formed column by column from ``action``
    and exponentiated by ``scipy.linalg.expm`` (the exact modes of
    ``TimeEvoMode``, ``time_evolution.py:621-655``; small tensors only)."""
    import scipy.linalg
    n = psi.size
    H = np.empty((n, n), dtype=complex)
    for i in range(n):
        e = np.zeros(n, dtype=complex)
        e[i] = 1.0
        H[:, i] = np.asarray(action(e.reshape(psi.shape))).reshape(-1)
    return (scipy.linalg.expm(exp_factor * dt * H) @ psi.reshape(-1)).reshape(psi.shape)


def ode_exp_action(psi, action, dt, exp_factor, method="RK45", **options):
    """The ODE modes of ``TimeEvoMode.time_evolve_action``
    (``time_evolution.py:595-615``): ``scipy.integrate.solve_ivp`` on
    y' = exp_factor H y over (0, dt), read at t_eval = [dt]."""
    from scipy.integrate import solve_ivp
    shape = psi.shape

    def rhs(t, y):
        return exp_factor * np.asarray(action(y.reshape(shape))).reshape(-1)
    res = solve_ivp(rhs, (0, dt), np.asarray(psi, dtype=complex).reshape(-1), method=method,
                    t_eval=[dt], **options)
    return res.y[:, 0].reshape(shape)


def _postorder(tree: OTree, nid):
    if tree.is_leaf(nid):
        return [nid]
    out = []
    for c in tree.lchildren[nid]:
        out += _postorder(tree, c)
    return out + [nid]


def leaf_to_root_path(tree: OTree):
    """``TDVPUpdatePathFinder_LeafToRoot.find_path``
    (``time_evolution/time_evo_util/update_path.py:63-254``)."""
    root = tree.root
    dist = tree.distance_to_node(root)
    start = max(dist, key=dist.get)
    main = tree.path_to_root(start)
    path = []
    for origin in main:
        if origin != root:
            path += [x for c in tree.lchildren[origin] if c not in main
                     for x in _postorder(tree, c)] + [origin]
            continue
        if len(tree.lchildren[root]) == 1:
            path += [root]
            continue
        leaves = [nid for nid in tree.nodes if tree.is_leaf(nid) and nid not in path]
        ld = {nid: d for nid, d in dist.items() if nid in leaves}
        last = max(ld, key=ld.get)
        down = list(reversed(tree.path_to_root(last)))
        for o in down:
            if o == root:
                excl = (main[-2], down[1])
                path += [x for c in tree.lchildren[root] if c not in excl
                         for x in _postorder(tree, c)] + [root]
            else:
                path += [x for c in tree.lchildren[o] if c not in down
                         for x in _postorder(tree, c)] + [o]
    return path


def leaf_to_leaf_path(tree: OTree):
    """``TDVPUpdatePathFinder_LeafToLeaf.find_path`` (``update_path.py:255-396``):
    the first pair of leaves at maximal distance (leaves in node order, the
    root counted when it has one neighbour), the path between them, and every
    off-path subtree visited children first just before the main-path node it
    hangs from."""
    leaves = [nid for nid in tree.nodes if tree.is_leaf(nid)]
    if len(tree.lneighbours(tree.root)) == 1:
        leaves.append(tree.root)
    best, pair = -1, (leaves[0], leaves[0])
    for i in range(len(leaves)):
        di = tree.distance_to_node(leaves[i])
        for j in range(i + 1, len(leaves)):
            if di[leaves[j]] > best:
                best, pair = di[leaves[j]], (leaves[i], leaves[j])
    main = tree.path_from_to(*pair)
    visited, path = set(), []

    def sub(nid):
        if nid in visited or nid in main:
            return []
        visited.add(nid)
        out = []
        p = tree.parent[nid]
        if p is not None and p not in main and p not in visited:
            out += sub(p)
        for c in tree.lchildren[nid]:
            if c not in main and c not in visited:
                out += sub(c)
        return out + [nid]
    for origin in main:
        p = tree.parent[origin]
        if p is not None and p not in main and p not in visited:
            path += sub(p)
        for c in tree.lchildren[origin]:
            if c not in main:
                path += sub(c)
        if origin not in visited:
            visited.add(origin)
            path.append(origin)
    return path


def orthogonalisation_paths(tree: OTree, path):
    """``find_orthogonalisation_path`` (``update_path.py:400-421``)."""
    return [tree.path_from_to(path[i], path[i + 1])[1:] for i in range(len(path) - 1)]


# ----------------------------------------------------------------------------
# one-site TDVP drivers
# ----------------------------------------------------------------------------
class _OneSiteBase:
    """Shared machinery of ``TDVPAlgorithm`` / ``OneSiteTDVP``
    (``tdvp_algorithms/tdvp_algorithm.py:58-221``, ``onesitetdvp.py:17-134``)."""

    def __init__(self, state: OState, W: dict, dt: float, krylov_tol=1e-10,
                 max_krylov_dim=None, path_mode: str = "LeafToRoot", exact: bool = False,
                 ode: dict | None = None):
        self.exact = exact
        self.ode = ode
        self.state = state.copy()
        self.W = W
        self.dt = dt
        self.tol = krylov_tol
        self.maxdim = max_krylov_dim
        self.krylov_dims = []
        init_tree = state.tree.copy()
        self.update_path = leaf_to_leaf_path(init_tree) if path_mode == "LeafToLeaf" else leaf_to_root_path(init_tree)
        self.orth_paths = orthogonalisation_paths(init_tree, self.update_path)
        if self.state.orth_center is None:
            canonical_form(self.state, self.update_path[0])
        else:
            move_orth_center(self.state, self.update_path[0])
        self.envs = init_cache_but_one(self.state, W, self.update_path[0])

    def _krylov(self, x, action, factor, exp_factor):
        if self.ode is not None:
            return ode_exp_action(x, action, self.dt * factor, exp_factor, **self.ode)
        if self.exact:
            return dense_exp_action(x, action, self.dt * factor, exp_factor)
        return krylov_exp_action(x, action, self.dt * factor, exp_factor,
                                 krylov_tol=self.tol, max_krylov_dim=self.maxdim,
                                 stats=self.krylov_dims)

    def update_site(self, nid, factor=1.0):
        tree = self.state.tree
        W = self.W[nid]
        act = lambda y: heff_apply(y, tree, nid, W, self.envs)
        self.state.tensors[nid] = self._krylov(self.state.tensors[nid], act, factor, -1j)

    def update_link(self, nid, nxt, factor=1.0):
        assert self.state.orth_center == nid
        tree = self.state.tree
        r = qr_keep_split(self.state, nid, nxt)
        self.envs[(nid, nxt)] = env_update(tree, nid, nxt, self.state.tensors[nid],
                                           self.W[nid], self.envs)
        e_q, e_n = self.envs[(nid, nxt)], self.envs[(nxt, nid)]
        act = lambda y: bond_apply(y, e_q, e_n)
        r = self._krylov(r, act, factor, +1j)
        absorb_r(self.state, r, nid, nxt, link_variant=True)
        self.state.orth_center = nxt

    def move_orth_and_update_cache(self, path):
        if len(path) == 0:
            return
        assert self.state.orth_center == path[0]
        tree = self.state.tree
        for prev, nid in zip(path[:-1], path[1:]):
            move_orth_center(self.state, nid)
            self.envs[(prev, nid)] = env_update(tree, prev, nid, self.state.tensors[prev],
                                                self.W[prev], self.envs)


class FirstOrderOneSiteTDVPOracle(_OneSiteBase):
    """``FirstOrderOneSiteTDVP.run_one_time_step`` (``firstorderonesite.py:23-104``)."""

    def run_one_time_step(self):
        path = self.update_path
        for i, nid in enumerate(path):
            if i == len(path) - 1:
                if len(self.orth_paths) > 0:
                    self.move_orth_and_update_cache(self.orth_paths[-1])
                self.update_site(nid)
                move_orth_center(self.state, path[0])
                self.envs = init_cache_but_one(self.state, self.W, path[0])
            elif i == 0:
                self.update_site(nid)
                self.update_link(nid, self.orth_paths[0][0])
            else:
                self.move_orth_and_update_cache(self.orth_paths[i - 1])
                self.update_site(nid)
                self.update_link(nid, self.orth_paths[i][0])


class SecondOrderOneSiteTDVPOracle(_OneSiteBase):
    """``SecondOrderOneSiteTDVP.run_one_time_step`` (``secondorderonesite.py:60-193``)."""

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        self.back_path = list(reversed(self.update_path))
        tree = self.state.tree
        bo = []
        for i, nid in enumerate(self.back_path[1:-1]):
            bo.append(tree.path_from_to(nid, self.back_path[i + 2])[:-1])
        bo.append([self.back_path[-1]])
        self.back_orth = bo

    def run_one_time_step(self):
        path = self.update_path
        for i, nid in enumerate(path[:-1]):
            if i > 0:
                self.move_orth_and_update_cache(self.orth_paths[i - 1])
            nxt = self.orth_paths[i][0]
            self.update_site(nid, 0.5)
            self.update_link(nid, nxt, 0.5)
        self.update_site(path[-1], 1.0)
        bp = self.back_path
        self.update_link(self.state.orth_center, bp[1], 0.5)
        for i, nid in enumerate(bp[1:-1]):
            idx = i + 1
            self.update_site(nid, 0.5)
            self.move_orth_and_update_cache(self.back_orth[idx - 1])
            self.update_link(self.state.orth_center, bp[idx + 1], 0.5)
        self.update_site(bp[-1], 0.5)


# ----------------------------------------------------------------------------
# fixed-rank BUG (basis update and Galerkin)
# ----------------------------------------------------------------------------
def _split_toward(A, ax):
    """QR of A with leg ``ax`` as the column index: (Q with A's legs, R)."""
    At = np.moveaxis(A, ax, -1)
    k = At.shape[-1]
    q, r = np.linalg.qr(At.reshape(-1, k), mode="reduced")
    if q.shape[1] < k:
        q = np.pad(q, [(0, 0), (0, k - q.shape[1])])
        r = np.pad(r, [(0, k - r.shape[0]), (0, 0)])
    return np.moveaxis(q.reshape(At.shape), -1, ax), r


def _bug_basis(T):
    """New basis of a non-root node: QR of its evolved tensor with the parent
    leg (leg 0) as the column index, KEEP (``compute_fixed_size_new_basis_tensor``,
    ``time_evo_util/bug_util.py:93-121``; leaf: ``common_bug.py:94-101``)."""
    Q, _ = _split_toward(T, 0)
    return Q


def _in_new_child_bases(T, tree, nid, Ms):
    """Contract each child's basis change tensor M_g (old, new) into T's leg
    toward g (``contract_all_children``)."""
    for g in tree.children[nid]:
        a = tree.axis(nid, g)
        T = np.moveaxis(np.tensordot(T, Ms[g], axes=([a], [0])), -1, a)
    return T


def _bug_exp(x, action, dt, setting):
    """exp(-i dt H) x for a BUG node: ``setting`` is a Krylov tolerance, or
    the ``solve_ivp`` arguments (method and options) of an ODE mode."""
    if isinstance(setting, dict):
        return ode_exp_action(x, action, dt, -1j, **setting)
    return krylov_exp_action(x, action, dt, -1j, krylov_tol=setting)


def _bug_update_node(c, P, envs_p, tree, W, dt, tol, child_tol):
    """``update_node`` / ``update_leaf_node`` / ``update_non_leaf_node``
    (``time_evo_util/common_bug.py:47-309``) with fixed rank. ``P`` has its
    orthogonality centre at c's parent and ``envs_p`` all environments toward
    it. Returns (new basis tensors of c's subtree, environment of c toward its
    parent in the new basis, basis change tensor (old, new)). The reference
    passes its solver options only to the root's children; deeper nodes run
    with the defaults (``child_tol``)."""
    p = tree.parent[c]
    Q, R = _split_toward(P[p], tree.axis(p, c))
    cur = dict(P)
    cur[p] = Q
    cur[c] = np.tensordot(R, P[c], axes=([1], [0]))
    envs = dict(envs_p)
    envs[(p, c)] = env_update(tree, p, c, cur[p], W[p], envs)
    envs.pop((c, p), None)
    new, Ms, blocks = {}, {}, {}
    for g in tree.children[c]:
        # every child starts from the environments as they were before any
        # sibling was updated
        sub, blocks[g], Ms[g] = _bug_update_node(g, cur, envs, tree, W, dt, child_tol, child_tol)
        new.update(sub)
    for g, b in blocks.items():
        envs[(g, c)] = b
    x = _in_new_child_bases(cur[c], tree, c, Ms)
    upd = _bug_exp(x, lambda y: heff_apply(y, tree, c, W[c], envs), dt, tol)
    U = _bug_basis(upd)
    old = _in_new_child_bases(P[c], tree, c, Ms)
    legs = list(range(1, U.ndim))
    M = np.tensordot(old, U.conj(), axes=(legs, legs))
    new[c] = U
    return new, env_update(tree, c, p, U, W[c], envs), M


def _split_reduced(A, ax):
    """QR with SplitMode.REDUCED: the bond shrinks to the row count when A is wide."""
    At = np.moveaxis(A, ax, -1)
    k = At.shape[-1]
    q, r = np.linalg.qr(At.reshape(-1, k), mode="reduced")
    return np.moveaxis(q.reshape(At.shape[:-1] + (q.shape[1],)), -1, ax), r


def _move_center(state: OState, target: str, reduced: bool):
    tree = state.tree
    path = tree.path_from_to(state.orth_center, target)
    for a, b in zip(path[:-1], path[1:]):
        split = _split_reduced if reduced else _split_toward
        Q, R = split(state.tensors[a], tree.axis(a, b))
        state.tensors[a] = Q
        ax = tree.axis(b, a)
        state.tensors[b] = np.moveaxis(np.tensordot(R, state.tensors[b], axes=([1], [ax])), 0, ax)
    state.orth_center = target


def svd_truncation(state: OState, params: SVDParams) -> OState:
    """``svd_truncation`` with one-site compressions (``core/truncation/svd_truncation.py``):
    along the leaf-to-leaf path, the centre moves to each non-root node (REDUCED
    QR) and the bond to its parent is cut by a truncated SVD, U staying at the
    node and S V^H going into the parent (``compress_parent_leg``)."""
    tree = state.tree
    path = leaf_to_leaf_path(tree)
    _move_center(state, path[0], reduced=True)
    for nid in path:
        if nid == tree.root:
            continue
        _move_center(state, nid, reduced=True)
        T = state.tensors[nid]
        k = T.shape[0]
        u, s, vh = np.linalg.svd(T.reshape(k, -1).T, full_matrices=False)
        r, new_s = truncate_singular_values(s, params)
        state.tensors[nid] = u[:, :r].T.reshape((r,) + T.shape[1:])
        p = tree.parent[nid]
        ax = tree.axis(p, nid)
        svh = new_s[:, None] * vh[:r]
        state.tensors[p] = np.moveaxis(np.tensordot(svh, state.tensors[p], axes=([1], [ax])), 0, ax)
        state.orth_center = p
    return state


def _adaptive_bug_update_node(c, P, envs_p, tree, W, dt, tol, child_tol):
    """``update_node`` of the rank-adaptive BUG (``common_bug.py:47-309`` with
    ``fixed_rank=False``): REDUCED moves, and the new basis spans the old and
    the evolved tensor (``compute_new_basis_tensor``, ``bug_util.py:123-157``;
    a leaf concatenates its old basis tensor, an inner node its old centre
    tensor in the children's new bases)."""
    p = tree.parent[c]
    Q, R = _split_reduced(P[p], tree.axis(p, c))
    cur = dict(P)
    cur[p] = Q
    cur[c] = np.tensordot(R, P[c], axes=([1], [0]))
    envs = dict(envs_p)
    envs[(p, c)] = env_update(tree, p, c, cur[p], W[p], envs)
    envs.pop((c, p), None)
    new, Ms, blocks = {}, {}, {}
    for g in tree.children[c]:
        sub, blocks[g], Ms[g] = _adaptive_bug_update_node(g, cur, envs, tree, W, dt, child_tol, child_tol)
        new.update(sub)
    for g, b in blocks.items():
        envs[(g, c)] = b
    x = _in_new_child_bases(cur[c], tree, c, Ms)
    upd = krylov_exp_action(x, lambda y: heff_apply(y, tree, c, W[c], envs), dt, -1j, krylov_tol=tol)
    old = _in_new_child_bases(P[c], tree, c, Ms)
    first = old if not tree.children[c] else x
    U, _ = _split_reduced(np.concatenate([first, upd], axis=0), 0)
    legs = list(range(1, U.ndim))
    M = np.tensordot(old, U.conj(), axes=(legs, legs))
    new[c] = U
    return new, env_update(tree, c, p, U, W[c], envs), M


def adaptive_bug_step(state: OState, W: dict, dt: float, svd: SVDParams, krylov_tol=1e-10,
                      default_tol=1e-10) -> OState:
    """One step of the rank-adaptive ``BUG`` (``time_evolution/bug.py:84-117``):
    the augmented-basis root update, then ``svd_truncation`` and the centre
    back at the root."""
    tree = state.tree
    root = tree.root
    assert state.orth_center == root
    envs = init_cache_but_one(state, W, root)
    new, Ms, blocks = {}, {}, {}
    for c in tree.children[root]:
        sub, blocks[c], Ms[c] = _adaptive_bug_update_node(c, state.tensors, envs, tree, W, dt, krylov_tol,
                                                          default_tol)
        new.update(sub)
    for c, b in blocks.items():
        envs[(c, root)] = b
    x = _in_new_child_bases(state.tensors[root], tree, root, Ms)
    new[root] = krylov_exp_action(x, lambda y: heff_apply(y, tree, root, W[root], envs), dt, -1j,
                                  krylov_tol=krylov_tol)
    out = OState(tree, new)
    out.orth_center = root
    svd_truncation(out, svd)
    _move_center(out, root, reduced=False)
    return out


def fixed_bug_step(state: OState, W: dict, dt: float, krylov_tol=1e-10, default_tol=1e-10,
                   ode: dict | None = None) -> OState:
    """One step of ``FixedBUG`` (``time_evolution/fixed_bug.py:83-97``,
    ``root_update`` in ``time_evo_util/common_bug.py:311-378``): every child of
    the root updates its subtree recursively from the current state, then the
    root tensor, expressed in the children's new bases, evolves by dt in the
    new environments. The state must have its orthogonality centre at the root.
    ``ode`` (``solve_ivp`` method and options) selects an ODE mode; nodes below
    the root's children then run it with ``solve_ivp``'s own tolerances."""
    if ode is not None:
        krylov_tol, default_tol = ode, {"method": ode["method"]}
    tree = state.tree
    root = tree.root
    assert state.orth_center == root
    envs = init_cache_but_one(state, W, root)
    new, Ms, blocks = {}, {}, {}
    for c in tree.children[root]:
        sub, blocks[c], Ms[c] = _bug_update_node(c, state.tensors, envs, tree, W, dt, krylov_tol, default_tol)
        new.update(sub)
    for c, b in blocks.items():
        envs[(c, root)] = b
    x = _in_new_child_bases(state.tensors[root], tree, root, Ms)
    new[root] = _bug_exp(x, lambda y: heff_apply(y, tree, root, W[root], envs), dt, krylov_tol)
    out = OState(tree, new)
    out.orth_center = root
    return out


# ----------------------------------------------------------------------------
# zip-up application of a TTNO
# ----------------------------------------------------------------------------
def zipup_apply(state: OState, W: dict, params: SVDParams) -> OState:
    """Non-canonical zip-up (``ttns/ttns_ttno/zipup.py:55-105,191-253``): from
    the leaves up, each node's state tensor, its TTNO tensor and the blocks of
    its children are contracted and split by a truncated SVD, the node keeping
    U (new bond toward the parent) and the parent receiving S V^H with legs
    (state bond, operator bond, new bond); the root keeps everything."""
    tree = state.tree
    order = _postorder(tree, tree.root)
    cache, new = {}, {}
    for v in order:
        nb = tree.neighbours(v)
        n = len(nb)
        T = np.tensordot(state.tensors[v], W[v], axes=([n], [n + 1]))
        legs = [("a", k) for k in range(n)] + [("b", k) for k in range(n)] + ["t"]
        kids = [k for k, x in enumerate(nb) if x != tree.parent[v]]
        for k in kids:
            T = np.tensordot(T, cache.pop(nb[k]), axes=([legs.index(("a", k)), legs.index(("b", k))], [0, 1]))
            legs = [l for l in legs if l not in (("a", k), ("b", k))] + [("n", k)]
        if tree.parent[v] is None:
            new[v] = np.transpose(T, [legs.index(("n", k)) for k in kids] + [legs.index("t")])
            continue
        order_legs = [("n", k) for k in kids] + ["t", ("a", 0), ("b", 0)]
        T = np.transpose(T, [legs.index(l) for l in order_legs])
        rows, cp, wp = T.shape[:-2], T.shape[-2], T.shape[-1]
        u, sv, vh = np.linalg.svd(T.reshape(-1, cp * wp), full_matrices=False)
        r, new_s = truncate_singular_values(sv, params)
        new[v] = np.moveaxis(u[:, :r].reshape(rows + (r,)), -1, 0)
        cache[v] = np.transpose((new_s[:, None] * vh[:r]).reshape(r, cp, wp), (1, 2, 0))
    out = OState(tree, new)
    return out


# ----------------------------------------------------------------------------
# observables and full contractions
# ----------------------------------------------------------------------------
def expect_product(state: OState, ops: dict, bra: OState | None = None) -> complex:
    """<bra| prod_i O_i |ket> for single-site operators (``TTNS.tensor_product_expectation_value``,
    ``ttns/ttns.py:240-264``; bra defaults to the state)."""
    bra = state if bra is None else bra
    tree = state.tree

    def rec(nid, toward):
        A = state.tensors[nid]
        if nid in ops:
            A = np.moveaxis(np.tensordot(ops[nid], A, axes=([1], [A.ndim - 1])), 0, -1)
        nbrs = tree.neighbours(nid)
        T = _L(A, [f"a{k}" for k in range(len(nbrs))] + ["s"])
        for k, nb in enumerate(nbrs):
            if nb != toward:
                T = T.dot(_L(rec(nb, nid), [f"a{k}", f"c{k}"]), [f"a{k}"])
        B = _L(bra.tensors[nid].conj(), [f"c{k}" if nb != toward else "z"
                                          for k, nb in enumerate(nbrs)] + ["s"])
        E = T.dot(B, [f"c{k}" for k, nb in enumerate(nbrs) if nb != toward] + ["s"])
        if toward is None:
            return E.t
        k = nbrs.index(toward)
        return E.out([f"a{k}", "z"])
    return complex(rec(tree.root, None))


def scalar_product(a: OState, b: OState) -> complex:
    """<a|b> (``contract_two_ttns``, ``contractions/state_state_contraction.py:29-66``)."""
    return expect_product(b, {}, bra=a)


def state_vector(state: OState, site_order):
    """Dense state vector with sites in ``site_order`` (small trees only)."""
    tree = state.tree

    def rec(nid, toward):
        A = state.tensors[nid]
        legs = tree.neighbours(nid)
        sites = [nid]
        T = A
        cur = list(legs) + ["#" + nid]
        for nb in legs:
            if nb == toward:
                continue
            sub, subsites = rec(nb, nid)
            ax = cur.index(nb)
            T = np.tensordot(T, sub, axes=([ax], [0]))
            cur = cur[:ax] + cur[ax + 1:] + ["#" + s for s in subsites]
            sites += subsites
        if toward is not None:
            ax = cur.index(toward)
            T = np.moveaxis(T, ax, 0)
            cur = [cur[ax]] + cur[:ax] + cur[ax + 1:]
        return T, [c[1:] for c in cur if c.startswith("#")]
    T, sites = rec(tree.root, None)
    perm = [sites.index(s) for s in site_order]
    return np.transpose(T, perm).reshape(-1)


# ----------------------------------------------------------------------------
# truncated SVD and two-site TDVP
# ----------------------------------------------------------------------------
class SVDParams:
    """Fields of ``SVDParameters`` (``util/tensor_splitting.py:253-328``)."""

    def __init__(self, max_bond_dim=100, rel_tol=1e-15, total_tol=1e-15, renorm=False,
                 sum_trunc=False, sum_renorm=False):
        self.max_bond_dim = max_bond_dim
        self.rel_tol = rel_tol
        self.total_tol = total_tol
        self.renorm = renorm
        self.sum_trunc = sum_trunc
        self.sum_renorm = sum_renorm


def truncate_singular_values(s, p: SVDParams):
    """Number of singular values kept and their (possibly renormalised) values
    (``truncate_singular_values``, ``value_truncation``, ``_sum_truncation_index``,
    ``renormalise_singular_values``; ``util/tensor_splitting.py:330-486``).
    ``s`` is sorted in descending order."""
    s = np.asarray(s, dtype=float)
    if len(s) == 0:
        raise ValueError("No singular values to truncate!")
    if p.sum_trunc:
        normsq = float(np.linalg.norm(s)) ** 2
        keep = 0
        if normsq != 0.0:
            acc = 0.0
            for i, v in enumerate(s[::-1]):
                acc += v * v
                if (acc / normsq if p.sum_renorm else acc) > p.total_tol ** 2:
                    keep = len(s) - i
                    break
    else:
        cut = max(p.rel_tol * s[0], p.total_tol)
        keep = int(np.count_nonzero(s > cut))
    keep = min(keep, p.max_bond_dim)
    if keep == 0:
        keep = 1
    new_s = s[:keep].copy()
    if p.renorm:
        new_s = new_s * np.linalg.norm(s) / np.linalg.norm(new_s)
    return keep, new_s


def two_site_merge(state: OState, u: str, v: str):
    """Contract the tensors of neighbours ``u`` and ``v`` (``contract_nodes``,
    ``contractions/node_contraction.py:12-141``). Returns the merged tensor
    with legs (u's other neighbours in physical order, s_u, v's other
    neighbours in physical order, s_v) and the two neighbour lists."""
    tree = state.tree
    nu = [x for x in tree.neighbours(u) if x != v]
    nv = [x for x in tree.neighbours(v) if x != u]
    A = _L(state.tensors[u], [f"u:{x}" if x != v else "bond" for x in tree.neighbours(u)] + ["su"])
    B = _L(state.tensors[v], [f"v:{x}" if x != u else "bond" for x in tree.neighbours(v)] + ["sv"])
    T = A.dot(B, ["bond"])
    return T.out([f"u:{x}" for x in nu] + ["su"] + [f"v:{x}" for x in nv] + ["sv"]), nu, nv


# Largest intermediate (elements) for which the two-site H_eff follows the
# reference's contraction order.
TWO_SITE_REFERENCE_ORDER_MAX = 10 ** 8


def two_site_heff_apply(x, nu, nv, u, v, Wu, Wv, tree: OTree, envs):
    """H_eff of the merged pair applied to ``x`` (legs as ``two_site_merge``)
    (``effective_two_site_evolution``, ``time_evo_util/effective_time_evolution.py:326-410``:
    the two TTNO tensors joined over their shared bond, then the single-site
    contraction of ``contract_ket_ham_with_envs``)."""
    lab_x = [f"au{k}" for k in range(len(nu))] + ["su"] + [f"av{k}" for k in range(len(nv))] + ["sv"]
    T = _L(x, lab_x)
    wl_u = [f"bu{nu.index(y)}" if y != v else "bw" for y in tree.neighbours(u)] + ["tu", "su"]
    wl_v = [f"bv{nv.index(y)}" if y != u else "bw" for y in tree.neighbours(v)] + ["tv", "sv"]
    wu = [envs[(nb, u)].shape[1] for nb in nu]
    wv = [envs[(nb, v)].shape[1] for nb in nv]
    w_bw = Wu.shape[tree.neighbours(u).index(v)]
    peak = x.size * max(int(np.prod(wu)), w_bw * int(np.prod(wv)))
    if peak <= TWO_SITE_REFERENCE_ORDER_MAX:
        # the reference's order: every environment of a side, then its TTNO tensor
        for k, nb in enumerate(nu):
            T = T.dot(_L(envs[(nb, u)], [f"au{k}", f"bu{k}", f"cu{k}"]), [f"au{k}"])
        T = T.dot(_L(Wu, wl_u), [f"bu{k}" for k in range(len(nu))] + ["su"])
        for k, nb in enumerate(nv):
            T = T.dot(_L(envs[(nb, v)], [f"av{k}", f"bv{k}", f"cv{k}"]), [f"av{k}"])
        T = T.dot(_L(Wv, wl_v), [f"bv{k}" for k in range(len(nv))] + ["bw", "sv"])
    else:
        # too large for that order (the TTNO bond legs of a whole side pile
        # up): each side in the single-site order instead (half of its
        # environments, its TTNO tensor, the rest) -- the same sum
        hu = len(nu) // 2
        for k in range(hu):
            T = T.dot(_L(envs[(nu[k], u)], [f"au{k}", f"bu{k}", f"cu{k}"]), [f"au{k}"])
        T = T.dot(_L(Wu, wl_u), [f"bu{k}" for k in range(hu)] + ["su"])
        for k in range(hu, len(nu)):
            T = T.dot(_L(envs[(nu[k], u)], [f"au{k}", f"bu{k}", f"cu{k}"]), [f"au{k}", f"bu{k}"])
        hv = len(nv) // 2
        for k in range(hv):
            T = T.dot(_L(envs[(nv[k], v)], [f"av{k}", f"bv{k}", f"cv{k}"]), [f"av{k}"])
        T = T.dot(_L(Wv, wl_v), [f"bv{k}" for k in range(hv)] + ["bw", "sv"])
        for k in range(hv, len(nv)):
            T = T.dot(_L(envs[(nv[k], v)], [f"av{k}", f"bv{k}", f"cv{k}"]), [f"av{k}", f"bv{k}"])
    return T.out([f"cu{k}" for k in range(len(nu))] + ["tu"] + [f"cv{k}" for k in range(len(nv))] + ["tv"])


def two_site_split(state: OState, merged, nu, nv, u: str, v: str, params: SVDParams):
    """Truncated SVD split of the merged pair; singular values go to ``v``
    (``split_node_svd`` -> ``contr_truncated_svd_splitting`` with VCONTR,
    ``core/ttn.py:1476-1497``, ``util/tensor_splitting.py:488-572``).
    Rows are matricised in the reference's order (parent, logical children,
    physical) on each side. Logical order afterwards: the node that gains a
    child through the split lists it first (``core/ttn.py:1400-1448``).
    Returns the kept singular values."""
    tree = state.tree

    def side(node, other, nbrs):
        p = tree.parent[node]
        order = ([p] if (p is not None and p != other) else []) + [c for c in tree.lchildren[node] if c != other]
        return [nbrs.index(x) for x in order]
    iu = side(u, v, nu)
    iv = side(v, u, nv)
    nuu = len(nu)
    row_axes = iu + [nuu]
    col_axes = [nuu + 1 + i for i in iv] + [nuu + 1 + len(nv)]
    mat = np.transpose(merged, row_axes + col_axes)
    rshape = mat.shape[:len(row_axes)]
    cshape = mat.shape[len(row_axes):]
    mat = mat.reshape(int(np.prod(rshape)), int(np.prod(cshape)))
    U, s, Vh = np.linalg.svd(mat, full_matrices=False)
    r, new_s = truncate_singular_values(s, params)
    U = U[:, :r].reshape(list(rshape) + [r])
    SV = (new_s[:, None] * Vh[:r, :]).reshape([r] + list(cshape))
    # U legs: (u's row legs in reference order, bond) -> u's physical layout
    labels_u = [nu[i] for i in iu] + ["#phys", v]
    tgt_u = tree.neighbours(u) + ["#phys"]
    state.tensors[u] = np.ascontiguousarray(np.transpose(U, [labels_u.index(x) for x in tgt_u]))
    labels_v = [u] + [nv[i] for i in iv] + ["#phys"]
    tgt_v = tree.neighbours(v) + ["#phys"]
    state.tensors[v] = np.ascontiguousarray(np.transpose(SV, [labels_v.index(x) for x in tgt_v]))
    if tree.parent[v] == u:
        tree.lchildren[u] = [v] + [c for c in tree.lchildren[u] if c != v]
    else:
        tree.lchildren[v] = [u] + [c for c in tree.lchildren[v] if c != u]
    return new_s


class _TwoSiteBase(_OneSiteBase):
    """``TwoSiteTDVP`` (``tdvp_algorithms/twositetdvp.py:29-146``)."""

    def __init__(self, state: OState, W: dict, dt: float, svd: SVDParams, krylov_tol=1e-10,
                 max_krylov_dim=None, path_mode: str = "LeafToRoot", ode: dict | None = None,
                 exact: bool = False):
        super().__init__(state, W, dt, krylov_tol, max_krylov_dim, path_mode=path_mode, ode=ode, exact=exact)
        self.svd = svd
        self.bond_history = []

    def update_two_sites(self, u, v, factor=1.0):
        """``_update_two_site_nodes`` (``twositetdvp.py:89-125``)."""
        assert self.state.orth_center == u
        tree = self.state.tree
        x, nu, nv = two_site_merge(self.state, u, v)
        act = lambda y: two_site_heff_apply(y, nu, nv, u, v, self.W[u], self.W[v], tree, self.envs)
        x = self._krylov(x, act, factor, -1j)
        s = two_site_split(self.state, x, nu, nv, u, v, self.svd)
        self.bond_history.append(len(s))
        self.state.orth_center = v
        self.envs[(u, v)] = env_update(tree, u, v, self.state.tensors[u], self.W[u], self.envs)

    def backward_site(self, nid, factor=1.0):
        """``_single_site_backwards_update`` (``twositetdvp.py:127-138``)."""
        self.update_site(nid, -factor)


class SecondOrderTwoSiteTDVPOracle(_TwoSiteBase):
    """``SecondOrderTwoSiteTDVP.run_one_time_step`` (``secondordertwosite.py:55-193``)."""

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        self.back_path = list(reversed(self.update_path))
        self.back_orth = [list(reversed(p)) for p in reversed(self.orth_paths)]

    def run_one_time_step(self):
        path, orth = self.update_path, self.orth_paths
        for i, nid in enumerate(path[:-2]):
            if i > 0:
                self.move_orth_and_update_cache(orth[i - 1])
            nxt = orth[i][0]
            self.update_two_sites(nid, nxt, 0.5)
            self.backward_site(nxt, 0.5)
        self.update_two_sites(path[-2], path[-1], 0.5)
        bp = self.back_path
        for i in range(len(bp) - 1):
            if i == 0:
                self.update_two_sites(bp[0], bp[1], 0.5)
                continue
            op = self.back_orth[i]
            self.move_orth_and_update_cache(op)
            tgt = op[-1]
            self.backward_site(tgt, 0.5)
            self.update_two_sites(tgt, bp[i + 1], 0.5)


class FirstOrderTwoSiteTDVPOracle(_TwoSiteBase):
    """``FirstOrderTwoSiteTDVP.run_one_time_step`` (``firstordertwosite.py:11-30``) as
    intended: the partner of update-path node i is the first node of the
    i-th orthogonalisation sub-path, and the environments are rebuilt after
    the centre returns to the start (as ``firstorderonesite.py:66-75`` does).
    The reference indexes sub-path i+1 and raises ValueError on the second
    pair of any tree with a branching root."""

    def run_one_time_step(self):
        path, orth = self.update_path, self.orth_paths
        for i, nid in enumerate(path[:-2]):
            nxt = orth[i][0]
            self.update_two_sites(nid, nxt)
            self.backward_site(nxt)
            self.move_orth_and_update_cache(orth[i])
        self.update_two_sites(path[-2], path[-1])
        move_orth_center(self.state, path[0])
        self.envs = init_cache_but_one(self.state, self.W, path[0])


# ----------------------------------------------------------------------------
# TEBD
# ----------------------------------------------------------------------------
def tebd_apply_gate(state: OState, op, ids, params: SVDParams):
    """One exponentiated Trotter operator (``TEBD._apply_one_trotter_step``,
    ``time_evolution/tebd.py:84-155``): a one-site gate is absorbed into the
    physical leg (``absorb_into_open_legs``, ``core/ttn.py:929-964``); a two-site
    gate (legs out_1, out_2, in_1, in_2 for ids = (u, v)) acts on the merged
    pair, which is split again by the truncated SVD with the singular values
    moved into v."""
    op = np.asarray(op)
    if len(ids) == 1:
        A = state.tensors[ids[0]]
        state.tensors[ids[0]] = np.moveaxis(np.tensordot(op, A, axes=([1], [A.ndim - 1])), 0, -1)
        return None
    if len(ids) != 2:
        raise NotImplementedError("More than two-site interactions are not implemented.")
    u, v = ids
    x, nu, nv = two_site_merge(state, u, v)
    iu, iv = len(nu), x.ndim - 1
    y = np.tensordot(x, op, axes=([iu, iv], [2, 3]))          # (nu..., nv..., gu, gv)
    y = np.moveaxis(y, [y.ndim - 2, y.ndim - 1], [iu, y.ndim - 1])
    return two_site_split(state, y, nu, nv, u, v, params)


class TEBDOracle:
    """``TEBD.run_one_time_step`` (``time_evolution/tebd.py:84-155``): every
    exponentiated Trotter operator applied once, in order."""

    def __init__(self, state: OState, gates, params: SVDParams):
        self.state = state.copy()
        self.gates = list(gates)
        self.params = params

    def run_one_time_step(self):
        for op, ids in self.gates:
            tebd_apply_gate(self.state, op, ids, self.params)


def ttno_expectation(state: OState, W: dict) -> complex:
    """<psi| H |psi> for a TTNO (``TTNS.ttno_expectation_value`` through
    ``expectation_value``, ``contractions/state_operator_contraction.py:26-74``):
    every environment toward the root, then the root's H_eff applied to the
    root tensor and contracted with its conjugate."""
    root = state.tree.root
    envs = init_cache_but_one(state, W, root)
    x = state.tensors[root]
    y = heff_apply(x, state.tree, root, W[root], envs)
    return complex(np.vdot(x.reshape(-1), y.reshape(-1)))
