"""PyTreeNet's contraction helpers on the GPU engine.

Drop-in counterparts of the helpers a PyTreeNet user composes into custom
algorithms: ``SandwichCache`` (``contractions/sandwich_caching.py:14-126``),
``contract_ket_ham_with_envs`` (``contractions/state_operator_contraction.py:227-273``),
``contract_any`` (``:407-461``), ``effective_single_site_evolution``
(``time_evolution/time_evo_util/effective_time_evolution.py:257-324``) and the
dense ``get_effective_single_site_hamiltonian(_nodes)``
(``contractions/effective_hamiltonians.py:109-157``). Tensors
come and go as NumPy arrays in the reference's leg conventions: a site tensor
in its node's logical leg order (parent, children, physical), a cache entry
E(node -> next) with legs (ket, ham, bra). The environments themselves stay on
the device inside the cache; the contractions run through the same plans as
the drivers.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import CDT, DeviceNetwork
from .tdvp import EvoDirection, TimeEvoMode


class SandwichCache:
    """Environments of a TTNO sandwiched between a TTNS and its conjugate,
    one device buffer per directed edge (``sandwich_caching.py:14-126``)."""

    def __init__(self, state, hamiltonian, precision: str = "plain"):
        self.state = state
        self.hamiltonian = hamiltonian
        self.net = DeviceNetwork(state, hamiltonian, precision=precision)
        self._valid: set = set()

    @classmethod
    def init_cache_but_one(cls, state, hamiltonian, node_id: str, precision: str = "plain") -> "SandwichCache":
        """Every environment pointing toward ``node_id`` (``sandwich_caching.py:97-126``)."""
        cache = cls(state, hamiltonian, precision=precision)
        cache.net.init_cache_but_one(node_id)

        def rec(nid, toward):
            for nb in cache.net.nbrs(nid):
                if nb != toward:
                    rec(nb, nid)
            if toward is not None:
                cache._valid.add((nid, toward))
        rec(node_id, None)
        return cache

    @classmethod
    def of_network(cls, net: DeviceNetwork, hamiltonian=None) -> "SandwichCache":
        """The environments a driver's device network holds, as a cache (the
        drivers' ``partial_tree_cache``); no buffers are copied."""
        cache = cls.__new__(cls)
        cache.state = net.state
        cache.hamiltonian = hamiltonian
        cache.net = net
        cache._valid = None
        return cache

    def update_tree_cache(self, node_id: str, next_node_id: str):
        """Recompute E(node_id -> next_node_id) from the current tensors
        (``sandwich_caching.py:79-95``)."""
        self.net.update_env(node_id, next_node_id)
        if self._valid is not None:
            self._valid.add((node_id, next_node_id))

    def __contains__(self, key) -> bool:
        if self._valid is None:
            return tuple(key) in self.net.env
        return tuple(key) in self._valid

    def get_entry(self, node_id: str, next_node_id: str) -> np.ndarray:
        """E(node_id -> next_node_id) as a NumPy array with legs (ket, ham, bra)."""
        if (node_id, next_node_id) not in self:
            raise KeyError(f"no cached environment from {node_id} to {next_node_id}")
        return self.net.env_buf(node_id, next_node_id).detach().cpu().numpy()


def _to_phys(state, nid, tensor) -> np.ndarray:
    inv = np.argsort(state.logical_perm(nid))
    return np.ascontiguousarray(np.transpose(np.asarray(tensor, dtype=np.complex128), inv))


def _from_phys(state, nid, tensor) -> np.ndarray:
    return np.transpose(tensor, state.logical_perm(nid))


def _node_id(node) -> str:
    return node if isinstance(node, str) else node.identifier


def contract_ket_ham_with_envs(ket_node, ket_tensor, ham_node, ham_tensor, dictionary: SandwichCache) -> np.ndarray:
    """H_eff applied to ``ket_tensor`` with the cached environments of all the
    node's neighbours (``state_operator_contraction.py:227-273``). The TTNO
    tensor is the cache's; the result has the ket tensor's leg order."""
    nid = _node_id(ket_node)
    net = dictionary.net
    st = dictionary.state
    x = torch.from_numpy(_to_phys(st, nid, ket_tensor)).to(net.device, CDT)
    if list(x.shape) != net.shape(nid):
        raise ValueError(f"tensor shape {tuple(x.shape)} does not match node {nid} {tuple(net.shape(nid))}")
    y = torch.empty_like(x)
    net.heff_plan(nid).run(x.data_ptr(), y.data_ptr())
    return _from_phys(st, nid, y.cpu().numpy())


def contract_any(node_id: str, next_node_id: str, state, operator, dictionary: SandwichCache,
                 bra_state=None, bra_state_conjugated: bool = True, id_trafo_op=None, id_trafo_bra=None) -> np.ndarray:
    """E(node_id -> next_node_id) from the node's current tensor and the cached
    environments of its other neighbours (``state_operator_contraction.py:407-461``),
    legs (ket, ham, bra). The bra is the conjugate of the ket state; other bras
    and identifier transformations are not provided."""
    if bra_state is not None or id_trafo_op is not None or id_trafo_bra is not None or not bra_state_conjugated:
        raise NotImplementedError("contract_any on the GPU engine sandwiches the state with its own conjugate")
    dictionary.update_tree_cache(node_id, next_node_id)
    return dictionary.get_entry(node_id, next_node_id)


def effective_single_site_evolution(state_tensor, state_node, hamiltonian_tensor, hamiltonian_node,
                                    time_step_size: float, tensor_cache: SandwichCache,
                                    mode: TimeEvoMode = TimeEvoMode.FASTEST,
                                    forward: EvoDirection = EvoDirection.FORWARD, **options) -> np.ndarray:
    """exp(-i dt H_eff) applied to ``state_tensor`` (``effective_time_evolution.py:257-324``):
    the matrix-free Krylov exponential (options ``krylov_tol``, ``max_krylov_dim``,
    ``hermitian``; the exact modes run it to machine precision), or for RK45,
    RK23 and DOP853 the adaptive Runge-Kutta integration with ``solve_ivp``'s
    options. ``forward`` gives the sign of the exponent as in the reference;
    ``exp_factor`` replaces the forward factor -i (backward: its negation)."""
    from .tdvp import check_time_evo_mode, ode_options
    options = check_time_evo_mode(mode, options, tensor_cache.net.precision)
    nid = _node_id(state_node)
    net = tensor_cache.net
    st = tensor_cache.state
    x = torch.from_numpy(_to_phys(st, nid, state_tensor)).to(net.device, CDT)
    if list(x.shape) != net.shape(nid):
        raise ValueError(f"tensor shape {tuple(x.shape)} does not match node {nid} {tuple(net.shape(nid))}")
    p = net.heff_plan(nid)
    is_forward = forward is EvoDirection.FORWARD if isinstance(forward, EvoDirection) else bool(forward)
    override = options.get("exp_factor")
    if override is None:
        exp_factor = -1j if is_forward else 1j
    else:
        exp_factor = override if is_forward else -override

    def apply(xp, yp):
        p.run(xp, yp)
    out = torch.empty_like(x)
    ode = ode_options(mode, options)
    if ode is not None:
        from .ode import RungeKuttaSolver
        RungeKuttaSolver(net.ws).integrate(x, apply, time_step_size, exp_factor, out=out, **ode)
    else:
        net.krylov.expm(x, apply, time_step_size, exp_factor, options.get("krylov_tol", 1e-10),
                        options.get("max_krylov_dim"), hermitian=options.get("hermitian", True), out=out,
                        tridiagonal=net.levels > 0)
    return _from_phys(st, nid, out.cpu().numpy())


def _dense_site_hamiltonian(cache: SandwichCache, nid: str, W=None) -> np.ndarray:
    from .adjoint import site_apply
    net = cache.net
    shape = net.shape(nid)
    N = int(np.prod(shape))
    eye = torch.eye(N, dtype=CDT, device=net.device).reshape([N] + shape)
    envs = [net.env_buf(x, nid) for x in net.nbrs(nid)]
    Y = site_apply(eye, envs, net.W[nid] if W is None else W, batch=True)
    H_phys = Y.reshape(N, N).transpose(0, 1).cpu().numpy()      # column r = H e_r
    P = np.arange(N).reshape(shape).transpose(cache.state.logical_perm(nid)).reshape(-1)
    return H_phys[np.ix_(P, P)]


def get_effective_single_site_hamiltonian(node_id: str, state, hamiltonian, tensor_cache: SandwichCache) -> np.ndarray:
    """H_eff of a site as an N x N matrix acting on the site tensor flattened in
    its leg order (``get_effective_single_site_hamiltonian``,
    ``contractions/effective_hamiltonians.py:133-157``). The matrix is built on
    the device by applying the matvec chain to the N unit vectors at once;
    meant for small sites, as in the reference."""
    return _dense_site_hamiltonian(tensor_cache, node_id)


def get_effective_single_site_hamiltonian_nodes(state_node, hamiltonian_node, hamiltonian_tensor,
                                                tensor_cache: SandwichCache) -> np.ndarray:
    """As :func:`get_effective_single_site_hamiltonian`, with the TTNO tensor given
    in ``hamiltonian_node``'s leg order (``effective_hamiltonians.py:109-131``)."""
    nid = _node_id(state_node)
    W = None
    if hamiltonian_tensor is not None:
        net = tensor_cache.net
        order = tensor_cache.state.nodes[nid].phys_neighbours()
        hn = hamiltonian_node.neighbouring_nodes()
        n = len(hn)
        perm = [hn.index(x) for x in order] + [n, n + 1]
        Wn = np.transpose(np.asarray(hamiltonian_tensor, dtype=np.complex128), perm)
        W = torch.from_numpy(np.ascontiguousarray(Wn)).to(net.device)
    return _dense_site_hamiltonian(tensor_cache, nid, W)


# ----------------------------------------------------------------------------
# bond pieces with a plain environment dictionary
# ----------------------------------------------------------------------------
class PartialTreeCachDict(dict):
    """Environment tensors keyed by (node, next node), legs (ket, ham, bra)
    (``contractions/tree_cach_dict.py:16-150``); values may be NumPy arrays
    or device tensors."""

    def get_entry(self, node_id: str, next_node_id: str):
        return self[(node_id, next_node_id)]

    def add_entry(self, node_id: str, next_node_id: str, tensor):
        self[(node_id, next_node_id)] = tensor

    def delete_entry(self, node_id: str, next_node_id: str):
        del self[(node_id, next_node_id)]

    def contains(self, node_id: str, next_node_id: str) -> bool:
        return (node_id, next_node_id) in self

    def change_next_id_for_entry(self, node_id: str, old_next_id: str, new_next_id: str):
        self[(node_id, new_next_id)] = self.pop((node_id, old_next_id))

    def num_legs(self, node_id: str, next_node_id: str) -> int:
        return len(self[(node_id, next_node_id)].shape)

    def copy(self) -> "PartialTreeCachDict":
        return PartialTreeCachDict(self)

    def close_to(self, other: "PartialTreeCachDict") -> bool:
        if set(self) != set(other):
            return False
        return all(np.allclose(np.asarray(_host(self[k])), np.asarray(_host(other[k]))) for k in self)


def _host(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else t


def _dev(t) -> torch.Tensor:
    from . import engine as E
    if isinstance(t, torch.Tensor):
        return t.to(E.DEFAULT_DEVICE if t.device.type == "cpu" else t.device, CDT).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(t, dtype=np.complex128))).to(E.DEFAULT_DEVICE)


def _bond_envs(state_node, tensor_cache):
    """(E_parent, E_child) of a bond node: the parent's environment toward the
    child and the child's toward the parent."""
    parent = state_node.parent
    children = list(state_node.children)
    if parent is None or len(children) != 1:
        raise ValueError("The node must have exactly two neighbours (a parent and one child) "
                         "to represent a bond!")
    return tensor_cache.get_entry(parent, children[0]), tensor_cache.get_entry(children[0], parent)


def _bond_apply(r: torch.Tensor, ep: torch.Tensor, ec: torch.Tensor, out: torch.Tensor | None = None):
    from .adjoint import _raw_contract
    t = _raw_contract(ep, ["a", "b", "p"], r, ["a", "c"], ["b", "p", "c"], ["a"])
    return _raw_contract(t, ["b", "p", "c"], ec, ["c", "b", "q"], ["p", "q"], ["b", "c"], out=out)


def contract_bond_tensor(tensor, state_node, tensor_cache) -> np.ndarray:
    """H_eff applied to a bond tensor (legs: parent side, child side)
    (``contract_bond_tensor``, ``state_operator_contraction.py:984-1040``):
    y[a', c'] = sum E_p[a, b, a'] x[a, c] E_c[c, b, c'], two device contractions."""
    ep, ec = _bond_envs(state_node, tensor_cache)
    y = _bond_apply(_dev(tensor), _dev(ep), _dev(ec))
    return y if isinstance(tensor, torch.Tensor) else y.cpu().numpy()


def get_effective_bond_hamiltonian_tensor(state_node, tensor_cache) -> np.ndarray:
    """H[a', c', a, c] = sum_b E_p[a, b, a'] E_c[c, b, c']
    (``effective_hamiltonians.py:159-206``), one device contraction."""
    from .adjoint import _raw_contract
    ep, ec = _bond_envs(state_node, tensor_cache)
    h = _raw_contract(_dev(ep), ["a", "b", "p"], _dev(ec), ["c", "b", "q"], ["p", "q", "a", "c"], ["b"])
    return h.cpu().numpy()


def get_effective_bond_hamiltonian_nodes(state_node, tensor_cache) -> np.ndarray:
    """The bond Hamiltonian as a matrix (output legs rows, input legs columns)."""
    h = get_effective_bond_hamiltonian_tensor(state_node, tensor_cache)
    d = h.shape[0] * h.shape[1]
    return h.reshape(d, d)


def get_effective_bond_hamiltonian(bond_node_id: str, state, tensor_cache) -> np.ndarray:
    return get_effective_bond_hamiltonian_nodes(state.nodes[bond_node_id], tensor_cache)


def effective_bond_evolution(state_tensor, state_node, time_step_size: float, tensor_cache,
                             mode: TimeEvoMode = TimeEvoMode.FASTEST,
                             forward: EvoDirection = EvoDirection.FORWARD, **options) -> np.ndarray:
    """A bond tensor evolved by its effective Hamiltonian
    (``effective_time_evolution.py:205-255``): the action modes (KRYLOV, the
    solve_ivp modes) apply the bond matvec on the device; the exact modes
    evolve by the dense bond Hamiltonian, on the device as well."""
    ep, ec = _bond_envs(state_node, tensor_cache)
    ep, ec = _dev(ep), _dev(ec)
    x = _dev(state_tensor)
    if mode.action_evolvable():
        def action(t, y):
            return _bond_apply(y, ep, ec)
        out = mode.time_evolve_action(x, action, time_step_size, forward=forward, **options)
    else:
        h = get_effective_bond_hamiltonian_nodes(state_node, tensor_cache)
        out = mode.time_evolve(x, h, time_step_size, forward=forward, **options)
    return out if isinstance(state_tensor, torch.Tensor) else out.cpu().numpy()


def bond_time_evolution(node_id: str, state, time_step_size: float, tensor_cache,
                        forward: EvoDirection = EvoDirection.FORWARD, mode: TimeEvoMode = TimeEvoMode.FASTEST,
                        solver_options: dict | None = None) -> np.ndarray:
    """``bond_time_evolution`` (``effective_time_evolution.py:28-68``)."""
    node = state.nodes[node_id]
    return effective_bond_evolution(state.tensors[node_id], node, time_step_size, tensor_cache, mode=mode,
                                    forward=forward, **(solver_options or {}))


def single_site_time_evolution(node_id: str, state, hamiltonian, time_step_size: float,
                               tensor_cache: SandwichCache, forward: EvoDirection = EvoDirection.FORWARD,
                               mode: TimeEvoMode = TimeEvoMode.FASTEST,
                               solver_options: dict | None = None) -> np.ndarray:
    """``single_site_time_evolution`` (``effective_time_evolution.py:70-115``):
    the node's tensor evolved by its effective Hamiltonian with the cache's
    environments."""
    return effective_single_site_evolution(state.tensors[node_id], state.nodes[node_id], None,
                                           hamiltonian.nodes[node_id], time_step_size, tensor_cache,
                                           mode=mode, forward=forward, **(solver_options or {}))
