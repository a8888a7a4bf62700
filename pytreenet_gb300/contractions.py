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
                                    mode: TimeEvoMode = TimeEvoMode.KRYLOV,
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
