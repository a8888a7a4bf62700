"""Fixed-rank BUG (basis update and Galerkin) on the GPU engine.

``FixedBUG`` (``time_evolution/fixed_bug.py:21-97``) with the recursion of
``time_evo_util/common_bug.py:47-378``: starting from a state whose
orthogonality centre is the root, each child of the root updates its subtree
recursively -- the centre moves into the child (QR of the parent toward it,
R absorbed), the child's own children update first, the child's tensor is
expressed in their new bases and evolved by exp(-i dt H_eff), and the QR of
the result (rows: children and physical leg, column: parent leg, bond kept)
is the child's new basis; the basis change tensor <old|new> and the child's
environment in the new basis go back to the parent. Last, the root tensor in
its children's new bases evolves by dt. Siblings all start from the
environments as they were before any of them was updated.

Every contraction is ``ptn_zcontract``, every QR ``ptn_zqr_keep``, every
local exponential the engine's Krylov solver; tensors keep the engine's
physical leg layout, so the reference's basis-change nodes become
contractions on a leg in place. As in the reference, the solver options
reach the root and its children only; deeper nodes use the default Krylov
tolerance 1e-10 (an ODE mode there runs at ``solve_ivp``'s own tolerances).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import ctypes

import torch

from . import _lib
from . import engine as E
from .adjoint import (_SiteOp, _raw_contract, _solver, _tensor_apply, absorb, env_apply, qr_keep_raw)
from .engine import CDT, DeviceNetwork, check
from .ode import RungeKuttaSolver
from .tdvp import (TTNTimeEvolutionConfig, TimeEvoMode, _tensor_copy, check_time_evo_mode,
                   compute_num_time_steps, ode_options)
from .results import RunLoop, init_operators
from .svd_truncation import TreeOps, move_center, qr_split, truncate_tensors
from .truncation import SVDParameters

DEFAULT_KRYLOV_TOL = 1e-10


@dataclass
class CommonBUGConfig(TTNTimeEvolutionConfig):
    """``time_evo_util/common_bug.py:32-45``."""
    deep: bool = False
    fixed_rank: bool = False
    time_evo_mode: TimeEvoMode = TimeEvoMode.FASTEST


@dataclass
class FixedBUGConfig(CommonBUGConfig):
    """``fixed_bug.py:12-19``."""

    def __post_init__(self):
        self.fixed_rank = True


@dataclass
class BUGConfig(CommonBUGConfig, SVDParameters):
    """``bug.py:15-27``: the BUG options and the truncation of ``svd_truncation``."""

    def __post_init__(self):
        SVDParameters.__post_init__(self)
        assert self.fixed_rank is False, "Fixed rank is not supported for BUG!"


def small_svd(R: torch.Tensor):
    """Jacobi SVD (``ptn_zsvd_jacobi``) of a k x k device matrix: returns U and V
    as k x k tensors whose row j holds column j (U = Ut^T, V = Vt^T) and S on
    the host, with R = U diag(S) V^H."""
    lib = _lib.load()
    k = R.shape[0]
    R = R.contiguous()
    Ut = torch.empty((k, k), dtype=CDT, device=R.device)
    Vt = torch.empty((k, k), dtype=CDT, device=R.device)
    Sb = torch.zeros((k + 2,), dtype=torch.float64, device=R.device)
    work = torch.empty(((int(lib.ptn_zsvd_work_bytes(k, k)) + 15) // 16,), dtype=CDT, device=R.device)
    d = _lib.SvdDesc()
    d.A, d.m, d.n, d.row_stride, d.col_stride = R.data_ptr(), k, k, k, 1
    d.U, d.ldu, d.S, d.V, d.ldv = Ut.data_ptr(), k, Sb.data_ptr(), Vt.data_ptr(), k
    d.work = work.data_ptr()
    d.status = Sb[k:].data_ptr()
    check(lib.ptn_zsvd_jacobi(ctypes.byref(d), E._stream_ptr()), "ptn_zsvd_jacobi")
    host = Sb.cpu()
    code = int(host[k:k + 1].view(torch.int32)[0])
    if code != 0:
        raise _lib.PtnError(code, "Jacobi SVD")
    return Ut, Vt, host[:k].numpy().copy()


class FixedBUG(RunLoop):
    """Fixed-rank BUG driver with PyTreeNet's constructor and stepping API."""

    config_class = FixedBUGConfig

    def __init__(self, initial_state, hamiltonian, time_step_size: float, final_time: float, operators,
                 config: FixedBUGConfig | None = None, solver_options: dict[str, Any] | None = None):
        if time_step_size <= 0 or final_time <= 0:
            raise ValueError("time step and final time must be positive")
        self.config = config if config is not None else self.config_class()
        self.solver_options = check_time_evo_mode(self.config.time_evo_mode, solver_options)
        # the reference hands its options to the root and its children only;
        # deeper nodes run the mode's defaults (the exact modes need no options)
        mode = self.config.time_evo_mode
        exact = mode.is_exact()
        # local solver settings (Krylov stop, Krylov dimension cap, ODE options)
        self._top = (self.solver_options.get("krylov_tol", DEFAULT_KRYLOV_TOL),
                     self.solver_options.get("max_krylov_dim"), ode_options(mode, self.solver_options))
        self._deep = (self.solver_options["krylov_tol"] if exact else DEFAULT_KRYLOV_TOL,
                      self.solver_options.get("max_krylov_dim") if exact else None, ode_options(mode, {}))
        self.time_step_size = float(time_step_size)
        self.final_time = float(final_time)
        self.num_time_steps = compute_num_time_steps(final_time, time_step_size)
        self.operators = init_operators(operators)
        self.hamiltonian = hamiltonian
        initial_state._finalise()
        self._loschmidt_state = _tensor_copy(initial_state) if getattr(self.config, "record_loschmidt_amplitude", False) else None
        self._initial_state = initial_state.copy_structure()
        self._setup_state()
        root = self.root
        self.nbrs = {nid: list(self.net.nbrs(nid)) for nid in self.state._order}
        self.children = {nid: list(self.state.nodes[nid].phys_children) for nid in self.state._order}
        self.parent = {nid: self.state.nodes[nid].parent for nid in self.state._order}
        self.results = None
        self.times = []

    def _setup_state(self):
        self.state = self._initial_state.copy_structure()
        self.net = DeviceNetwork(self.state, self.hamiltonian)
        self.root = self.state.root_id
        if self.state.orthogonality_center_id is None:
            self.net.canonical_form(self.root)
        else:
            self.net.move_orth_center(self.root)
        self.results = None
        self.times = []

    @property
    def initial_state(self):
        return self._initial_state

    def reset_to_initial_state(self):
        """``TimeEvolution.reset_to_initial_state``."""
        if getattr(self.config, "time_dep", False):
            self.hamiltonian.reset()
        self._setup_state()

    # -- local pieces --------------------------------------------------------------
    def _ax(self, u, v):
        return self.nbrs[u].index(v)

    def _env(self, nid, nxt, A, envs):
        ev = [envs[(x, nid)] if x != nxt else None for x in self.nbrs[nid]]
        return env_apply(A, ev, self.net.W[nid], self._ax(nid, nxt))

    def _evolve(self, nid, x, envs, setting):
        tol, maxdim, ode = setting
        nb = self.nbrs[nid]
        params = [envs[(v, nid)] for v in nb] + [self.net.W[nid]]
        y = torch.empty_like(x)
        apply = _tensor_apply(_SiteOp(len(nb)), params, x.shape)
        if ode is not None:
            if self._rk is None:
                self._rk = RungeKuttaSolver(_solver(x.device).ws)
            self._rk.integrate(x.contiguous(), apply, self.time_step_size, -1j, out=y, **ode)
        else:
            _solver(x.device).expm(x.contiguous(), apply, self.time_step_size, -1j, tol, maxdim, out=y)
        return y

    def _in_new_child_bases(self, T, nid, Ms):
        for g in self.children[nid]:
            ax = self._ax(nid, g)
            lT = [f"i{j}" for j in range(T.dim())]
            lout = [l if j != ax else "new" for j, l in enumerate(lT)]
            T = _raw_contract(T, lT, Ms[g], [lT[ax], "new"], lout, [lT[ax]])
        return T

    _adaptive = False
    _rk = None

    def _update_node(self, c, P, envs_p, setting):
        """``update_node`` + ``update_leaf_node`` / ``update_non_leaf_node``."""
        p = self.parent[c]
        Q, R = qr_split(P[p], self._ax(p, c), reduced=self._adaptive)
        cur = dict(P)
        cur[p] = Q
        cur[c] = absorb(R, P[c], self._ax(c, p))
        envs = dict(envs_p)
        envs[(p, c)] = self._env(p, c, Q, envs)
        envs.pop((c, p), None)
        new, Ms, blocks = {}, {}, {}
        for g in self.children[c]:
            sub, blocks[g], Ms[g] = self._update_node(g, cur, envs, self._deep)
            new.update(sub)
        envs.update({(g, c): b for g, b in blocks.items()})
        x = self._in_new_child_bases(cur[c], c, Ms)
        upd = self._evolve(c, x, envs, setting)
        old = self._in_new_child_bases(P[c], c, Ms)
        if self._adaptive:
            # the new basis spans the old and the evolved tensor
            # (``compute_new_basis_tensor``, ``bug_util.py:123-157``): a leaf
            # stacks its old basis tensor, an inner node its old centre tensor
            first = old if not self.children[c] else x
            U, _ = qr_split(torch.cat([first, upd], dim=0), 0, reduced=True)
        else:
            U, _ = qr_keep_raw(upd, 0)
        legs = [f"i{j}" for j in range(1, U.dim())]
        M = _raw_contract(old, ["p"] + legs, U, ["q"] + legs, ["p", "q"], legs, conj_b=True)
        new[c] = U
        return new, self._env(c, p, U, envs), M

    def _root_update(self, A):
        """``root_update`` (``common_bug.py:311-378``)."""
        root = self.root
        envs = {}

        def rec(nid, toward):
            for x in self.nbrs[nid]:
                if x != toward:
                    rec(x, nid)
            if toward is not None:
                envs[(nid, toward)] = self._env(nid, toward, A[nid], envs)
        rec(root, None)
        new, Ms, blocks = {}, {}, {}
        for c in self.children[root]:
            sub, blocks[c], Ms[c] = self._update_node(c, A, envs, self._top)
            new.update(sub)
        envs.update({(c, root): b for c, b in blocks.items()})
        new[root] = self._evolve(root, self._in_new_child_bases(A[root], root, Ms), envs, self._top)
        return new

    def update_hamiltonian(self):
        """A time-dependent TTNO advanced by one step and copied to the device."""
        self.hamiltonian.update(self.time_step_size)
        self.hamiltonian.modify_state(self.state)
        self.net.refresh_hamiltonian(self.hamiltonian)

    def _store(self, new: dict):
        for nid, t in new.items():
            if tuple(t.shape) == tuple(self.net.t[nid].shape):
                self.net.t[nid].copy_(t)
            else:
                self.net._forget_node(nid)
                self.net._set_node_tensor(nid, t.contiguous())
        self.state.orthogonality_center_id = self.root

    # -- driver API ------------------------------------------------------------------
    def run_one_time_step(self, **kwargs):
        with torch.no_grad():
            self._store(self._root_update(dict(self.net.t)))

    def evaluate_operator(self, operator) -> complex:
        from .ttn import TreeTensorNetworkOperator
        if isinstance(operator, TreeTensorNetworkOperator):
            return self.net.expect_ttno(operator)
        return self.net.expect_local(dict(operator))

class BUG(FixedBUG):
    """Rank-adaptive BUG (``time_evolution/bug.py:30-117``): every basis is
    augmented with the evolved tensor (bond dimensions up to double), the
    centre moves with REDUCED QRs, and after the root update ``svd_truncation``
    (``core/truncation/svd_truncation.py``) cuts every bond by a truncated SVD
    along the leaf-to-leaf path: the centre moves to each non-root node, its
    parent leg is factored (Householder QR, then Jacobi SVD of the k x k R),
    U stays and S V^H goes into the parent, with the rule of
    ``truncate_singular_values`` (``BUGConfig``'s SVD fields). The centre then
    returns to the root. The reference orders that path by its node
    dictionary, which its BUG update rebuilds in a hash-dependent order; a bond
    cap that binds can therefore make its result depend on the process, while
    tolerance-limited truncations agree to the tolerance."""

    config_class = BUGConfig
    _adaptive = True

    def truncation(self, A):
        ops = TreeOps(self.state)
        center = truncate_tensors(ops, A, self.root, self.config)
        move_center(ops, A, center, self.root, False)
        return A

    def run_one_time_step(self, **kwargs):
        with torch.no_grad():
            A = dict(self.net.t)
            A.update(self._root_update(A))
            self._store(self.truncation(A))
