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
tolerance 1e-10.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

from .adjoint import (_SiteOp, _raw_contract, _solver, _tensor_apply, absorb, env_apply, qr_keep_raw)
from .engine import DeviceNetwork
from .tdvp import (TTNTimeEvolutionConfig, TensorProduct, TimeEvoMode, compute_num_time_steps)

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


class FixedBUG:
    """Fixed-rank BUG driver with PyTreeNet's constructor and stepping API."""

    config_class = FixedBUGConfig

    def __init__(self, initial_state, hamiltonian, time_step_size: float, final_time: float, operators,
                 config: FixedBUGConfig | None = None, solver_options: dict[str, Any] | None = None):
        if time_step_size <= 0 or final_time <= 0:
            raise ValueError("time step and final time must be positive")
        self.config = config if config is not None else self.config_class()
        if self.config.time_evo_mode is not TimeEvoMode.KRYLOV:
            raise NotImplementedError(
                f"time_evo_mode={self.config.time_evo_mode}: the GPU engine runs the matrix-free "
                "KRYLOV exponential only")
        opts = dict(solver_options or {})
        bad = set(opts) - TimeEvoMode.valid_solver_options(TimeEvoMode.KRYLOV)
        if bad:
            raise ValueError(f"solver options {sorted(bad)} are not valid for KRYLOV")
        self.solver_options = opts
        self.time_step_size = float(time_step_size)
        self.final_time = float(final_time)
        self.num_time_steps = compute_num_time_steps(final_time, time_step_size)
        self.operators = operators if operators is not None else []
        self.hamiltonian = hamiltonian
        initial_state._finalise()
        self.state = initial_state.copy_structure()
        self.net = DeviceNetwork(self.state, hamiltonian)
        root = self.state.root_id
        if self.state.orthogonality_center_id is None:
            self.net.canonical_form(root)
        else:
            self.net.move_orth_center(root)
        self.root = root
        self.nbrs = {nid: list(self.net.nbrs(nid)) for nid in self.state._order}
        self.children = {nid: list(self.state.nodes[nid].phys_children) for nid in self.state._order}
        self.parent = {nid: self.state.nodes[nid].parent for nid in self.state._order}
        self.results = None
        self.times = []

    # -- local pieces --------------------------------------------------------------
    def _ax(self, u, v):
        return self.nbrs[u].index(v)

    def _env(self, nid, nxt, A, envs):
        ev = [envs[(x, nid)] if x != nxt else None for x in self.nbrs[nid]]
        return env_apply(A, ev, self.net.W[nid], self._ax(nid, nxt))

    def _evolve(self, nid, x, envs, tol):
        nb = self.nbrs[nid]
        params = [envs[(v, nid)] for v in nb] + [self.net.W[nid]]
        y = torch.empty_like(x)
        _solver(x.device).expm(x.contiguous(), _tensor_apply(_SiteOp(len(nb)), params, x.shape), self.time_step_size,
                               -1j, tol, self.solver_options.get("max_krylov_dim"), out=y)
        return y

    def _in_new_child_bases(self, T, nid, Ms):
        for g in self.children[nid]:
            ax = self._ax(nid, g)
            lT = [f"i{j}" for j in range(T.dim())]
            lout = [l if j != ax else "new" for j, l in enumerate(lT)]
            T = _raw_contract(T, lT, Ms[g], [lT[ax], "new"], lout, [lT[ax]])
        return T

    def _update_node(self, c, P, envs_p, tol):
        """``update_node`` + ``update_leaf_node`` / ``update_non_leaf_node``."""
        p = self.parent[c]
        Q, R = qr_keep_raw(P[p], self._ax(p, c))
        cur = dict(P)
        cur[p] = Q
        cur[c] = absorb(R, P[c], self._ax(c, p))
        envs = dict(envs_p)
        envs[(p, c)] = self._env(p, c, Q, envs)
        envs.pop((c, p), None)
        new, Ms, blocks = {}, {}, {}
        for g in self.children[c]:
            sub, blocks[g], Ms[g] = self._update_node(g, cur, envs, DEFAULT_KRYLOV_TOL)
            new.update(sub)
        envs.update({(g, c): b for g, b in blocks.items()})
        upd = self._evolve(c, self._in_new_child_bases(cur[c], c, Ms), envs, tol)
        U, _ = qr_keep_raw(upd, 0)
        old = self._in_new_child_bases(P[c], c, Ms)
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
        tol = self.solver_options.get("krylov_tol", DEFAULT_KRYLOV_TOL)
        new, Ms, blocks = {}, {}, {}
        for c in self.children[root]:
            sub, blocks[c], Ms[c] = self._update_node(c, A, envs, tol)
            new.update(sub)
        envs.update({(c, root): b for c, b in blocks.items()})
        new[root] = self._evolve(root, self._in_new_child_bases(A[root], root, Ms), envs, tol)
        return new

    # -- driver API ------------------------------------------------------------------
    def run_one_time_step(self, **kwargs):
        with torch.no_grad():
            new = self._root_update(dict(self.net.t))
            for nid, t in new.items():
                self.net.t[nid].copy_(t)
        self.state.orthogonality_center_id = self.root

    def evaluate_operator(self, operator) -> complex:
        from .ttn import TreeTensorNetworkOperator
        if isinstance(operator, TreeTensorNetworkOperator):
            return self.net.expect_ttno(operator)
        return self.net.expect_local(dict(operator))

    def evaluate_operators(self):
        ops = self.operators
        if isinstance(ops, dict):
            ops = list(ops.values())
        elif isinstance(ops, TensorProduct):
            ops = [ops]
        return np.array([self.evaluate_operator(o) for o in ops])

    def run(self, evaluation_time: int = 1, pgbar: bool = False):
        """``TimeEvolution.run`` (``time_evolution/time_evolution.py:346-368``)."""
        res = [self.evaluate_operators()]
        self.times = [0.0]
        for i in range(self.num_time_steps):
            self.run_one_time_step()
            if evaluation_time != "inf" and (i + 1) % evaluation_time == 0:
                res.append(self.evaluate_operators())
                self.times.append((i + 1) * self.time_step_size)
        self.results = np.array(res)
        return self.results
