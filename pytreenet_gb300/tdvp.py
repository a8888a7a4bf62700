"""One-site and two-site TDVP drivers running on the GB300 engine.

Public surface mirrors PyTreeNet's drivers
(``time_evolution/tdvp_algorithms/*.py``): the constructor
``(initial_state, hamiltonian, time_step_size, final_time, operators,
config=None, solver_options=None)``, ``run_one_time_step()``, ``run()``,
``update_path``, ``orthogonalization_path``, ``state`` and ``results``.
"""
from __future__ import annotations

from dataclasses import dataclass
from enum import Enum
from typing import Any

import numpy as np

from .engine import DeviceNetwork
from .truncation import SVDParameters
from .results import RunLoop, init_operators
from .ttn import TreeTensorNetworkOperator, TreeTensorNetworkState


class TimeEvoMode(Enum):
    """Local exponential method (``time_evolution/time_evolution.py:431-655``).

    KRYLOV is the matrix-free Lanczos exponential with the adaptive stop at
    ``krylov_tol``. The exact modes (FASTEST, which the reference maps to
    CHEBYSHEV, EXPM, CHEBYSHEV, SPARSE) build the N x N effective Hamiltonian
    in the reference; here they compute the same exp(-i dt H_eff) x
    matrix-free, with the Krylov stop at 1e-14 (1e-11 on the reduced-precision
    path) and at most 64 vectors. RK45, RK23 and DOP853 integrate the local
    equation with the same adaptive explicit Runge-Kutta pairs and step
    control as ``solve_ivp``, on device vectors (``ode.py``); BDF (implicit,
    needs the N x N Jacobian) is not provided."""
    FASTEST = "fastest"
    EXPM = "expm"
    CHEBYSHEV = "chebyshev"
    SPARSE = "sparse"
    RK45 = "RK45"
    RK23 = "RK23"
    DOP853 = "DOP853"
    BDF = "BDF"
    KRYLOV = "krylov"

    def __str__(self) -> str:
        return self.value

    @staticmethod
    def default_solver_options(mode) -> dict:
        if mode is TimeEvoMode.KRYLOV:
            return {"krylov_tol": 1e-10}
        if mode in (TimeEvoMode.RK45, TimeEvoMode.RK23, TimeEvoMode.DOP853, TimeEvoMode.BDF):
            return {"atol": 1e-10, "rtol": 1e-10}
        return {}

    @staticmethod
    def valid_solver_options(mode) -> set:
        if mode is TimeEvoMode.KRYLOV:
            return {"krylov_tol", "max_krylov_dim", "hermitian", "exp_factor"}
        if mode in TimeEvoMode.scipy_modes():
            return {"atol", "rtol", "max_step", "first_step", "jac", "jac_sparsity",
                    "lband", "uband", "min_step", "hermitian", "exp_factor"}
        return {"exp_factor"}

    @staticmethod
    def scipy_modes() -> list:
        return [TimeEvoMode.RK45, TimeEvoMode.RK23, TimeEvoMode.DOP853, TimeEvoMode.BDF]

    @staticmethod
    def fastest_equivalent() -> "TimeEvoMode":
        return TimeEvoMode.CHEBYSHEV

    def is_exact(self) -> bool:
        """The matrix-exponential modes (everything but KRYLOV and the ODE solvers)."""
        return self is not TimeEvoMode.KRYLOV and self not in TimeEvoMode.scipy_modes()

    def is_scipy(self) -> bool:
        """A ``solve_ivp`` mode (FASTEST counts as its equivalent, CHEBYSHEV)."""
        if self is TimeEvoMode.FASTEST:
            return TimeEvoMode.fastest_equivalent().is_scipy()
        return self in TimeEvoMode.scipy_modes()

    def action_evolvable(self) -> bool:
        """Modes that evolve through an action instead of a dense matrix."""
        return self.is_scipy() or self is TimeEvoMode.KRYLOV

    def time_evolve_action(self, psi, time_evo_action, time_difference: float, forward=None, **options):
        """psi evolved by y' = c A(t) y on the device, A given as
        ``time_evo_action(t, y)`` (``time_evolution.py:536-615``); see
        ``local_evolution.time_evolve_action``."""
        from .local_evolution import time_evolve_action
        return time_evolve_action(self, psi, time_evo_action, time_difference,
                                  EvoDirection.FORWARD if forward is None else forward, **options)

    def time_evolve(self, psi, hamiltonian, time_difference: float, forward=None, **options):
        """psi evolved by a dense Hamiltonian with the caller's options only
        (``time_evolution.py:617-655``); see ``local_evolution``."""
        from .local_evolution import evolve_dense
        return evolve_dense(self, psi, hamiltonian, time_difference,
                            EvoDirection.FORWARD if forward is None else forward, options)


# the exact modes run the Krylov exponential to these stops
EXACT_KRYLOV_TOL = {"plain": 1e-14, "reduced": 1e-11}
EXACT_MAX_KRYLOV_DIM = 64


def check_time_evo_mode(mode, solver_options, precision: str = "plain"):
    """Validate the mode and options as the reference does and return the
    options the engine's Krylov exponential runs with."""
    if mode is TimeEvoMode.BDF:
        raise NotImplementedError(
            f"time_evo_mode={mode}: the implicit BDF solver is not provided; use RK45, RK23, DOP853, "
            "KRYLOV or an exact mode")
    # the drivers hand the caller's options to the solver as they are: an ODE
    # mode given none runs at solve_ivp's own tolerances (``ode_options``)
    opts = {} if mode in TimeEvoMode.scipy_modes() else TimeEvoMode.default_solver_options(mode)
    opts.update(solver_options or {})
    bad = set(opts) - TimeEvoMode.valid_solver_options(mode)
    if bad:
        raise ValueError(f"solver options {sorted(bad)} are not valid for {mode}")
    if mode.is_exact():
        opts = dict(opts, krylov_tol=EXACT_KRYLOV_TOL["plain" if precision == "plain" else "reduced"],
                    max_krylov_dim=EXACT_MAX_KRYLOV_DIM)
    return opts


ODE_OPTIONS = ("atol", "rtol", "max_step", "first_step")
# solve_ivp's tolerances when the caller sets none
ODE_DEFAULT_TOLERANCES = {"atol": 1e-6, "rtol": 1e-3}


def ode_options(mode, solver_options) -> dict | None:
    """The Runge-Kutta settings of an ODE mode (None for the exponential
    modes): the method and the ``solve_ivp`` options that explicit methods
    read (``jac``, ``lband`` and the like have no effect on them). The
    reference's drivers pass their options to ``solve_ivp`` unchanged
    (``time_evolution.py:595-615``), so tolerances not given are
    ``solve_ivp``'s: atol 1e-6, rtol 1e-3."""
    if mode not in TimeEvoMode.scipy_modes():
        return None
    opts = dict(ODE_DEFAULT_TOLERANCES)
    opts.update({k: v for k, v in (solver_options or {}).items() if k in ODE_OPTIONS})
    opts["method"] = mode.value
    return opts


class EvoDirection(Enum):
    """``time_evolution/time_evolution.py:384-429``: FORWARD = exp(-i H t)."""
    FORWARD = -1
    BACKWARD = 1

    @staticmethod
    def from_bool(forward: bool) -> "EvoDirection":
        return EvoDirection.FORWARD if forward else EvoDirection.BACKWARD

    def exp_sign(self) -> int:
        return self.value

    def exp_factor(self) -> complex:
        return 1.0j * self.value


class PathFinderMode(Enum):
    LeafToLeaf = "LeafToLeaf"
    LeafToRoot = "LeafToRoot"


@dataclass
class TTNTimeEvolutionConfig:
    record_bond_dim: bool = False
    record_max_bdim: bool = False
    record_average_bdim: bool = False
    record_total_size: bool = False
    record_norm: bool = False
    record_loschmidt_amplitude: bool = False
    time_dep: bool = False


@dataclass
class TDVPConfig(TTNTimeEvolutionConfig):
    """``tdvp_algorithms/tdvp_algorithm.py:23-34``."""
    time_evo_mode: TimeEvoMode = TimeEvoMode.FASTEST
    main_path_mode: PathFinderMode = PathFinderMode.LeafToRoot


def _tensor_copy(ttn):
    """A TTN sharing no tensor with ``ttn`` (the state at time zero)."""
    out = ttn.copy_structure()
    out._phys = {k: (v.copy() if isinstance(v, np.ndarray) else v.clone()) for k, v in out._phys.items()}
    return out


def compute_num_time_steps(final_time: float, time_step_size: float) -> int:
    """``TimeEvolution._compute_num_time_steps`` (``time_evolution/time_evolution.py:104-116``):
    the integer part of final_time / dt, plus one when the fractional part is
    at least 0.1 (so 0.3 / 0.05 = 5.999... gives 6, not 7)."""
    import math
    frac, whole = math.modf(final_time / time_step_size)
    return int(whole) if frac < 0.1 else int(whole + 1)


def _postorder(ttn, nid):
    node = ttn.nodes[nid]
    if node.is_leaf():
        return [nid]
    out = []
    for c in node.children:
        out += _postorder(ttn, c)
    return out + [nid]


def leaf_to_root_update_path(ttn) -> list[str]:
    """``TDVPUpdatePathFinder_LeafToRoot.find_path``
    (``time_evolution/time_evo_util/update_path.py:63-254``)."""
    root = ttn.root_id
    dist = ttn.distance_to_node(root)
    start = max(dist, key=dist.get)
    main = ttn.find_path_to_root(start)
    path = []
    for origin in main:
        if origin != root:
            path += [x for c in ttn.nodes[origin].children if c not in main
                     for x in _postorder(ttn, c)] + [origin]
            continue
        if len(ttn.nodes[root].children) == 1:
            path += [root]
            continue
        leaves = [x for x in ttn.get_leaves() if x not in path]
        ld = {x: d for x, d in dist.items() if x in leaves}
        if not ld:
            raise AssertionError("no unvisited leaf left")
        last = max(ld, key=ld.get)
        down = list(reversed(ttn.find_path_to_root(last)))
        for o in down:
            if o == root:
                excl = (main[-2], down[1])
                path += [x for c in ttn.nodes[root].children if c not in excl
                         for x in _postorder(ttn, c)] + [root]
            else:
                path += [x for c in ttn.nodes[o].children if c not in down
                         for x in _postorder(ttn, c)] + [o]
    return path


def leaf_to_leaf_update_path(ttn) -> list[str]:
    """``TDVPUpdatePathFinder_LeafToLeaf.find_path``
    (``time_evolution/time_evo_util/update_path.py:255-396``): the first pair of
    leaves at maximal distance (leaves in node order, the root included when it
    has a single neighbour), the path between them, and every off-path subtree,
    children first, just before the main-path node it hangs from."""
    leaves = [nid for nid in ttn._order if ttn.nodes[nid].is_leaf()]
    if ttn.nodes[ttn.root_id].nneighbours() == 1:
        leaves.append(ttn.root_id)
    best, pair = -1, (leaves[0], leaves[0])
    for i in range(len(leaves)):
        di = ttn.distance_to_node(leaves[i])
        for j in range(i + 1, len(leaves)):
            if di[leaves[j]] > best:
                best, pair = di[leaves[j]], (leaves[i], leaves[j])
    main = ttn.path_from_to(*pair)
    on_main = set(main)
    visited: set = set()
    path: list[str] = []

    def subtree(nid):
        if nid in visited or nid in on_main:
            return []
        visited.add(nid)
        node = ttn.nodes[nid]
        out = []
        if node.parent is not None and node.parent not in on_main and node.parent not in visited:
            out += subtree(node.parent)
        for c in node.children:
            if c not in on_main and c not in visited:
                out += subtree(c)
        return out + [nid]
    for origin in main:
        node = ttn.nodes[origin]
        if node.parent is not None and node.parent not in on_main and node.parent not in visited:
            path += subtree(node.parent)
        for c in node.children:
            if c not in on_main:
                path += subtree(c)
        if origin not in visited:
            visited.add(origin)
            path.append(origin)
    return path


def find_update_path(ttn, mode: "PathFinderMode") -> list[str]:
    """``find_path`` (``update_path.py:15-31``) for the two path modes."""
    if mode is PathFinderMode.LeafToLeaf:
        return leaf_to_leaf_update_path(ttn)
    return leaf_to_root_update_path(ttn)


class TensorProduct(dict):
    """Single-site operators keyed by node id (``operators/tensorproduct.py:33-430``),
    numeric or symbolic (strings resolved through a conversion dictionary)."""

    @classmethod
    def from_operators(cls, operators) -> "TensorProduct":
        out = cls()
        for op in operators:
            assert len(op.node_identifiers) == 1
            out[op.node_identifiers[0]] = op.operator
        return out

    def add_operator(self, node_id: str, operator):
        self[node_id] = operator

    def add_suffix(self, suffix: str) -> "TensorProduct":
        return TensorProduct({k + suffix: v for k, v in self.items()})

    def num_sites(self) -> int:
        return len(self)

    def allclose(self, other) -> bool:
        return len(self) == len(other) and all(k in other and np.allclose(v, other[k]) for k, v in self.items())

    def pad_with_identities(self, ttn, symbolic: bool = False) -> "TensorProduct":
        """Identities on every node of ``ttn`` without an operator."""
        missing = set(self) - set(ttn.nodes)
        if missing:
            raise KeyError("Single site operators in this tensor product are applied to nodes "
                           "that do not exist in the TTN!")
        out = TensorProduct(self)
        for nid in ttn.nodes:
            if nid not in out:
                d = int(ttn.phys(nid).shape[-1])
                out[nid] = f"I{d}" if symbolic else np.eye(d)
        return out

    def into_operator(self, conversion_dict=None, order=None):
        """The Kronecker product of the factors (``order`` defaults to the keys)."""
        from .tebd import NumericOperator
        order = list(self.keys()) if order is None else order
        total = np.ones((1, 1), dtype=complex)
        for nid in order:
            op = self[nid]
            if isinstance(op, str):
                if conversion_dict is None:
                    raise TypeError("If the tensor_product contains symbolic operators, there must be a "
                                    "dictionary for conversion!")
                op = conversion_dict[op]
            total = np.kron(total, np.asarray(op))
        return NumericOperator(total, list(order))

    def exp(self, factor=1):
        """exp(factor * A_1 x A_2 x ...)."""
        import scipy.linalg
        from .tebd import NumericOperator
        op = self.into_operator()
        return NumericOperator(scipy.linalg.expm(factor * op.operator), op.node_identifiers)

    def _local(self, fn, invariance=None, suffix=""):
        out = TensorProduct()
        for k, v in self.items():
            if isinstance(v, str):
                out[k] = v if (invariance is not None and invariance.get(v)) else v + suffix
            else:
                out[k] = fn(np.asarray(v))
        return out

    def transpose(self, sym_dict=None, transpose_suffix: str = "_T") -> "TensorProduct":
        return self._local(np.transpose, sym_dict, transpose_suffix)

    def conjugate(self, real_dict=None, conjugate_suffix: str = "_conj") -> "TensorProduct":
        return self._local(np.conjugate, real_dict, conjugate_suffix)

    def conjugate_transpose(self, herm_dict=None, herm_suffix: str = "_H") -> "TensorProduct":
        return self._local(lambda a: a.conj().T, herm_dict, herm_suffix)

    def otimes(self, other, to_copy: bool = True) -> "TensorProduct":
        out = TensorProduct(self) if to_copy else self
        for k, v in other.items():
            if k in out:
                raise ValueError("The tensor products have a common identifier!")
            out[k] = v
        return out

    def multiply(self, other, identity_dict=None, conversion_dict=None, multi_inset: str = "_mult_"):
        """Site-wise matrix products (numeric factors; symbolic ones need the
        conversion dictionary, into which the products are entered)."""
        out = TensorProduct()
        for k in set(self) | set(other):
            if k in self and k in other:
                a, b = self[k], other[k]
                if isinstance(a, str) or isinstance(b, str):
                    if conversion_dict is None:
                        raise TypeError("symbolic factors need a conversion dictionary")
                    name = f"{a}{multi_inset}{b}"
                    conversion_dict[name] = np.asarray(conversion_dict[a] if isinstance(a, str) else a) @ \
                        np.asarray(conversion_dict[b] if isinstance(b, str) else b)
                    out[k] = name
                else:
                    out[k] = np.asarray(a) @ np.asarray(b)
            else:
                out[k] = self[k] if k in self else other[k]
        return out

    def __matmul__(self, other):
        return self.multiply(other)


class OneSiteTDVP(RunLoop):
    """Common machinery of the one-site TDVP drivers
    (``tdvp_algorithms/tdvp_algorithm.py:37-221``, ``onesitetdvp.py:17-134``)."""

    config_class = TDVPConfig

    def __init__(self, initial_state: TreeTensorNetworkState, hamiltonian: TreeTensorNetworkOperator,
                 time_step_size: float, final_time: float, operators, config: TDVPConfig | None = None,
                 solver_options: dict[str, Any] | None = None, precision: str = "plain"):
        if len(initial_state.nodes) != len(hamiltonian.nodes):
            raise AssertionError("state and Hamiltonian must have the same nodes")
        from .time_dep import AbstractTimeDepTTNO
        if config is not None and config.time_dep and not isinstance(hamiltonian, AbstractTimeDepTTNO):
            raise TypeError("The Hamiltonian must be from the AbstractTimeDepTTNO class "
                            "if the time evolution is time-dependent!")
        if time_step_size <= 0 or final_time <= 0:
            raise ValueError("time step and final time must be positive")
        self.config = config if config is not None else self.config_class()
        self.solver_options = check_time_evo_mode(self.config.time_evo_mode, solver_options, precision)
        self.time_step_size = float(time_step_size)
        self.final_time = float(final_time)
        self.num_time_steps = compute_num_time_steps(final_time, time_step_size)
        self.operators = init_operators(operators)
        self.hamiltonian = hamiltonian
        initial_state._finalise()
        self._loschmidt_state = _tensor_copy(initial_state) if self.config.record_loschmidt_amplitude else None
        self._initial_state = initial_state.copy_structure()
        self.update_path = find_update_path(self._initial_state, self.config.main_path_mode)
        self.orthogonalization_path = [self._initial_state.path_from_to(self.update_path[i],
                                                                        self.update_path[i + 1])[1:]
                                       for i in range(len(self.update_path) - 1)]
        self.precision = precision
        self._setup_state()

    def _setup_state(self):
        """The working state from the initial one: a device copy in canonical
        form at the first site of the update path, environments toward it
        (``tdvp_algorithm.py:58-163``)."""
        self.state = self._initial_state.copy_structure()
        self.net = DeviceNetwork(self.state, self.hamiltonian, precision=self.precision)
        self.net.ode = ode_options(self.config.time_evo_mode, self.solver_options)
        if self.state.orthogonality_center_id is None:
            self.net.canonical_form(self.update_path[0])
        else:
            self.net.move_orth_center(self.update_path[0])
        self.net.init_cache_but_one(self.update_path[0])
        self.results = None
        self.times = []

    @property
    def initial_state(self):
        return self._initial_state

    def reset_to_initial_state(self):
        """``TimeEvolution.reset_to_initial_state`` (``time_evolution.py:370-390``):
        the state back to the initial one, results cleared, a time-dependent
        Hamiltonian reset. The initial tensors must not have been modified
        (the engine evolves device copies)."""
        if self.config.time_dep:
            self.hamiltonian.reset()
        self._setup_state()

    @property
    def partial_tree_cache(self):
        """The environments of the sweep (``TDVPAlgorithm.partial_tree_cache``,
        ``tdvp_algorithm.py:108,156-163``) as a ``SandwichCache`` over the
        device buffers."""
        from .contractions import SandwichCache
        return SandwichCache.of_network(self.net, self.hamiltonian)

    def update_tree_cache(self, node_id: str, next_node_id: str):
        """``TDVPAlgorithm.update_tree_cache`` (``tdvp_algorithm.py:165-182``):
        E(node_id -> next_node_id) from the current tensors."""
        self.net.update_env(node_id, next_node_id)

    # -- Krylov options ------------------------------------------------------------
    def _kry(self):
        o = self.solver_options
        return o.get("krylov_tol", 1e-10), o.get("max_krylov_dim", None)

    def _factor(self, forward: bool) -> complex:
        override = self.solver_options.get("exp_factor")
        if override is None:
            return -1j if forward else 1j
        return override if forward else -override

    # -- building blocks --------------------------------------------------------------
    def _update_site(self, node_id, time_step_factor=1.0):
        tol, maxdim = self._kry()
        self.net.evolve_site(node_id, self.time_step_size * time_step_factor, self._factor(True), tol, maxdim,
                             hermitian=self.solver_options.get("hermitian", True))

    def _update_link(self, node_id, next_node_id, time_step_factor=1.0):
        st = self.state
        assert st.orthogonality_center_id == node_id
        R = self.net.qr_split(node_id, next_node_id)
        self.net.update_env(node_id, next_node_id)
        tol, maxdim = self._kry()
        self.net.evolve_bond(R, node_id, next_node_id, self.time_step_size * time_step_factor,
                             self._factor(False), tol, maxdim, hermitian=self.solver_options.get("hermitian", True))
        self.net.absorb(R, node_id, next_node_id, link_variant=True)
        st.orthogonality_center_id = next_node_id

    def _move_orth_and_update_cache_for_path(self, path):
        if len(path) == 0:
            return
        assert self.state.orthogonality_center_id == path[0]
        for prev, nid in zip(path[:-1], path[1:]):
            self.net.move_orth_center(nid)
            self.net.update_env(prev, nid)

    # -- observables -----------------------------------------------------------------
    def evaluate_operator(self, operator) -> complex:
        """``TTNTimeEvolution.evaluate_operator`` (``time_evolution/ttn_time_evolution.py:181-211``):
        a TensorProduct of one-site operators, or a TTNO on the state's tree."""
        from .ttn import TreeTensorNetworkOperator
        if isinstance(operator, TreeTensorNetworkOperator):
            return self.net.expect_ttno(operator)
        return self.net.expect_local(dict(operator))

    def update_hamiltonian(self):
        """Advance a time-dependent TTNO by one step and copy its tensors into
        the device buffers (the environments are kept, as in the reference)."""
        self.hamiltonian.update(self.time_step_size)
        self.hamiltonian.modify_state(self.state)
        self.net.refresh_hamiltonian(self.hamiltonian)

    def reset_hamiltonian(self):
        self.hamiltonian.reset()
        self.net.refresh_hamiltonian(self.hamiltonian)

class FirstOrderOneSiteTDVP(OneSiteTDVP):
    """``tdvp_algorithms/firstorderonesite.py:7-104``."""

    def run_one_time_step(self):
        path = self.update_path
        op = self.orthogonalization_path
        for i, nid in enumerate(path):
            if i == len(path) - 1:
                if len(op) > 0:
                    self._move_orth_and_update_cache_for_path(op[-1])
                self._update_site(nid)
                self.net.move_orth_center(path[0])
                # environments whose side of the tree the sweep's last moves
                # did not touch are still exact: keep them
                self.net.init_cache_but_one(path[0], reuse=True)
            elif i == 0:
                assert self.state.orthogonality_center_id == nid
                self._update_site(nid)
                self._update_link(nid, op[0][0])
            else:
                self._move_orth_and_update_cache_for_path(op[i - 1])
                self._update_site(nid)
                self._update_link(nid, op[i][0])


class SecondOrderOneSiteTDVP(OneSiteTDVP):
    """``tdvp_algorithms/secondorderonesite.py:11-193``."""

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.backwards_update_path = list(reversed(self.update_path))
        bp = self.backwards_update_path
        bo = [self.state.path_from_to(nid, bp[i + 2])[:-1] for i, nid in enumerate(bp[1:-1])]
        bo.append([bp[-1]])
        self.backwards_orth_path = bo

    def run_one_time_step(self):
        path, op = self.update_path, self.orthogonalization_path
        for i, nid in enumerate(path[:-1]):
            if i > 0:
                self._move_orth_and_update_cache_for_path(op[i - 1])
            self._update_site(nid, 0.5)
            self._update_link(nid, op[i][0], 0.5)
        self._update_site(path[-1])
        bp = self.backwards_update_path
        self._update_link(self.state.orthogonality_center_id, bp[1], 0.5)
        for i, nid in enumerate(bp[1:-1]):
            idx = i + 1
            self._update_site(nid, 0.5)
            self._move_orth_and_update_cache_for_path(self.backwards_orth_path[idx - 1])
            self._update_link(self.state.orthogonality_center_id, bp[idx + 1], 0.5)
        self._update_site(bp[-1], 0.5)


# ----------------------------------------------------------------------------
# two-site TDVP
# ----------------------------------------------------------------------------
@dataclass
class TwoSiteTDVPConfig(TDVPConfig, SVDParameters):
    """``tdvp_algorithms/twositetdvp.py:18-27``: TDVP options plus the truncation
    parameters of the SVD split."""


class TwoSiteTDVP(OneSiteTDVP):
    """``tdvp_algorithms/twositetdvp.py:29-146``: two neighbouring sites are
    merged, evolved together and split by a truncated SVD."""

    config_class = TwoSiteTDVPConfig

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        if len(self.state.nodes) < 2:
            raise ValueError("Two-site TDVP cannot be used for systems with less than 2 sites!")
        if not hasattr(self.config, "max_bond_dim"):
            raise TypeError("two-site TDVP needs a TwoSiteTDVPConfig (truncation parameters)")
        self.bond_dims_history: list[int] = []

    def _setup_state(self):
        super()._setup_state()
        # bond dimensions change from step to step, so captured QR launch
        # sequences would mostly be captured once and dropped: launch eagerly
        self.net.use_graphs = False
        self.bond_dims_history = []

    def _update_two_site_nodes(self, target_node_id, next_node_id, time_step_factor=1.0):
        """``_update_two_site_nodes`` (``twositetdvp.py:89-125``)."""
        tol, maxdim = self._kry()
        s = self.net.evolve_two_site(target_node_id, next_node_id, self.time_step_size * time_step_factor,
                                     self._factor(True), tol, maxdim, self.config,
                                     hermitian=self.solver_options.get("hermitian", True))
        self.bond_dims_history.append(len(s))

    def _single_site_backwards_update(self, node_id, time_step_factor=1.0):
        """``_single_site_backwards_update`` (``twositetdvp.py:127-138``): the site
        evolves with the time step negated."""
        self._update_site(node_id, -1 * time_step_factor)

    @staticmethod
    def create_two_site_id(node_id: str, next_node_id: str) -> str:
        return "TwoSite_" + node_id + "_contr_" + next_node_id


class FirstOrderTwoSiteTDVP(TwoSiteTDVP):
    """``tdvp_algorithms/firstordertwosite.py:11-30``, run as intended: the
    partner of update-path node i is the first node of the i-th
    orthogonalisation sub-path, and the environments are rebuilt once the
    centre is back at the start (as the first-order one-site driver does).
    The reference indexes sub-path i + 1 and raises ValueError on the second
    pair of any tree whose root has more than one child."""

    def run_one_time_step(self):
        path, op = self.update_path, self.orthogonalization_path
        for i, nid in enumerate(path[:-2]):
            nxt = op[i][0]
            self._update_two_site_nodes(nid, nxt)
            self._single_site_backwards_update(nxt)
            self._move_orth_and_update_cache_for_path(op[i])
        self._update_two_site_nodes(path[-2], path[-1])
        self.net.move_orth_center(path[0])
        self.net.init_cache_but_one(path[0])


class SecondOrderTwoSiteTDVP(TwoSiteTDVP):
    """``tdvp_algorithms/secondordertwosite.py:11-193``: forward sweep with
    half steps, then the mirrored backward sweep."""

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.backwards_update_path = list(reversed(self.update_path))
        self.backwards_orth_path = [list(reversed(p)) for p in reversed(self.orthogonalization_path)]

    def forward_sweep(self):
        path, op = self.update_path, self.orthogonalization_path
        for i, nid in enumerate(path[:-2]):
            if i > 0:
                self._move_orth_and_update_cache_for_path(op[i - 1])
            assert self.state.orthogonality_center_id == nid
            nxt = op[i][0]
            self._update_two_site_nodes(nid, nxt, 0.5)
            self._single_site_backwards_update(nxt, 0.5)
        self._update_two_site_nodes(path[-2], path[-1], 0.5)

    def backwards_sweep(self):
        bp, bo = self.backwards_update_path, self.backwards_orth_path
        for i in range(len(bp) - 1):
            if i == 0:
                self._update_two_site_nodes(bp[0], bp[1], 0.5)
                continue
            self._move_orth_and_update_cache_for_path(bo[i])
            target = bo[i][-1]
            self._single_site_backwards_update(target, 0.5)
            self._update_two_site_nodes(target, bp[i + 1], 0.5)

    def run_one_time_step(self):
        self.forward_sweep()
        self.backwards_sweep()
