"""TEBD on the GB300 engine, and a nearest-neighbour Trotter splitting.

Public surface mirrors PyTreeNet's ``TEBD`` (``time_evolution/tebd.py:18-155``):
``TEBD(initial_state, trotter_splitting, time_step_size, final_time, operators,
svd_parameters=None, config=None)`` with ``exponents``, ``trotter_splitting``,
``run_one_time_step()`` and ``run()``. Any object with
``exponentiate_splitting(delta_time, ttn)`` returning operators that carry
``.operator`` (legs: outputs, then inputs) and ``.node_identifiers`` can be
passed as the splitting -- PyTreeNet's own ``TrotterSplitting`` included. The
module's ``SWAPlist`` / ``TrotterStep`` / ``TrotterSplitting``
(``time_evolution/trotter.py:15-322``) build the gate list, with SWAP gates
before and after a step to bring the sites of a non-neighbouring term next to
each other.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.linalg
import torch

from .engine import CDT, DeviceNetwork
from .results import RunLoop, init_operators
from .tdvp import TTNTimeEvolutionConfig, TensorProduct, _tensor_copy, compute_num_time_steps
from .truncation import SVDParameters


@dataclass
class NumericOperator:
    """``operators/operator.py:18-60``: a matrix or tensor (outputs, then inputs)
    and the node identifiers its legs act on, in the same order."""
    operator: np.ndarray
    node_identifiers: list


def swap_gate(dimension: int = 2) -> np.ndarray:
    """SWAP of two sites of dimension d as a d^2 x d^2 matrix: |i j> -> |j i>."""
    d = int(dimension)
    m = np.zeros((d * d, d * d), dtype=complex)
    for i in range(d):
        for j in range(d):
            m[j * d + i, i * d + j] = 1.0
    return m


def _open_dimension(ttn, nid) -> int:
    return int(ttn.phys(nid).shape[-1])


class SWAPlist(list):
    """``time_evolution/trotter.py:15-103``: SWAP gates of neighbouring nodes,
    each pair in the leg order of its gate."""

    def __init__(self, swap_list=None):
        swap_list = [] if swap_list is None else list(swap_list)
        for pair in swap_list:
            if len(pair) != 2:
                raise ValueError("SWAPs can only happen between exactly two nodes!")
        super().__init__(swap_list)

    def is_compatible_with_ttn(self, ttn) -> bool:
        for a, b in self:
            if a not in ttn.nodes:
                return False
            if b not in ttn.nodes[a].neighbouring_nodes():
                return False
            if _open_dimension(ttn, a) != _open_dimension(ttn, b):
                return False
        return True

    def into_operators(self, ttn=None, dim=None) -> list:
        if ttn is None and dim is None and len(self) != 0:
            raise ValueError("`ttn` and `dim` cannot both be `None`!")
        out = []
        for a, b in self:
            d = _open_dimension(ttn, a) if ttn is not None else dim
            out.append(NumericOperator(swap_gate(d).reshape(d, d, d, d), [a, b]))
        return out


class TrotterStep:
    """``time_evolution/trotter.py:105-194``: a tensor product of one-site
    operators, the factor of its exponent, and SWAP gates applied before and
    after the exponentiated operator."""

    def __init__(self, operator: TensorProduct | dict, factor: float, swaps_before=None, swaps_after=None):
        self.operator = dict(operator)
        self.factor = factor
        self.swaps_before = SWAPlist() if swaps_before is None else SWAPlist(swaps_before)
        self.swaps_after = SWAPlist() if swaps_after is None else SWAPlist(swaps_after)

    def exponentiate_operator(self, delta_time: float, ttn=None, dim=None) -> NumericOperator:
        """exp(-i factor dt (A_1 x A_2 x ...)) with the factors in the tensor
        product's order, reshaped to (out_1, ..., out_n, in_1, ..., in_n)."""
        ids = list(self.operator)
        mats = [np.asarray(self.operator[i], dtype=complex) for i in ids]
        full = mats[0]
        for m in mats[1:]:
            full = np.kron(full, m)
        u = scipy.linalg.expm(-1j * self.factor * delta_time * full)
        dims = [m.shape[0] for m in mats]
        return NumericOperator(u.reshape(dims + dims), ids)

    def realise_swaps(self, ttn=None, dim=None):
        return self.swaps_before.into_operators(ttn, dim), self.swaps_after.into_operators(ttn, dim)


class TrotterSplitting(list):
    """``time_evolution/trotter.py:196-322``: the Trotter steps in order."""

    def __init__(self, trotter_steps=None):
        super().__init__([] if trotter_steps is None else trotter_steps)

    @classmethod
    def from_lists(cls, tensor_products, splitting=None, swaps_before=None, swaps_after=None):
        """Steps from a list of tensor products: ``splitting`` gives (index,
        factor) pairs (or bare indices, factor 1; default: every product once
        in order); the SWAP lists are indexed like the products."""
        if splitting is None:
            splitting = [(i, 1) for i in range(len(tensor_products))]
        steps = []
        for split in splitting:
            index, factor = (split, 1) if isinstance(split, (int, np.integer)) else (split[0], split[1])
            steps.append(TrotterStep(tensor_products[index], factor,
                                     swaps_before=None if swaps_before is None else swaps_before[index],
                                     swaps_after=None if swaps_after is None else swaps_after[index]))
        return cls(steps)

    def exponentiate_splitting(self, delta_time: float, ttn=None, dim=None) -> list:
        """The gates of one time step: for every step its SWAPs before, the
        exponentiated operator, its SWAPs after."""
        out = []
        for step in self:
            before, after = step.realise_swaps(ttn=ttn, dim=dim)
            out.extend(before)
            out.append(step.exponentiate_operator(delta_time, ttn=ttn, dim=dim))
            out.extend(after)
        return out


class TEBD(RunLoop):
    """``time_evolution/tebd.py:18-155``."""

    def __init__(self, initial_state, trotter_splitting, time_step_size: float, final_time: float,
                 operators, svd_parameters: SVDParameters | None = None,
                 config: TTNTimeEvolutionConfig | None = None, precision: str = "plain"):
        if time_step_size <= 0 or final_time <= 0:
            raise ValueError("time step and final time must be positive")
        self.config = config if config is not None else TTNTimeEvolutionConfig()
        self._trotter_splitting = trotter_splitting
        self.svd_parameters = svd_parameters if svd_parameters is not None else SVDParameters()
        self.time_step_size = float(time_step_size)
        self.final_time = float(final_time)
        self.num_time_steps = compute_num_time_steps(final_time, time_step_size)
        self.operators = init_operators(operators)
        initial_state._finalise()
        self._loschmidt_state = _tensor_copy(initial_state) if getattr(self.config, "record_loschmidt_amplitude", False) else None
        self.initial_state = initial_state
        self.state = initial_state.copy_structure()
        self.state.orthogonality_center_id = None
        self._exponents = trotter_splitting.exponentiate_splitting(self.time_step_size, self.state)
        self.net = DeviceNetwork(self.state, None, precision=precision)
        self._dev_ops = [torch.from_numpy(np.ascontiguousarray(np.asarray(u.operator, dtype=np.complex128)))
                         .to(self.net.device, CDT) for u in self._exponents]
        self.results = None
        self.times = []

    def reset_to_initial_state(self):
        """``TimeEvolution.reset_to_initial_state``: a fresh device copy of the
        initial state, results cleared."""
        self.state = self.initial_state.copy_structure()
        self.state.orthogonality_center_id = None
        self.net = DeviceNetwork(self.state, None, precision=self.net.precision)
        self.results = None
        self.times = []

    @property
    def exponents(self) -> list:
        return self._exponents

    @property
    def trotter_splitting(self):
        return self._trotter_splitting

    def _apply_one_trotter_step(self, index: int):
        """``_apply_one_trotter_step`` (``tebd.py:127-147``)."""
        unitary = self._exponents[index]
        ids = list(unitary.node_identifiers) if not isinstance(unitary.node_identifiers, str) \
            else [unitary.node_identifiers]
        if len(ids) == 0:
            return
        if len(ids) == 1:
            self.net.apply_single_site_gate(ids[0], self._dev_ops[index])
        elif len(ids) == 2:
            a, b = ids
            if self.state.nodes[a].parent != b and self.state.nodes[b].parent != a:
                raise ValueError(f"nodes {a} and {b} are not neighbours; bring them together with SWAP gates")
            self.net.apply_two_site_gate(a, b, self._dev_ops[index], self.svd_parameters)
        else:
            raise NotImplementedError("More than two-site interactions are not implemented.")

    def run_one_time_step(self, **kwargs):
        """Every exponentiated Trotter operator applied once (``tebd.py:149-155``)."""
        for i in range(len(self._exponents)):
            self._apply_one_trotter_step(i)

    def evaluate_operator(self, operator) -> complex:
        """``TTNTimeEvolution.evaluate_operator`` (``time_evolution/ttn_time_evolution.py:181-211``):
        a TensorProduct of one-site operators, or a TTNO on the state's tree."""
        from .ttn import TreeTensorNetworkOperator
        if isinstance(operator, TreeTensorNetworkOperator):
            return self.net.expect_ttno(operator)
        return self.net.expect_local(dict(operator))
