"""Results of a time evolution and the measuring run loop
(``time_evolution/results.py``, ``time_evolution/time_evolution.py:118-368``,
``time_evolution/ttn_time_evolution.py:88-211``).

``Results`` keeps one array per operator name plus the times, with the
reference's accessors. ``RunLoop`` is the ``run`` of the reference's drivers:
operators are named (list -> "0", "1", ...; dict -> its keys; a single
operator -> "0"), measured every ``evaluation_time`` steps (or only at the
end with "inf"), and with the configuration's ``record_*`` flags also the
bond dimensions, their maximum and average, the total size, the norm and
the Loschmidt amplitude <psi(0)|psi(t)>. HDF5 files need h5py, which is not
part of this engine's environment.
"""
from __future__ import annotations

import re
from typing import Any, Hashable

import numpy as np

TIMES_ID = "times"
MAX_BOND_DIM_ID = "max_bond_dim"
AVERAGE_BOND_DIM_ID = "average_bond_dim"
TOTAL_SIZE_ID = "total_size"
BOND_DIM_ATRR = "bond_dim"


class Results:
    """``Results`` (``time_evolution/results.py:17-485``) without the HDF5 files."""

    def __init__(self, metadata: dict[str, Any] | None = None):
        self.results: dict[Hashable, np.ndarray] = {}
        self.attributes: dict[str, list] = {}
        self.metadata = metadata if metadata is not None else {}

    def close_to(self, other: "Results") -> bool:
        if len(self.results) != len(other.results):
            return False
        return all(k in other.results and np.allclose(v, other.results[k]) for k, v in self.results.items())

    def num_results(self) -> int:
        return len([k for k in self.results if k != TIMES_ID])

    def results_length(self) -> int:
        self.not_initialized_error()
        return len(next(iter(self.results.values())))

    def shape(self) -> tuple[int, int]:
        return self.num_results(), self.results_length()

    def is_initialized(self) -> bool:
        return len(self.results) > 0

    def not_initialized_error(self):
        if not self.is_initialized():
            raise ValueError("Results object is not initialized!")

    def initialize(self, operators: dict, num_time_steps: int, with_time: bool = True):
        if self.is_initialized():
            raise ValueError("Results object is already initialized!")
        if with_time:
            self.results[TIMES_ID] = np.zeros((num_time_steps + 1,), dtype=np.float64)
        for op, dtype in operators.items():
            if isinstance(op, int):
                raise ValueError("Operator names mustn't be integers!")
            self.results[op] = np.zeros((num_time_steps + 1,), dtype=np.complex128 if dtype is None else dtype)

    def set_attribute(self, operator_id, attribute_name: str, value):
        if operator_id not in self.results:
            self.attributes[operator_id] = []
        self.attributes.setdefault(operator_id, []).append((attribute_name, value))

    def set_element(self, operator, index: int, value):
        self.results[operator][index] = value

    def get_element(self, operator, index: int):
        return self.results[operator][index]

    def set_operator_result(self, operator, values):
        self.results[operator] = values

    def set_time(self, index: int, time: float):
        self.results[TIMES_ID][index] = time

    def get_time(self, index: int) -> float:
        return self.results[TIMES_ID][index]

    def times(self) -> np.ndarray:
        self.not_initialized_error()
        return self.results[TIMES_ID]

    def result_real(self, operator) -> bool:
        r = self.results.get(operator)
        return bool(np.isrealobj(r) or np.allclose(np.imag(r), 0))

    def results_real(self) -> bool:
        return all(self.result_real(k) for k in self.results)

    def operator_result(self, operator, realise: bool = False) -> np.ndarray:
        self.not_initialized_error()
        r = self.results[operator]
        return np.real(r) if realise and not np.isrealobj(r) else r

    def _desired(self, key, operators) -> bool:
        if operators is None:
            return key != TIMES_ID
        if isinstance(operators, list):
            return key in operators
        if isinstance(operators, re.Pattern):
            if not isinstance(key, str):
                raise TypeError("Operators must be strings to match against a regex pattern!")
            return bool(operators.match(key))
        raise TypeError("Operators must be a list of Hashable or a regex pattern!")

    def get_results(self, operators=None, realise: bool = False) -> dict:
        self.not_initialized_error()
        if isinstance(operators, str):
            operators = re.compile(r"^" + operators + r"\d+$")
        return {k: self.operator_result(k, realise=realise) for k in self.results if self._desired(k, operators)}

    def operator_results(self, operators=None, realise: bool = False) -> np.ndarray:
        """The selected results stacked as rows."""
        return np.array(list(self.get_results(operators, realise).values()))

    def save_to_h5(self, *args, **kwargs):
        raise NotImplementedError("HDF5 results need h5py, which is not available")

    @classmethod
    def load_from_h5(cls, *args, **kwargs):
        raise NotImplementedError("HDF5 results need h5py, which is not available")


def init_operators(operators) -> dict:
    """``TimeEvolution.init_operators`` (``time_evolution.py:118-139``)."""
    from .tdvp import TensorProduct
    from .ttn import TreeTensorNetworkOperator
    if operators is None:
        return {}
    if isinstance(operators, (TensorProduct, TreeTensorNetworkOperator, np.ndarray)):
        return {"0": operators}
    if isinstance(operators, (list, tuple)):
        return {str(i): op for i, op in enumerate(operators)}
    if isinstance(operators, dict):
        return dict(operators)
    return {"0": operators}


class RunLoop:
    """The measuring ``run`` shared by the drivers. A driver provides
    ``operators`` (a dict from ``init_operators``), ``num_time_steps``,
    ``time_step_size``, ``config``, ``run_one_time_step``, ``evaluate_operator``
    and, for tree states, ``state`` (and ``_loschmidt_state`` when the
    Loschmidt amplitude is recorded)."""

    def update_hamiltonian(self):
        raise NotImplementedError("This time evolution has no time-dependent Hamiltonian")

    def _flag(self, name) -> bool:
        return bool(getattr(self.config, name, False))

    def result_init_dictionary(self) -> dict:
        d = {k: complex for k in self.operators}
        if self._flag("record_bond_dim"):
            for key in self.state.bond_dims():
                d[key] = int
                self.results.set_attribute(key, BOND_DIM_ATRR, True)
        if self._flag("record_max_bdim"):
            d[MAX_BOND_DIM_ID] = int
        if self._flag("record_average_bdim"):
            d[AVERAGE_BOND_DIM_ID] = float
        if self._flag("record_total_size"):
            d[TOTAL_SIZE_ID] = int
        if self._flag("record_norm"):
            d["norm"] = complex
        if self._flag("record_loschmidt_amplitude"):
            d["loschmidt_amplitude"] = complex
        return d

    def init_results(self, evaluation_time=1):
        self.results = Results()
        num = 1 if evaluation_time == "inf" else self.num_time_steps // evaluation_time
        self.results.initialize(self.result_init_dictionary(), num)

    def evaluate_operator_values(self) -> list:
        """The current value of every operator, in the order of their names.
        A driver on a device network measures all products of one-site
        operators in one pass over the tree (``DeviceNetwork.expect_many``) and
        each TTNO on its own; the reference evaluates them one at a time
        (``time_evolution/ttn_time_evolution.py:181-197``)."""
        ops = list(self.operators.values())
        net = getattr(self, "net", None)
        if net is None or not hasattr(net, "expect_many"):
            return [self.evaluate_operator(op) for op in ops]
        from .ttn import TreeTensorNetworkOperator
        vals = [None] * len(ops)
        local = [i for i, op in enumerate(ops) if not isinstance(op, TreeTensorNetworkOperator)]
        if local:
            for i, v in zip(local, net.expect_many([ops[i] for i in local])):
                vals[i] = complex(v)
        return [v if v is not None else self.evaluate_operator(op) for v, op in zip(vals, ops)]

    def evaluate_operators_at(self, index: int):
        for key, value in zip(self.operators, self.evaluate_operator_values()):
            self.results.set_element(key, index, value)
        if self._flag("record_bond_dim"):
            for key, value in self.state.bond_dims().items():
                self.results.set_element(key, index, value)
        if self._flag("record_max_bdim"):
            self.results.set_element(MAX_BOND_DIM_ID, index, self.state.max_bond_dim())
        if self._flag("record_average_bdim"):
            self.results.set_element(AVERAGE_BOND_DIM_ID, index, self.state.avg_bond_dim())
        if self._flag("record_total_size"):
            self.results.set_element(TOTAL_SIZE_ID, index, self.state.size())
        if self._flag("record_norm"):
            self.results.set_element("norm", index, self.state.norm())
        if self._flag("record_loschmidt_amplitude"):
            self.results.set_element("loschmidt_amplitude", index,
                                     self.state.scalar_product(other=self._loschmidt_state))

    def evaluate_operators(self):
        """The current expectation values in the order of the operator names."""
        return np.array(self.evaluate_operator_values())

    def run(self, evaluation_time=1, pgbar: bool = True):
        """``TimeEvolution.run`` (``time_evolution.py:346-368``): step, measure
        (every ``evaluation_time`` steps, or only at the end with "inf"), then
        update a time-dependent Hamiltonian. Returns the operator results as an
        array (rows: measurements)."""
        self.init_results(evaluation_time)
        for i in range(self.num_time_steps + 1):
            if i != 0:
                self.run_one_time_step()
            every = evaluation_time != "inf" and i % evaluation_time == 0
            end = evaluation_time == "inf" and i == self.num_time_steps
            if every or end:
                index = 0 if evaluation_time == "inf" else i // evaluation_time
                self.evaluate_operators_at(index)
                self.results.set_time(index, i * self.time_step_size)
            if self._flag("time_dep") and i != 0:
                self.update_hamiltonian()
        self.times = list(self.results.times())
        keys = list(self.operators)
        return np.array([self.results.operator_result(k) for k in keys]).T if keys else np.zeros((0, 0))
