"""Exact (state-vector) time evolution on the device (``time_evolution/exact_time_evolution.py``).

A validation tool for small systems: the state is a dense vector (or, with
``config.open``, a vectorised density matrix) and the Hamiltonian a dense
matrix. As in the reference, the one-step propagator exp(-i dt H) is formed
once with ``scipy.linalg.expm`` on the host; every step multiplies it into the
device-resident state (``ptn_zcontract``) and expectation values are the
contractions <psi|O|psi> (or tr(O rho)) on the device.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np
import scipy.linalg
import torch

from . import engine as E
from .adjoint import _raw_contract
from .engine import CDT
from .results import RunLoop, init_operators
from .tdvp import compute_num_time_steps


@dataclass
class ExactTimeEvolutionConfig:
    """``exact_time_evolution.py:12-20``."""
    open: bool = False


class ExactTimeEvolution(RunLoop):
    """``ExactTimeEvolution(initial_state, hamiltonian, time_step_size, final_time,
    operators, config=None, solver_options=None)`` with ``run_one_time_step``,
    ``evaluate_operator`` and ``run``."""

    config_class = ExactTimeEvolutionConfig

    def __init__(self, initial_state, hamiltonian, time_step_size: float, final_time: float, operators,
                 config: ExactTimeEvolutionConfig | None = None, solver_options: dict[str, Any] | None = None,
                 device=None):
        if time_step_size <= 0 or final_time <= 0:
            raise ValueError("time step and final time must be positive")
        if not torch.cuda.is_available():
            raise RuntimeError("pytreenet_gb300 needs a CUDA device (no CPU fallback)")
        self.config = config if config is not None else self.config_class()
        self.device = torch.device(device or E.DEFAULT_DEVICE)
        self.time_step_size = float(time_step_size)
        self.final_time = float(final_time)
        self.num_time_steps = compute_num_time_steps(final_time, time_step_size)
        self.operators = init_operators(operators)
        self.hamiltonian = np.asarray(hamiltonian, dtype=complex)
        u = scipy.linalg.expm(-1j * self.time_step_size * self.hamiltonian)
        self._u = torch.from_numpy(np.ascontiguousarray(u)).to(self.device, CDT)
        self._psi = torch.from_numpy(np.ascontiguousarray(np.asarray(initial_state, dtype=complex))).to(self.device, CDT)
        self._dev_ops: dict = {}
        self.results = None
        self.times = []

    @property
    def state(self) -> np.ndarray:
        return self._psi.cpu().numpy()

    def run_one_time_step(self, **kwargs):
        self._psi = _raw_contract(self._u, ["i", "j"], self._psi, ["j"], ["i"], ["j"])

    def _dev(self, operator):
        key = id(operator)
        if key not in self._dev_ops:
            self._dev_ops[key] = (operator, torch.from_numpy(
                np.ascontiguousarray(np.asarray(operator, dtype=complex))).to(self.device, CDT))
        return self._dev_ops[key][1]

    def evaluate_operator(self, operator) -> complex:
        """<psi| O |psi>, or tr(O rho) for an open system (``exact_time_evolution.py:88-105``)."""
        O = self._dev(operator)
        if self.config.open:
            dim = O.shape[0]
            rho = self._psi.view(dim, dim)
            return complex(_raw_contract(O, ["i", "j"], rho, ["j", "i"], [], ["i", "j"]).item())
        opsi = _raw_contract(O, ["i", "j"], self._psi, ["j"], ["i"], ["j"])
        return complex(_raw_contract(self._psi, ["i"], opsi, ["i"], [], ["i"], conj_a=True).item())
