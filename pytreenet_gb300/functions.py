"""PyTreeNet's module-level functions around the path, on the engine's data model.

Each is the reference function of the same name and arguments; the
contractions behind them run on the device through the TTNS methods.

* ``expectation_value(state, operator)``: <psi|H|psi> for a TTNO
  (``contractions/state_operator_contraction.py:26-74``);
* ``contract_two_ttns(ttn1, ttn2)``: the bilinear contraction of two states
  over all legs, no conjugation (``contractions/state_state_contraction.py:29-66``;
  ``scalar_product`` conjugates its argument first);
* ``completely_contract_tree``, ``canonical_form``,
  ``multi_single_site_expectation_value``: the TTN / TTNS methods as functions
  (``contractions/tree_contraction.py:20``, ``core/canonical_form.py:162-208``,
  ``ttns/ttns_util.py:95``);
* ``pauli_matrices``, ``spin_jumps``, ``hadamard``, ``bosonic_operators``
  (``operators/common_operators.py:16-100``);
* ``TDVPUpdatePathFinder(state, mode).find_path()``
  (``time_evolution/time_evo_util/update_path.py:33-61``; its default mode is
  LeafToLeaf, while ``TDVPConfig``'s is LeafToRoot).
"""
from __future__ import annotations

import numpy as np

from .tdvp import PathFinderMode, find_update_path


def expectation_value(state, operator) -> complex:
    return state.ttno_expectation_value(operator)


def contract_two_ttns(ttn1, ttn2, id_trafo=None) -> complex:
    if id_trafo is not None:
        raise NotImplementedError("identifier transformations between the two states are not provided")
    return ttn1.scalar_product(ttn2.conjugate())


def completely_contract_tree(ttn, to_copy: bool = False, order: list | None = None):
    return ttn.completely_contract_tree(to_copy=to_copy, order=order)


def canonical_form(ttn, orthogonality_center_id: str, mode=None):
    ttn.canonical_form(orthogonality_center_id, mode=mode)


def multi_single_site_expectation_value(ttns, operators, move_orth: bool = False) -> dict:
    return ttns.multi_single_site_expectation_value(operators, move_orth=move_orth)


def pauli_matrices() -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """X, Y, Z in the Z basis."""
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
    Z = np.array([[1, 0], [0, -1]], dtype=complex)
    return X, Y, Z


def spin_jumps() -> tuple[np.ndarray, np.ndarray]:
    """S+ = (X + iY) / 2 and S- = (X - iY) / 2."""
    X, Y, _ = pauli_matrices()
    return 0.5 * (X + 1j * Y), 0.5 * (X - 1j * Y)


def hadamard() -> np.ndarray:
    return np.array([[1, 1], [1, -1]], dtype=complex) / np.sqrt(2)


def bosonic_operators(dimension: int = 2) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Creation, annihilation and number operator truncated to ``dimension`` levels."""
    if dimension <= 0:
        raise ValueError("dimension must be positive")
    creation = np.diag(np.sqrt(np.arange(1, dimension)).astype(complex), k=-1)
    annihilation = creation.T
    return creation, annihilation, creation @ annihilation


class TDVPUpdatePathFinder:
    """The order in which a TDVP sweep visits the nodes."""

    def __init__(self, state, mode: PathFinderMode = PathFinderMode.LeafToLeaf):
        if not isinstance(mode, PathFinderMode):
            raise ValueError(f"Unsupported mode: {mode}")
        self.state = state
        self.mode = mode

    def find_path(self) -> list:
        return find_update_path(self.state, self.mode)
