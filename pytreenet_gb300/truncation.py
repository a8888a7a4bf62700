"""Truncation parameters and the singular-value truncation rule.

Mirrors ``SVDParameters`` and ``truncate_singular_values`` of PyTreeNet
(``util/tensor_splitting.py:253-486``). The rule needs only the singular values,
which the GPU SVD copies to the host; it decides the kept rank, and the device
then writes the kept factors into the two node tensors.
"""
from __future__ import annotations

from dataclasses import dataclass
from numbers import Integral
from warnings import warn

import numpy as np


@dataclass
class SVDParameters:
    """``SVDParameters`` (``util/tensor_splitting.py:253-328``).

    Keep s > max(rel_tol * s_0, total_tol) (or, with ``sum_trunc``, drop the
    tail whose squared sum is below total_tol^2), at most ``max_bond_dim``
    values and at least one; ``renorm`` rescales the kept values to the 2-norm
    of all of them. With ``random`` the reference factors by a randomised SVD
    and keeps exactly ``max_bond_dim`` values; the engine keeps the same number
    of exact leading values."""
    max_bond_dim: int = 100
    rel_tol: float = 1e-15
    total_tol: float = 1e-15
    renorm: bool = False
    sum_trunc: bool = False
    sum_renorm: bool = False
    random: bool = False

    def __post_init__(self):
        self.check_truncation_parameters()

    def check_truncation_parameters(self):
        mbd = self.max_bond_dim
        if not isinstance(mbd, Integral) and mbd != float("inf"):
            raise TypeError(f"'max_bond_dim' has to be an integer or inf, not {type(mbd)}!")
        if mbd <= 0:
            raise ValueError("'max_bond_dim' has to be positive.")
        if self.rel_tol < 0 and self.rel_tol != float("-inf"):
            raise ValueError("'rel_tol' has to be positive or -inf.")
        if self.total_tol < 0 and self.total_tol != float("-inf"):
            raise ValueError("'total_tol' has to be positive or -inf.")
        if self.random and self.max_bond_dim == float("inf"):
            raise ValueError("a randomised SVD needs a finite 'max_bond_dim' (its rank)")


def renormalise_singular_values(s: np.ndarray, new_s: np.ndarray) -> np.ndarray:
    """Scale ``new_s`` to the 2-norm of ``s`` (``util/tensor_splitting.py:330-352``)."""
    return new_s * np.linalg.norm(s) / np.linalg.norm(new_s)


def _sum_truncation_index(s: np.ndarray, total_tol: float, norming: bool) -> int:
    """``_sum_truncation_index`` (``util/tensor_splitting.py:353-396``)."""
    normsq = float(np.linalg.norm(s)) ** 2
    if normsq == 0:
        return 0
    acc = 0.0
    for i, v in enumerate(s[::-1]):
        acc += float(v) ** 2
        if (acc / normsq if norming else acc) > total_tol ** 2:
            return len(s) - i
    return 0


def truncate_singular_values(s: np.ndarray, svd_params) -> tuple[np.ndarray, np.ndarray]:
    """(kept, truncated) singular values (``truncate_singular_values``,
    ``util/tensor_splitting.py:448-486``); ``s`` sorted in descending order."""
    s = np.asarray(s, dtype=float)
    if len(s) == 0:
        raise ValueError("No singular values to truncate!")
    if getattr(svd_params, "random", False):
        # ``truncated_tensor_svd`` with ``random`` keeps the max_bond_dim leading
        # values of its randomised factorisation and applies no tolerance
        # (``util/tensor_splitting.py:488-527``); the engine factors exactly and
        # keeps the same number
        k = min(int(svd_params.max_bond_dim), len(s))
        return s[:k].copy(), s[k:]
    if getattr(svd_params, "sum_trunc", False):
        s_temp = s[:_sum_truncation_index(s, svd_params.total_tol, getattr(svd_params, "sum_renorm", False))]
    else:
        cut = max(svd_params.rel_tol * s[0], svd_params.total_tol)
        s_temp = s[s > cut]
    mbd = svd_params.max_bond_dim
    if len(s_temp) > mbd:
        new_s, s_trunc = s_temp[:int(mbd)], s[int(mbd):]
    elif len(s_temp) == 0:
        warn("All singular values were truncated. Returning only the largest singular value.")
        new_s, s_trunc = np.array([s[0]]), s[1:]
    else:
        new_s, s_trunc = s_temp, s[len(s_temp):]
    if getattr(svd_params, "renorm", False):
        new_s = renormalise_singular_values(s, new_s)
    return new_s, s_trunc
