"""Parameter gradients of time-evolved observables by finite differences.

For a Hamiltonian family H(theta) (for example per-site transverse fields
g_i and a coupling J), d<O>(T)/d theta_k is formed from 2 K (central) or
K + 1 (forward) complete time evolutions on the engine. Each evolution is an
ordinary driver run, so every one of them runs on the GPU path; the runs are
independent and can also be spread over ``run_realisations`` workers.
This is the checker for the adjoint in ``adjoint.py`` (one forward and one
backward sweep per gradient, whatever the number of parameters) and the
fallback for parameters the adjoint does not cover.
"""
from __future__ import annotations

from typing import Callable

import numpy as np

from .batch import run_realisations


def finite_difference_gradient(evolve: Callable[[np.ndarray], float], theta: np.ndarray, step: float = 1e-5,
                               central: bool = True, workers: int = 1) -> np.ndarray:
    """Gradient of ``evolve(theta)`` (a real observable after a time evolution)
    by central (default) or forward differences with step ``step``."""
    theta = np.asarray(theta, dtype=float)
    K = theta.size
    points = []
    for k in range(K):
        e = np.zeros(K)
        e[k] = step
        points.append(theta + e)
        if central:
            points.append(theta - e)
    if not central:
        points.append(theta.copy())

    class _Run:
        def __init__(self, p):
            self.p = p
            self.value = None

        def run_one_time_step(self):
            self.value = float(evolve(self.p))
    vals = run_realisations(lambda i: _Run(points[i]), len(points), 1, workers=workers,
                            on_done=lambda i, r: r.value)
    g = np.empty(K)
    for k in range(K):
        if central:
            g[k] = (vals[2 * k] - vals[2 * k + 1]) / (2 * step)
        else:
            g[k] = (vals[k] - vals[-1]) / step
    return g


def tfim_z_root_evolution(n: int = 31, chi: int = 64, dt: float = 0.02, steps: int = 30, seed: int = 0,
                          precision: str = "plain") -> Callable[[np.ndarray], float]:
    """The observable of a gradient study on the heap-ordered binary tree:
    theta = (g_1 .. g_n, J) of H = -J sum Z Z - sum g_i X_i, the state a
    seeded product state zero-padded to ``chi``, ``steps`` first-order
    one-site TDVP steps of ``dt``; returns <Z_root>(T)."""
    from .tdvp import FirstOrderOneSiteTDVP, TDVPConfig, TimeEvoMode, TensorProduct
    from .operators import tfim_ttno
    from .workloads import binary_tfim_product_state
    Z = np.diag([1.0, -1.0]).astype(complex)

    def evolve(theta: np.ndarray) -> float:
        st, _, spec, _ = binary_tfim_product_state(n=n, chi=chi, seed=seed)
        g = {nid: float(theta[i]) for i, (nid, _) in enumerate(spec)}
        H = tfim_ttno(st, J=float(theta[n]), g=g)
        algo = FirstOrderOneSiteTDVP(st, H, dt, dt * steps, {}, config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV),
                                     solver_options={"krylov_tol": 1e-12}, precision=precision)
        for _ in range(steps):
            algo.run_one_time_step()
        return float(np.real(algo.evaluate_operator(TensorProduct({spec[0][0]: Z}))))
    return evolve
