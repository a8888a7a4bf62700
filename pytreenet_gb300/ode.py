"""Explicit Runge-Kutta integration of the local equation y' = c H_eff y on the device.

The reference's ODE modes (``TimeEvoMode.RK45 / RK23 / DOP853``,
``time_evolution/time_evolution.py:595-615``) hand the effective
Schroedinger equation to ``scipy.integrate.solve_ivp`` (SciPy >= 1.15, 1.18.1
where the fixtures were made) with ``t_eval=[dt]``: an embedded explicit
Runge-Kutta pair with adaptive steps, started by the initial-step rule of
Hairer, Norsett & Wanner, "Solving Ordinary Differential Equations I",
Sec. II.4, and controlled by the RMS norm of the embedded error weighted by
atol + rtol max(|y|, |y_new|) (safety 0.9, step factor within [0.2, 10], no
growth right after a rejection). The pairs are Dormand-Prince 5(4) (RK45),
Bogacki-Shampine 3(2) (RK23) and Dormand-Prince 8(5,3) (DOP853, with its
combined fifth/third-order error estimate).

Here the same integration runs on device vectors: every stage is one
``ptn_zcombine`` of the current point and the stored actions (their Butcher
coefficients times h times c, one launch) followed by one H_eff application;
the error vector is another ``ptn_zcombine``; the step decisions are taken on
the host from one weighted norm per trial step. The Butcher tableaux are
read from SciPy's solver classes, so the coefficients are the ones the
reference integrates with. The solution at dt is the endpoint of the last
step (SciPy evaluates its dense output there, which reproduces the endpoint
up to rounding). BDF, an implicit method whose Newton iteration needs the
N x N Jacobian, is not provided.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib
from . import engine as E
from .engine import Workspace, check

SAFETY = 0.9
MIN_FACTOR = 0.2
MAX_FACTOR = 10.0
RK_METHODS = ("RK45", "RK23", "DOP853")


class _Tableau:
    """Butcher tableau of an embedded explicit pair (from SciPy's classes)."""

    def __init__(self, method: str):
        import scipy.integrate as si
        if method not in RK_METHODS:
            raise NotImplementedError(f"ODE method {method!r} is not provided (explicit pairs: {RK_METHODS})")
        cls = getattr(si, method)
        self.method = method
        self.n_stages = int(cls.n_stages)
        self.A = np.asarray(cls.A, dtype=float)[:self.n_stages, :self.n_stages]
        self.B = np.asarray(cls.B, dtype=float)[:self.n_stages]
        self.C = np.asarray(cls.C, dtype=float)[:self.n_stages]
        if method == "DOP853":
            self.E = None
            self.E3 = np.asarray(cls.E3, dtype=float)
            self.E5 = np.asarray(cls.E5, dtype=float)
        else:
            self.E = np.asarray(cls.E, dtype=float)
        self.error_exponent = -1.0 / (int(cls.error_estimator_order) + 1)
        self.order = int(cls.error_estimator_order)


_TABLEAUX: dict[str, _Tableau] = {}


def tableau(method: str) -> _Tableau:
    if method not in _TABLEAUX:
        _TABLEAUX[method] = _Tableau(method)
    return _TABLEAUX[method]


class RungeKuttaSolver:
    """Adaptive explicit Runge-Kutta exponential action on device vectors."""

    def __init__(self, ws: Workspace):
        self.ws = ws
        self.steps: list[int] = []      # accepted steps per integration
        self.evaluations: list[int] = []

    # -- device pieces -------------------------------------------------------------
    def _combine(self, rows: torch.Tensor, coeffs, out: torch.Tensor):
        lib = _lib.load()
        n = out.numel()
        c = np.ascontiguousarray(np.asarray(coeffs, dtype=np.complex128))
        cdev = self.ws.get("ode_c", 64)[:len(c)]
        cdev.copy_(torch.from_numpy(c).to(cdev.device))
        check(lib.ptn_zcombine(rows.data_ptr(), n, len(c), cdev.data_ptr(), out.data_ptr(), n, E._stream_ptr()),
              "zcombine")

    @staticmethod
    def _rms(v: torch.Tensor, scale: torch.Tensor) -> float:
        return float(torch.linalg.vector_norm(v / scale).item()) / math.sqrt(v.numel())

    def integrate(self, x: torch.Tensor, apply, dt: float, exp_factor: complex, method: str = "RK45",
                  atol: float = 1e-10, rtol: float = 1e-10, max_step: float = math.inf,
                  first_step: float | None = None, out: torch.Tensor | None = None, **ignored) -> torch.Tensor:
        """y(dt) for y' = exp_factor H y, y(0) = x, where ``apply(xp, yp)``
        writes H applied to the vector at ``xp`` into ``yp`` (device pointers,
        or tensors when ``apply.takes_tensors``; with ``apply.takes_time`` it
        is called as ``apply(t, xp, yp)`` for an operator H(t)). Options that
        SciPy ignores for explicit methods (``jac``, ``lband``, ...) are
        accepted and ignored."""
        tab = tableau(method)
        if rtol < 100 * np.finfo(float).eps:
            rtol = 100 * np.finfo(float).eps
        if max_step <= 0:
            raise ValueError("`max_step` must be positive.")
        n = x.numel()
        out = x if out is None else out
        s = tab.n_stages
        # rows: 0 = y, 1 + i = H k_i for the stages, 1 + s = H y_new (FSAL)
        S = self.ws.get("ode_rows", (s + 2) * n)[:(s + 2) * n].view(s + 2, n)
        tmp = self.ws.get("ode_tmp", n)[:n]
        ynew = self.ws.get("ode_ynew", n)[:n]
        tensor_apply = getattr(apply, "takes_tensors", False)
        timed = getattr(apply, "takes_time", False)
        evals = 0

        def H(src: torch.Tensor, dst: torch.Tensor, at: float):
            nonlocal evals
            evals += 1
            a, b = (src, dst) if tensor_apply else (src.data_ptr(), dst.data_ptr())
            if timed:
                apply(at, a, b)
            else:
                apply(a, b)

        S[0].copy_(x.reshape(-1))
        t, t_bound = 0.0, float(dt)
        if t_bound == 0.0:
            if out.data_ptr() != x.data_ptr():
                out.copy_(x)
            return out
        ef = complex(exp_factor)
        # a negative dt integrates backward from 0 to dt, as solve_ivp does
        direction = 1.0 if t_bound > 0 else -1.0
        interval = abs(t_bound)
        H(S[0], S[1], t)
        # initial step (Hairer, Norsett & Wanner II.4; SciPy's select_initial_step)
        if first_step is not None:
            if first_step <= 0 or first_step > interval:
                raise ValueError("`first_step` must be positive and not exceed the interval")
            h_abs = float(first_step)
        else:
            y0 = S[0]
            f0 = S[1] * ef
            scale = atol + y0.abs() * rtol
            d0, d1 = self._rms(y0, scale), self._rms(f0, scale)
            h0 = 1e-6 if (d0 < 1e-5 or d1 < 1e-5) else 0.01 * d0 / d1
            h0 = min(h0, interval)
            self._combine(S[:2], [1.0, h0 * direction * ef], tmp)
            H(tmp, ynew, t + h0 * direction)
            d2 = self._rms((ynew - S[1]) * ef, scale) / h0
            if d1 <= 1e-15 and d2 <= 1e-15:
                h1 = max(1e-6, h0 * 1e-3)
            else:
                h1 = (0.01 / max(d1, d2)) ** (1.0 / (tab.order + 1))
            h_abs = min(100 * h0, h1, interval, max_step)
        accepted_steps = 0
        while direction * (t - t_bound) < 0:
            min_step = 10 * abs(np.nextafter(t, direction * np.inf) - t)
            h_abs = min(max(h_abs, min_step), max_step)
            rejected = False
            while True:
                if h_abs < min_step:
                    raise _lib.PtnError(3, f"{method}: required step size is less than spacing between numbers")
                t_new = t + h_abs * direction
                if direction * (t_new - t_bound) > 0:
                    t_new = t_bound
                h = t_new - t
                h_abs = abs(h)
                for i in range(1, s):
                    self._combine(S[:1 + i], [1.0] + [h * ef * a for a in tab.A[i, :i]], tmp)
                    H(tmp, S[1 + i], t + tab.C[i] * h)
                self._combine(S[:1 + s], [1.0] + [h * ef * b for b in tab.B], ynew)
                H(ynew, S[1 + s], t + h)
                scale = atol + torch.maximum(S[0].abs(), ynew.abs()) * rtol
                if tab.E is not None:
                    self._combine(S[1:2 + s], [h * ef * e for e in tab.E], tmp)
                    err = self._rms(tmp, scale)
                else:
                    self._combine(S[1:2 + s], [ef * e for e in tab.E5], tmp)
                    e5 = float(torch.linalg.vector_norm(tmp / scale).item()) ** 2
                    self._combine(S[1:2 + s], [ef * e for e in tab.E3], tmp)
                    e3 = float(torch.linalg.vector_norm(tmp / scale).item()) ** 2
                    err = 0.0 if (e5 == 0 and e3 == 0) else abs(h) * e5 / math.sqrt((e5 + 0.01 * e3) * n)
                if err < 1:
                    factor = MAX_FACTOR if err == 0 else min(MAX_FACTOR, SAFETY * err ** tab.error_exponent)
                    if rejected:
                        factor = min(1.0, factor)
                    h_abs *= factor
                    break
                h_abs *= max(MIN_FACTOR, SAFETY * err ** tab.error_exponent)
                rejected = True
            t = t_new
            S[0].copy_(ynew)
            S[1].copy_(S[1 + s])
            accepted_steps += 1
        self.steps.append(accepted_steps)
        self.evaluations.append(evals)
        out.view(-1).copy_(S[0])
        return out
