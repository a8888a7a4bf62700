"""Local exponentials of a dense matrix or an action, on the device.

PyTreeNet's module functions ``time_evolve`` and ``krylov_exp_action``
(``time_evolution/time_evolution.py:657-821``) with the same arguments:

* ``time_evolve(psi, hamiltonian, time_difference, forward, mode, **options)``
  evolves psi by exp(-/+ i dt H) for a dense H. H goes to the device once and
  every application is one ``ptn_zcontract`` (a complex matrix-vector
  product); KRYLOV runs the engine's Lanczos exponential, RK45 / RK23 /
  DOP853 the Runge-Kutta integration with ``solve_ivp``'s steps, the exact
  modes (FASTEST, EXPM, CHEBYSHEV, SPARSE) the Arnoldi exponential to a
  1e-14 stop. As in the reference the mode's default
  options are laid under the caller's (``time_evolution.py:686-694``), and
  ``exp_factor`` replaces the forward factor -i (backward: its negation).
* ``krylov_exp_action(psi, action, time_difference, exp_factor, krylov_tol,
  max_krylov_dim, hermitian)``: ``action`` maps an array of psi's shape to
  one of the same shape. A NumPy action is the caller's host code (each
  Krylov step copies the vector to the host and back); an action written on
  torch tensors runs where they live and no copy is made.
* ``TimeEvoMode.time_evolve_action`` / ``TimeEvoMode.time_evolve``: the
  enum's methods, with the caller's options only.

NumPy inputs give NumPy results, device tensors device tensors.
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine as E
from .engine import CDT
from .tdvp import EXACT_KRYLOV_TOL, EvoDirection, TimeEvoMode, ode_options


def _to_device(psi):
    if isinstance(psi, torch.Tensor):
        return psi.to(E.DEFAULT_DEVICE if psi.device.type == "cpu" else psi.device, CDT).contiguous(), False
    return torch.from_numpy(np.ascontiguousarray(np.asarray(psi, dtype=np.complex128))).to(E.DEFAULT_DEVICE), True


def _solvers(device):
    from .adjoint import _solver
    from .ode import RungeKuttaSolver
    kry = _solver(device)
    rk = getattr(kry, "_rk", None)
    if rk is None:
        rk = kry._rk = RungeKuttaSolver(kry.ws)
    return kry, rk


def _tensor_action(fn):
    fn.takes_tensors = True
    return fn


def _host_or_device_action(action, shape, numpy_action: bool):
    if numpy_action:
        def ap(xq, w):
            y = np.asarray(action(xq.detach().cpu().numpy().reshape(shape)), dtype=np.complex128)
            w.copy_(torch.from_numpy(np.ascontiguousarray(y).reshape(-1)).to(w.device))
    else:
        def ap(xq, w):
            w.copy_(action(xq.view(shape)).reshape(-1))
    return _tensor_action(ap)


def krylov_exp_action(psi, action, time_difference: float, exp_factor: complex, krylov_tol: float = 1e-10,
                      max_krylov_dim: int | None = None, hermitian: bool = True):
    """exp(exp_factor dt A) psi for the operator ``action`` by the matrix-free
    Lanczos (``hermitian``) or Arnoldi exponential with the reference's
    adaptive stop (``krylov_exp_action``, ``time_evolution.py:721-821``)."""
    x, was_numpy = _to_device(psi)
    shape = tuple(x.shape)
    kry, _ = _solvers(x.device)
    apply = _host_or_device_action(action, shape, was_numpy)
    out = torch.empty_like(x)
    kry.expm(x.reshape(-1), apply, time_difference, exp_factor, krylov_tol, max_krylov_dim,
             hermitian=hermitian, out=out.view(-1))
    return out.cpu().numpy() if was_numpy else out


def _exp_factor(forward, override) -> complex:
    if isinstance(forward, bool):
        forward = EvoDirection.from_bool(forward)
    if override is None:
        return forward.exp_factor()
    return override if forward is EvoDirection.FORWARD else -override


def time_evolve_action(mode: TimeEvoMode, psi, time_evo_action, time_difference: float,
                       forward=EvoDirection.FORWARD, **options):
    """``TimeEvoMode.time_evolve_action`` (``time_evolution.py:536-615``):
    psi evolved under y' = c A(t) y with A given as ``time_evo_action(t, y)``
    (NumPy or torch, as for ``krylov_exp_action``). KRYLOV calls it at t = 0;
    the Runge-Kutta modes at their stage times. ``exp_factor`` and
    ``hermitian`` are read here; options the mode does not read are ignored."""
    options = dict(options)
    exp_factor = _exp_factor(forward, options.pop("exp_factor", None))
    hermitian = options.pop("hermitian", True)
    if mode is TimeEvoMode.KRYLOV:
        return krylov_exp_action(psi, lambda y: time_evo_action(0.0, y), time_difference, exp_factor,
                                 krylov_tol=options.get("krylov_tol", 1e-10),
                                 max_krylov_dim=options.get("max_krylov_dim"), hermitian=hermitian)
    if not mode.is_scipy():
        raise NotImplementedError("The time evolution via action is not implemented for this mode: "
                                  + str(mode.value))
    if mode is TimeEvoMode.BDF:
        raise NotImplementedError("the implicit BDF solver is not provided")
    x, was_numpy = _to_device(psi)
    shape = tuple(x.shape)
    _, rk = _solvers(x.device)
    if was_numpy:
        def ap(t, xq, w):
            y = np.asarray(time_evo_action(t, xq.detach().cpu().numpy().reshape(shape)), dtype=np.complex128)
            w.copy_(torch.from_numpy(np.ascontiguousarray(y).reshape(-1)).to(w.device))
    else:
        def ap(t, xq, w):
            w.copy_(time_evo_action(t, xq.view(shape)).reshape(-1))
    ap.takes_time = True
    _tensor_action(ap)
    out = torch.empty_like(x)
    rk.integrate(x.reshape(-1), ap, time_difference, exp_factor, out=out.view(-1), **ode_options(mode, options))
    return out.cpu().numpy() if was_numpy else out


def evolve_dense(mode: TimeEvoMode, psi, hamiltonian, time_difference: float, forward, options: dict):
    """``TimeEvoMode.time_evolve`` (``time_evolution.py:617-655``) for a dense
    H with exactly the caller's options (an ODE mode given none runs at
    ``solve_ivp``'s own tolerances); options the mode does not read are
    ignored, as in the reference."""
    from .adjoint import _raw_contract
    if mode is TimeEvoMode.BDF:
        raise NotImplementedError("the implicit BDF solver is not provided")
    opts = dict(options)
    exp_factor = _exp_factor(forward, opts.pop("exp_factor", None))
    x, was_numpy = _to_device(psi)
    n = x.numel()
    Hd, _ = _to_device(hamiltonian)
    Hd = Hd.to(x.device)
    if tuple(Hd.shape) != (n, n):
        raise ValueError(f"Hamiltonian of shape {tuple(Hd.shape)} does not act on a vector of {n} entries")

    def ap(xq, w):
        _raw_contract(Hd, ["i", "j"], xq, ["j"], ["i"], ["j"], out=w)
    ap = _tensor_action(ap)
    kry, rk = _solvers(x.device)
    out = torch.empty(n, dtype=CDT, device=x.device)
    ode = ode_options(mode, opts)
    if ode is not None:
        rk.integrate(x.reshape(-1), ap, time_difference, exp_factor, out=out, **ode)
    elif mode is TimeEvoMode.KRYLOV:
        kry.expm(x.reshape(-1), ap, time_difference, exp_factor, opts.get("krylov_tol", 1e-10),
                 opts.get("max_krylov_dim"), hermitian=opts.get("hermitian", True), out=out)
    else:
        # the exact modes: the Krylov exponential to machine precision, with
        # the general (Arnoldi) projection since H need not be Hermitian here
        # and no cap on the basis (at n vectors the projection is exact)
        kry.expm(x.reshape(-1), ap, time_difference, exp_factor, EXACT_KRYLOV_TOL["plain"],
                 None, hermitian=False, out=out)
    out = out.view(x.shape)
    return out.cpu().numpy() if was_numpy else out


def time_evolve(psi, hamiltonian, time_difference: float, forward=EvoDirection.FORWARD,
                mode: TimeEvoMode = TimeEvoMode.FASTEST, **options):
    """psi(t +/- dt) = exp(-/+ i H dt) psi for a dense matrix H
    (``time_evolve``, ``time_evolution.py:657-694``): the mode's default
    options laid under the caller's."""
    opts = TimeEvoMode.default_solver_options(mode)
    opts.update(options)
    return evolve_dense(mode, psi, hamiltonian, time_difference, forward, opts)
