"""Gradients of one-site TDVP observables by a hand-written adjoint on the engine.

The first-order one-site TDVP step (``tdvp_algorithms/firstorderonesite.py:92-104``
with the link update of ``onesitetdvp.py:29-127``) is written here as a pure
function of the site tensors and the TTNO tensors, built from three
differentiable primitives whose forward AND backward passes run in
libptn_gb300:

* ``contract`` -- one pairwise tensor contraction (``ptn_zcontract`` through
  ``ptn_exec_ops``). Its adjoint is two more contractions of the same kind:
  for C = A . op(B), dA = dC . conj(op(B)) over B's free legs and
  dB = dC . conj(A) (or conj(dC) . A when B enters conjugated) over A's.
* ``krylov_expm`` -- y = exp(z H) x for an anti-Hermitian z H (z = c dt, c
  imaginary) with H given by a contraction chain of environments and TTNO
  tensors. Backward: x_bar = exp(-z H) y_bar (another matrix-free Krylov
  exponential), and the parameter gradient of
  Re(z int_0^1 <w(s)| dH |v(s)> ds), with v(s) = exp(s z H) x and
  w(s) = exp(-(1-s) z H) y_bar. Both trajectories live in the Krylov bases
  of x and y_bar; the s-integral of their coefficient products is a small
  matrix M computed exactly from the eigenpairs of the two projections
  (phi_1 functions), and its SVD turns the integral into a few bilinear
  forms <a_r| H |b_r>, whose gradients are one batched pass of the chain
  forward and back.
* ``qr`` -- the Householder QR of ``ptn_zqr_keep`` (LAPACK convention, real
  diagonal of R). Backward: A_bar = [Q_bar + Q herm(N)] R^-H with
  N = R_bar R^H - Q^H Q_bar and herm(N) the Hermitian matrix with N's upper
  triangle and the real part of its diagonal; the k x k factors are formed
  on the host.

``torch.autograd`` only records the order of these calls; every step is
checkpointed (``torch.utils.checkpoint``), so the environments are rebuilt
from the step's input tensors in the backward pass and only the site tensors
of each step boundary stay resident.

The derivative is the derivative of the exact local exponentials; the Krylov
tolerance bounds the difference to the derivative of the truncated series.
QR splits must be tall and of full rank (bond dimensions no larger than the
subtree dimensions): the QR of a rank-deficient matrix has no derivative.
"""
from __future__ import annotations

import ctypes
from typing import Callable

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import _lib
from . import engine as E
from .engine import CDT, KrylovSolver, Operand, Step, Workspace, check, ttno_site_tensors


# ----------------------------------------------------------------------------
# pairwise contraction
# ----------------------------------------------------------------------------
_DESCS: dict = {}


# Contraction precision of the adjoint: 0 = complex128 (ptn_zcontract), 3 =
# BF16x6 tensor-core products with FP32 accumulation (ptn_cgemm_bf16x3). Set
# by OneSiteTDVPAdjoint around its forward and backward passes; the Krylov
# exponentials, QR splits and the phi-function integral stay in FP64.
_LEVELS = {"levels": 0}
_MIXED_PLANS: dict = {}
_MIXED_WS: dict = {}


class _Ptr:
    """A plan operand whose device address is set before each run."""

    def __init__(self):
        self.p = 0

    def data_ptr(self):
        return self.p


def _mixed_contract(a, la, b, lb, lc, klabels, conj_a, conj_b, out, levels):
    key = (tuple(la), tuple(a.shape), tuple(lb), tuple(b.shape), tuple(lc), tuple(klabels),
           bool(conj_a), bool(conj_b), levels)
    ent = _MIXED_PLANS.get(key)
    if ent is None:
        dev = str(a.device)
        ws = _MIXED_WS.setdefault(dev, Workspace(a.device))
        holder = _Ptr()
        dims = {**dict(zip(la, a.shape)), **dict(zip(lb, b.shape))}
        cb = E.ChainBuilder(ws)
        cb.contract(Operand.contiguous(("in",), list(la), list(a.shape)),
                    Operand.contiguous(("fixed", holder), list(lb), list(b.shape)), list(klabels),
                    out=Operand.contiguous(("out",), list(lc), [dims[l] for l in lc]),
                    conj_a=conj_a, conj_b=conj_b)
        ent = (cb.mixed_plan(levels), holder, ws)
        _MIXED_PLANS[key] = ent
    plan, holder, ws = ent
    holder.p = b.data_ptr()
    plan.run(a.data_ptr(), out.data_ptr())
    return out


def _raw_contract(a, la, b, lb, lc, klabels, conj_a=False, conj_b=False, out=None, beta=0.0):
    """C[lc] = beta C + sum_k op(A)[la] op(B)[lb] in one ``ptn_exec_ops`` call
    (on the tensor cores when the adjoint runs in mixed precision and beta = 0)."""
    if a.dtype != CDT or b.dtype != CDT:
        raise TypeError("contractions take complex128 tensors")
    if a.dim() != len(la) or b.dim() != len(lb):
        raise ValueError("one label per leg")
    a = a.contiguous()
    b = b.contiguous()
    dims = dict(zip(la, a.shape))
    for l, d in zip(lb, b.shape):
        if dims.setdefault(l, d) != d:
            raise ValueError(f"dimension mismatch on leg {l}")
    shape_c = [dims[l] for l in lc]
    if out is None:
        if beta != 0.0:
            raise ValueError("beta needs an output tensor")
        out = torch.empty(shape_c, dtype=CDT, device=a.device)
    elif list(out.shape) != shape_c or not out.is_contiguous() or out.dtype != CDT:
        raise ValueError(f"output tensor {tuple(out.shape)} does not match the contraction's {tuple(shape_c)}")
    if _LEVELS["levels"] and beta == 0.0 and klabels:
        return _mixed_contract(a, la, b, lb, lc, klabels, conj_a, conj_b, out, _LEVELS["levels"])
    key = (tuple(la), tuple(a.shape), tuple(lb), tuple(b.shape), tuple(lc), tuple(klabels),
           bool(conj_a), bool(conj_b), complex(beta))
    ent = _DESCS.get(key)
    if ent is None:
        st = Step(Operand.contiguous(("fixed", None), la, list(a.shape)),
                  Operand.contiguous(("fixed", None), lb, list(b.shape)), list(klabels),
                  Operand.contiguous(("fixed", None), lc, shape_c), conj_a=conj_a, conj_b=conj_b, beta=beta)
        ops = (_lib.ExecOp * 1)()
        ops[0].kind = _lib.OP_ZCONTRACT
        ops[0].a, ops[0].b, ops[0].c = 2, 3, 4
        ops[0].desc = ctypes.addressof(st.desc)
        ent = (st, ops)
        _DESCS[key] = ent
    st, ops = ent
    ptrs = (ctypes.c_void_p * 5)(None, None, a.data_ptr(), b.data_ptr(), out.data_ptr())
    check(_lib.load().ptn_exec_ops(ops, 1, ptrs, 5, E._stream_ptr()), "ptn_exec_ops")
    return out


class _Contract(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, b, la, lb, lc, conj_b):
        k = [l for l in la if l in lb]
        if any(l in lc for l in k):
            raise ValueError("a leg shared by both operands must be contracted")
        ctx.save_for_backward(a, b)
        ctx.meta = (la, lb, lc, k, conj_b)
        return _raw_contract(a, la, b, lb, lc, k, conj_b=conj_b)

    @staticmethod
    def backward(ctx, g):
        a, b = ctx.saved_tensors
        la, lb, lc, k, conj_b = ctx.meta
        g = g.contiguous()
        ga = gb = None
        if ctx.needs_input_grad[0]:
            nlab = [l for l in lb if l not in k]
            ga = _raw_contract(g, lc, b, lb, la, nlab, conj_b=not conj_b)
        if ctx.needs_input_grad[1]:
            mlab = [l for l in la if l not in k]
            if conj_b:
                gb = _raw_contract(g, lc, a, la, lb, mlab, conj_a=True)
            else:
                gb = _raw_contract(g, lc, a, la, lb, mlab, conj_b=True)
        return ga, gb, None, None, None, None


def contract(a, la, b, lb, lc, conj_b=False, out=None):
    """Differentiable C[lc] = sum A[la] op(B)[lb] over the legs A and B share.
    With ``out`` (no gradient recorded) the result is written there."""
    if out is not None or not torch.is_grad_enabled() or not (a.requires_grad or b.requires_grad):
        k = [l for l in la if l in lb]
        return _raw_contract(a, la, b, lb, lc, k, conj_b=conj_b, out=out)
    return _Contract.apply(a, b, tuple(la), tuple(lb), tuple(lc), bool(conj_b))


# ----------------------------------------------------------------------------
# local operators (the contraction chains of the site, environment and bond)
# ----------------------------------------------------------------------------
def _site_chain(x, lx, envs, W, n, open_k=None):
    """Environments of the first half of the neighbours, then W, then the rest
    (the order of the engine's matvec). Leaves neighbour ``open_k`` open."""
    ks = [k for k in range(n) if k != open_k]
    half = len(ks) // 2
    T, lT = x, list(lx)
    for k in ks[:half]:
        le = [f"a{k}", f"b{k}", f"c{k}"]
        lnew = [l for l in lT if l != f"a{k}"] + [f"b{k}", f"c{k}"]
        T, lT = contract(T, lT, envs[k], le, lnew), lnew
    lW = [f"b{k}" for k in range(n)] + ["t", "s"]
    cl = [f"b{k}" for k in ks[:half]] + ["s"]
    lnew = [l for l in lT if l not in cl] + [l for l in lW if l not in cl]
    T, lT = contract(T, lT, W, lW, lnew), lnew
    return T, lT, ks[half:]


def site_apply(x, envs, W, batch=False, out=None):
    """y = H_eff x for a site with ``len(envs)`` neighbours (environment k has
    legs (ket, ham, bra) of neighbour k -> site; W legs (neighbours, out, in))."""
    n = len(envs)
    lead = ["r"] if batch else []
    T, lT, rest = _site_chain(x, lead + [f"a{k}" for k in range(n)] + ["s"], envs, W, n)
    for i, k in enumerate(rest):
        last = i == len(rest) - 1
        lnew = (lead + [f"c{j}" for j in range(n)] + ["t"]) if last else \
            [l for l in lT if l not in (f"a{k}", f"b{k}")] + [f"c{k}"]
        T, lT = contract(T, lT, envs[k], [f"a{k}", f"b{k}", f"c{k}"], lnew, out=out if last else None), lnew
    return T


def env_apply(A, envs, W, k0):
    """E(site -> neighbour k0), legs (ket, ham, bra), from the site tensor A,
    W and the environments of the other neighbours."""
    n = A.dim() - 1
    T, lT, rest = _site_chain(A, [f"a{k}" for k in range(n)] + ["s"], envs, W, n, open_k=k0)
    for k in rest:
        lnew = [l for l in lT if l not in (f"a{k}", f"b{k}")] + [f"c{k}"]
        T, lT = contract(T, lT, envs[k], [f"a{k}", f"b{k}", f"c{k}"], lnew), lnew
    lB = [f"c{k}" if k != k0 else "z" for k in range(n)] + ["t"]
    return contract(T, lT, A, lB, [f"a{k0}", f"b{k0}", "z"], conj_b=True)


def bond_apply(r, e_q, e_n, batch=False, out=None):
    """Bond matvec on R (legs: Q side, neighbour side) with E(site -> nbr) = e_q
    and E(nbr -> site) = e_n."""
    lead = ["r"] if batch else []
    T = contract(e_q, ["a", "b", "x"], r, lead + ["a", "c"], ["b", "x"] + lead + ["c"])
    return contract(T, ["b", "x"] + lead + ["c"], e_n, ["c", "b", "y"], lead + ["x", "y"], out=out)


class _SiteOp:
    def __init__(self, n):
        self.n = n

    def apply(self, x, params, batch=False, out=None):
        return site_apply(x, list(params[:self.n]), params[self.n], batch=batch, out=out)


class _BondOp:
    def apply(self, x, params, batch=False, out=None):
        return bond_apply(x, params[0], params[1], batch=batch, out=out)


# ----------------------------------------------------------------------------
# Krylov exponential and its adjoint
# ----------------------------------------------------------------------------
_SOLVERS: dict = {}


def _solver(device) -> KrylovSolver:
    key = str(device)
    if key not in _SOLVERS:
        _SOLVERS[key] = KrylovSolver(Workspace(torch.device(device)))
    return _SOLVERS[key]


def _tensor_apply(op, params, shape):
    def ap(xq, w):
        op.apply(xq.view(shape), params, out=w.view(shape))
    ap.takes_tensors = True
    return ap


def _phi1(z):
    z = np.asarray(z, dtype=complex)
    small = np.abs(z) < 1e-8
    safe = np.where(small, 1.0, z)
    return np.where(small, 1.0 + z / 2 + z * z / 6, np.expm1(safe) / safe)


def coupling_matrix(Tv, beta_v, Tw, beta_w, z):
    """M_ij = int_0^1 conj(a_i(s)) b_j(s) ds with b(s) = beta_v exp(s z Tv) e_1 and
    a(s) = beta_w exp(-(1-s) z Tw) e_1 (Hermitian parts of the projections,
    z imaginary), in closed form from their eigenpairs."""
    lam, P = np.linalg.eigh(0.5 * (Tv + Tv.conj().T))
    mu, S = np.linalg.eigh(0.5 * (Tw + Tw.conj().T))
    p = P[0].conj()
    s = S[0].conj()
    K = np.exp(z * mu)[:, None] * _phi1(z * (lam[None, :] - mu[:, None]))
    return beta_v * beta_w * (S.conj() * s.conj()[None, :]) @ K @ (P * p[None, :]).T


# Deepest Krylov basis of a solve whose operator is a reduced-precision product
# (a guard: the Lanczos stop triggers at the FP64 path's depths, 7-12 here).
MIXED_MAX_KRYLOV_DIM = 96


def _krylov_mode(maxdim):
    """With tensor-core contractions the Krylov exponential projects on the
    Lanczos tridiagonal (alpha_j, beta_j), as the engine's mixed path does: the
    full symmetrised Arnoldi projection turns the operator's rounding far from
    the diagonal into a coupling that keeps its adaptive stop from ever
    triggering. Returns (tridiagonal, max Krylov dimension)."""
    if not _LEVELS["levels"]:
        return False, maxdim
    cap = MIXED_MAX_KRYLOV_DIM if maxdim is None else min(int(maxdim), MIXED_MAX_KRYLOV_DIM)
    return True, cap


class _KrylovExp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op, dt, c, tol, maxdim, *params):
        if abs(complex(c).real) > 0:
            raise ValueError("the adjoint needs an imaginary exponent factor (unitary evolution)")
        x = x.contiguous()
        y = torch.empty_like(x)
        bx = {}
        tri, maxdim = _krylov_mode(maxdim)
        _solver(x.device).expm(x.detach(), _tensor_apply(op, [p.detach() for p in params], x.shape),
                               dt, c, tol, maxdim, out=y, basis=bx, tridiagonal=tri)
        # the basis of x is kept for the backward pass (under checkpointing it
        # lives only while its step is being differentiated)
        ctx.save_for_backward(x, bx["Q"] if bx["m"] else x.new_zeros(0), *params)
        ctx.meta = (op, dt, complex(c), tol, maxdim, bx["T"], bx["beta0"], bx["m"])
        return y

    @staticmethod
    def backward(ctx, gy):
        x, Qx, *params = ctx.saved_tensors
        op, dt, c, tol, maxdim, Tx, beta_x, mx = ctx.meta
        gy = gy.contiguous()
        det = [p.detach() for p in params]
        ap = _tensor_apply(op, det, x.shape)
        solver = _solver(x.device)
        bx = {"Q": Qx, "T": Tx, "beta0": beta_x, "m": mx}
        bw = {}
        gx = torch.empty_like(x)
        tri, maxdim = _krylov_mode(maxdim)
        solver.expm(gy, ap, dt, -c, tol, maxdim, out=gx, basis=bw, tridiagonal=tri)
        grads = [None] * len(params)
        need = list(ctx.needs_input_grad[6:])
        if any(need) and bx["m"] > 0 and bw["m"] > 0:
            z = c * dt
            M = coupling_matrix(bx["T"], bx["beta0"], bw["T"], bw["beta0"], z)
            U, sig, Yh = np.linalg.svd(M)
            # M's singular values fall off geometrically; terms below 1e-13 of the
            # largest change the gradient far below the Krylov tolerance
            keep = int(np.sum(sig > 1e-13 * sig[0])) if sig[0] > 0 else 0
            if keep:
                n = x.numel()
                lib = _lib.load()
                a = torch.empty((keep, n), dtype=CDT, device=x.device)
                b = torch.empty((keep, n), dtype=CDT, device=x.device)
                ca = np.conj(z) * U[:, :keep].conj().T           # rows r: conj(z) conj(U[:, r])
                cb = sig[:keep, None] * Yh[:keep]
                if max(bw["m"], bx["m"]) > 64:
                    raise NotImplementedError("adjoint of a Krylov exponential deeper than 64 vectors")
                for r in range(keep):
                    for coef, basis, dst in ((ca[r], bw["Q"], a[r]), (cb[r], bx["Q"], b[r])):
                        cd = torch.from_numpy(np.ascontiguousarray(coef)).to(x.device)
                        check(lib.ptn_zcombine(basis.data_ptr(), n, basis.shape[0], cd.data_ptr(), dst.data_ptr(), n,
                                               E._stream_ptr()), "zcombine")
                with torch.enable_grad():
                    ps = [p.detach().requires_grad_(nd) for p, nd in zip(params, need)]
                    yb = op.apply(b.view((keep,) + tuple(x.shape)), ps, batch=True)
                    want = [p for p in ps if p.requires_grad]
                    got = torch.autograd.grad(yb, want, grad_outputs=a.view(yb.shape), allow_unused=True)
                it = iter(got)
                grads = [next(it) if nd else None for nd in need]
        return (gx, None, None, None, None, None, *grads)


def krylov_expm(x, op, params, dt, c, tol=1e-12, maxdim=None):
    """Differentiable exp(c dt H(params)) x by the engine's Krylov exponential."""
    return _KrylovExp.apply(x, op, float(dt), complex(c), float(tol), maxdim, *params)


# ----------------------------------------------------------------------------
# QR split and its adjoint
# ----------------------------------------------------------------------------
_ROWOFF: dict = {}


def _rowoff(shape, ax, device):
    key = (tuple(shape), ax, str(device))
    if key not in _ROWOFF:
        strides = [int(np.prod(shape[i + 1:])) for i in range(len(shape))]
        idx = np.zeros(1, dtype=np.int64)
        for a in range(len(shape)):
            if a != ax:
                idx = (idx[:, None] + np.arange(shape[a], dtype=np.int64)[None, :] * strides[a]).reshape(-1)
        _ROWOFF[key] = (torch.from_numpy(idx).to(device), strides[ax])
    return _ROWOFF[key]


def qr_keep_raw(A, ax):
    """Householder QR (``ptn_zqr_keep``, KEEP: Q zero-padded when A is wide)
    with leg ``ax`` as the column index: (Q with A's legs, R k x k)."""
    shape = list(A.shape)
    k = shape[ax]
    m = A.numel() // k
    lib = _lib.load()
    Q = A.detach().contiguous().clone()
    rowoff, cs = _rowoff(shape, ax, A.device)
    R = torch.zeros((k, k), dtype=CDT, device=A.device)
    work = torch.empty(((int(lib.ptn_zqr_work_bytes(m, k)) + 15) // 16,), dtype=CDT, device=A.device)
    check(lib.ptn_zqr_keep(Q.data_ptr(), rowoff.data_ptr(), m, k, cs, R.data_ptr(), work.data_ptr(),
                           E._stream_ptr()), "ptn_zqr_keep")
    return Q, R


class _QR(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, ax):
        k = A.shape[ax]
        m = A.numel() // k
        if m < k:
            raise ValueError(f"QR split of a {m} x {k} matrix: the adjoint needs tall splits "
                             "(bond dimensions no larger than the subtree dimensions)")
        Q, R = qr_keep_raw(A, ax)
        ctx.save_for_backward(Q, R)
        ctx.ax = ax
        return Q, R

    @staticmethod
    def backward(ctx, gQ, gR):
        Q, R = ctx.saved_tensors
        ax = ctx.ax
        n = Q.dim()
        k = Q.shape[ax]
        lab = [f"i{j}" for j in range(n)]
        lp = [l if j != ax else "p" for j, l in enumerate(lab)]
        lq = [l if j != ax else "q" for j, l in enumerate(lab)]
        rows = [l for j, l in enumerate(lab) if j != ax]
        Rh = R.cpu().numpy()
        d = np.abs(np.diag(Rh))
        if d.min() <= 1e-12 * max(d.max(), 1e-300):
            raise ValueError("QR adjoint of a rank-deficient split")
        N = -_raw_contract(Q, lp, gQ.contiguous(), lq, ["p", "q"], rows, conj_a=True).cpu().numpy()
        N += gR.cpu().numpy() @ Rh.conj().T
        Hm = np.triu(N, 1)
        Hm = Hm + Hm.conj().T + np.diag(np.diag(N).real)
        RinvH = np.linalg.inv(Rh).conj().T
        dev = Q.device
        RinvH_d = torch.from_numpy(np.ascontiguousarray(RinvH)).to(dev)
        HR_d = torch.from_numpy(np.ascontiguousarray(Hm @ RinvH)).to(dev)
        # A_bar = Q_bar R^-H + Q (herm(N) R^-H)
        gA = _raw_contract(gQ.contiguous(), lq, RinvH_d, ["q", "p"], lp, ["q"])
        _raw_contract(Q, lq, HR_d, ["q", "p"], lp, ["q"], out=gA, beta=1.0)
        return gA, None


def qr(A, ax):
    """Differentiable Householder QR of A matricised with leg ``ax`` as the
    column index: returns (Q with A's legs, R (k x k; new bond, old bond))."""
    return _QR.apply(A, ax)


def absorb(R, T, ax):
    """T[..., new, ...] = sum_a R[new, a] T[..., a, ...] on leg ``ax``."""
    n = T.dim()
    lT = [f"i{j}" for j in range(n)]
    lout = [l if j != ax else "new" for j, l in enumerate(lT)]
    return contract(T, lT, R, ["new", lT[ax]], lout)


def expect_product(A: dict, nbrs: dict, root: str, ops: dict):
    """<psi| prod_i O_i |psi> (``TTNS.tensor_product_expectation_value``,
    ``ttns/ttns.py:240-264``), differentiable."""
    def rec(nid, toward):
        T = A[nid]
        nb = nbrs[nid]
        n = len(nb)
        lT = [f"a{k}" for k in range(n)] + ["s"]
        if nid in ops:
            O = torch.as_tensor(np.asarray(ops[nid], dtype=np.complex128)).to(T.device)
            T = contract(T, lT, O, ["t", "s"], [f"a{k}" for k in range(n)] + ["t"])
            lT = [f"a{k}" for k in range(n)] + ["t"]
            lT = [l if l != "t" else "s" for l in lT]
        for k, x in enumerate(nb):
            if x == toward:
                continue
            sub = rec(x, nid)
            lnew = [l for l in lT if l != f"a{k}"] + [f"c{k}"]
            T, lT = contract(T, lT, sub, [f"a{k}", f"c{k}"], lnew), lnew
        lB = [f"c{k}" if nb[k] != toward else "z" for k in range(n)] + ["s"]
        if toward is None:
            return contract(T, lT, A[nid], lB, [], conj_b=True)
        k0 = nb.index(toward)
        return contract(T, lT, A[nid], lB, [f"a{k0}", "z"], conj_b=True)
    return rec(root, None)


# ----------------------------------------------------------------------------
# the differentiable sweep
# ----------------------------------------------------------------------------
class _precision:
    """Contraction precision of the adjoint for the duration of a block (the
    backward pass runs inside ``expectation_and_gradient``'s block)."""

    def __init__(self, levels):
        self.levels = levels

    def __enter__(self):
        self.saved = _LEVELS["levels"]
        _LEVELS["levels"] = self.levels

    def __exit__(self, *a):
        _LEVELS["levels"] = self.saved
        if self.levels and a[0] is None:
            # a bounded wait that ran out inside a tensor-core product
            for ws in _MIXED_WS.values():
                st = ws.bufs.get("tc_status")
                if st is not None and int(st.item()) != 0:
                    code = int(st.item())
                    st.zero_()
                    raise _lib.PtnError(code, "tensor-core contraction in the adjoint")


class OneSiteTDVPAdjoint:
    """One-site TDVP (``FirstOrderOneSiteTDVP``, or ``SecondOrderOneSiteTDVP``
    with ``second_order``) as a differentiable
    map (site tensors, TTNO tensors) -> site tensors after ``num_steps`` steps,
    with the observable <psi(T)| prod O_i |psi(T)> and its gradients.

    The initial state is brought into canonical form at the first site of the
    update path by the engine (as the driver does), and with ``normalise``
    scaled to unit norm; gradients with respect to the state are gradients
    with respect to those canonical tensors."""

    def __init__(self, initial_state, hamiltonian, time_step_size: float, num_steps: int,
                 krylov_tol: float = 1e-12, max_krylov_dim=None, use_checkpoint: bool = True,
                 normalise: bool = False, second_order: bool = False, precision: str = "plain"):
        """``precision``: "plain" (complex128 contractions) or "mixed" (every
        contraction of the forward and backward passes as BF16x6 tensor-core
        products with FP32 accumulation; Krylov vectors, QR, the small
        exponentials and the phi-function integral stay FP64)."""
        from .tdvp import leaf_to_root_update_path
        if precision not in ("plain", "mixed"):
            raise ValueError("precision must be 'plain' or 'mixed'")
        self.levels = 3 if precision == "mixed" else 0
        if time_step_size <= 0 or num_steps <= 0:
            raise ValueError("time step and number of steps must be positive")
        initial_state._finalise()
        init = initial_state.copy_structure()
        st = initial_state.copy_structure()
        st._phys = {k: (v.copy() if isinstance(v, np.ndarray) else v.clone()) for k, v in st._phys.items()}
        self.update_path = leaf_to_root_update_path(init)
        self.orth_paths = [st.path_from_to(self.update_path[i], self.update_path[i + 1])[1:]
                           for i in range(len(self.update_path) - 1)]
        self.second_order = bool(second_order)
        bp = list(reversed(self.update_path))
        self.back_path = bp
        self.back_orth = [st.path_from_to(nid, bp[i + 2])[:-1] for i, nid in enumerate(bp[1:-1])] + [[bp[-1]]]
        net = E.DeviceNetwork(st, None)
        if st.orthogonality_center_id is None:
            net.canonical_form(self.update_path[0])
        else:
            net.move_orth_center(self.update_path[0])
        if normalise:
            net.normalise_center()
        self.device = net.device
        self.order = list(st._order)
        self.nbrs = {nid: list(net.nbrs(nid)) for nid in self.order}
        self.root = st.root_id
        self.tree = st
        self.A0 = {nid: net.t[nid].clone() for nid in self.order}
        self.hamiltonian = hamiltonian
        self.W0 = self.ttno_tensors(hamiltonian)
        self.dt = float(time_step_size)
        self.num_steps = int(num_steps)
        self.tol = float(krylov_tol)
        self.maxdim = max_krylov_dim
        self.use_checkpoint = use_checkpoint

    def ttno_tensors(self, hamiltonian) -> dict:
        return {nid: torch.from_numpy(Wn).to(self.device)
                for nid, Wn in ttno_site_tensors(self.tree, hamiltonian).items()}

    def _ax(self, u, v):
        return self.nbrs[u].index(v)

    def _env(self, nid, nxt, A, W, envs):
        nb = self.nbrs[nid]
        ev = [envs[(x, nid)] if x != nxt else None for x in nb]
        return env_apply(A[nid], ev, W[nid], nb.index(nxt))

    def _hop(self, A, a, b):
        Q, R = qr(A[a], self._ax(a, b))
        A[a] = Q
        A[b] = absorb(R, A[b], self._ax(b, a))

    # -- building blocks of the sweeps (functional counterparts of the driver's) --
    def _envs_toward(self, A, W, center) -> dict:
        """All environments pointing toward ``center`` (``init_cache_but_one``)."""
        envs = {}

        def rec(nid, toward):
            for x in self.nbrs[nid]:
                if x != toward:
                    rec(x, nid)
            if toward is not None:
                envs[(nid, toward)] = self._env(nid, toward, A, W, envs)
        rec(center, None)
        return envs

    def _site(self, A, envs, W, nid, factor):
        """``_update_site`` (``tdvp_algorithm.py:183-201``)."""
        nb = self.nbrs[nid]
        params = [envs[(x, nid)] for x in nb] + [W[nid]]
        A[nid] = krylov_expm(A[nid], _SiteOp(len(nb)), params, self.dt * factor, -1j, self.tol, self.maxdim)

    def _link(self, A, envs, W, nid, nxt, factor):
        """``_update_link`` (``onesitetdvp.py:103-127``): QR split toward ``nxt``,
        new environment, backward bond evolution, R absorbed into ``nxt``."""
        Q, R = qr(A[nid], self._ax(nid, nxt))
        A[nid] = Q
        envs[(nid, nxt)] = self._env(nid, nxt, A, W, envs)
        R = krylov_expm(R, _BondOp(), [envs[(nid, nxt)], envs[(nxt, nid)]], self.dt * factor, 1j,
                        self.tol, self.maxdim)
        A[nxt] = absorb(R, A[nxt], self._ax(nxt, nid))

    def _move(self, A, envs, W, path):
        """``_move_orth_and_update_cache_for_path`` (``tdvp_algorithm.py:203-221``)."""
        for prev, cur in zip(path[:-1], path[1:]):
            self._hop(A, prev, cur)
            envs[(prev, cur)] = self._env(prev, cur, A, W, envs)

    def step(self, A: dict, W: dict) -> dict:
        """One time step. First order (``firstorderonesite.py:92-104``): every site
        forward by dt with the links backward in between, then the
        orthogonality centre goes back to the first site and the environments
        are rebuilt. Second order (``secondorderonesite.py:101-193``): a
        half-step sweep along the update path, the last site by dt, and a
        half-step sweep back. Every step starts from environments rebuilt from
        its input tensors; the second-order driver carries them over, and
        they equal the rebuilt ones because each points toward the centre and
        was computed from the tensors as they are."""
        A = dict(A)
        path, op = self.update_path, self.orth_paths
        envs = self._envs_toward(A, W, path[0])
        if not self.second_order:
            for i, nid in enumerate(path):
                if i > 0:
                    self._move(A, envs, W, op[i - 1])
                self._site(A, envs, W, nid, 1.0)
                if i < len(path) - 1:
                    self._link(A, envs, W, nid, op[i][0], 1.0)
                else:
                    back = self.tree.path_from_to(nid, path[0])
                    for a, b in zip(back[:-1], back[1:]):
                        self._hop(A, a, b)
            return A
        for i, nid in enumerate(path[:-1]):
            if i > 0:
                self._move(A, envs, W, op[i - 1])
            self._site(A, envs, W, nid, 0.5)
            self._link(A, envs, W, nid, op[i][0], 0.5)
        center = op[len(path) - 2][0] if len(path) > 1 else path[0]
        self._site(A, envs, W, path[-1], 1.0)
        bp, bo = self.back_path, self.back_orth
        if len(bp) > 1:
            self._link(A, envs, W, center, bp[1], 0.5)
            center = bp[1]
            for i, nid in enumerate(bp[1:-1]):
                idx = i + 1
                self._site(A, envs, W, nid, 0.5)
                sub = bo[idx - 1]
                if sub:
                    self._move(A, envs, W, sub)
                    center = sub[-1]
                self._link(A, envs, W, center, bp[idx + 1], 0.5)
                center = bp[idx + 1]
            self._site(A, envs, W, bp[-1], 0.5)
        return A

    def _step_flat(self, *flat):
        k = len(self.order)
        A = dict(zip(self.order, flat[:k]))
        W = dict(zip(self.order, flat[k:]))
        out = self.step(A, W)
        return tuple(out[nid] for nid in self.order)

    def evolve(self, A: dict, W: dict) -> dict:
        flat = tuple(A[nid] for nid in self.order)
        Wl = tuple(W[nid] for nid in self.order)
        with _precision(self.levels):
            for _ in range(self.num_steps):
                if self.use_checkpoint and torch.is_grad_enabled():
                    flat = checkpoint(self._step_flat, *flat, *Wl, use_reentrant=False)
                else:
                    flat = self._step_flat(*flat, *Wl)
        return dict(zip(self.order, flat))

    def expectation_and_gradient(self, ops: dict, W: dict | None = None, wrt_state: bool = False):
        """Re <psi(T)| prod O_i |psi(T)> and its gradients: a dict node -> dL/dW
        (torch's convention for complex leaves: dL/dRe + i dL/dIm, TTNO legs as
        in ``ttno_tensors``) and, with ``wrt_state``, node -> dL/dA0."""
        W = self.W0 if W is None else W
        Wl = {nid: W[nid].detach().clone().requires_grad_(True) for nid in self.order}
        A = {nid: self.A0[nid].detach().clone().requires_grad_(wrt_state) for nid in self.order}
        with torch.enable_grad(), _precision(self.levels):
            At = self.evolve(A, Wl)
            val = expect_product(At, self.nbrs, self.root, ops)
            loss = val.real.sum()
            want = [Wl[nid] for nid in self.order] + ([A[nid] for nid in self.order] if wrt_state else [])
            got = torch.autograd.grad(loss, want, allow_unused=True)
        gW = {nid: (g if g is not None else torch.zeros_like(Wl[nid])) for nid, g in zip(self.order, got)}
        gA = None
        if wrt_state:
            gA = {nid: (g if g is not None else torch.zeros_like(A[nid]))
                  for nid, g in zip(self.order, got[len(self.order):])}
        return float(loss.detach().cpu()), gW, gA


def coupling_gradient(adj: OneSiteTDVPAdjoint, hamiltonian_of: Callable[[np.ndarray], object],
                      theta, ops: dict, affine_check: float = 1e-12):
    """d Re<psi(T)| prod O_i |psi(T)> / d theta for a TTNO family H(theta) that is
    affine in theta (every coupling multiplies fixed operator entries, as for
    the TFIM fields g_i and the coupling J). The tensors' derivatives are probed
    once per parameter; the chain rule over the TTNO tensors runs on the host."""
    theta = np.asarray(theta, dtype=float)
    base = {k: v.cpu().numpy() for k, v in adj.ttno_tensors(hamiltonian_of(theta)).items()}
    D = []
    for j in range(theta.size):
        e = np.zeros_like(theta)
        e[j] = 1.0
        Wj = {k: v.cpu().numpy() for k, v in adj.ttno_tensors(hamiltonian_of(theta + e)).items()}
        D.append({k: Wj[k] - base[k] for k in base})
        Wh = {k: v.cpu().numpy() for k, v in adj.ttno_tensors(hamiltonian_of(theta + 0.5 * e)).items()}
        err = max(np.max(np.abs(Wh[k] - base[k] - 0.5 * D[-1][k])) for k in base)
        if err > affine_check * max(1.0, max(np.max(np.abs(v)) for v in base.values())):
            raise ValueError(f"the TTNO is not affine in parameter {j} (deviation {err:.2e})")
    W = {k: torch.from_numpy(v).to(adj.device) for k, v in base.items()}
    val, gW, _ = adj.expectation_and_gradient(ops, W)
    gWh = {k: v.cpu().numpy() for k, v in gW.items()}
    grad = np.array([sum(float(np.real(np.vdot(D[j][k], gWh[k]))) for k in base) for j in range(theta.size)])
    return val, grad
