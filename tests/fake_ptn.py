"""NumPy stand-in for libptn_gb300 used by the host-logic tests on CPU.

It implements the C ABI's semantics (include/ptn_gb300.h) on host memory so
the engine's planning code (strides, leg orders, QR row tables, Krylov
control flow) can be exercised without a GPU. It is test infrastructure: the
product never loads it, and GPU tests load the real library.
"""
import ctypes

import numpy as np


def _view(ptr, n, dtype=np.complex128):
    itemsize = np.dtype(dtype).itemsize
    buf = (ctypes.c_char * (int(n) * itemsize)).from_address(int(ptr))
    return np.frombuffer(buf, dtype=dtype, count=int(n))


def _extent(dims, strides):
    return 1 + sum((d - 1) * s for d, s in zip(dims, strides))


def _strided(ptr, dims, strides):
    n = _extent(dims, strides)
    base = _view(ptr, n)
    return np.lib.stride_tricks.as_strided(base, shape=tuple(dims),
                                           strides=tuple(16 * s for s in strides), writeable=True)


class FakeLib:
    calls = 0

    def ptn_zcontract(self, desc_ref, stream):
        d = desc_ref._obj
        self.calls += 1

        def grp(m, which):
            dims = [m.dim[i] for i in range(m.n)]
            return dims, [getattr(m, which)[i] for i in range(m.n)]
        md, ma = grp(d.m, "stride_a")
        _, mc = grp(d.m, "stride_c")
        nd, nb = grp(d.n, "stride_b")
        _, nc = grp(d.n, "stride_c")
        kd, ka = grp(d.k, "stride_a")
        _, kb = grp(d.k, "stride_b")
        A = _strided(d.A, md + kd, ma + ka).reshape(int(np.prod(md)), int(np.prod(kd)))
        B = _strided(d.B, kd + nd, kb + nb).reshape(int(np.prod(kd)), int(np.prod(nd)))
        if d.conj_a:
            A = A.conj()
        if d.conj_b:
            B = B.conj()
        res = (complex(d.alpha_re, d.alpha_im) * (A @ B)).reshape(md + nd)
        C = _strided(d.C, md + nd, mc + nc)
        beta = complex(d.beta_re, d.beta_im)
        if beta != 0:
            res = res + beta * C
        C[...] = res
        return 0

    def ptn_krylov_partials(self, n):
        return 64

    def ptn_zdot_multi(self, Q, ldq, nq, w, n, h, acc, part, stream):
        Qm = _view(Q, (nq - 1) * ldq + n).copy()
        wv = _view(w, n)
        hv = _view(h, nq)
        vals = np.array([np.vdot(Qm[i * ldq:i * ldq + n], wv) for i in range(nq)])
        hv[:] = hv + vals if acc else vals
        return 0

    def ptn_zaxpy_multi(self, Q, ldq, nq, h, w, n, stream):
        Qm = _view(Q, (nq - 1) * ldq + n)
        hv = _view(h, nq)
        wv = _view(w, n)
        for i in range(nq):
            wv -= hv[i] * Qm[i * ldq:i * ldq + n]
        return 0

    def ptn_dznrm2(self, w, n, out, part, stream):
        _view(out, 1, np.float64)[0] = np.linalg.norm(_view(w, n))
        return 0

    def ptn_zscal_inv(self, w, scale, y, n, stream):
        s = _view(scale, 1, np.float64)[0]
        _view(y, n)[:] = _view(w, n) / s
        return 0

    def ptn_zcombine(self, Q, ldq, nq, c, out, n, stream):
        Qm = _view(Q, (nq - 1) * ldq + n)
        cv = _view(c, nq)
        o = np.zeros(n, dtype=complex)
        for i in range(nq):
            o += cv[i] * Qm[i * ldq:i * ldq + n]
        _view(out, n)[:] = o
        return 0

    def ptn_zqr_work_bytes(self, m, k):
        return 16

    def ptn_zqr_keep(self, A, rowoff, m, k, cs, R, work, stream):
        ro = _view(rowoff, m, np.int64)
        ext = int(ro.max()) + (k - 1) * cs + 1
        a = _view(A, ext)
        idx = ro[:, None] + np.arange(k)[None, :] * cs
        mat = a[idx]
        q, r = np.linalg.qr(mat, mode="reduced")
        if q.shape[1] < k:
            q = np.pad(q, [(0, 0), (0, k - q.shape[1])])
            r = np.pad(r, [(0, k - r.shape[0]), (0, 0)])
        a[idx] = q
        _view(R, k * k)[:] = r.reshape(-1)
        return 0

    def ptn_check_finite(self, x, n, flag, stream):
        if not np.all(np.isfinite(_view(x, n))):
            _view(flag, 1, np.int32)[0] = 1
        return 0


def install(monkeypatch):
    """Route the engine to FakeLib and host tensors."""
    import torch
    import pytreenet_gb300._lib as L
    import pytreenet_gb300.engine as E
    fake = FakeLib()
    monkeypatch.setattr(L, "load", lambda: fake)
    monkeypatch.setattr(E, "_stream_ptr", lambda: None)
    monkeypatch.setattr(E, "DEFAULT_DEVICE", "cpu")
    monkeypatch.setattr(torch.cuda, "is_available", lambda: True)
    return fake
