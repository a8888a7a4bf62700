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

    def ptn_zscal_ratio(self, w, num, den, y, n, stream):
        a, b = _view(num, 1, np.float64)[0], _view(den, 1, np.float64)[0]
        f = a / b if b > 0 else 1.0
        _view(y, n)[:] = _view(w, n) * f
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


# ---- mixed-precision entry points (BF16 hi/lo splits emulated in NumPy) ----------
def _bf16_bits(x):
    """float64 -> bf16 bit patterns (round to nearest even), as uint16."""
    f = np.asarray(x, dtype=np.float32).view(np.uint32)
    rounded = f + 0x7FFF + ((f >> 16) & 1)
    return (rounded >> 16).astype(np.uint16)


def _bf16_val(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def _split_levels(v, L):
    # the library's split: the first piece from the double, its remainder
    # (exact in double) rounded once to FP32, the later pieces split in FP32
    b = _bf16_bits(v)
    out = [b]
    r = (v - _bf16_val(b)).astype(np.float32)
    for _ in range(1, L):
        b = _bf16_bits(r)
        out.append(b)
        r = (r - _bf16_val(b).astype(np.float32)).astype(np.float32)
    return out


def _modes(m, field):
    return [m.dim[i] for i in range(m.n)], [getattr(m, field)[i] for i in range(m.n)]


def _offsets(dims, strides):
    idx = np.zeros(1, dtype=np.int64)
    for d, s in zip(dims, strides):
        idx = (idx[:, None] + np.arange(d, dtype=np.int64)[None, :] * s).reshape(-1)
    return idx


def _gather(ptr, rows, cols, conj):
    rd, rs = _modes(rows, "stride_a")
    cd, cs = _modes(cols, "stride_a")
    ro, co = _offsets(rd, rs), _offsets(cd, cs)
    ext = int(ro.max() + co.max()) + 1
    src = _view(ptr, ext)
    v = src[ro[:, None] + co[None, :]]
    return v.conj() if conj else v


def _fake_to_planes(self, d_ref, stream):
    d = d_ref._obj
    v = _gather(d.src, d.rows, d.cols, d.conj)
    M, K = v.shape
    L = d.levels
    dst = _view(d.dst, (2 * L - 1) * d.plane + M * d.ld, np.uint16)
    for p, part in enumerate([v.real, v.imag]):
        for lvl, arr in enumerate(_split_levels(part, L)):
            plane = (2 * lvl + p) * d.plane
            blk = dst[plane:plane + M * d.ld].reshape(M, d.ld)
            blk[:, :K] = arr
    return 0


def _fake_expand_b(self, d_ref, stream):
    d = d_ref._obj
    v = _gather(d.src, d.rows, d.cols, d.conj)
    N, K = v.shape
    L = d.levels
    blk = N * d.ld
    dst = _view(d.dst, 3 * L * blk, np.uint16)
    re = _split_levels(v.real, L)
    im = _split_levels(v.imag, L)
    for lv in range(L):
        for b, arr in enumerate([_bf16_bits(-_bf16_val(im[lv])), re[lv], im[lv]]):
            i = 3 * lv + b
            dst[i * blk:(i + 1) * blk].reshape(N, d.ld)[:, :K] = arr
    return 0


def _fake_cgemm(self, d_ref, stream):
    d = d_ref._obj
    M, K, N, L = d.M, d.K, d.N, d.levels
    # the library's argument checks (ptn_cgemm_bf16x3): lda a multiple of 8
    # except on the CUDA-core path (K <= 32, N <= 128), ldb always, planes too
    smallk = K <= 32 and N <= 128
    if (not smallk and d.lda % 8) or d.ldb % 8 or d.lda < K or d.ldb < K or d.a_plane % 8:
        return 1
    a = _view(d.A, (2 * L - 1) * d.a_plane + M * d.lda, np.uint16)

    def plane(p):
        return _bf16_val(a[p * d.a_plane:p * d.a_plane + M * d.lda].reshape(M, d.lda)[:, :K])
    A = sum(plane(2 * lv) + 1j * plane(2 * lv + 1) for lv in range(L))
    b = _view(d.Bx, 3 * L * N * d.ldb, np.uint16)

    def blk(i):
        return _bf16_val(b[i * N * d.ldb:(i + 1) * N * d.ldb].reshape(N, d.ldb)[:, :K])
    B = sum(blk(3 * lv + 1) + 1j * blk(3 * lv + 2) for lv in range(L))
    # FP32 accumulation, as the tensor cores: the rounding error scales with
    # sum |a||b|, not with |C|
    C = (A.astype(np.complex64) @ B.T.astype(np.complex64)).astype(np.complex128)
    md, ms = _modes(d.m_out, "stride_c")
    nd, ns = _modes(d.n_out, "stride_c")
    off = _offsets(md, ms)[:, None] + _offsets(nd, ns)[None, :]
    C = C.astype(np.complex64).astype(np.complex128)
    if d.out_kind == 0:
        out = _view(d.C, int(off.max()) + 1)
        out[off] = C
    else:
        out = _view(d.C, (2 * L - 1) * d.c_plane + int(off.max()) + 1, np.uint16)
        for p, part in enumerate([C.real, C.imag]):
            for lv, arr in enumerate(_split_levels(part.astype(np.float32).astype(np.float64), L)):
                out[(2 * lv + p) * d.c_plane + off] = arr
    return 0


FakeLib.ptn_to_planes = _fake_to_planes
FakeLib.ptn_expand_b = _fake_expand_b
FakeLib.ptn_cgemm_bf16x3 = _fake_cgemm
FakeLib.ptn_launch_counter = lambda self: 0
FakeLib.ptn_stream_synchronize = lambda self, stream: 0


# ---- SVD and permute ------------------------------------------------------------
def _fake_svd_work_bytes(self, m, n):
    return 256


def _fake_svd(self, d_ref, stream):
    d = d_ref._obj
    m, n = d.m, d.n
    A = _strided(d.A, [m, n], [d.row_stride, d.col_stride]).copy()
    u, s, vh = np.linalg.svd(A, full_matrices=False)
    U = _strided(d.U, [n, m], [d.ldu, 1])
    U[...] = u.T
    _view(d.S, n, np.float64)[:] = s
    V = _strided(d.V, [n, n], [d.ldv, 1])
    V[...] = vh.conj()
    return 0


def _fake_permute(self, d_ref, stream):
    d = d_ref._obj
    dims = [d.dim[i] for i in range(d.n)]
    src = _strided(d.src, dims, [d.stride_src[i] for i in range(d.n)]).copy()
    if d.conj:
        src = src.conj()
    if d.scale:
        sc = _view(d.scale, dims[d.scale_mode], np.float64)
        shp = [1] * d.n
        shp[d.scale_mode] = dims[d.scale_mode]
        src = src * sc.reshape(shp)
    dst = _strided(d.dst, dims, [d.stride_dst[i] for i in range(d.n)])
    dst[...] = src
    return 0


FakeLib.ptn_zsvd_work_bytes = _fake_svd_work_bytes
FakeLib.ptn_zsvd_jacobi = _fake_svd
FakeLib.ptn_zpermute = _fake_permute


# ---- native executor -------------------------------------------------------------
def _fake_exec_ops(self, ops, nops, ptrs, nptrs, stream):
    import pytreenet_gb300._lib as L
    for i in range(nops):
        op = ops[i]
        if op.kind == L.OP_ZCONTRACT:
            d = L.ContractDesc.from_buffer_copy(ctypes.cast(op.desc, ctypes.POINTER(L.ContractDesc)).contents)
            d.A, d.B, d.C = ptrs[op.a], (ptrs[op.b] if op.b >= 0 else None), ptrs[op.c]
            self.ptn_zcontract(ctypes.byref(d), stream)
        elif op.kind == L.OP_CGEMM:
            d = L.CgemmDesc.from_buffer_copy(ctypes.cast(op.desc, ctypes.POINTER(L.CgemmDesc)).contents)
            d.A, d.Bx, d.C = ptrs[op.a], (ptrs[op.b] if op.b >= 0 else None), ptrs[op.c]
            self.ptn_cgemm_bf16x3(ctypes.byref(d), stream)
        else:
            d = L.ConvertDesc.from_buffer_copy(ctypes.cast(op.desc, ctypes.POINTER(L.ConvertDesc)).contents)
            d.src, d.dst = ptrs[op.a], ptrs[op.c]
            if op.kind == L.OP_TO_PLANES:
                self.ptn_to_planes(ctypes.byref(d), stream)
            else:
                self.ptn_expand_b(ctypes.byref(d), stream)
    return 0


def _fake_gs_step(self, Q, ldq, nq, w, n, h, part, norms, qnext, stream):
    self.ptn_dznrm2(w, n, norms, part, stream)
    for off in (0, nq):
        hp = int(h) + 16 * off
        self.ptn_zdot_multi(Q, ldq, nq, w, n, hp, 0, part, stream)
        self.ptn_zaxpy_multi(Q, ldq, nq, hp, w, n, stream)
    self.ptn_dznrm2(w, n, int(norms) + 8, part, stream)
    if qnext:
        self.ptn_zscal_inv(w, int(norms) + 8, qnext, n, stream)
    return 0


FakeLib.ptn_exec_ops = _fake_exec_ops
FakeLib.ptn_krylov_gs_step = _fake_gs_step


# ---- CholeskyQR2 factors and the zero-row scan --------------------------------------
def _fake_chol_upper(self, G, ldg, k, R, Rinv, ratio, series, series_tol, status, work, stream):
    g = _view(G, (k - 1) * ldg + k).copy()
    g = np.stack([g[i * ldg:i * ldg + k] for i in range(k)])
    g = 0.5 * (g + g.conj().T)
    if series and np.linalg.norm(g - np.eye(k)) <= series_tol:
        e = g - np.eye(k)
        u = np.triu(e, 1) + 0.5 * np.diag(np.diag(e).real)
        _view(R, k * k)[:] = (np.eye(k) + u).reshape(-1)
        _view(Rinv, k * k)[:] = (np.eye(k) - u).reshape(-1)
        return 0
    try:
        lc = np.linalg.cholesky(g)
    except np.linalg.LinAlgError:
        _view(status, 1, np.int32)[0] = 5
        return 0
    d = np.abs(np.diag(lc))
    if not d.min() > ratio * d.max():
        _view(status, 1, np.int32)[0] = 5
        return 0
    r = lc.conj().T
    _view(R, k * k)[:] = r.reshape(-1)
    _view(Rinv, k * k)[:] = np.triu(np.linalg.inv(r)).reshape(-1)
    return 0


def _fake_tri_mul(self, A, B, C, k, stream):
    a = _view(A, k * k).reshape(k, k)
    b = _view(B, k * k).reshape(k, k)
    _view(C, k * k)[:] = np.triu(np.triu(a) @ np.triu(b)).reshape(-1)
    return 0


def _fake_nonzero_rows(self, A, rowoff, m, k, cs, out, stream):
    ro = _view(rowoff, m, np.int64)
    ext = int(ro.max()) + (k - 1) * cs + 1
    mat = _view(A, ext)[ro[:, None] + np.arange(k)[None, :] * cs]
    nz = np.nonzero(np.any(mat != 0, axis=1))[0]
    _view(out, 1, np.int64)[0] = int(nz[-1]) + 1 if nz.size else 0
    return 0


def _fake_qr_keep_rows(self, A, rowoff, m, m_used, k, cs, R, work, stream):
    ro = _view(rowoff, m, np.int64)
    ext = int(ro.max()) + (k - 1) * cs + 1
    a = _view(A, ext)
    idx = ro[:, None] + np.arange(k)[None, :] * cs
    mat = a[idx]
    assert not np.any(mat[m_used:]), "rows past m_used must be zero"
    p = min(m, k)
    q = np.zeros((m, k), dtype=complex)
    r = np.zeros((k, k), dtype=complex)
    qs, rs = np.linalg.qr(mat[:m_used], mode="reduced")
    q[:m_used, :qs.shape[1]] = qs
    r[:rs.shape[0], :] = rs
    for j in range(min(m_used, k), p):
        q[j, j] = 1.0
    a[idx] = q
    _view(R, k * k)[:] = r.reshape(-1)
    return 0


FakeLib.ptn_zchol_work_bytes = lambda self, k: 16
FakeLib.ptn_zchol_max_k = lambda self: 256
FakeLib.ptn_zchol_upper = _fake_chol_upper
FakeLib.ptn_ztri_mul_upper = _fake_tri_mul


def _fake_tri_inv_newton(self, X, R0, R, work, k, stream):
    x = np.triu(_view(X, k * k).reshape(k, k))
    r0 = np.triu(_view(R0, k * k).reshape(k, k))
    _view(R, k * k)[:] = np.triu(r0 @ (2 * np.eye(k) - x @ r0)).reshape(-1)
    return 0


FakeLib.ptn_ztri_inv_newton = _fake_tri_inv_newton
FakeLib.ptn_znonzero_rows = _fake_nonzero_rows
FakeLib.ptn_zqr_keep_rows = _fake_qr_keep_rows
# the stand-in GEMM never splits K
FakeLib.ptn_cgemm_partial_bytes = lambda self, M, N, K: 0
FakeLib.ptn_zqr_path = lambda self, m, k: 0
