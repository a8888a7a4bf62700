"""CUDA kernels of libptn_gb300 against NumPy, through the C ABI."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(11)


def crandn(*shape):
    return (RNG.normal(size=shape) + 1j * RNG.normal(size=shape)) / np.sqrt(2)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def lib():
    from pytreenet_gb300 import _lib, build
    build.build()
    return _lib.load()


CASES = [
    # (A dims/labels, B dims/labels, contracted labels, output order)
    (("ab", (5, 7)), ("bc", (7, 3)), "b", "ac"),
    (("abcs", (6, 5, 4, 2)), ("bxy", (5, 3, 6)), "b", "acsxy"),
    (("abcs", (6, 5, 4, 2)), ("xbsy", (3, 5, 2, 7)), "bs", "yacx"),
    (("abs", (70, 65, 2)), ("axb", (70, 5, 65)), "ab", "sx"),
    (("pqrs", (3, 130, 2, 9)), ("rqt", (2, 130, 11)), "qr", "tsp"),
    (("ab", (1, 1)), ("bc", (1, 1)), "b", "ac"),
    (("abc", (9, 8, 7)), ("d", (4,)), "", "dabc"),
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("conj_b", [False, True])
def test_zcontract_matches_numpy(lib, case, conj_b):
    from pytreenet_gb300.engine import Operand, Step, ChainBuilder, Workspace, Plan
    (la, da), (lb, db), kl, lo = case
    A, B = crandn(*da), crandn(*db)
    dims = {**dict(zip(la, da)), **dict(zip(lb, db))}
    Ad, Bd = dev(A), dev(B)
    C = torch.zeros([dims[l] for l in lo], dtype=torch.complex128, device="cuda")
    st = Step(Operand.contiguous(("fixed", Ad), list(la), list(da)),
              Operand.contiguous(("fixed", Bd), list(lb), list(db)), list(kl),
              Operand.contiguous(("fixed", C), list(lo), [dims[l] for l in lo]), conj_b=conj_b)
    Plan(Workspace("cuda"), [st], {}).run()
    ref = np.einsum(f"{la},{lb}->{lo}", A, B.conj() if conj_b else B)
    got = C.cpu().numpy()
    assert np.max(np.abs(got - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))


def test_zcontract_beta_and_alpha(lib):
    from pytreenet_gb300.engine import Operand, Step, Workspace, Plan
    A, B, C0 = crandn(40, 33), crandn(33, 17), crandn(40, 17)
    Ad, Bd, Cd = dev(A), dev(B), dev(C0)
    st = Step(Operand.contiguous(("fixed", Ad), ["m", "k"], [40, 33]),
              Operand.contiguous(("fixed", Bd), ["k", "n"], [33, 17]), ["k"],
              Operand.contiguous(("fixed", Cd), ["m", "n"], [40, 17]), alpha=0.5 - 2j, beta=1.5j)
    Plan(Workspace("cuda"), [st], {}).run()
    ref = (0.5 - 2j) * A @ B + 1.5j * C0
    assert np.max(np.abs(Cd.cpu().numpy() - ref)) < 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("n,nq", [(1, 1), (1000, 3), (100003, 9), (70000, 20)])
def test_krylov_vector_kernels(lib, n, nq):
    from pytreenet_gb300.engine import _stream_ptr
    Q, w, c = crandn(nq, n), crandn(n), crandn(nq)
    Qd, wd, cd = dev(Q), dev(w), dev(c)
    h = torch.zeros(nq, dtype=torch.complex128, device="cuda")
    part = torch.zeros(int(lib.ptn_krylov_partials(n)) + 8, dtype=torch.complex128, device="cuda")
    s = _stream_ptr()
    assert lib.ptn_zdot_multi(Qd.data_ptr(), n, nq, wd.data_ptr(), n, h.data_ptr(), 0, part.data_ptr(), s) == 0
    ref_h = Q.conj() @ w
    assert np.max(np.abs(h.cpu().numpy() - ref_h)) < 1e-11 * np.sqrt(n)
    assert lib.ptn_zaxpy_multi(Qd.data_ptr(), n, nq, h.data_ptr(), wd.data_ptr(), n, s) == 0
    w2 = w - Q.T @ ref_h
    assert np.max(np.abs(wd.cpu().numpy() - w2)) < 1e-10 * np.sqrt(n)
    nrm = torch.zeros(2, dtype=torch.float64, device="cuda")
    assert lib.ptn_dznrm2(wd.data_ptr(), n, nrm.data_ptr(), part.data_ptr(), s) == 0
    assert abs(nrm[0].item() - np.linalg.norm(w2)) < 1e-10 * np.linalg.norm(w2)
    out = torch.zeros(n, dtype=torch.complex128, device="cuda")
    assert lib.ptn_zcombine(Qd.data_ptr(), n, nq, cd.data_ptr(), out.data_ptr(), n, s) == 0
    assert np.max(np.abs(out.cpu().numpy() - c @ Q)) < 1e-11 * np.sqrt(nq)
    assert lib.ptn_zscal_inv(wd.data_ptr(), nrm.data_ptr(), out.data_ptr(), n, s) == 0
    assert abs(np.linalg.norm(out.cpu().numpy()) - 1.0) < 1e-12


def _qr_case(lib, A, row_perm=None):
    """QR of A (m x k) stored column-major-ish inside a buffer through a row table."""
    m, k = A.shape
    # store as a (k, m) row-major buffer: element (i, c) at c * m + phys_row(i)
    phys = np.arange(m) if row_perm is None else np.asarray(row_perm)
    buf = np.zeros((k, m), dtype=complex)
    buf[:, phys] = A.T
    Ad = dev(buf.reshape(-1))
    rowoff = torch.from_numpy(phys.astype(np.int64)).cuda()
    R = torch.zeros((k, k), dtype=torch.complex128, device="cuda")
    work = torch.zeros((int(lib.ptn_zqr_work_bytes(m, k)) + 15) // 16, dtype=torch.complex128, device="cuda")
    from pytreenet_gb300.engine import _stream_ptr
    assert lib.ptn_zqr_keep(Ad.data_ptr(), rowoff.data_ptr(), m, k, m, R.data_ptr(), work.data_ptr(),
                            _stream_ptr()) == 0
    out = Ad.cpu().numpy().reshape(k, m)[:, phys].T
    return out, R.cpu().numpy()


@pytest.mark.parametrize("m,k", [(6, 4), (300, 40), (2, 8), (2048, 64), (5, 5), (1, 3), (3000, 130),
                                 (512, 256), (768, 100), (64, 80), (700, 33), (769, 64)])
def test_qr_matches_lapack_convention(lib, m, k):
    A = crandn(m, k)
    q, r = _qr_case(lib, A, row_perm=RNG.permutation(m))
    qn, rn = np.linalg.qr(A, mode="reduced")
    p = min(m, k)
    assert np.max(np.abs(q[:, :p] - qn)) < 1e-12 * max(1, np.sqrt(m))
    assert np.max(np.abs(r[:p] - rn)) < 1e-12 * np.max(np.abs(rn)) * max(1, np.sqrt(m))
    assert np.all(q[:, p:] == 0) and np.all(r[p:] == 0)


def test_qr_rank_deficient_exact_structure(lib):
    """Zero-padded tensor: rank 1 with exact zero columns; the Householder
    complement must equal LAPACK's (unit vectors through the first reflector)."""
    m, k = 128, 8
    A = np.zeros((m, k), dtype=complex)
    A[:2, 0] = [0.6, 0.8j]
    A[:, 3] = 0
    q, r = _qr_case(lib, A)
    qn, rn = np.linalg.qr(A, mode="reduced")
    assert np.max(np.abs(q - qn)) < 1e-15
    assert np.max(np.abs(r - rn)) < 1e-15
    B = np.zeros((m, k), dtype=complex)
    B[:4, :] = crandn(4, k)
    q, r = _qr_case(lib, B)
    qn, rn = np.linalg.qr(B, mode="reduced")
    assert np.max(np.abs(q - qn)) < 1e-13
    assert np.all(q[4:, 4:] == qn[4:, 4:])
    # the panel (blocked) path: rank 4 in a 256 x 64 matrix, exact identity complement
    C = np.zeros((256, 64), dtype=complex)
    C[:4, :] = crandn(4, 64)
    q, r = _qr_case(lib, C)
    qn, rn = np.linalg.qr(C, mode="reduced")
    assert np.max(np.abs(q - qn)) < 1e-13
    assert np.all(q[4:, 4:] == qn[4:, 4:])


@pytest.mark.parametrize("n,nq", [(1, 1), (1000, 3), (131072, 8), (70001, 16), (4097, 17)])
def test_krylov_gs_step_matches_numpy(n, nq):
    """One Gram-Schmidt step (ptn_krylov_gs_step) against NumPy's two-pass
    classical Gram-Schmidt."""
    import ctypes
    from pytreenet_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(n + nq)
    Qn = rng.normal(size=(nq, n)) + 1j * rng.normal(size=(nq, n))
    for i in range(nq):                       # orthonormal rows, as in a Krylov basis
        for j in range(i):
            Qn[i] -= np.vdot(Qn[j], Qn[i]) * Qn[j]
        Qn[i] /= np.linalg.norm(Qn[i])
    wn = rng.normal(size=n) + 1j * rng.normal(size=n)
    Q = torch.from_numpy(Qn).cuda()
    w = torch.from_numpy(wn.copy()).cuda()
    h = torch.zeros(2 * nq, dtype=torch.complex128, device="cuda")
    part = torch.zeros(int(lib.ptn_krylov_partials(n)) + 8, dtype=torch.complex128, device="cuda")
    norms = torch.zeros(2, dtype=torch.float64, device="cuda")
    qn = torch.zeros(n, dtype=torch.complex128, device="cuda")
    st = lib.ptn_krylov_gs_step(Q.data_ptr(), n, nq, w.data_ptr(), n, h.data_ptr(), part.data_ptr(),
                                norms.data_ptr(), qn.data_ptr(),
                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    w1 = wn.copy()
    h1 = Qn.conj() @ w1
    w1 = w1 - h1 @ Qn
    h2 = Qn.conj() @ w1
    w1 = w1 - h2 @ Qn
    scale = np.linalg.norm(wn)
    np.testing.assert_allclose(norms.cpu().numpy()[0], np.linalg.norm(wn), rtol=1e-13)
    np.testing.assert_allclose(h.cpu().numpy(), np.concatenate([h1, h2]), atol=1e-12 * scale)
    np.testing.assert_allclose(w.cpu().numpy(), w1, atol=1e-12 * scale)
    b = np.linalg.norm(w1)
    np.testing.assert_allclose(norms.cpu().numpy()[1], b, rtol=1e-10, atol=1e-13 * scale)
    if b > 1e-8 * scale:
        np.testing.assert_allclose(qn.cpu().numpy(), w1 / b, atol=1e-10)
