"""Device CholeskyQR2 factors, the zero-row scan and the row-skipping Householder
QR, through the C ABI, against NumPy/LAPACK; and the engine's QR split routed
through them on the reduced-precision path."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RNG = np.random.default_rng(23)


def crandn(*shape):
    return (RNG.normal(size=shape) + 1j * RNG.normal(size=shape)) / np.sqrt(2)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def lib():
    from pytreenet_gb300 import _lib, build
    build.build()
    return _lib.load()


def _chol(lib, G, ratio=1e-3, series=0, tol=0.0):
    from pytreenet_gb300.engine import _stream_ptr
    k = G.shape[0]
    Gd = dev(G)
    R = torch.zeros((k, k), dtype=torch.complex128, device="cuda")
    Ri = torch.zeros_like(R)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    work = torch.zeros((int(lib.ptn_zchol_work_bytes(k)) + 15) // 16, dtype=torch.complex128, device="cuda")
    assert lib.ptn_zchol_upper(Gd.data_ptr(), k, k, R.data_ptr(), Ri.data_ptr(), ratio, series, tol,
                               st.data_ptr(), work.data_ptr(), _stream_ptr()) == 0
    torch.cuda.synchronize()
    return R.cpu().numpy(), Ri.cpu().numpy(), int(st.item())


@pytest.mark.parametrize("m,k", [(3, 1), (40, 17), (200, 64), (300, 100), (512, 256)])
def test_zchol_upper_matches_lapack(lib, m, k):
    A = crandn(m, k)
    G = A.conj().T @ A
    R, Ri, st = _chol(lib, G)
    assert st == 0
    ref = np.linalg.cholesky(G).conj().T           # positive real diagonal, as LAPACK
    assert np.allclose(np.tril(R, -1), 0) and np.allclose(np.tril(Ri, -1), 0)
    # FP32 factorisation: relative error at the single-precision level times kappa(G)
    kap = np.linalg.cond(G)
    assert np.linalg.norm(R - ref) / np.linalg.norm(ref) < 2e-7 * kap
    assert np.linalg.norm(R @ Ri - np.eye(k)) / np.sqrt(k) < 2e-7 * kap


def test_zchol_upper_rejects_rank_deficient(lib):
    A = crandn(96, 40)
    A[:, 7] = A[:, 3] * (0.5 - 1j)
    _, _, st = _chol(lib, A.conj().T @ A)
    assert st == 5
    B = crandn(96, 40)
    B[:, 9] *= 1e-5                       # full rank, but below the pivot ratio
    _, _, st = _chol(lib, B.conj().T @ B, ratio=1e-3)
    assert st == 5
    _, _, st = _chol(lib, B.conj().T @ B, ratio=1e-7)
    assert st == 0


def test_zchol_upper_series_near_identity(lib):
    k = 48
    E = crandn(k, k) * 1e-6
    G = np.eye(k) + 0.5 * (E + E.conj().T)
    R, Ri, st = _chol(lib, G, series=1, tol=1e-3)
    assert st == 0
    ref = np.linalg.cholesky(G).conj().T
    assert np.max(np.abs(R - ref)) < 1e-10                  # O(|E|^2)
    assert np.max(np.abs(Ri - np.linalg.inv(ref))) < 1e-10
    # above the tolerance the full factorisation runs
    G2 = np.eye(k) + 0.05 * (E + E.conj().T) * 1e6 / 1e3
    R2, _, st = _chol(lib, G2, series=1, tol=1e-6)
    assert st == 0 and np.linalg.norm(R2 - np.linalg.cholesky(G2).conj().T) < 1e-5


def test_ztri_mul_upper_and_newton_inverse(lib):
    from pytreenet_gb300.engine import _stream_ptr
    k = 70
    A, B = np.triu(crandn(k, k)), np.triu(crandn(k, k))
    Ad, Bd = dev(A), dev(B)
    C = torch.zeros((k, k), dtype=torch.complex128, device="cuda")
    assert lib.ptn_ztri_mul_upper(Ad.data_ptr(), Bd.data_ptr(), C.data_ptr(), k, _stream_ptr()) == 0
    assert np.max(np.abs(C.cpu().numpy() - A @ B)) < 1e-12 * k
    # one Newton step from an FP32-accurate inverse gives the FP64 one
    X = np.triu(crandn(k, k)) + 4 * np.eye(k)
    Xi = np.linalg.inv(X)
    R0 = np.triu((Xi * (1 + 1e-7 * crandn(k, k))))
    Xd, R0d = dev(X), dev(R0)
    R = torch.zeros_like(C)
    W = torch.zeros_like(C)
    assert lib.ptn_ztri_inv_newton(Xd.data_ptr(), R0d.data_ptr(), R.data_ptr(), W.data_ptr(), k,
                                   _stream_ptr()) == 0
    Rn = R.cpu().numpy()
    assert np.allclose(np.tril(Rn, -1), 0)
    assert np.max(np.abs(Rn @ X - np.eye(k))) < 1e-12


def _rowoff(shape, row_axes):
    strides = [int(np.prod(shape[i + 1:])) for i in range(len(shape))]
    idx = np.zeros(1, dtype=np.int64)
    for ax in row_axes:
        idx = (idx[:, None] + np.arange(shape[ax], dtype=np.int64)[None, :] * strides[ax]).reshape(-1)
    return idx, strides


@pytest.mark.parametrize("shape,m_used", [((256, 64, 2), 12), ((40, 60, 2), 7), ((300, 20, 2), 20),
                                          ((16, 1200, 2), 600), ((64, 1500, 2), 1000), ((8, 200, 2), 3)])
def test_zqr_keep_rows_equals_full_householder(lib, shape, m_used):
    """Rows past m_used zero (rows = legs 1 and 2, columns = leg 0): the row
    skipping QR returns exactly what the full Householder QR returns."""
    from pytreenet_gb300.engine import _stream_ptr
    T = crandn(*shape)
    idx, strides = _rowoff(shape, [1, 2])
    flat = T.reshape(-1)
    k = shape[0]
    m = idx.size
    mat = flat[idx[:, None] + np.arange(k)[None, :] * strides[0]]
    mat[m_used:] = 0.0
    flat[idx[:, None] + np.arange(k)[None, :] * strides[0]] = mat
    ro = dev(idx)
    w = torch.zeros((int(lib.ptn_zqr_work_bytes(m, k)) + 15) // 16, dtype=torch.complex128, device="cuda")
    out = []
    for rows in (None, m_used):
        A = dev(T.copy())
        R = torch.zeros(k * k, dtype=torch.complex128, device="cuda")
        if rows is None:
            st = lib.ptn_zqr_keep(A.data_ptr(), ro.data_ptr(), m, k, strides[0], R.data_ptr(), w.data_ptr(),
                                  _stream_ptr())
        else:
            st = lib.ptn_zqr_keep_rows(A.data_ptr(), ro.data_ptr(), m, rows, k, strides[0], R.data_ptr(),
                                       w.data_ptr(), _stream_ptr())
        assert st == 0
        out.append((A.cpu().numpy(), R.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    nz = torch.zeros(1, dtype=torch.int64, device="cuda")
    Ad = dev(T)
    assert lib.ptn_znonzero_rows(Ad.data_ptr(), ro.data_ptr(), m, k, strides[0], nz.data_ptr(), _stream_ptr()) == 0
    last = np.nonzero(np.any(mat != 0, axis=1))[0]
    assert int(nz.item()) == (int(last[-1]) + 1 if last.size else 0)


def test_engine_cholqr2_split_matches_lapack_up_to_phase(lib):
    """A 512 x 256 split (an arm site of the chi=256 T-tree, split toward its
    parent) on the reduced-precision path goes through CholeskyQR2 on the
    device; Q R reproduces A, Q is orthonormal, and Q, R equal LAPACK's up to
    a diagonal phase, all at the tensor-core (FP32-level) accuracy."""
    import pytreenet_gb300 as P
    from pytreenet_gb300.engine import DeviceNetwork
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    st, spec, tensors = t_tree_state(arm_len=2, chi=256, seed=5)
    H, _ = t_tree_heisenberg(st, seed=6)
    net = DeviceNetwork(st, H, precision="mixed")
    nid, nbr = "a0_0", "root"
    A0 = net.t[nid].cpu().numpy().copy()          # legs (parent, child, phys)
    R = net.qr_split(nid, nbr).cpu().numpy()
    assert net.cholqr_count == 1 and net.householder_count == 0
    Q = net.t[nid].cpu().numpy()
    Am = A0.transpose(1, 2, 0).reshape(512, 256)
    Qm = Q.transpose(1, 2, 0).reshape(512, 256)
    # Q R = A up to the one tensor-core product A X (FP32 level); R is the
    # FP64 inverse of X, so the FP32 Cholesky factors do not enter
    assert np.linalg.norm(Qm @ R - Am) / np.linalg.norm(Am) < 2e-7
    assert np.max(np.abs(Qm.conj().T @ Qm - np.eye(256))) < 2e-6
    q_ref, r_ref = np.linalg.qr(Am)
    # R_ref = D R and Q_ref = Q D^-1 for a diagonal unitary D
    ph = np.diag(r_ref) / np.diag(R)
    assert np.allclose(np.abs(ph), 1.0, atol=1e-6)
    ph = ph / np.abs(ph)
    assert np.max(np.abs(Qm * ph.conj()[None, :] - q_ref)) < 1e-5
    assert np.linalg.norm(ph[:, None] * R - r_ref) / np.linalg.norm(r_ref) < 1e-5


def test_engine_rank_deficient_split_takes_householder(lib):
    """A padded split (rows past the rank exactly zero) fails the pivot test,
    takes the row-skipping Householder path, and equals the plain path's QR."""
    from pytreenet_gb300.engine import DeviceNetwork
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    st, spec, tensors = t_tree_state(arm_len=2, chi=128, seed=7)
    t = st._phys["a0_0"]
    t[:, 3:, :] = 0.0             # child bond used only on 3 indices: 6 nonzero rows of 256
    H, _ = t_tree_heisenberg(st, seed=8)
    outs = []
    for prec in ("plain", "mixed"):
        s2 = st.copy_structure()
        s2._phys = {k: np.array(v, copy=True) for k, v in tensors.items()}
        s2._phys["a0_0"] = np.array(t, copy=True)
        net = DeviceNetwork(s2, H, precision=prec)
        R = net.qr_split("a0_0", "root").cpu().numpy()
        outs.append((net.t["a0_0"].cpu().numpy(), R, net))
    assert outs[1][2].cholqr_count == 0 and outs[1][2].householder_count == 1
    assert outs[1][2].qr_rows_skipped == 256 - 6
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("shape,pad", [((256, 256, 2), 0), ((256, 256, 2), 100), ((24, 24, 2), 0),
                                       ((40, 7, 2), 0), ((8, 300, 2), 0), ((64, 1000, 2), 0), ((3, 1, 2), 0),
                                       ((512, 100, 2), 0)])
def test_zqr_one_launch_path_equals_launch_sequence(lib, shape, pad):
    """The one-launch Householder QR (reflectors handed between CTAs through
    flags) returns the same bits as the per-step launch sequence, full-rank
    and with zero-padded columns (KEEP complements), tall and wide."""
    from pytreenet_gb300.engine import _stream_ptr
    T = crandn(*shape)
    if pad:
        T[:, shape[1] - pad:, :] = 0.0           # the trailing child indices unused: rank-deficient rows
    idx, strides = _rowoff(shape, [1, 2])
    k, m = shape[0], idx.size
    if m <= 2048:
        assert lib.ptn_zqr_path(m, k) == 1
    ro = dev(idx)
    w = torch.zeros((int(lib.ptn_zqr_work_bytes(m, k)) + 15) // 16, dtype=torch.complex128, device="cuda")
    out = []
    for fn in (lib.ptn_zqr_keep, lib.ptn_zqr_keep_steps):
        A = dev(T.copy())
        R = torch.zeros(k * k, dtype=torch.complex128, device="cuda")
        assert fn(A.data_ptr(), ro.data_ptr(), m, k, strides[0], R.data_ptr(), w.data_ptr(), _stream_ptr()) == 0
        torch.cuda.synchronize()
        out.append((A.cpu().numpy(), R.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    # and it is a QR: Q R = A
    mat = T.reshape(-1)[idx[:, None] + np.arange(k)[None, :] * strides[0]]
    q = out[0][0].reshape(-1)[idx[:, None] + np.arange(k)[None, :] * strides[0]]
    r = out[0][1].reshape(k, k)
    assert np.max(np.abs(q @ r - mat)) < 1e-12 * max(1.0, np.max(np.abs(mat)))
