"""The QR entry point that allocates nothing (ptn_zqr_keep_noalloc).

Callers that cannot allocate device memory -- a host framework bound through a
plain C FFI that owns no CUDA allocator, or code that must not allocate while
a stream is captured -- use this variant. It must give the same Q and R as
ptn_zqr_keep with a caller-provided work buffer, call after call (its scratch
is a fixed array shared by every call), and reject problems whose scratch
would not fit.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _qr_inputs(rng, m, k):
    A = (rng.normal(size=(k, m)) + 1j * rng.normal(size=(k, m))).reshape(-1)
    perm = rng.permutation(m).astype(np.int64)
    return A, perm


def test_qr_noalloc_matches_allocating_entry_point():
    from pytreenet_gb300 import _lib, build
    from pytreenet_gb300.engine import _stream_ptr
    build.build()
    lib = _lib.load()
    rng = np.random.default_rng(5)
    for call, (m, k) in enumerate([(3000, 130), (512, 256)]):
        A, perm = _qr_inputs(rng, m, k)
        A1 = torch.from_numpy(A).cuda()
        A2 = A1.clone()
        rowoff = torch.from_numpy(perm).cuda()
        R1 = torch.zeros((k, k), dtype=torch.complex128, device="cuda")
        R2 = torch.zeros((k, k), dtype=torch.complex128, device="cuda")
        work = torch.zeros((int(lib.ptn_zqr_work_bytes(m, k)) + 15) // 16, dtype=torch.complex128,
                           device="cuda")
        s = _stream_ptr()
        assert lib.ptn_zqr_keep(A1.data_ptr(), rowoff.data_ptr(), m, k, m, R1.data_ptr(), work.data_ptr(), s) == 0
        assert lib.ptn_zqr_keep_noalloc(A2.data_ptr(), rowoff.data_ptr(), m, k, m, R2.data_ptr(), s) == 0
        torch.cuda.synchronize()
        q1, q2 = A1.cpu().numpy(), A2.cpu().numpy()
        r1, r2 = R1.cpu().numpy(), R2.cpu().numpy()
        assert np.max(np.abs(q1 - q2)) < 1e-12, call
        assert np.max(np.abs(r1 - r2)) < 1e-12 * max(1.0, np.max(np.abs(r1))), call


def test_qr_noalloc_rejects_oversized_problem():
    from pytreenet_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    cap = int(lib.ptn_zqr_noalloc_max_bytes())
    m, k = 1 << 20, 1024
    assert int(lib.ptn_zqr_work_bytes(m, k)) > cap
    dummy = torch.zeros(8, dtype=torch.complex128, device="cuda")
    rowoff = torch.zeros(8, dtype=torch.int64, device="cuda")
    # the size check happens on the host before any launch; nothing is dereferenced
    assert lib.ptn_zqr_keep_noalloc(dummy.data_ptr(), rowoff.data_ptr(), m, k, m, dummy.data_ptr(), None) == 6
