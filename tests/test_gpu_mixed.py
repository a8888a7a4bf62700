"""Tensor-core (tcgen05, BF16x3) contraction path on the GPU."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(21)


def crandn(*shape):
    return (RNG.normal(size=shape) + 1j * RNG.normal(size=shape)) / np.sqrt(2)


@pytest.fixture(scope="module")
def lib():
    from pytreenet_gb300 import _lib, build
    build.build()
    return _lib.load()


def _bf16_round(x):
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(torch.bfloat16)


@pytest.fixture(scope="module")
def selftest_lib(lib):
    """The descriptor self-test kernel, built into a test-only library."""
    import ctypes
    import os
    import subprocess
    from pytreenet_gb300 import build
    here = os.path.dirname(os.path.abspath(__file__))
    out_dir = os.path.join(here, "native", "_build")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "libtc_selftest.so")
    cmd = [build.nvcc(), *build.ARCH, *build.NVCC_FLAGS, "-shared", "-I", build.CSRC,
           os.path.join(here, "native", "tc_selftest.cu"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    t = ctypes.CDLL(so)
    t.tc_selftest.restype = ctypes.c_int
    t.tc_selftest.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int32, ctypes.c_void_p]
    return t


@pytest.mark.parametrize("sw64", [0, 1, 2])
def test_tcgen05_descriptor_selftest(selftest_lib, sw64):
    from pytreenet_gb300.engine import _stream_ptr
    A = _bf16_round(RNG.normal(size=(128, 64)))
    B = _bf16_round(RNG.normal(size=(128, 64)))
    D = torch.zeros((128, 128), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    Ad, Bd = A.cuda(), B.cuda()
    assert selftest_lib.tc_selftest(Ad.data_ptr(), Bd.data_ptr(), D.data_ptr(), st.data_ptr(), sw64,
                                    _stream_ptr()) == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.float().numpy() @ B.float().numpy().T
    assert np.max(np.abs(D.cpu().numpy() - ref)) < 1e-3


@pytest.mark.parametrize("levels,tol", [(2, 5e-5), (3, 2e-6)])
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (200, 70, 100), (1000, 130, 256), (4096, 512, 1280),
                                   (37, 5, 10), (131072 // 32, 256, 256)])
def test_cgemm_bf16_matches_complex128(lib, M, N, K, levels, tol):
    """C = A B^T with BF16 splits: error ~ 2^-16 (2 levels) / 2^-24 (3 levels) per term."""
    from pytreenet_gb300.engine import Operand, ChainBuilder, Workspace
    A, B = crandn(M, K), crandn(N, K)
    Ad = torch.from_numpy(A).cuda()
    Bd = torch.from_numpy(B).cuda()
    C = torch.zeros((M, N), dtype=torch.complex128, device="cuda")
    ws = Workspace("cuda")
    cb = ChainBuilder(ws)
    cb.contract(Operand.contiguous(("fixed", Ad), ["m", "k"], [M, K]),
                Operand.contiguous(("fixed", Bd), ["n", "k"], [N, K]), ["k"],
                out=Operand.contiguous(("fixed", C), ["m", "n"], [M, N]))
    p = cb.mixed_plan(levels)
    p.run()
    torch.cuda.synchronize()
    assert int(ws.bufs["tc_status"].item()) == 0
    ref = A @ B.T
    err = np.max(np.abs(C.cpu().numpy() - ref)) / np.sqrt(K)
    assert err < tol, err


def test_cgemm_chain_matches_fp64_plan(lib):
    """The degree-2 and degree-3 site matvecs on both paths, same operands."""
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    from pytreenet_gb300.engine import DeviceNetwork
    st, spec, tensors = t_tree_state(arm_len=3, chi=32, seed=2)
    H, _ = t_tree_heisenberg(st, seed=3)
    ref = DeviceNetwork(st, H, precision="plain")
    ref.canonical_form("a0_1")
    ref.init_cache_but_one("a0_1")
    ref.init_cache_but_one("root")
    for nid in ("a0_1", "root"):
        outs = {}
        for prec in ("plain", "bf16x3", "bf16x6"):
            st2, _, _ = t_tree_state(arm_len=3, chi=32, seed=2)
            net = DeviceNetwork(st2, H, precision=prec)
            for key, e in ref.env.items():
                net.env_buf(*key).copy_(e)
            x = ref.t[nid].clone()
            y = torch.zeros_like(x)
            net.heff_plan(nid).run(x.data_ptr(), y.data_ptr())
            torch.cuda.synchronize()
            outs[prec] = y.cpu().numpy()
        rel3 = np.linalg.norm(outs["bf16x3"] - outs["plain"]) / np.linalg.norm(outs["plain"])
        rel6 = np.linalg.norm(outs["bf16x6"] - outs["plain"]) / np.linalg.norm(outs["plain"])
        assert rel3 < 1e-4, (nid, rel3)
        assert rel6 < 2e-6, (nid, rel6)


@pytest.mark.parametrize("name", ["ttree3_heis_chi6_o1", "ternary2_xxz_chi4_o1"])
def test_gpu_mixed_tdvp_matches_reference(name):
    import oracle as O
    import pytreenet_gb300 as P
    from golden_util import build_ttn, load_case, oracle_state, fidelity_and_dist
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"] * c["steps"], {},
                                   config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                   solver_options={"krylov_tol": c["krylov_tol"]}, precision="mixed")
    for _ in range(c["steps"]):
        algo.run_one_time_step()
    got = O.OState(oracle_state(c).tree, {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]})
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), got)
    assert one_minus_f < 1e-11


def test_gpu_cholqr2_split_is_isometric():
    """Mixed path, tall full-rank split (CholeskyQR2 on the tensor cores):
    Q is an isometry and Q R reproduces the tensor."""
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    from pytreenet_gb300.engine import DeviceNetwork
    st, spec, tensors = t_tree_state(arm_len=1, chi=64, seed=4)
    H, _ = t_tree_heisenberg(st, seed=5)
    net = DeviceNetwork(st, H, precision="mixed")
    A0 = net.t["root"].clone()
    R = net.qr_split("root", "a1_0").clone()
    torch.cuda.synchronize()
    Qm = net.t["root"].permute(0, 2, 3, 1).reshape(-1, 64).cpu().numpy()
    Am = A0.permute(0, 2, 3, 1).reshape(-1, 64).cpu().numpy()
    assert np.max(np.abs(Qm.conj().T @ Qm - np.eye(64))) < 1e-6
    assert np.max(np.abs(Qm @ R.cpu().numpy() - Am)) < 1e-6 * np.max(np.abs(Am))


def test_gpu_qr_graph_replay_matches_eager():
    """The captured QR launch sequence gives the same Q and R as eager launches."""
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    from pytreenet_gb300.engine import DeviceNetwork
    outs = []
    for graphs in (False, True):
        # the root split has 48 * 48 * 2 = 4608 rows: the multi-kernel path that graphs capture
        st, spec, tensors = t_tree_state(arm_len=1, chi=48, seed=6)
        H, _ = t_tree_heisenberg(st, seed=7)
        net = DeviceNetwork(st, H, precision="plain")
        net.use_graphs = graphs
        rs = []
        for _ in range(3):     # eager, capture + replay, replay
            x = net.t["root"]
            x.copy_(torch.from_numpy(tensors["root"]).cuda())
            rs.append((net.qr_split("root", "a0_0").clone(), net.t["root"].clone()))
        outs.append(rs)
    for (r0, q0), (r1, q1) in zip(outs[0], outs[1]):
        assert torch.equal(r0, r1) and torch.equal(q0, q1)
    assert net.qr_graphs, "the multi-kernel split was not captured"


def test_cgemm_abort_mid_kernel_drains_and_recovers(lib):
    """A nonzero status word written from another stream while tensor-core
    GEMMs run makes them stop early: the running CTAs leave their waits, drain
    the loads and MMAs they issued, free TMEM and exit; later launches see the
    word and skip. The status stays nonzero, and once it is cleared the same
    GEMM runs again and reproduces its earlier output exactly."""
    from pytreenet_gb300.engine import Operand, ChainBuilder, Workspace
    M, N, K = 65536, 512, 2048
    g = torch.Generator(device="cuda").manual_seed(5)
    Ad = torch.randn((M, K), dtype=torch.complex128, device="cuda", generator=g)
    Bd = torch.randn((N, K), dtype=torch.complex128, device="cuda", generator=g)
    C = torch.zeros((M, N), dtype=torch.complex128, device="cuda")
    ws = Workspace("cuda")
    cb = ChainBuilder(ws)
    cb.contract(Operand.contiguous(("fixed", Ad), ["m", "k"], [M, K]),
                Operand.contiguous(("fixed", Bd), ["n", "k"], [N, K]), ["k"],
                out=Operand.contiguous(("fixed", C), ["m", "n"], [M, N]))
    p = cb.mixed_plan(3)
    p.run()
    torch.cuda.synchronize()
    status = ws.bufs["tc_status"]
    assert int(status.item()) == 0
    C_ok = C.clone()
    side = torch.cuda.Stream()
    for _ in range(8):
        p.run()
    with torch.cuda.stream(side):
        torch.cuda._sleep(2_000_000)          # ~1 ms, while the GEMMs above run
        status.fill_(99)
    torch.cuda.synchronize()
    assert int(status.item()) != 0
    status.zero_()
    C.zero_()
    p.run()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(C, C_ok)


@pytest.mark.parametrize("M,N,K", [(256, 256, 16384), (200, 70, 4096), (1280, 256, 2048)])
def test_cgemm_split_k_matches_complex128(lib, M, N, K):
    """Few output tiles and a long K: the product is split over K (FP32
    partial sums added in FP64) and matches complex128 at the BF16x6 level."""
    from pytreenet_gb300.engine import Operand, ChainBuilder, Workspace
    assert lib.ptn_cgemm_partial_bytes(M, N, K) > 0
    A, B = crandn(M, K), crandn(N, K)
    Ad, Bd = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    C = torch.zeros((M, N), dtype=torch.complex128, device="cuda")
    ws = Workspace("cuda")
    cb = ChainBuilder(ws)
    cb.contract(Operand.contiguous(("fixed", Ad), ["m", "k"], [M, K]),
                Operand.contiguous(("fixed", Bd), ["n", "k"], [N, K]), ["k"],
                out=Operand.contiguous(("fixed", C), ["m", "n"], [M, N]))
    p = cb.mixed_plan(3)
    p.run()
    torch.cuda.synchronize()
    assert int(ws.bufs["tc_status"].item()) == 0
    assert "tc_partial" in ws.bufs
    err = np.max(np.abs(C.cpu().numpy() - A @ B.T)) / np.sqrt(K)
    assert err < 2e-6, err
    # deterministic: a second run gives the same bits
    C0 = C.clone()
    p.run()
    torch.cuda.synchronize()
    assert torch.equal(C, C0)


def test_cgemm_split_k_into_planes(lib):
    """A split first step writes its sum as BF16 planes for the next step."""
    from pytreenet_gb300.engine import Operand, ChainBuilder, Workspace
    M, K, N, P = 200, 8192, 100, 60
    assert lib.ptn_cgemm_partial_bytes(M, N, K) > 0
    A, B, D = crandn(M, K), crandn(N, K), crandn(N, P)
    Ad, Bd, Dd = (torch.from_numpy(x).cuda() for x in (A, B, D))
    C = torch.zeros((M, P), dtype=torch.complex128, device="cuda")
    ws = Workspace("cuda")
    cb = ChainBuilder(ws)
    T = cb.contract(Operand.contiguous(("fixed", Ad), ["m", "k"], [M, K]),
                    Operand.contiguous(("fixed", Bd), ["n", "k"], [N, K]), ["k"])
    cb.contract(T, Operand.contiguous(("fixed", Dd), ["n", "p"], [N, P]), ["n"],
                out=Operand.contiguous(("fixed", C), ["m", "p"], [M, P]))
    cb.mixed_plan(3).run()
    torch.cuda.synchronize()
    assert int(ws.bufs["tc_status"].item()) == 0
    ref = (A @ B.T) @ D
    err = np.max(np.abs(C.cpu().numpy() - ref)) / (np.sqrt(K) * np.sqrt(N))
    assert err < 2e-6, err


@pytest.mark.parametrize("K", [2, 4, 6, 10, 7, 20])
def test_cgemm_small_k_chain_matches_fp64(lib, K):
    """Products with K <= 32 run on the CUDA-core kernel compiled for their K
    (7 takes the generic instance); when the next step contracts the inner
    row leg of this step's output, the rows come in adjacent pairs and the
    paired kernel writes bf16x2 (K = 2, 4, 6, 10). Chain
    T[m1, m2, n] = sum_k A[m1, m2, k] B[n, k], then sum_m2 T[m1, m2, n] D[m2, p],
    on the tensor-core path against the FP64 plan."""
    from pytreenet_gb300.engine import Operand, ChainBuilder, Workspace
    m1, m2, N, P = 96, 38, 50, 24
    A, B, D = crandn(m1, m2, K), crandn(N, K), crandn(m2, P)
    Ad, Bd, Dd = (torch.from_numpy(x).cuda() for x in (A, B, D))
    outs = []
    for mixed in (True, False):
        C = torch.zeros((m1, N, P), dtype=torch.complex128, device="cuda")
        ws = Workspace("cuda")
        cb = ChainBuilder(ws)
        T = cb.contract(Operand.contiguous(("fixed", Ad), ["a", "b", "k"], [m1, m2, K]),
                        Operand.contiguous(("fixed", Bd), ["n", "k"], [N, K]), ["k"])
        cb.contract(T, Operand.contiguous(("fixed", Dd), ["b", "p"], [m2, P]), ["b"],
                    out=Operand.contiguous(("fixed", C), ["a", "n", "p"], [m1, N, P]))
        p = cb.mixed_plan(3) if mixed else cb.plan()
        p.run()
        torch.cuda.synchronize()
        if mixed:
            assert int(ws.bufs["tc_status"].item()) == 0
        outs.append(C.cpu().numpy())
    ref = np.einsum("abk,nk,bp->anp", A, B, D)
    assert np.max(np.abs(outs[1] - ref)) < 1e-10 * np.max(np.abs(ref))
    assert np.max(np.abs(outs[0] - outs[1])) < 2e-6 * np.max(np.abs(ref))
