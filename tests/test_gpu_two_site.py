"""GPU: Jacobi SVD, strided permute, and two-site TDVP against the reference's fixtures."""
import ctypes

import numpy as np
import pytest

import oracle as O
from golden_util import TWO_SITE_CASES, build_ttn, case_solver, load_case, oracle_state, fidelity_and_dist

pytestmark = pytest.mark.gpu
Zm = np.diag([1.0, -1.0]).astype(complex)


def _svd_gpu(A_np, transpose_input=False):
    import torch
    from pytreenet_gb300 import _lib
    lib = _lib.load()
    m, n = A_np.shape
    if transpose_input:
        src = torch.from_numpy(np.ascontiguousarray(A_np)).cuda()          # row-major: (i, j) at i*n + j
        rs, cs = n, 1
    else:
        src = torch.from_numpy(np.ascontiguousarray(A_np.T)).cuda()        # column-major
        rs, cs = 1, m
    U = torch.zeros(n * m, dtype=torch.complex128, device="cuda")
    V = torch.zeros(n * n, dtype=torch.complex128, device="cuda")
    S = torch.zeros(n + 2, dtype=torch.float64, device="cuda")
    work = torch.zeros((lib.ptn_zsvd_work_bytes(m, n) + 15) // 16, dtype=torch.complex128, device="cuda")
    d = _lib.SvdDesc()
    d.A, d.m, d.n, d.row_stride, d.col_stride = src.data_ptr(), m, n, rs, cs
    d.U, d.ldu, d.S, d.V, d.ldv = U.data_ptr(), m, S.data_ptr(), V.data_ptr(), n
    d.work, d.status = work.data_ptr(), S[n:].data_ptr()
    st = lib.ptn_zsvd_jacobi(ctypes.byref(d), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    h = S.cpu()
    code = int(h[n:n + 1].view(torch.int32)[0])
    Uh = U.cpu().numpy().reshape(n, m).T
    Vh = V.cpu().numpy().reshape(n, n).T
    return Uh, h[:n].numpy(), Vh, code


def _graded(rng, m, n, rank=None, spread=1e-12):
    k = min(m, n)
    r = k if rank is None else rank
    Qa, _ = np.linalg.qr(rng.normal(size=(m, k)) + 1j * rng.normal(size=(m, k)))
    Qb, _ = np.linalg.qr(rng.normal(size=(n, k)) + 1j * rng.normal(size=(n, k)))
    s = np.zeros(k)
    s[:r] = np.geomspace(1.0, spread, r)
    return (Qa * s) @ Qb.conj().T, s


@pytest.mark.parametrize("m,n,rank,spread,transpose", [
    (1, 1, None, 1.0, False), (7, 5, None, 1e-3, False), (64, 64, None, 1e-12, False),
    (200, 37, None, 1e-10, True), (96, 96, 10, 1e-6, False), (513, 129, None, 1e-13, False),
    (300, 256, None, 1e-9, True), (256, 32, None, 1e-11, False), (100, 20, 6, 1e-8, True),
    (257, 32, None, 1e-6, False), (40, 33, None, 1e-6, False)])
def test_jacobi_svd_matches_lapack(m, n, rank, spread, transpose):
    rng = np.random.default_rng(m * 1000 + n)
    A, s_true = _graded(rng, m, n, rank, spread)
    U, s, V, code = _svd_gpu(A, transpose)
    assert code == 0
    s_ref = np.linalg.svd(A, compute_uv=False)
    assert np.all(np.diff(s) <= 0)
    np.testing.assert_allclose(s, s_ref, rtol=0, atol=1e-14 * max(1.0, s_ref[0]) * np.sqrt(m))
    # the input itself fixes small singular values only to ~eps * |A| (absolute)
    nz = s_true > 0
    assert np.max(np.abs(s[:nz.sum()] - s_true[nz])) < 1e-13 * np.sqrt(m)
    rec = (U * s) @ V.conj().T
    assert np.linalg.norm(rec - A) <= 1e-13 * np.linalg.norm(A) * np.sqrt(m)
    k = int(np.sum(s > 1e-12 * s[0]))
    assert np.linalg.norm(U[:, :k].conj().T @ U[:, :k] - np.eye(k)) < 1e-12 * np.sqrt(m)
    assert np.linalg.norm(V.conj().T @ V - np.eye(n)) < 1e-12 * np.sqrt(n)


def test_permute_kernel():
    import torch
    from pytreenet_gb300.engine import DeviceNetwork
    rng = np.random.default_rng(3)
    a = rng.normal(size=(3, 4, 5, 6)) + 1j * rng.normal(size=(3, 4, 5, 6))
    scale = rng.normal(size=5)
    src = torch.from_numpy(a).cuda()
    dst = torch.zeros((6, 5, 3, 4), dtype=torch.complex128, device="cuda")
    sc = torch.from_numpy(scale).cuda()
    dims = [3, 4, 5, 6]
    s_src = list(np.array(a.strides) // 16)
    s_dst = [4, 1, 12, 60]
    DeviceNetwork._permute(None, src.data_ptr(), dst.data_ptr(), dims, s_src, s_dst, conj=True,
                           scale_ptr=sc.data_ptr(), scale_mode=2)
    torch.cuda.synchronize()
    ref = np.transpose(a.conj() * scale[None, None, :, None], (3, 2, 0, 1))
    np.testing.assert_array_equal(dst.cpu().numpy(), ref)


def _run_two_site(name, precision="plain", with_algo=False):
    import pytreenet_gb300 as P
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    mode, opts = case_solver(c, P)
    cfg = P.TwoSiteTDVPConfig(time_evo_mode=mode, main_path_mode=P.PathFinderMode[c["path_mode"]],
                              **c["svd"])
    algo = P.SecondOrderTwoSiteTDVP(st, H, c["dt"], c["dt"] * c["steps"], {}, config=cfg,
                                    solver_options=opts, precision=precision)
    zs = []
    for k in range(c["steps"]):
        algo.run_one_time_step()
        zs.append([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    if with_algo:
        return c, O.OState(oracle_state(c).tree, out), np.array(zs), algo
    return c, O.OState(oracle_state(c).tree, out), np.array(zs)


C2 = "c2_ternary3_xxz_neel_chi16"


def _c2_bond_history():
    import os
    from golden_util import GOLDEN
    return [int(x) for x in np.load(os.path.join(GOLDEN, C2 + ".npz"))["bond_history"]]


def test_gpu_c2_ternary_depth3_chi16_plain_matches_oracle():
    """Config 2 at full tree size: second-order two-site TDVP on the ternary
    tree of depth 3 (40 sites), XXZ, Neel start, max_bond_dim 16, cutoff
    1e-10, 10 steps of dt = 0.02, complex128 on the GPU against the oracle
    (tests/golden/make_oracle_fixtures.py; the reference's order cannot run
    this size): the same bond dimension after every one of the 780 splits,
    fidelity error below 1e-10 and <Z_i> to 1e-8 after every step."""
    c, got, zs, algo = _run_two_site(C2, with_algo=True)
    assert list(algo.bond_dims_history) == _c2_bond_history()
    fin = oracle_state(c, "final")
    for nid in fin.tensors:
        assert fin.tensors[nid].shape == got.tensors[nid].shape, nid
    one_minus_f, _ = fidelity_and_dist(fin, got)
    assert one_minus_f < 1e-10
    assert np.max(np.abs(zs - c["z"])) < 1e-8


def test_gpu_c2_ternary_depth3_chi16_mixed_matches_oracle():
    """The same run with BF16x6 tensor-core contractions (FP64 Krylov, SVD and
    truncation). Singular values within the BF16x6 rounding (~1e-7 relative)
    of the 1e-10 cutoff are kept or dropped differently from the complex128
    run, so some splits keep another rank: measured on a GB300, 40 of the 780
    (at most 3 apart), fidelity error 3.7e-10 and <Z_i> within 1.5e-6 after
    10 steps. Bounds: at least 90 % of the ranks equal and none more than 4
    apart, 1 - F < 2e-9, |d<Z_i>| < 5e-6."""
    c, got, zs, algo = _run_two_site(C2, precision="mixed", with_algo=True)
    hist, ref = list(algo.bond_dims_history), _c2_bond_history()
    assert len(hist) == len(ref)
    same = sum(a == b for a, b in zip(hist, ref))
    assert same >= 0.9 * len(ref)
    assert max(abs(a - b) for a, b in zip(hist, ref)) <= 4
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), got)
    assert one_minus_f < 2e-9
    assert np.max(np.abs(zs - c["z"])) < 5e-6


@pytest.mark.parametrize("name", TWO_SITE_CASES)
def test_gpu_two_site_tdvp_matches_reference(name):
    c, got, zs = _run_two_site(name)
    fin = oracle_state(c, "final")
    for nid in fin.tensors:
        assert fin.tensors[nid].shape == got.tensors[nid].shape, nid
    one_minus_f, dist = fidelity_and_dist(fin, got)
    assert np.max(np.abs(zs - c["z"])) < 1e-10
    assert one_minus_f < 1e-12


def test_gpu_two_site_tdvp_mixed():
    """Tensor-core (BF16x6) contractions in the two-site path: FP32-level parity."""
    c, got, zs = _run_two_site("ternary2_xxz_neel_2tdvp", precision="mixed")
    one_minus_f, dist = fidelity_and_dist(oracle_state(c, "final"), got)
    assert np.max(np.abs(zs - c["z"])) < 1e-6
    assert one_minus_f < 1e-9


def test_gpu_two_site_ternary_chi16_vs_oracle():
    """Ternary depth 2 from a random chi=6 state, truncation to 16: bond
    growth, QR-reduced SVD on both orientations, against the oracle."""
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import ternary_state, ternary_xxz
    st, spec, tensors = ternary_state(depth=2, chi=6, seed=11)
    H, Wphys = ternary_xxz(st, seed=12)
    svd = dict(max_bond_dim=16, rel_tol=1e-10, total_tol=1e-10)
    cfg = P.TwoSiteTDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV, **svd)
    algo = P.SecondOrderTwoSiteTDVP(st, H, 0.02, 0.04, {}, config=cfg, solver_options={"krylov_tol": 1e-12})
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    ora = O.SecondOrderTwoSiteTDVPOracle(O.OState(tree, tensors), Wphys, 0.02, O.SVDParams(**svd),
                                         krylov_tol=1e-12)
    for _ in range(2):
        algo.run_one_time_step()
        ora.run_one_time_step()
    assert algo.bond_dims_history == ora.bond_history
    got = O.OState(tree, {nid: algo.state.get_phys_numpy(nid) for nid, _ in spec})
    one_minus_f, dist = fidelity_and_dist(ora.state, got)
    assert one_minus_f < 1e-11


def test_gpu_two_site_subspace_split(monkeypatch):
    """Subspace-iteration reduction (forced on small pairs) against the oracle."""
    import pytreenet_gb300.engine as E
    from test_engine_host import _two_site_vs_oracle
    monkeypatch.setattr(E.DeviceNetwork, "SVD_DIRECT_MAX", 8)
    calls = []
    orig = E.DeviceNetwork._subspace_factor
    monkeypatch.setattr(E.DeviceNetwork, "_subspace_factor", lambda self, *a: calls.append(a[1:]) or orig(self, *a))
    algo, ora, (one_minus_f, dist) = _two_site_vs_oracle(12, 5)
    assert calls
    assert algo.bond_dims_history == ora.bond_history
    assert one_minus_f < 1e-11


@pytest.mark.parametrize("n", [2, 3, 4, 8, 16, 32])
def test_jacobi_svd_converges_on_many_small_matrices(n):
    """Small and triangular matrices (the R factors the split feeds in), many seeds."""
    rng = np.random.default_rng(100 + n)
    for trial in range(24):
        A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        if trial % 2:
            A = np.triu(A)
        if trial % 3 == 0:
            A[:, -1] *= 1e-9
        U, s, V, code = _svd_gpu(A, transpose_input=bool(trial % 4 == 1))
        assert code == 0, (n, trial)
        np.testing.assert_allclose(s, np.linalg.svd(A, compute_uv=False), rtol=0, atol=1e-13 * s[0])
        assert np.linalg.norm((U * s) @ V.conj().T - A) <= 1e-13 * np.linalg.norm(A)


def test_gpu_tebd_matches_reference():
    from golden_util import TEBD_CASES, run_tebd_case
    for name in TEBD_CASES:
        c, got, zs, algo = run_tebd_case(name)
        fin = oracle_state(c, "final")
        for nid in fin.tensors:
            assert fin.tensors[nid].shape == got.tensors[nid].shape
        one_minus_f, _ = fidelity_and_dist(fin, got)
        assert np.max(np.abs(zs - c["z"])) < 1e-12 * np.max(np.abs(c["z"]))
        assert one_minus_f < 1e-13


def test_gpu_ttno_expectation():
    import pytreenet_gb300 as P
    for name in ["ttree3_heis_chi6_o1", "ternary2_xxz_chi4_o1", "c1_binary15_tfim_chi8"]:
        c = load_case(name)
        st = build_ttn(P.TTNS, c["spec"], c["final"])
        H = build_ttn(P.TTNO, c["spec"], c["ttno"])
        algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"], {},
                                       config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV))
        e = algo.evaluate_operator(H)
        assert abs(e - c["energy_final"]) < 1e-11 * max(1.0, abs(c["energy_final"]))


def test_gpu_contraction_helpers_match_oracle():
    """The contraction helpers on the real library against the oracle."""
    import pytreenet_gb300 as P
    from pytreenet_gb300 import contractions as C
    c = load_case("ttree3_heis_chi6_o1")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    ost = oracle_state(c)
    center = "root"
    cache = C.SandwichCache.init_cache_but_one(st, H, center)
    envs = O.init_cache_but_one(ost, c["ttno"], center)
    for key, e in envs.items():
        np.testing.assert_allclose(cache.get_entry(*key), e, atol=1e-12)
    x = st.tensors[center]
    y = C.contract_ket_ham_with_envs(st.nodes[center], x, H.nodes[center], None, cache)
    yo = O.heff_apply(ost.tensors[center], ost.tree, center, c["ttno"][center], envs)
    np.testing.assert_allclose(y, np.transpose(yo, st.logical_perm(center)), atol=1e-12)
    z = C.effective_single_site_evolution(x, st.nodes[center], None, H.nodes[center], 0.05, cache,
                                          mode=P.TimeEvoMode.KRYLOV, krylov_tol=1e-12)
    zo = O.krylov_exp_action(ost.tensors[center], lambda v: O.heff_apply(v, ost.tree, center, c["ttno"][center],
                                                                         envs), 0.05, -1j, krylov_tol=1e-12)
    np.testing.assert_allclose(z, np.transpose(zo, st.logical_perm(center)), atol=1e-11)


def test_gpu_dense_effective_hamiltonian():
    """get_effective_single_site_hamiltonian(_nodes) on the GB300 against the reference."""
    from golden_util import check_heff_fixture
    check_heff_fixture()


def test_gpu_ttns_observable_methods():
    """TTNS.scalar_product / operator_expectation_value on the GB300 against
    values the reference computed."""
    import os
    import pytreenet_gb300 as P
    from golden_util import GOLDEN
    Zm = np.diag([1.0, -1.0]).astype(complex)
    st = P.TTNS.load(os.path.join(GOLDEN, "saved_ttns"))
    vals = np.load(os.path.join(GOLDEN, "saved_ttns_values.npz"))
    assert abs(st.scalar_product() - vals["norm2"]) < 1e-12
    for i, nid in enumerate(str(x) for x in vals["ids"]):
        assert abs(st.operator_expectation_value(P.TensorProduct({nid: Zm})) - vals["z"][i]) < 1e-12
    c = load_case("ttree3_heis_chi6_o1")
    fin = build_ttn(P.TTNS, c["spec"], c["final"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    assert abs(fin.operator_expectation_value(H) - c["energy_final"]) < 1e-10


def test_gpu_exact_time_evolution():
    """ExactTimeEvolution on the GB300 against the reference's run."""
    import os
    from golden_util import GOLDEN
    from pytreenet_gb300.exact import ExactTimeEvolution, ExactTimeEvolutionConfig
    d = np.load(os.path.join(GOLDEN, "exact_evolution.npz"))
    ops = [d["op0"], d["op1"]]
    res = ExactTimeEvolution(d["psi"], d["H"], float(d["dt"]), float(d["final"]), ops).run()
    assert np.max(np.abs(res[1:] - d["closed_values"])) < 1e-12
    ev2 = ExactTimeEvolution(d["rho"], d["L"], float(d["dt"]), float(d["final"]), [d["O"]],
                             config=ExactTimeEvolutionConfig(open=True))
    for _ in range(4):
        ev2.run_one_time_step()
    assert abs(ev2.evaluate_operator(d["O"]) - d["open_final"]) < 1e-12


def test_gpu_direct_ttno_application():
    """apply_ttno_to_ttns (DIRECT) on the GB300 against dense H|psi>."""
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import binary_tfim_random_state
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Zm = np.diag([1.0, -1.0]).astype(complex)
    st, spec, tens, _, _ = binary_tfim_random_state(n=7, chi=8, seed=9)
    ids = [n for n, _ in spec]
    H = P.TTNO.from_hamiltonian(P.Hamiltonian([P.TensorProduct({"s3": X, "s0": Zm}),
                                               P.TensorProduct({"s2": X})]), st)

    def dense(ops):
        mats = [ops.get(n, np.eye(2)) for n in ids]
        out = mats[0]
        for m in mats[1:]:
            out = np.kron(out, m)
        return out
    psi = st.to_dense(ids)
    ref = (dense({"s3": X, "s0": Zm}) + dense({"s2": X})) @ psi
    got = P.apply_ttno_to_ttns(st, H).to_dense(ids)
    assert np.max(np.abs(got - ref)) < 1e-12 * np.max(np.abs(ref))


def test_gpu_apply_and_truncate():
    """apply_and_truncate(DIRECT, SVD) on the GB300: a tolerance-only truncation
    keeps H|psi>, a bond cap of 3 is respected."""
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import binary_tfim_random_state
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Zm = np.diag([1.0, -1.0]).astype(complex)
    st, spec, tens, _, _ = binary_tfim_random_state(n=7, chi=2, seed=4)
    ids = [n for n, _ in spec]
    terms = [P.TensorProduct({p: -Zm, n: Zm}) for n, p in spec if p is not None]
    terms += [P.TensorProduct({n: -0.7 * X}) for n, _ in spec]
    H = P.TTNO.from_hamiltonian(P.Hamiltonian(terms), st)
    ref = P.apply_ttno_to_ttns(st, H).to_dense(ids)
    loose = P.apply_and_truncate(st, H, P.ApplicationMethod.DIRECT, P.TruncationMethod.SVD,
                                 trunc_args=(P.SVDParameters(max_bond_dim=100, rel_tol=1e-13, total_tol=1e-13),))
    assert np.max(np.abs(loose.to_dense(ids) - ref)) < 1e-11 * np.max(np.abs(ref))
    tight = P.apply_and_truncate(st, H, P.ApplicationMethod.DIRECT, P.TruncationMethod.SVD,
                                 trunc_args=(P.SVDParameters(max_bond_dim=3, rel_tol=1e-10, total_tol=1e-10),))
    assert max(tight.phys(n).shape[0] for n in ids if n != "s0") <= 3


def test_gpu_recorded_run_matches_reference():
    """run(evaluation_time=2) with every record flag on the GB300 against the
    reference's Results (operators, bond dimensions, norm, Loschmidt amplitude)."""
    from golden_util import run_recorded_case
    res, ref = run_recorded_case()
    for name, arr in ref.items():
        key = tuple(name.split("/")[1:]) if name.startswith("bond/") else name
        got = res.operator_result(key) if key != "times" else res.times()
        assert np.max(np.abs(got - arr)) < 1e-9 * max(1.0, np.max(np.abs(arr))), name


@pytest.mark.parametrize("tag", ["cap", "tol"])
def test_gpu_zipup_matches_reference(tag):
    """Zip-up TTNO application on the GB300 against the reference's zipup."""
    from golden_util import check_zipup_fixture
    check_zipup_fixture(tag)


@pytest.mark.parametrize("tag", ["t4", "t6"])
def test_gpu_ttno_from_tensor(tag):
    """TTNO.from_tensor on the GB300: QR-mode node tensors equal the
    reference's; the SVD modes give the same operator."""
    import pytreenet_gb300 as P
    from golden_util import GOLDEN
    d = np.load(f"{GOLDEN}/ttno_from_tensor.npz")
    ids = [str(x) for x in d[f"{tag}/spec_ids"]]
    spec = list(zip(ids, [str(x) or None for x in d[f"{tag}/spec_parents"]]))
    tree = build_ttn(P.TTNS, spec, {nid: d[f"{tag}/init/{nid}"] for nid in ids})
    leg_dict = {nid: int(d[f"{tag}/leg/{nid}"]) for nid in ids}
    op = d[f"{tag}/op"]
    ttno = P.TTNO.from_tensor(tree, op, leg_dict)
    for nid in ids:
        ref = d[f"{tag}/ttno/{nid}"]
        got = np.asarray(ttno.tensors[nid])
        assert got.shape == ref.shape, nid
        assert np.abs(got - ref).max() < 1e-12 * max(1.0, np.abs(ref).max()), nid
    half = op.ndim // 2
    perm = [leg_dict[n] for n in ids] + [half + leg_dict[n] for n in ids]
    dim = int(np.prod([op.shape[leg_dict[n]] for n in ids]))
    dense = np.transpose(op, perm).reshape(dim, dim)
    for mode in (P.Decomposition.SVD, P.Decomposition.tSVD):
        m, _ = P.TTNO.from_tensor(tree, op, leg_dict, mode=mode).as_matrix(ids)
        assert np.abs(m - dense).max() < 1e-11 * np.abs(dense).max(), mode
