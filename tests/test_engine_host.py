"""Engine host logic on CPU: planning, leg orders, QR row tables, Krylov control.

The CUDA library is replaced by tests/fake_ptn.py (NumPy implementation of the
same C ABI), so these tests check everything the Python layer decides; the GPU
tests check the kernels through the real library.
"""
import numpy as np
import torch
import pytest

import fake_ptn
from golden_util import CASES, build_ttn, load_case, oracle_state, fidelity_and_dist

Zm = np.diag([1.0, -1.0]).astype(complex)


def _run_case(name, steps=None):
    import pytreenet_gb300 as P
    import oracle as O
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    cls = P.FirstOrderOneSiteTDVP if c["order"] == 1 else P.SecondOrderOneSiteTDVP
    algo = cls(st, H, c["dt"], c["dt"] * c["steps"], {},
               config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
               solver_options={"krylov_tol": c["krylov_tol"]})
    assert algo.update_path == c["update_path"]
    steps = c["steps"] if steps is None else steps
    zerr = 0.0
    for k in range(steps):
        algo.run_one_time_step()
        z = [algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]]
        zerr = max(zerr, float(np.max(np.abs(np.array(z) - c["z"][k]))))
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    return c, out, zerr


@pytest.mark.parametrize("name", [n for n in CASES if n != "c1_binary15_tfim_chi8"])
def test_engine_host_matches_reference(monkeypatch, name):
    fake_ptn.install(monkeypatch)
    c, out, zerr = _run_case(name)
    import oracle as O
    got = O.OState(oracle_state(c).tree, out)
    one_minus_f, dist = fidelity_and_dist(oracle_state(c, "final"), got)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12


def test_engine_host_c1_padded(monkeypatch):
    """Padded product state: the reference itself moves by ~2e-6 in state and
    ~5e-9 in <Z> under a 1e-15 input perturbation (noise-level Householder
    complements), so parity is bounded by that floor."""
    fake_ptn.install(monkeypatch)
    c, out, zerr = _run_case("c1_binary15_tfim_chi8", steps=10)
    assert zerr < 2e-8


@pytest.mark.parametrize("name,precision", [("ttree3_heis_chi6_o1", "bf16x6"), ("ternary2_xxz_chi4_o1", "bf16x3"),
                                            ("binary7_tfim_chi4_o2", "bf16x6"),
                                            ("c3shape_ttree20_heis_chi8_o1", "bf16x6")])
def test_engine_host_mixed_layouts(monkeypatch, name, precision):
    """The tensor-core plans (operand layouts chosen per step, epilogue strides)
    give the reference's result up to BF16x3 rounding."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    import oracle as O
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    cls = P.FirstOrderOneSiteTDVP if c["order"] == 1 else P.SecondOrderOneSiteTDVP
    algo = cls(st, H, c["dt"], c["dt"] * c["steps"], {},
               config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
               solver_options={"krylov_tol": c["krylov_tol"]}, precision=precision)
    for _ in range(c["steps"]):
        algo.run_one_time_step()
    got = O.OState(oracle_state(c).tree, {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]})
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), got)
    assert one_minus_f < (1e-8 if precision == "bf16x3" else 1e-11)


def test_engine_host_cholqr2_split(monkeypatch):
    """Mixed path, tall full-rank split: CholeskyQR2 (tensor-core Gram and
    solves) gives an isometric Q with Q R = A, like the Householder split."""
    fake_ptn.install(monkeypatch)
    import torch
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    from pytreenet_gb300.engine import DeviceNetwork
    st, spec, tensors = t_tree_state(arm_len=1, chi=64, seed=4)
    H, _ = t_tree_heisenberg(st, seed=5)
    net = DeviceNetwork(st, H, precision="mixed")
    A0 = net.t["root"].clone()
    R = net.qr_split("root", "a1_0").clone()
    Q = net.t["root"]
    # root legs (a0_0, a1_0, a2_0, s); split toward a1_0 (axis 1)
    Qm = Q.permute(0, 2, 3, 1).reshape(-1, 64).numpy()
    Am = A0.permute(0, 2, 3, 1).reshape(-1, 64).numpy()
    assert np.max(np.abs(Qm.conj().T @ Qm - np.eye(64))) < 1e-6
    assert np.max(np.abs(Qm @ R.numpy() - Am)) < 1e-6 * np.max(np.abs(Am))
    assert np.allclose(np.tril(R.numpy(), -1), 0)
    assert net.state.nodes["root"].children[0] == "a1_0"


# ---------------------------------------------------------------------------
# two-site TDVP (truncated SVD split) on the fake library
# ---------------------------------------------------------------------------
from golden_util import TWO_SITE_CASES, case_solver  # noqa: E402


def _run_two_site(name, precision="plain", order=2, dt=None, steps=None):
    import pytreenet_gb300 as P
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    mode, opts = case_solver(c, P)
    cfg = P.TwoSiteTDVPConfig(time_evo_mode=mode, main_path_mode=P.PathFinderMode[c["path_mode"]],
                              **c["svd"])
    cls = P.SecondOrderTwoSiteTDVP if order == 2 else P.FirstOrderTwoSiteTDVP
    dt = c["dt"] if dt is None else dt
    algo = cls(st, H, dt, dt * c["steps"], {}, config=cfg, solver_options=opts, precision=precision)
    assert algo.update_path == c["update_path"]
    zs = []
    for k in range(c["steps"] if steps is None else steps):
        algo.run_one_time_step()
        zs.append([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    return c, algo, out, np.array(zs)


@pytest.mark.parametrize("name", TWO_SITE_CASES)
def test_engine_host_two_site_matches_reference(monkeypatch, name):
    fake_ptn.install(monkeypatch)
    import oracle as O
    c, algo, out, zs = _run_two_site(name)
    got = O.OState(oracle_state(c).tree, out)
    fin = oracle_state(c, "final")
    for nid in fin.tensors:
        assert fin.tensors[nid].shape == out[nid].shape, nid
    one_minus_f, dist = fidelity_and_dist(fin, got)
    assert np.max(np.abs(zs - c["z"])) < 1e-10
    assert one_minus_f < 1e-12
    # the logical children order follows the reference's split rules
    for nid, _ in c["spec"]:
        assert algo.state.nodes[nid].children == algo.net.state.nodes[nid].children


from golden_util import CONFIG_SHAPE_CASES, CONFIG_SHAPE_TWO_SITE_CASES  # noqa: E402


@pytest.mark.parametrize("name", CONFIG_SHAPE_CASES)
def test_engine_host_config_shape_one_site(monkeypatch, name):
    """The engine's planning and Krylov control on the 61-site T-tree and the
    31-site binary TFIM with per-site fields, against the reference's runs."""
    fake_ptn.install(monkeypatch)
    import oracle as O
    c, out, zerr = _run_case(name)
    got = O.OState(oracle_state(c).tree, out)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), got)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", CONFIG_SHAPE_TWO_SITE_CASES)
def test_engine_host_config_shape_two_site(monkeypatch, name):
    """Two-site TDVP with bond growth on the 40-site ternary tree and the
    31-site binary tree with random fields, against the reference's runs:
    same final bond dimensions, <Z_i> to 1e-10, 1-F < 1e-12."""
    fake_ptn.install(monkeypatch)
    import oracle as O
    c, algo, out, zs = _run_two_site(name)
    fin = oracle_state(c, "final")
    for nid in fin.tensors:
        assert fin.tensors[nid].shape == out[nid].shape, nid
    one_minus_f, _ = fidelity_and_dist(fin, O.OState(oracle_state(c).tree, out))
    assert np.max(np.abs(zs - c["z"])) < 1e-10
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", CONFIG_SHAPE_TWO_SITE_CASES)
def test_engine_host_config_shape_two_site_mixed(monkeypatch, name):
    """The BF16x6 plans of the two-site path (emulated by the stand-in
    library) on the same trees: measured |dZ| 2e-7 to 4e-7 and 1-F below
    3e-13 against the reference, with the same final bond dimensions."""
    fake_ptn.install(monkeypatch)
    import oracle as O
    c, algo, out, zs = _run_two_site(name, precision="mixed")
    fin = oracle_state(c, "final")
    for nid in fin.tensors:
        assert fin.tensors[nid].shape == out[nid].shape, nid
    one_minus_f, _ = fidelity_and_dist(fin, O.OState(oracle_state(c).tree, out))
    assert np.max(np.abs(zs - c["z"])) < 2e-6
    assert one_minus_f < 1e-10


def test_engine_host_first_order_two_site_matches_oracle(monkeypatch):
    fake_ptn.install(monkeypatch)
    import oracle as O
    c, algo, out, zs = _run_two_site("ternary2_xxz_neel_2tdvp", order=1, dt=0.01, steps=3)
    ora = O.FirstOrderTwoSiteTDVPOracle(oracle_state(c), c["ttno"], 0.01, O.SVDParams(**c["svd"]),
                                        krylov_tol=c["krylov_tol"])
    for _ in range(3):
        ora.run_one_time_step()
    got = O.OState(oracle_state(c).tree, out)
    one_minus_f, dist = fidelity_and_dist(ora.state, got)
    assert one_minus_f < 1e-12
    assert algo.bond_dims_history == ora.bond_history


def test_svd_parameters_validation():
    import pytreenet_gb300 as P
    with pytest.raises(TypeError):
        P.SVDParameters(max_bond_dim=2.5)
    with pytest.raises(ValueError):
        P.SVDParameters(rel_tol=-1.0)
    with pytest.raises(ValueError):
        P.SVDParameters(max_bond_dim=0)
    d = np.load(f"{__import__('golden_util').GOLDEN}/units.npz")
    for i in range(int(d["svd/n"])):
        maxd, rel, tot, renorm, sumt = d[f"svd/{i}/params"]
        p = P.SVDParameters(max_bond_dim=int(maxd), rel_tol=rel, total_tol=tot, renorm=bool(renorm),
                            sum_trunc=bool(sumt))
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            new_s, _ = P.truncate_singular_values(d[f"svd/{i}/s"], p)
        np.testing.assert_allclose(new_s, d[f"svd/{i}/out"], rtol=1e-15, atol=0)
    # random=True: the reference keeps exactly max_bond_dim values, no tolerance
    s = np.array([3.0, 1.0, 1e-12, 1e-14])
    kept, cut = P.truncate_singular_values(s, P.SVDParameters(max_bond_dim=3, rel_tol=1e-3, random=True))
    assert list(kept) == [3.0, 1.0, 1e-12] and list(cut) == [1e-14]
    with pytest.raises(ValueError):
        P.SVDParameters(random=True, max_bond_dim=float("inf"))


def _two_site_vs_oracle(chi, max_bond_dim, steps=2):
    import pytreenet_gb300 as P
    import oracle as O
    from pytreenet_gb300.workloads import ternary_state, ternary_xxz
    st, spec, tensors = ternary_state(depth=2, chi=chi, seed=11)
    H, Wphys = ternary_xxz(st, seed=12)
    svd = dict(max_bond_dim=max_bond_dim, rel_tol=1e-10, total_tol=1e-10)
    cfg = P.TwoSiteTDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV, **svd)
    algo = P.SecondOrderTwoSiteTDVP(st, H, 0.02, 0.02 * steps, {}, config=cfg,
                                    solver_options={"krylov_tol": 1e-12})
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    ora = O.SecondOrderTwoSiteTDVPOracle(O.OState(tree, tensors), Wphys, 0.02, O.SVDParams(**svd),
                                         krylov_tol=1e-12)
    for _ in range(steps):
        algo.run_one_time_step()
        ora.run_one_time_step()
    got = O.OState(tree, {nid: algo.state.get_phys_numpy(nid) for nid, _ in spec})
    return algo, ora, fidelity_and_dist(ora.state, got)


def test_engine_host_two_site_subspace_split(monkeypatch):
    """Subspace-iteration reduction of large merged pairs (forced on small ones)."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300.engine as E
    monkeypatch.setattr(E.DeviceNetwork, "SVD_DIRECT_MAX", 8)
    calls = []
    orig = E.DeviceNetwork._subspace_factor
    monkeypatch.setattr(E.DeviceNetwork, "_subspace_factor", lambda self, *a: calls.append(a[1:]) or orig(self, *a))
    algo, ora, (one_minus_f, dist) = _two_site_vs_oracle(12, 5)
    assert calls
    assert algo.bond_dims_history == ora.bond_history
    assert one_minus_f < 1e-12


def test_engine_host_qr_buffers_follow_bond_growth(monkeypatch):
    """Two-site splits grow bonds; every later QR split must find R and the
    work area large enough for its own (rows, k) -- sized by the library's own
    ptn_zqr_work_bytes (a host-only function of the real .so)."""
    import ctypes
    fake = fake_ptn.install(monkeypatch)
    from pytreenet_gb300.build import LIB, build
    build()
    real = ctypes.CDLL(LIB)
    real.ptn_zqr_work_bytes.restype = ctypes.c_int64
    real.ptn_zqr_work_bytes.argtypes = [ctypes.c_int64, ctypes.c_int64]
    monkeypatch.setattr(type(fake), "ptn_zqr_work_bytes", lambda self, m, k: int(real.ptn_zqr_work_bytes(m, k)))
    import pytreenet_gb300.engine as E
    orig = E.DeviceNetwork.qr_split
    checked = []

    def qr_split(self, nid, nbr):
        R = orig(self, nid, nbr)
        k = self.shape(nid)[self.state.phys_axis(nid, nbr)]
        m = self.t[nid].numel() // k
        assert self.qr_R.numel() >= k * k
        assert self.qr_work.numel() * 16 >= real.ptn_zqr_work_bytes(m, k), (nid, nbr, m, k)
        checked.append((m, k))
        return R
    monkeypatch.setattr(E.DeviceNetwork, "qr_split", qr_split)
    # chi = 12: the first splits shrink a depth-1 node's leg to 2, so its QR
    # toward the root drops from 3456 rows (multi-kernel path) to 576 rows
    # (one-launch path, whose V buffer needs m * min(m, k) entries)
    algo, ora, (one_minus_f, dist) = _two_site_vs_oracle(12, 5, steps=1)
    assert checked
    assert one_minus_f < 1e-12


def test_engine_host_tebd_matches_reference(monkeypatch):
    fake_ptn.install(monkeypatch)
    from golden_util import TEBD_CASES, run_tebd_case
    for name in TEBD_CASES:
        c, got, zs, algo = run_tebd_case(name)
        fin = oracle_state(c, "final")
        for nid in fin.tensors:
            assert fin.tensors[nid].shape == got.tensors[nid].shape
        one_minus_f, _ = fidelity_and_dist(fin, got)
        assert np.max(np.abs(zs - c["z"])) < 1e-13 * np.max(np.abs(c["z"]))
        assert one_minus_f < 1e-13


def test_engine_host_trotter_splitting_matches_fixture_gates(monkeypatch):
    """The engine's own TrotterSplitting gives the gates the reference built."""
    import pytreenet_gb300 as P
    c = load_case("binary7_tfim_tebd")
    Xm = np.array([[0, 1], [1, 0]], dtype=complex)
    steps = [P.TrotterStep({p: -1.0 * Zm, nid: Zm}, 1.0) for nid, p in c["spec"] if p is not None]
    steps += [P.TrotterStep({nid: -0.7 * Xm}, 1.0) for nid, _ in c["spec"]]
    ops = P.TrotterSplitting(steps).exponentiate_splitting(c["dt"])
    assert len(ops) == len(c["gates"])
    for mine, (op, ids) in zip(ops, c["gates"]):
        assert list(mine.node_identifiers) == ids
        np.testing.assert_allclose(mine.operator, op, atol=1e-14)


def test_engine_host_ttno_expectation(monkeypatch):
    """<psi|H|psi> through a TDVP driver's evaluate_operator, against the
    reference's value on the reference's final state."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    for name in ["ttree3_heis_chi6_o1", "ternary2_xxz_chi4_o1"]:
        c = load_case(name)
        st = build_ttn(P.TTNS, c["spec"], c["final"])
        H = build_ttn(P.TTNO, c["spec"], c["ttno"])
        algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"], {},
                                       config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV))
        e = algo.evaluate_operator(H)
        assert abs(e - c["energy_final"]) < 1e-11 * max(1.0, abs(c["energy_final"]))


def test_engine_host_realisations_concurrent_equals_sequential(monkeypatch):
    """Independent realisations run by several worker threads give exactly the
    results of running them one after the other."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import binary_neel_random_field

    def make(i):
        st, H, spec, _, _ = binary_neel_random_field(n=7, seed=i)
        cfg = P.TwoSiteTDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV, max_bond_dim=4, rel_tol=1e-9,
                                  total_tol=1e-9)
        return P.SecondOrderTwoSiteTDVP(st, H, 0.05, 1.0, {}, config=cfg, solver_options={"krylov_tol": 1e-10})

    def done(i, algo):
        return (list(algo.bond_dims_history), {nid: algo.state.get_phys_numpy(nid).copy() for nid in algo.state._order})
    seq = P.run_realisations(make, 5, 2, workers=1, on_done=done)
    par = P.run_realisations(make, 5, 2, workers=3, on_done=done)
    for (h1, s1), (h2, s2) in zip(seq, par):
        assert h1 == h2
        for nid in s1:
            np.testing.assert_array_equal(s1[nid], s2[nid])
    assert seq[0][0] != seq[1][0] or any(not np.array_equal(seq[0][1][k], seq[1][1][k]) for k in seq[0][1])


_CHILD_STANDIN = None


def _standin_disorder_make(i):
    """Realisation builder for a spawned worker process: the process starts
    without the CPU stand-in for the library, so it installs it first."""
    global _CHILD_STANDIN
    if _CHILD_STANDIN is None:
        _CHILD_STANDIN = pytest.MonkeyPatch()
        fake_ptn.install(_CHILD_STANDIN)
    from pytreenet_gb300.workloads import disorder_realisation
    return disorder_realisation(i, caps=(2, 4), precision="plain", n=7)


def _realisation_result(i, algo):
    return (list(algo.bond_dims_history), {nid: algo.state.get_phys_numpy(nid).copy() for nid in algo.state._order})


def test_realisations_in_worker_processes_equal_sequential(monkeypatch):
    """run_realisations over two spawned worker processes returns, in
    realisation order, exactly the results of running the realisations one
    after the other in this process; without on_done it refuses."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import disorder_realisation
    seq = P.run_realisations(lambda i: disorder_realisation(i, caps=(2, 4), precision="plain", n=7), 4, 2,
                             workers=1, on_done=_realisation_result)
    par = P.run_realisations(_standin_disorder_make, 4, 2, workers=1, on_done=_realisation_result, processes=2)
    for (h1, s1), (h2, s2) in zip(seq, par):
        assert h1 == h2
        for nid in s1:
            np.testing.assert_array_equal(s1[nid], s2[nid])
    with pytest.raises(ValueError):
        P.run_realisations(_standin_disorder_make, 2, 1, processes=2)


def test_contraction_helpers_match_oracle(monkeypatch):
    """SandwichCache / contract_ket_ham_with_envs / contract_any /
    effective_single_site_evolution in the reference's conventions, against the
    oracle's restatement."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from pytreenet_gb300 import contractions as C
    import oracle as O
    c = load_case("ttree3_heis_chi6_o1")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    ost = oracle_state(c)
    center = "a0_1"
    cache = C.SandwichCache.init_cache_but_one(st, H, center)
    envs = O.init_cache_but_one(ost, c["ttno"], center)
    for key, e in envs.items():
        assert key in cache
        np.testing.assert_allclose(cache.get_entry(*key), e, atol=1e-12)
    # matvec in the node's logical leg order
    x = st.tensors[center]
    y = C.contract_ket_ham_with_envs(st.nodes[center], x, H.nodes[center], None, cache)
    yo = O.heff_apply(ost.tensors[center], ost.tree, center, c["ttno"][center], envs)
    np.testing.assert_allclose(y, np.transpose(yo, st.logical_perm(center)), atol=1e-12)
    # environment recomputed toward a neighbour
    e = C.contract_any(center, "a0_2", st, H, cache)
    eo = O.env_update(ost.tree, center, "a0_2", ost.tensors[center], c["ttno"][center], envs)
    np.testing.assert_allclose(e, eo, atol=1e-12)
    # Krylov exponential of the site
    z = C.effective_single_site_evolution(x, st.nodes[center], None, H.nodes[center], 0.05, cache,
                                          mode=P.TimeEvoMode.KRYLOV, krylov_tol=1e-12)
    zo = O.krylov_exp_action(ost.tensors[center], lambda v: O.heff_apply(v, ost.tree, center,
                                                                         c["ttno"][center], envs),
                             0.05, -1j, krylov_tol=1e-12)
    np.testing.assert_allclose(z, np.transpose(zo, st.logical_perm(center)), atol=1e-11)
    # the node-id form with the default mode (FASTEST: exact) against the dense exponential
    zf = C.single_site_time_evolution(center, st, H, 0.05, cache)
    zd = O.dense_exp_action(ost.tensors[center], lambda v: O.heff_apply(v, ost.tree, center, c["ttno"][center],
                                                                        envs), 0.05, -1j)
    np.testing.assert_allclose(zf, np.transpose(zd, st.logical_perm(center)), atol=1e-12)
    # a tensor of another shape is refused before anything runs on the device
    with pytest.raises(ValueError):
        C.effective_single_site_evolution(x[..., :1], st.nodes[center], None, H.nodes[center], 0.05, cache)
    with pytest.raises(ValueError):
        C.contract_ket_ham_with_envs(st.nodes[center], x[..., :1], H.nodes[center], None, cache)


def test_finite_difference_gradient_matches_oracle(monkeypatch):
    """d<Z_root>(T)/d(g_i, J) on a 3-site tree: the engine's finite-difference
    gradient equals the same differences taken with the oracle's evolution,
    and the derivative of the exact (dense) evolution to the FD accuracy."""
    fake_ptn.install(monkeypatch)
    import scipy.linalg
    import oracle as O
    from pytreenet_gb300.gradients import finite_difference_gradient, tfim_z_root_evolution
    from pytreenet_gb300.workloads import binary_tfim_product_state
    from pytreenet_gb300.operators import tfim_ttno
    n, chi, dt, steps = 3, 2, 0.05, 4
    f = tfim_z_root_evolution(n=n, chi=chi, dt=dt, steps=steps, seed=3)
    theta = np.array([0.4, 0.5, 0.6, 1.0])
    g = finite_difference_gradient(f, theta, step=1e-5, workers=2)
    # exact evolution on the 8-dimensional Hilbert space
    st, _, spec, tensors = binary_tfim_product_state(n=n, chi=chi, seed=3)
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    ids = [s[0] for s in spec]
    psi0 = O.state_vector(O.OState(tree, tensors), ids)
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Zm_ = np.diag([1.0, -1.0]).astype(complex)

    def op(site, M):
        mats = [np.eye(2, dtype=complex)] * n
        mats[site] = M
        out = mats[0]
        for m_ in mats[1:]:
            out = np.kron(out, m_)
        return out

    def exact(th):
        Hd = -th[n] * (op(0, Zm_) @ op(1, Zm_) + op(0, Zm_) @ op(2, Zm_))
        Hd = Hd - sum(th[i] * op(i, X) for i in range(n))
        psi = scipy.linalg.expm(-1j * dt * steps * Hd) @ psi0
        return float(np.real(np.vdot(psi, op(0, Zm_) @ psi)) / np.vdot(psi, psi).real)
    ge = np.array([(exact(theta + 1e-5 * np.eye(4)[k]) - exact(theta - 1e-5 * np.eye(4)[k])) / 2e-5
                   for k in range(4)])
    assert np.max(np.abs(g - ge)) < 1e-5


@pytest.mark.parametrize("name", ["binary7_tfim_driven_o1", "binary7_tfim_driven_o2"])
def test_engine_host_time_dependent_hamiltonian(monkeypatch, name):
    """Driven field through TimeDependentTTNO and config.time_dep: the engine's
    run() reproduces the reference's <Z_i>(t) and final state."""
    fake_ptn.install(monkeypatch)
    from golden_util import run_driven_case
    c, st, z = run_driven_case(name)
    assert np.max(np.abs(z - c["z"].real)) < 1e-10
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert one_minus_f < 1e-12


def test_time_dependent_ttno_api(monkeypatch):
    """time_dep without a time-dependent TTNO raises TypeError (as the
    reference); updates, resets and the discrete switcher act on the tensors
    in the reference's leg order."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from pytreenet_gb300.time_dep import DiscreetTimeTTNO, FactorUpdatable, TimeDependentTTNO
    c = load_case("binary7_tfim_driven_o1")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], {k: v.copy() for k, v in c["ttno"].items()})
    with pytest.raises(TypeError):
        P.FirstOrderOneSiteTDVP(st, H, 0.1, 1.0, {}, config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV,
                                                                          time_dep=True))
    base = H.get_tensor("s1").copy()
    D = np.ones((1, 1, 1, 2, 2))
    u = FactorUpdatable("s1", (0, 1, 2, slice(0, 2), slice(0, 2)), D, lambda t: 2.0 * t)
    T = TimeDependentTTNO([u], H)
    T.update(0.25)
    T.update(0.25)
    got = T.get_tensor("s1")
    exp = base.copy()
    exp[0, 1, 2] += 1.0
    assert np.allclose(got, exp)
    T.reset()
    assert np.allclose(T.get_tensor("s1"), base)
    H2 = build_ttn(P.TTNO, c["spec"], {k: 2 * v for k, v in c["ttno"].items()})
    Dt = DiscreetTimeTTNO([H, H2], dt=0.5)
    Dt.update(0.3)
    assert np.allclose(Dt.get_tensor("s0"), H.get_tensor("s0"))
    Dt.update(0.3)
    assert np.allclose(Dt.get_tensor("s0"), H2.get_tensor("s0"))
    Dt.reset()
    assert np.allclose(Dt.get_tensor("s0"), H.get_tensor("s0"))


def test_num_time_steps_rule():
    """``_compute_num_time_steps``: floor when the fractional part is below 0.1."""
    from pytreenet_gb300.tdvp import compute_num_time_steps
    assert compute_num_time_steps(0.3, 0.05) == 6          # 5.999... and 6.000...1 both give 6
    assert compute_num_time_steps(0.35, 0.1) == 4
    assert compute_num_time_steps(1.0, 0.3) == 4           # 3.33: fraction 0.33 -> one more step
    assert compute_num_time_steps(1.005, 0.1) == 10        # 10.05: fraction below 0.1 -> 10


def test_ttn_files_written_by_reference(monkeypatch, tmp_path):
    """PyTreeNet's save format (``core/ttn.py:1747-1838``): files written by the
    reference load into the engine's classes with the same values, and saving
    them again reproduces the files."""
    import json
    import os
    import pytreenet_gb300 as P
    from golden_util import GOLDEN
    st = P.TTNS.load(os.path.join(GOLDEN, "saved_ttns"))
    H = P.TTNO.load(os.path.join(GOLDEN, "saved_ttno"))
    vals = np.load(os.path.join(GOLDEN, "saved_ttns_values.npz"))
    ids = [str(x) for x in vals["ids"]]
    psi = st.to_dense(ids)
    n = len(ids)
    for i, nid in enumerate(ids):
        zi = np.ones(1)
        for j in range(n):
            zi = np.kron(zi, np.array([1.0, -1.0]) if j == i else np.ones(2))
        assert abs(np.vdot(psi, zi * psi) - vals["z"][i]) < 1e-12
    assert abs(np.vdot(psi, psi) - vals["norm2"]) < 1e-12
    assert st.orthogonality_center_id == "s3"
    for obj, name in ((st, "saved_ttns"), (H, "saved_ttno")):
        out = str(tmp_path / name)
        obj.save(out)
        with open(out + ".json") as f, open(os.path.join(GOLDEN, name + ".json")) as g:
            assert json.load(f) == json.load(g)
        a, b = np.load(out + ".npz"), np.load(os.path.join(GOLDEN, name + ".npz"))
        assert sorted(a.files) == sorted(b.files)
        for k in a.files:
            assert np.array_equal(a[k], b[k])
    # a loaded state and operator drive the engine
    fake_ptn.install(monkeypatch)
    algo = P.FirstOrderOneSiteTDVP(st, H, 0.05, 0.1, {}, config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV))
    algo.run_one_time_step()
    assert abs(algo.evaluate_operator(P.TensorProduct({})) - vals["norm2"]) < 1e-10


@pytest.mark.parametrize("name", ["binary15_tfim_fixed_bug", "ternary2_xxz_fixed_bug"])
def test_engine_host_fixed_bug_matches_reference(monkeypatch, name):
    """Fixed-rank BUG on the engine against the reference's FixedBUG."""
    fake_ptn.install(monkeypatch)
    from golden_util import run_bug_case
    c, st, z = run_bug_case(name)
    assert np.max(np.abs(z - c["z"])) < 1e-10
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", ["ttree3_heis_l2l_o1", "binary15_tfim_l2l_o2"])
def test_engine_host_leaf_to_leaf_path(monkeypatch, name):
    """TDVPConfig(main_path_mode=LeafToLeaf): the reference's path and results."""
    fake_ptn.install(monkeypatch)
    from golden_util import run_one_site_case
    c, st, zerr = run_one_site_case(name)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", ["binary7_tfim_bug", "ternary2_xxz_bug"])
def test_engine_host_adaptive_bug_matches_reference(monkeypatch, name):
    """Rank-adaptive BUG on the engine against the reference's BUG, bond
    dimensions included."""
    fake_ptn.install(monkeypatch)
    from golden_util import run_adaptive_bug_case
    c, st, z, bonds, ref_bonds = run_adaptive_bug_case(name)
    assert np.array_equal(bonds, ref_bonds)
    assert np.max(np.abs(z - c["z"])) < 1e-9
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert one_minus_f < 1e-11


@pytest.mark.parametrize("name", ["binary7_tfim_tebd_swaps", "binary7_tfim_tebd_strang"])
def test_engine_host_swap_splitting_matches_reference(monkeypatch, name):
    """TrotterSplitting.from_lists with SWAP lists or with a symmetric
    (Strang) order of factors: the same gate sequence as the reference's, and
    TEBD driven by it reproduces the reference's run."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from golden_util import swap_splitting
    c = load_case(name)
    split = swap_splitting(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    assert split[-1].swaps_before.is_compatible_with_ttn(st)
    gates = split.exponentiate_splitting(c["dt"], ttn=st)
    assert len(gates) == len(c["gates"])
    for g, (op, ids) in zip(gates, c["gates"]):
        assert list(g.node_identifiers) == ids
        assert np.allclose(g.operator, op, atol=1e-14)
    algo = P.TEBD(st, split, c["dt"], c["dt"] * c["steps"], {}, svd_parameters=P.SVDParameters(**c["svd"]))
    for k in range(c["steps"]):
        algo.run_one_time_step()
        z = np.array([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
        assert np.max(np.abs(z - c["z"][k])) < 1e-12 * np.max(np.abs(c["z"]))
    with pytest.raises(ValueError):
        bad = P.TrotterSplitting([P.TrotterStep({"s3": Zm, "s0": Zm}, 1.0)])
        P.TEBD(build_ttn(P.TTNS, c["spec"], c["init"]), bad, 0.1, 0.1, {}).run_one_time_step()


@pytest.mark.parametrize("name", ["ttree3_heis_fastest_o1", "binary7_tfim_fastest_o2"])
def test_engine_host_default_mode(monkeypatch, name):
    """TDVPConfig(time_evo_mode=FASTEST), the reference's default: the engine's
    matrix-free exponential at its exact-mode stop reproduces the reference's
    dense exponential."""
    fake_ptn.install(monkeypatch)
    from golden_util import run_one_site_case
    c, st, zerr = run_one_site_case(name)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert zerr < 1e-11
    assert one_minus_f < 1e-12


def test_engine_host_dense_effective_hamiltonian(monkeypatch):
    """get_effective_single_site_hamiltonian(_nodes) against the reference."""
    fake_ptn.install(monkeypatch)
    from golden_util import check_heff_fixture
    check_heff_fixture()


def test_ttns_observable_methods_match_reference(monkeypatch):
    """TTNS.scalar_product / norm / normalise / operator_expectation_value /
    distance on the engine against values the reference computed."""
    import os
    import oracle as O
    import pytreenet_gb300 as P
    from golden_util import GOLDEN
    fake_ptn.install(monkeypatch)
    st = P.TTNS.load(os.path.join(GOLDEN, "saved_ttns"))
    vals = np.load(os.path.join(GOLDEN, "saved_ttns_values.npz"))
    assert abs(st.scalar_product() - vals["norm2"]) < 1e-12
    for i, nid in enumerate(str(x) for x in vals["ids"]):
        assert abs(st.operator_expectation_value(P.TensorProduct({nid: Zm})) - vals["z"][i]) < 1e-12
        assert abs(st.single_site_operator_expectation_value(nid, Zm) - vals["z"][i]) < 1e-12
    # energy of a reference final state under its TTNO
    c = load_case("ttree3_heis_chi6_o1")
    fin = build_ttn(P.TTNS, c["spec"], c["final"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    assert abs(fin.operator_expectation_value(H) - c["energy_final"]) < 1e-10
    # overlaps between two states, against the oracle
    a = build_ttn(P.TTNS, c["spec"], c["init"])
    b = build_ttn(P.TTNS, c["spec"], c["final"])
    ref = O.scalar_product(oracle_state(c, "final"), oracle_state(c, "init"))   # sum init * conj(final)
    assert abs(a.scalar_product(b) - ref) < 1e-12 * max(1.0, abs(ref))
    d = a.distance(b)
    na, nb = O.scalar_product(oracle_state(c), oracle_state(c)).real, \
        O.scalar_product(oracle_state(c, "final"), oracle_state(c, "final")).real
    assert abs(d - np.sqrt(abs(na - 2 * abs(ref) + nb))) < 1e-10
    n0 = a.normalise()
    assert abs(n0 - np.sqrt(na)) < 1e-12 and abs(a.norm() - 1.0) < 1e-12
    with pytest.raises(TypeError):
        a.operator_expectation_value(3)


def _symbolic_tfim(spec, J, g):
    import pytreenet_gb300 as P
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    conv = {"mJZ": -J * Zm, "Z": Zm, "mgX": -g * X}
    terms = [P.TensorProduct({p: "mJZ", nid: "Z"}) for nid, p in spec if p is not None]
    terms += [P.TensorProduct({nid: "mgX"}) for nid, _ in spec]
    return P.Hamiltonian(terms, conv)


def test_ttno_from_hamiltonian_is_the_reference_operator():
    """TTNO.from_hamiltonian builds the same operator as the reference's TTNO
    (expectation values on random states with full bond dimensions), with the
    reference's bond dimension for nearest-neighbour models."""
    import oracle as O
    import pytreenet_gb300 as P
    c = load_case("binary7_tfim_fastest_o2")          # TFIM, J = 1, g = 0.9
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = P.TTNO.from_hamiltonian(_symbolic_tfim(c["spec"], 1.0, 0.9), st)
    W = {nid: H.phys(nid) for nid, _ in c["spec"]}
    assert max(max(w.shape[:-2], default=0) for w in W.values()) == 3
    rng = np.random.default_rng(0)
    from pytreenet_gb300.workloads import binary_tfim_random_state
    for _ in range(4):
        s, spec, tens, _, _ = binary_tfim_random_state(n=7, chi=8, seed=int(rng.integers(1 << 30)))
        ost = O.OState(oracle_state(c).tree, tens)
        a = O.ttno_expectation(ost, W)
        b = O.ttno_expectation(ost, c["ttno"])
        assert abs(a - b) < 1e-12 * max(1.0, abs(b))
    # a long-range, multi-site, symbolic-coefficient Hamiltonian against a dense sum
    from fractions import Fraction
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
    terms = [(Fraction(1, 2), "K", P.TensorProduct({"s3": "X", "s6": "Y", "s0": "Z"})),
             (Fraction(1), "1", P.TensorProduct({"s4": "Z", "s5": "Z"})),
             P.TensorProduct({"s2": X}), (Fraction(3), "K", P.TensorProduct({"s3": "X", "s6": "Y"}))]
    Hs = P.Hamiltonian(terms, {"X": X, "Y": Y, "Z": Zm}, {"K": 0.7})
    Ht = P.TTNO.from_hamiltonian(Hs, st)
    Wt = {nid: Ht.phys(nid) for nid, _ in c["spec"]}
    ids = [n for n, _ in c["spec"]]

    def dense(ops):
        mats = [ops.get(n, np.eye(2)) for n in ids]
        out = mats[0]
        for m in mats[1:]:
            out = np.kron(out, m)
        return out
    Hd = 0.35 * dense({"s3": X, "s6": Y, "s0": Zm}) + dense({"s4": Zm, "s5": Zm}) + dense({"s2": X}) \
        + 2.1 * dense({"s3": X, "s6": Y})
    for _ in range(3):
        s, spec, tens, _, _ = binary_tfim_random_state(n=7, chi=8, seed=int(rng.integers(1 << 30)))
        ost = O.OState(oracle_state(c).tree, tens)
        v = O.state_vector(ost, ids)
        assert abs(O.ttno_expectation(ost, Wt) - np.vdot(v, Hd @ v)) < 1e-12 * max(1.0, np.linalg.norm(v) ** 2)


def test_ttno_from_hamiltonian_drives_tdvp(monkeypatch):
    """One-site TDVP with a TTNO from TTNO.from_hamiltonian reproduces the
    reference's run, which used the reference's own TTNO."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    c = load_case("binary15_tfim_l2l_o2")              # TFIM, J = 1, g = 0.6
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = P.TTNO.from_hamiltonian(_symbolic_tfim(c["spec"], 1.0, 0.6), st)
    algo = P.SecondOrderOneSiteTDVP(st, H, c["dt"], c["dt"] * c["steps"], {},
                                    config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV,
                                                        main_path_mode=P.PathFinderMode.LeafToLeaf),
                                    solver_options={"krylov_tol": c["krylov_tol"]})
    for k in range(c["steps"]):
        algo.run_one_time_step()
        z = np.array([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
        assert np.max(np.abs(z - c["z"][k])) < 1e-10


def test_exact_time_evolution_matches_reference(monkeypatch):
    """ExactTimeEvolution (closed and open) against the reference's run."""
    import os
    fake_ptn.install(monkeypatch)
    from golden_util import GOLDEN
    from pytreenet_gb300.exact import ExactTimeEvolution, ExactTimeEvolutionConfig
    d = np.load(os.path.join(GOLDEN, "exact_evolution.npz"))
    ops = [d["op0"], d["op1"]]
    ev = ExactTimeEvolution(d["psi"], d["H"], float(d["dt"]), float(d["final"]), ops)
    assert ev.num_time_steps == 4
    for k in range(4):
        ev.run_one_time_step()
        got = [ev.evaluate_operator(o) for o in ops]
        assert np.max(np.abs(np.array(got) - d["closed_values"][k])) < 1e-12
    res = ExactTimeEvolution(d["psi"], d["H"], float(d["dt"]), float(d["final"]), ops).run()
    assert np.max(np.abs(res[1:] - d["closed_values"])) < 1e-12
    ev2 = ExactTimeEvolution(d["rho"], d["L"], float(d["dt"]), float(d["final"]), [d["O"]],
                             config=ExactTimeEvolutionConfig(open=True))
    for _ in range(4):
        ev2.run_one_time_step()
    assert abs(ev2.evaluate_operator(d["O"]) - d["open_final"]) < 1e-12


def test_direct_ttno_application(monkeypatch):
    """apply_ttno_to_ttns (DIRECT) and TTNS.apply_operator against dense H|psi>."""
    fake_ptn.install(monkeypatch)
    import oracle as O
    import pytreenet_gb300 as P
    from fractions import Fraction
    from pytreenet_gb300.workloads import binary_tfim_random_state
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
    st, spec, tens, _, _ = binary_tfim_random_state(n=7, chi=8, seed=9)
    ids = [n for n, _ in spec]
    terms = [(Fraction(1, 2), "K", P.TensorProduct({"s3": "X", "s6": "Y", "s0": "Z"})),
             P.TensorProduct({"s4": "Z", "s5": "Z"}), P.TensorProduct({"s2": X})]
    H = P.TTNO.from_hamiltonian(P.Hamiltonian(terms, {"X": X, "Y": Y, "Z": Zm}, {"K": 0.7}), st)

    def dense(ops):
        mats = [ops.get(n, np.eye(2)) for n in ids]
        out = mats[0]
        for m in mats[1:]:
            out = np.kron(out, m)
        return out
    Hd = 0.35 * dense({"s3": X, "s6": Y, "s0": Zm}) + dense({"s4": Zm, "s5": Zm}) + dense({"s2": X})
    psi = st.to_dense(ids)
    out = P.apply_ttno_to_ttns(st, H)
    got = out.to_dense(ids)
    assert np.max(np.abs(got - Hd @ psi)) < 1e-12 * np.max(np.abs(Hd @ psi))
    assert out.phys("s1").shape[0] == st.phys("s1").shape[0] * H.phys("s1").shape[0]
    st2, _, _, _, _ = binary_tfim_random_state(n=7, chi=8, seed=9)
    st2.apply_operator(P.TensorProduct({"s2": X, "s5": Zm}))
    assert np.max(np.abs(st2.to_dense(ids) - dense({"s2": X, "s5": Zm}) @ psi)) < 1e-12
    with pytest.raises(NotImplementedError):
        P.apply_ttno_to_ttns(st, H, method=P.ApplicationMethod.VARIATIONAL)


def test_apply_and_truncate_matches_oracle(monkeypatch):
    """apply_and_truncate(DIRECT, SVD): the engine's truncated H|psi> equals the
    oracle's svd_truncation of the same state (a binding bond cap), and without
    a cap the truncation only removes the zero directions."""
    fake_ptn.install(monkeypatch)
    import oracle as O
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import binary_tfim_random_state
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    st, spec, tens, _, _ = binary_tfim_random_state(n=7, chi=2, seed=4)
    ids = [n for n, _ in spec]
    H = P.TTNO.from_hamiltonian(_symbolic_tfim(spec, 1.0, 0.7), st)
    full = P.apply_ttno_to_ttns(st, H)
    ref_vec = full.to_dense(ids)
    loose = P.apply_and_truncate(st, H, P.ApplicationMethod.DIRECT, P.TruncationMethod.SVD,
                                 trunc_args=(P.SVDParameters(max_bond_dim=100, rel_tol=1e-13, total_tol=1e-13),))
    assert np.max(np.abs(loose.to_dense(ids) - ref_vec)) < 1e-11 * np.max(np.abs(ref_vec))
    params = P.SVDParameters(max_bond_dim=3, rel_tol=1e-10, total_tol=1e-10)
    tight = P.apply_and_truncate(st, H, P.ApplicationMethod.DIRECT, P.TruncationMethod.SVD, trunc_args=(params,))
    assert max(tight.phys(n).shape[0] for n in ids if n != "s0") <= 3
    ost = O.OState(oracle_state(load_case("binary7_tfim_fastest_o2")).tree,
                   {n: full.get_phys_numpy(n) for n in ids})
    O.canonical_form(ost, O.leaf_to_leaf_path(ost.tree)[0])
    O.svd_truncation(ost, O.SVDParams(max_bond_dim=3, rel_tol=1e-10, total_tol=1e-10))
    a, b = tight.to_dense(ids), O.state_vector(ost, ids)
    assert np.max(np.abs(a - b)) < 1e-10 * np.max(np.abs(b))


def test_run_results_match_reference(monkeypatch):
    """run(evaluation_time=2) with every record flag: the Results entries
    (times, operators, bond dimensions, their maximum and average, total size,
    norm, Loschmidt amplitude) equal the reference's."""
    fake_ptn.install(monkeypatch)
    from golden_util import run_recorded_case
    res, ref = run_recorded_case()
    for name, arr in ref.items():
        key = tuple(name.split("/")[1:]) if name.startswith("bond/") else name
        got = res.operator_result(key) if key != "times" else res.times()
        assert got.shape == arr.shape, name
        assert np.max(np.abs(got - arr)) < 1e-9 * max(1.0, np.max(np.abs(arr))), name
    assert set(res.get_results().keys()) == {tuple(n.split("/")[1:]) if n.startswith("bond/") else n
                                              for n in ref if n != "times"}


@pytest.mark.parametrize("tag", ["cap", "tol"])
def test_engine_zipup_matches_reference(monkeypatch, tag):
    fake_ptn.install(monkeypatch)
    from golden_util import check_zipup_fixture
    check_zipup_fixture(tag)


def test_direct_truncate_methods(monkeypatch):
    """DIRECT_TRUNCATE = DIRECT + SVD truncation; the random variant keeps
    exactly max_bond_dim values per bond (when the bond allows)."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import binary_tfim_random_state
    st, spec, tens, _, _ = binary_tfim_random_state(n=7, chi=2, seed=4)
    ids = [n for n, _ in spec]
    H = P.TTNO.from_hamiltonian(_symbolic_tfim(spec, 1.0, 0.7), st)
    ref = P.apply_ttno_to_ttns(st, H).to_dense(ids)
    a = P.apply_ttno_to_ttns(st, H, P.ApplicationMethod.DIRECT_TRUNCATE,
                             P.SVDParameters(max_bond_dim=100, rel_tol=1e-13, total_tol=1e-13))
    assert np.max(np.abs(a.to_dense(ids) - ref)) < 1e-11 * np.max(np.abs(ref))
    b = P.apply_ttno_to_ttns(st, H, P.ApplicationMethod.DIRECT_TRUNCATE_RANDOM,
                             params=P.SVDParameters(max_bond_dim=2))
    assert all(b.phys(n).shape[0] == 2 for n in ids if n != "s0")


def test_multi_single_site_expectation_value(monkeypatch):
    """TTNS.multi_single_site_expectation_value in its three input forms against
    the reference's values on its saved state."""
    import os
    import pytreenet_gb300 as P
    from golden_util import GOLDEN
    fake_ptn.install(monkeypatch)
    st = P.TTNS.load(os.path.join(GOLDEN, "saved_ttns"))
    vals = np.load(os.path.join(GOLDEN, "saved_ttns_values.npz"))
    ids = [str(x) for x in vals["ids"]]
    z = dict(zip(ids, vals["z"]))
    out = st.multi_single_site_expectation_value(P.TensorProduct({n: Zm for n in ids}))
    assert all(abs(out[n][0] - z[n]) < 1e-12 for n in ids)
    out = st.multi_single_site_expectation_value([P.TensorProduct({"s1": Zm}), P.TensorProduct({"s1": 2 * Zm})])
    assert abs(out["s1"][0] - z["s1"]) < 1e-12 and abs(out["s1"][1] - 2 * z["s1"]) < 1e-12
    out = st.multi_single_site_expectation_value({"s4": [P.TensorProduct({"s4": Zm})], "s5": P.TensorProduct({"s5": Zm})})
    assert abs(out["s4"][0] - z["s4"]) < 1e-12 and abs(out["s5"][0] - z["s5"]) < 1e-12
    with pytest.raises(TypeError):
        st.multi_single_site_expectation_value(3)


def test_reset_to_initial_state(monkeypatch):
    """reset_to_initial_state: the same evolution twice gives the same results."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    c = load_case("ttree3_heis_chi6_o1")
    st = build_ttn(P.TTNS, c["spec"], {k: v.copy() for k, v in c["init"].items()})
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    ops = {"z": P.TensorProduct({c["spec"][0][0]: Zm})}
    algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"] * 2, ops,
                                   config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                   solver_options={"krylov_tol": 1e-12})
    first = algo.run()
    algo.reset_to_initial_state()
    assert algo.results is None
    second = algo.run()
    assert np.max(np.abs(first - second)) < 1e-13


def test_reset_bug_and_tebd(monkeypatch):
    """reset_to_initial_state for BUG and TEBD repeats the run exactly."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from golden_util import FixedSplitting
    c = load_case("binary15_tfim_fixed_bug")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    ops = {"z": P.TensorProduct({"s0": Zm})}
    algo = P.FixedBUG(st, H, c["dt"], c["dt"] * 2, ops, config=P.FixedBUGConfig(time_evo_mode=P.TimeEvoMode.KRYLOV))
    a = algo.run()
    algo.reset_to_initial_state()
    assert np.max(np.abs(algo.run() - a)) < 1e-13
    t = load_case("binary7_tfim_tebd")
    st = build_ttn(P.TTNS, t["spec"], t["init"])
    tebd = P.TEBD(st, FixedSplitting(t["gates"]), t["dt"], t["dt"] * 2, ops, svd_parameters=P.SVDParameters(**t["svd"]))
    a = tebd.run()
    tebd.reset_to_initial_state()
    assert np.max(np.abs(tebd.run() - a)) < 1e-13


def test_ttns_canonical_form_methods(monkeypatch):
    """canonical_form / move_orthogonalization_center / is_in_canonical_form on
    the device: the state is unchanged, the centre carries the norm, REDUCED
    shrinks wide bonds and KEEP keeps them."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    c = load_case("binary7_tfim_chi4_o2")            # zero-padded product state, bonds 4
    ids = [n for n, _ in c["spec"]]
    st = build_ttn(P.TTNS, c["spec"], {k: v.copy() for k, v in c["init"].items()})
    v0 = st.to_dense(ids)
    assert not st.is_in_canonical_form()
    st.canonical_form("s3", mode=P.SplitMode.KEEP)
    assert st.orthogonality_center_id == "s3" and st.is_in_canonical_form()
    assert np.max(np.abs(st.to_dense(ids) - v0)) < 1e-12
    assert st.phys("s4").shape[0] == 4                  # KEEP: the leaf bond stays 4
    st.move_orthogonalization_center("s6")
    assert st.is_in_canonical_form() and np.max(np.abs(st.to_dense(ids) - v0)) < 1e-12
    st2 = build_ttn(P.TTNS, c["spec"], {k: v.copy() for k, v in c["init"].items()})
    st2.canonical_form("s0")                            # REDUCED: a leaf bond cannot exceed 2
    assert st2.phys("s4").shape[0] == 2 and np.max(np.abs(st2.to_dense(ids) - v0)) < 1e-12
    assert st2.ensure_root_orth_center() is True
    st3 = build_ttn(P.TTNS, c["spec"], {k: v.copy() for k, v in c["init"].items()})
    st3.orthogonalize_root()
    assert st3.orthogonality_center_id == st3.root_id and st3.is_in_canonical_form()
    assert np.max(np.abs(st3.to_dense(ids) - v0)) < 1e-12


def test_pad_bond_dimensions_reproduces_c1_fixture():
    """pad_bond_dimensions of a bond-1 product state gives the zero-padded
    tensors the padded binary-tree fixture was built from (same values, same leg layout)."""
    import pytreenet_gb300 as P
    c = load_case("c1_binary15_tfim_chi8")
    small = {}
    for nid, t in c["init"].items():
        small[nid] = t[tuple(slice(0, 1) for _ in range(t.ndim - 1)) + (slice(None),)].copy()
    st = build_ttn(P.TTNS, c["spec"], small)
    st.pad_bond_dimensions(8)
    for nid, t in c["init"].items():
        assert np.array_equal(st.phys(nid), t), nid
    assert st.max_bond_dim() == 8


def test_tensor_product_methods():
    import pytreenet_gb300 as P
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
    tp = P.TensorProduct({"a": X, "b": Zm})
    op = tp.into_operator()
    assert np.allclose(op.operator, np.kron(X, Zm)) and op.node_identifiers == ["a", "b"]
    import scipy.linalg
    assert np.allclose(tp.exp(-0.3j).operator, scipy.linalg.expm(-0.3j * np.kron(X, Zm)))
    assert (tp @ P.TensorProduct({"a": Y}))["a"].tolist() == (X @ Y).tolist()
    assert tp.otimes(P.TensorProduct({"c": Y})).num_sites() == 3
    with pytest.raises(ValueError):
        tp.otimes(P.TensorProduct({"a": Y}))
    assert np.allclose(P.TensorProduct({"a": Y}).conjugate_transpose()["a"], Y.conj().T)
    assert P.TensorProduct({"a": "X"}).transpose()["a"] == "X_T"
    c = load_case("binary7_tfim_tebd")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    padded = P.TensorProduct({"s1": X}).pad_with_identities(st)
    assert padded.num_sites() == 7 and np.allclose(padded["s0"], np.eye(2))
    assert P.TensorProduct({"a": X}).allclose(P.TensorProduct({"a": X.copy()}))


def test_ttno_as_matrix(monkeypatch):
    """TTNO.as_matrix (device contractions) equals the dense operator."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from fractions import Fraction
    from pytreenet_gb300.workloads import binary_tfim_random_state
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
    st, spec, tens, _, _ = binary_tfim_random_state(n=7, chi=2, seed=1)
    ids = [n for n, _ in spec]
    terms = [(Fraction(1, 2), "K", P.TensorProduct({"s3": "X", "s6": "Y", "s0": "Z"})),
             P.TensorProduct({"s4": "Z", "s5": "Z"}), P.TensorProduct({"s2": X})]
    H = P.TTNO.from_hamiltonian(P.Hamiltonian(terms, {"X": X, "Y": Y, "Z": Zm}, {"K": 0.7}), st)

    def dense(ops):
        mats = [ops.get(n, np.eye(2)) for n in ids]
        out = mats[0]
        for m in mats[1:]:
            out = np.kron(out, m)
        return out
    Hd = 0.35 * dense({"s3": X, "s6": Y, "s0": Zm}) + dense({"s4": Zm, "s5": Zm}) + dense({"s2": X})
    M, order = H.as_matrix(order=ids)
    assert order == ids and np.max(np.abs(M - Hd)) < 1e-12
    M2, sites = H.as_matrix()
    assert sorted(sites) == sorted(ids) and M2.shape == (128, 128)


def test_plans_refuse_mismatched_output_legs(monkeypatch):
    """A gate whose output dimension differs from the site's is refused when the
    plan is built (the kernel would otherwise write past the output buffer)."""
    fake_ptn.install(monkeypatch)
    import torch
    import pytreenet_gb300 as P
    from pytreenet_gb300.engine import DeviceNetwork, Operand, Step
    c = load_case("binary7_tfim_tebd")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    net = DeviceNetwork(st, None)
    with pytest.raises(ValueError):
        net.apply_single_site_gate("s1", torch.zeros((3, 2), dtype=torch.complex128))
    A = Operand.contiguous(("fixed", None), ["i", "k"], [4, 5])
    B = Operand.contiguous(("fixed", None), ["k", "j"], [5, 6])
    with pytest.raises(ValueError):
        Step(A, B, ["k"], Operand.contiguous(("fixed", None), ["i", "j"], [4, 7]))


def test_solver_option_hermitian_false(monkeypatch):
    """solver_options hermitian=False (the Arnoldi projection exponentiated as
    it is) reproduces the reference's run of a Hermitian problem."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    c = load_case("ttree3_heis_chi6_o1")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"] * c["steps"], {},
                                   config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                   solver_options={"krylov_tol": c["krylov_tol"], "hermitian": False})
    for k in range(c["steps"]):
        algo.run_one_time_step()
        z = np.array([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
        assert np.max(np.abs(z - c["z"][k])) < 1e-10


def test_ttn_structure_methods():
    import pytreenet_gb300 as P
    c = load_case("ttree3_heis_chi6_o1")
    st = build_ttn(P.TTNS, c["spec"], {k: v.copy() for k, v in c["init"].items()})
    node, t = st.root
    assert node.identifier == c["spec"][0][0] and st.num_nodes() == len(c["spec"])
    lin = st.linearise()
    assert lin[-1] == st.root_id and set(lin) == set(st.nodes)
    for n in lin:                                  # children before parents
        p = st.nodes[n].parent
        assert p is None or lin.index(p) > lin.index(n)
    assert st.linearise("parents_first")[0] == st.root_id
    ids = [n for n, _ in c["spec"]]
    v = st.to_dense(ids)
    assert np.allclose(st.conjugate().to_dense(ids), v.conj())
    full, order = st.completely_contract_tree(order=ids)
    assert np.allclose(full.reshape(-1), v) and order == ids
    leaf = ids[-1]
    st.replace_tensor(leaf, 2 * st.get_tensor(leaf))
    assert np.allclose(st.to_dense(ids), 2 * v)
    with pytest.raises(ValueError):
        st.replace_tensor(leaf, np.zeros((1, 1)))


@pytest.mark.parametrize("method", ["RK45", "RK23", "DOP853"])
def test_engine_host_runge_kutta_matches_solve_ivp(monkeypatch, method):
    """The device Runge-Kutta integration takes the same steps as
    scipy.integrate.solve_ivp (same number of right-hand-side evaluations,
    DOP853 less the three of its dense output) and lands on the same point,
    for either sign of the exponent factor and of dt (a negative dt integrates
    backward, as the two-site sweeps' backward site updates do), at tight and
    at loose tolerances with a step cap."""
    import torch
    from scipy.integrate import solve_ivp
    from pytreenet_gb300.engine import Workspace
    from pytreenet_gb300.ode import RungeKuttaSolver
    fake_ptn.install(monkeypatch)
    rng = np.random.default_rng(5)
    n = 40
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Hm = (A + A.conj().T) / 2
    x0 = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    Ht = torch.from_numpy(Hm)

    def ap(a, b):
        b.copy_(Ht @ a)
    ap.takes_tensors = True
    for ef, dt in ((-1j, 0.05), (1j, 0.2), (-1j, -0.1)):
        for opts in ({"atol": 1e-10, "rtol": 1e-10}, {"atol": 1e-6, "rtol": 1e-3, "max_step": 0.02}):
            ref = solve_ivp(lambda t, y: ef * (Hm @ y), (0, dt), x0, method=method, t_eval=[dt], **opts)
            solver = RungeKuttaSolver(Workspace(torch.device("cpu")))
            y = solver.integrate(torch.from_numpy(x0.copy()), ap, dt, ef, method, **opts).numpy()
            assert np.abs(y - ref.y[:, 0]).max() < 1e-13 * np.abs(ref.y[:, 0]).max()
            assert solver.evaluations[-1] == ref.nfev - (3 if method == "DOP853" else 0)


def test_engine_host_ode_options_follow_the_reference():
    """ODE modes: options pass through as given (solve_ivp's tolerances when
    none), solver-only keys are dropped, BDF is refused."""
    from pytreenet_gb300.tdvp import TimeEvoMode, check_time_evo_mode, ode_options
    assert ode_options(TimeEvoMode.KRYLOV, {"krylov_tol": 1e-9}) is None
    opts = check_time_evo_mode(TimeEvoMode.RK45, None)
    assert opts == {}
    assert ode_options(TimeEvoMode.RK45, opts) == {"atol": 1e-6, "rtol": 1e-3, "method": "RK45"}
    o = ode_options(TimeEvoMode.DOP853, check_time_evo_mode(TimeEvoMode.DOP853, {"rtol": 1e-9, "jac": None,
                                                                                 "hermitian": True}))
    assert o == {"atol": 1e-6, "rtol": 1e-9, "method": "DOP853"}
    with pytest.raises(NotImplementedError):
        check_time_evo_mode(TimeEvoMode.BDF, None)
    with pytest.raises(ValueError):
        check_time_evo_mode(TimeEvoMode.RK23, {"krylov_tol": 1e-9})


def test_engine_host_partial_tree_cache_matches_oracle(monkeypatch):
    """``partial_tree_cache`` exposes the sweep's environments: after a
    first-order step every environment the oracle's sweep holds is there, legs
    (ket, ham, bra), equal to rounding; ``update_tree_cache`` recomputes one."""
    import oracle as O
    from golden_util import build_ttn, load_case, oracle_state
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    c = load_case("ttree3_heis_chi6_o1")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"], {}, config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                   solver_options={"krylov_tol": c["krylov_tol"]})
    ref = O.FirstOrderOneSiteTDVPOracle(oracle_state(c), c["ttno"], c["dt"], krylov_tol=c["krylov_tol"])
    algo.run_one_time_step()
    ref.run_one_time_step()
    cache = algo.partial_tree_cache
    assert len(ref.envs) > 0
    for (u, v), E in ref.envs.items():
        assert (u, v) in cache
        got = cache.get_entry(u, v)
        assert got.shape == E.shape
        assert np.abs(got - E).max() < 1e-10 * max(1.0, np.abs(E).max())
    u, v = next(iter(ref.envs))
    before = cache.get_entry(u, v)
    algo.update_tree_cache(u, v)
    assert np.abs(cache.get_entry(u, v) - before).max() < 1e-10 * max(1.0, np.abs(before).max())


def test_engine_host_time_evolve_and_krylov_exp_action(monkeypatch):
    """``time_evolve`` on a dense matrix in every mode family against SciPy
    (expm for the exact and Krylov modes, solve_ivp with the mode defaults for
    RK45), forward and backward; ``krylov_exp_action`` with a NumPy action
    and with a torch action."""
    import scipy.linalg
    import torch
    from scipy.integrate import solve_ivp
    fake_ptn.install(monkeypatch)
    from pytreenet_gb300.local_evolution import krylov_exp_action, time_evolve
    from pytreenet_gb300.tdvp import EvoDirection, TimeEvoMode
    rng = np.random.default_rng(9)
    n = 30
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H = (A + A.conj().T) / 2
    psi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    psi /= np.linalg.norm(psi)
    dt = 0.1
    for fwd, f in ((EvoDirection.FORWARD, -1j), (EvoDirection.BACKWARD, 1j)):
        exact = scipy.linalg.expm(f * dt * H) @ psi
        for mode in (TimeEvoMode.FASTEST, TimeEvoMode.EXPM, TimeEvoMode.SPARSE):
            assert np.abs(time_evolve(psi, H, dt, forward=fwd, mode=mode) - exact).max() < 1e-12
        got = time_evolve(psi, H, dt, forward=fwd, mode=TimeEvoMode.KRYLOV, krylov_tol=1e-13)
        assert np.abs(got - exact).max() < 1e-11
        ref = solve_ivp(lambda t, y: f * (H @ y), (0, dt), psi, method="RK45", t_eval=[dt],
                        atol=1e-10, rtol=1e-10).y[:, 0]
        assert np.abs(time_evolve(psi, H, dt, forward=fwd, mode=TimeEvoMode.RK45) - ref).max() < 1e-13
    # a real exp_factor override: a diffusion-like flow exp(-dt H)
    got = time_evolve(psi, H, dt, mode=TimeEvoMode.EXPM, exp_factor=-1.0)
    assert np.abs(got - scipy.linalg.expm(-dt * H) @ psi).max() < 1e-12
    exact = scipy.linalg.expm(-1j * dt * H) @ psi
    got = krylov_exp_action(psi.reshape(5, 6), lambda y: (H @ y.reshape(-1)).reshape(5, 6), dt, -1j,
                            krylov_tol=1e-13)
    assert got.shape == (5, 6) and np.abs(got.reshape(-1) - exact).max() < 1e-11
    Ht = torch.from_numpy(H)
    got = krylov_exp_action(torch.from_numpy(psi.copy()), lambda y: Ht @ y, dt, -1j, krylov_tol=1e-13)
    assert isinstance(got, torch.Tensor) and np.abs(got.numpy() - exact).max() < 1e-11
    with pytest.raises(ValueError):
        time_evolve(psi, H[:5, :5], dt)
    with pytest.raises(NotImplementedError):
        time_evolve(psi, H, dt, mode=TimeEvoMode.BDF)


def test_engine_host_module_functions(monkeypatch):
    """Module-level functions with PyTreeNet's names: expectation_value gives
    the reference's final energy, contract_two_ttns is the bilinear product
    of the dense vectors, TDVPUpdatePathFinder's default (LeafToLeaf) gives the
    reference's leaf-to-leaf path, the operator helpers their matrices."""
    from golden_util import build_ttn, load_case
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    c = load_case("ttree3_heis_chi6_o1")
    final = build_ttn(P.TTNS, c["spec"], c["final"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    assert abs(P.expectation_value(final, H) - c["energy_final"]) < 1e-10
    a = build_ttn(P.TTNS, c["spec"], c["init"])
    b = build_ttn(P.TTNS, c["spec"], c["final"])
    order = [nid for nid, _ in c["spec"]]
    va, vb = a.to_dense(order), b.to_dense(order)
    assert abs(P.contract_two_ttns(a, b) - np.sum(va * vb)) < 1e-12
    assert abs(P.contract_two_ttns(a, b) - a.scalar_product(b)) > 1e-3   # no conjugation
    l2l = load_case("ttree3_heis_l2l_o1")
    st = build_ttn(P.TTNS, l2l["spec"], l2l["init"])
    assert P.TDVPUpdatePathFinder(st).find_path() == l2l["update_path"]
    assert P.TDVPUpdatePathFinder(st, P.PathFinderMode.LeafToRoot).find_path() == \
        P.leaf_to_root_update_path(st)
    X, Y, Z = P.pauli_matrices()
    assert np.allclose(X @ Y, 1j * Z)
    sp, sm = P.spin_jumps()
    assert np.allclose(sp, [[0, 1], [0, 0]]) and np.allclose(sm, [[0, 0], [1, 0]])
    cr, an, num = P.bosonic_operators(4)
    assert np.allclose(np.diag(num), [0, 1, 2, 3]) and np.isclose(cr[2, 1], np.sqrt(2)) and np.allclose(an, cr.T)
    assert np.allclose(P.hadamard() @ P.hadamard(), np.eye(2))


def test_engine_host_time_evo_mode_methods(monkeypatch):
    """TimeEvoMode / EvoDirection helpers and the enum's evolution methods
    with the checks of the reference's own mode tests (a random Hermitian
    24 x 24 generator on a (2, 3, 4) tensor, dt = 0.1, against expm): the
    action form for the solve_ivp modes at atol = rtol = 1e-9, the dense form
    for the exact and solve_ivp modes, the module function's mode defaults at
    dt = 1, and a time-dependent action against solve_ivp's own integration."""
    import scipy.linalg
    from scipy.integrate import solve_ivp
    fake_ptn.install(monkeypatch)
    from pytreenet_gb300.local_evolution import time_evolve
    from pytreenet_gb300.tdvp import EvoDirection, TimeEvoMode
    assert EvoDirection.from_bool(True) is EvoDirection.FORWARD
    assert EvoDirection.from_bool(False) is EvoDirection.BACKWARD
    assert EvoDirection.FORWARD.exp_sign() == -1 and EvoDirection.BACKWARD.exp_sign() == 1
    assert EvoDirection.FORWARD.exp_factor() == -1j and EvoDirection.BACKWARD.exp_factor() == 1j
    assert TimeEvoMode.fastest_equivalent() is TimeEvoMode.CHEBYSHEV
    for m, exp in ((TimeEvoMode.EXPM, False), (TimeEvoMode.CHEBYSHEV, False), (TimeEvoMode.SPARSE, False),
                   (TimeEvoMode.FASTEST, False), (TimeEvoMode.RK45, True), (TimeEvoMode.RK23, True),
                   (TimeEvoMode.DOP853, True), (TimeEvoMode.BDF, True)):
        assert m.is_scipy() is exp
        assert m.action_evolvable() is exp
    assert TimeEvoMode.KRYLOV.action_evolvable()
    rng = np.random.default_rng(21)
    shape = (2, 3, 4)
    n = 24
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Hm = (A + A.conj().T) / 2
    psi = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    Ht = Hm.reshape(2 * list(shape))

    def action(_, x):
        return np.tensordot(Ht, x, axes=([3, 4, 5], [0, 1, 2]))
    dt = 0.1
    ref = scipy.linalg.expm(-1j * Hm * dt) @ psi.reshape(-1)
    for m in (TimeEvoMode.RK45, TimeEvoMode.RK23, TimeEvoMode.DOP853):
        got = m.time_evolve_action(psi, action, dt, atol=1e-9, rtol=1e-9)
        assert got.shape == shape
        np.testing.assert_allclose(got.reshape(-1), ref)
    got = TimeEvoMode.KRYLOV.time_evolve_action(psi, action, dt, krylov_tol=1e-12)
    np.testing.assert_allclose(got.reshape(-1), ref)
    with pytest.raises(NotImplementedError):
        TimeEvoMode.EXPM.time_evolve_action(psi, action, dt)
    for m in (TimeEvoMode.EXPM, TimeEvoMode.CHEBYSHEV, TimeEvoMode.SPARSE, TimeEvoMode.RK45,
              TimeEvoMode.RK23, TimeEvoMode.DOP853):
        got = m.time_evolve(psi, Hm, dt, atol=1e-9, rtol=1e-9)
        assert got.shape == shape
        np.testing.assert_allclose(got.reshape(-1), ref)
    with pytest.raises(NotImplementedError):
        TimeEvoMode.BDF.time_evolve(psi, Hm, dt)
    ref1 = scipy.linalg.expm(-1j * Hm) @ psi.reshape(-1)
    for m in (TimeEvoMode.RK45, TimeEvoMode.RK23, TimeEvoMode.DOP853):
        # the module function lays the mode's 1e-10 defaults under the options;
        # the enum method alone runs at solve_ivp's 1e-3 and misses by far more
        np.testing.assert_allclose(time_evolve(psi, Hm, 1.0, mode=m).reshape(-1), ref1, atol=1e-6)
        assert np.abs(m.time_evolve(psi, Hm, 1.0).reshape(-1) - ref1).max() > 1e-6
    # H(t) = (1 + t) H: the stage times reach the action
    got = TimeEvoMode.RK45.time_evolve_action(psi, lambda t, x: (1 + t) * action(t, x), 0.3, atol=1e-10, rtol=1e-10)
    sol = solve_ivp(lambda t, y: -1j * (1 + t) * (Hm @ y), (0, 0.3), psi.reshape(-1), method="RK45",
                    t_eval=[0.3], atol=1e-10, rtol=1e-10).y[:, 0]
    assert np.abs(got.reshape(-1) - sol).max() < 1e-13
    exact = scipy.linalg.expm(-1j * (0.3 + 0.045) * Hm) @ psi.reshape(-1)
    assert np.abs(got.reshape(-1) - exact).max() < 1e-7


def test_engine_host_effective_bond_evolution(monkeypatch):
    """``effective_bond_evolution`` as the reference's own bond tests run it:
    a (4, 5) bond tensor between random non-Hermitian environments (4, 6, 4)
    and (5, 6, 5) in a ``PartialTreeCachDict``, every action mode (KRYLOV
    with hermitian=False and no early stop, the solve_ivp modes at 1e-10)
    and every exact mode against expm of the dense bond Hamiltonian, which
    itself matches a NumPy restatement."""
    import scipy.linalg
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from pytreenet_gb300.contractions import (PartialTreeCachDict, contract_bond_tensor,
                                              effective_bond_evolution, get_effective_bond_hamiltonian_nodes)
    rng = np.random.default_rng(17)

    def crandn(*s):
        return rng.standard_normal(s) + 1j * rng.standard_normal(s)
    node = P.Node("state_node")
    node.parent, node.children = "parent_node", ["child_node"]
    x = crandn(4, 5)
    cache = PartialTreeCachDict()
    ep, ec = crandn(4, 6, 4), crandn(5, 6, 5)
    cache.add_entry("parent_node", "child_node", ep)
    cache.add_entry("child_node", "parent_node", ec)
    H = np.einsum("abp,cbq->pqac", ep, ec).reshape(20, 20)
    np.testing.assert_allclose(get_effective_bond_hamiltonian_nodes(node, cache), H, rtol=1e-13)
    np.testing.assert_allclose(contract_bond_tensor(x, node, cache), (H @ x.reshape(-1)).reshape(4, 5), rtol=1e-13)
    dt = 0.1
    ref = (scipy.linalg.expm(-1j * dt * H) @ x.reshape(-1)).reshape(4, 5)
    for mode in (P.TimeEvoMode.RK45, P.TimeEvoMode.RK23, P.TimeEvoMode.DOP853):
        np.testing.assert_allclose(effective_bond_evolution(x, node, dt, cache, mode=mode, rtol=1e-10, atol=1e-10),
                                   ref)
    np.testing.assert_allclose(effective_bond_evolution(x, node, dt, cache, mode=P.TimeEvoMode.KRYLOV,
                                                        krylov_tol=0.0, hermitian=False), ref)
    for mode in (P.TimeEvoMode.FASTEST, P.TimeEvoMode.EXPM, P.TimeEvoMode.CHEBYSHEV, P.TimeEvoMode.SPARSE):
        np.testing.assert_allclose(effective_bond_evolution(x, node, dt, cache, mode=mode), ref)
    back = effective_bond_evolution(x, node, dt, cache, mode=P.TimeEvoMode.EXPM, forward=P.EvoDirection.BACKWARD)
    np.testing.assert_allclose(back, (scipy.linalg.expm(1j * dt * H) @ x.reshape(-1)).reshape(4, 5))
    assert cache.contains("parent_node", "child_node") and cache.num_legs("child_node", "parent_node") == 3
    bad = P.Node("leaf")
    bad.parent, bad.children = "parent_node", []
    with pytest.raises(ValueError):
        contract_bond_tensor(x, bad, cache)


@pytest.mark.parametrize("tag", ["t4", "t6"])
def test_engine_host_ttno_from_tensor(monkeypatch, tag):
    """``TTNO.from_tensor``: in QR mode the node tensors equal the reference's
    (same leg bookkeeping, Householder signs); the SVD modes give the same
    operator (as_matrix against the input tensor)."""
    from golden_util import GOLDEN, build_ttn
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    from pytreenet_gb300.ttno_decomposition import Decomposition
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
        assert list(ttno.nodes[nid].children) == [str(x) for x in d[f"{tag}/children/{nid}"]]
    half = op.ndim // 2
    order = ids
    perm = [leg_dict[n] for n in order] + [half + leg_dict[n] for n in order]
    dim = int(np.prod([op.shape[leg_dict[n]] for n in order]))
    dense = np.transpose(op, perm).reshape(dim, dim)
    for mode in (Decomposition.QR, Decomposition.SVD, Decomposition.tSVD):
        m, got_order = P.TTNO.from_tensor(tree, op, leg_dict, mode=mode).as_matrix(order)
        assert list(got_order) == order
        assert np.abs(m - dense).max() < 1e-11 * np.abs(dense).max(), mode


def test_engine_host_from_tensor_root_is_leaf(monkeypatch):
    """The reference's root-is-leaf case of ``from_tensor``: a 7-node tree whose
    root has one child, built with ``add_child_to_parent`` on chosen legs; the
    completely contracted TTNO (legs (out, in) per node, root first, then each
    child's subtree) equals the input tensor with its legs in that order."""
    fake_ptn.install(monkeypatch)
    import pytreenet_gb300 as P
    rng = np.random.default_rng(3)

    def crandn(shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    shapes = [(1, 1, 1, 2), (1, 1, 1, 2), (1, 2), (1, 2), (1, 2), (1, 1, 2), (1, 2)]
    t = [crandn(s) for s in shapes]
    tree = P.TTNS()
    tree.add_root("node4", t[4])
    tree.add_child_to_parent("node0", t[0], 0, "node4", 0)
    tree.add_child_to_parent("node1", t[1], 0, "node0", 1)
    tree.add_child_to_parent("node2", t[2], 0, "node1", 1)
    tree.add_child_to_parent("node3", t[3], 0, "node1", 2)
    tree.add_child_to_parent("node5", t[5], 0, "node0", 2)
    tree.add_child_to_parent("node6", t[6], 0, "node5", 1)
    n = len(shapes)
    start = crandn(2 * n * [2])
    leg_dict = {f"node{i}": i for i in range(n)}
    ttno = P.TTNO.from_tensor(tree, start.copy(), leg_dict)
    contracted, order = ttno.completely_contract_tree(to_copy=True)
    assert order == ["node4", "node0", "node1", "node2", "node3", "node5", "node6"]
    perm = [i for nid in order for i in (leg_dict[nid], leg_dict[nid] + n)]
    assert np.allclose(start.transpose(perm), contracted)
    # a state contracts to one leg per node in the same order
    vec, sorder = tree.completely_contract_tree()
    assert sorder == order and vec.shape == (2,) * n


def test_update_paths_match_reference():
    """``TDVPUpdatePathFinder`` in both modes gives the reference's paths on
    trees built leg by leg, including roots with a single child (which count
    as leaves, as in the reference's ``get_leaves``)."""
    from golden_util import GOLDEN
    import pytreenet_gb300 as P
    d = np.load(f"{GOLDEN}/update_paths.npz")
    names = sorted({k.split("/")[0] for k in d.files})
    assert len(names) >= 4
    for name in names:
        root = str(d[f"{name}/root"])
        edges = [(str(c), str(p), int(leg)) for c, p, leg in d[f"{name}/edges"]]
        nch = {root: 0}
        for c, p, _ in edges:
            nch[p] = nch.get(p, 0) + 1
            nch.setdefault(c, 0)

        def ones(n, is_root):
            return np.ones([1] * (nch[n] + (0 if is_root else 1)) + [2], dtype=complex)
        t = P.TTNS()
        t.add_root(root, ones(root, True))
        for c, p, leg in edges:
            t.add_child_to_parent(c, ones(c, False), 0, p, leg)
        for mode in ("LeafToRoot", "LeafToLeaf"):
            want = [str(x) for x in d[f"{name}/{mode}"]]
            assert P.TDVPUpdatePathFinder(t, P.PathFinderMode[mode]).find_path() == want, (name, mode)
    leaves = t.get_leaves(include_root=False)
    assert root not in leaves and set(leaves) <= set(nch)


def test_tree_structure_queries():
    """Leaves, subtrees and pairs at a distance (``core/tree_structure.py``):
    a node whose open leg is trivial is skipped when ``consider_open``."""
    import pytreenet_gb300 as P
    t = P.TTNS()
    t.add_root("r", np.ones((1, 1, 2), dtype=complex))
    t.add_child_to_parent("a", np.ones((1, 1, 1), dtype=complex), 0, "r", 0)   # trivial open leg
    t.add_child_to_parent("b", np.ones((1, 2), dtype=complex), 0, "r", 1)
    t.add_child_to_parent("c", np.ones((1, 2), dtype=complex), 0, "a", 1)
    assert sorted(t.get_leaves()) == ["b", "c"]
    assert set(t.find_subtree_of_node("a")) == {"a", "c"} and t.find_subtree_size_of_node("r") == 4
    assert set(t.leaves_under_node("a")) == {"c"}
    assert t.find_pairs_of_distance(1) == {frozenset(p) for p in [("r", "a"), ("r", "b"), ("a", "c")]}
    assert t.find_pairs_of_distance(2) == {frozenset(p) for p in [("a", "b"), ("r", "c")]}
    assert t.find_pairs_of_distance(1, consider_open=True) == {frozenset(p) for p in [("r", "b"), ("r", "c")]}
    assert t.find_pairs_of_distance(0, consider_open=True) == {frozenset([n]) for n in ("r", "b", "c")}
    assert sorted(tuple(sorted(p)) for p in t.nearest_neighbours()) == [("a", "c"), ("a", "r"), ("b", "r")]
    with pytest.raises(ValueError):
        t.find_pairs_of_distance(-1)


def test_ttn_scale_and_orth_assertion():
    """``scale`` multiplies the centre's tensor (the root's without a centre),
    in place or on a copy; ``assert_orth_center`` checks the centre."""
    import pytreenet_gb300 as P
    t = P.TTNS()
    t.add_root("r", np.ones((1, 2), dtype=complex))
    t.add_child_to_parent("a", np.full((1, 2), 2.0, dtype=complex), 0, "r", 0)
    c = t.scale(3.0, inplace=False)
    assert np.allclose(c.tensors["r"], 3.0) and np.allclose(t.tensors["r"], 1.0)
    t.orthogonality_center_id = "a"
    t.scale(0.5)
    assert np.allclose(t.tensors["a"], 1.0) and np.allclose(t.tensors["r"], 1.0)
    t.assert_orth_center("a")
    with pytest.raises(AssertionError):
        t.assert_orth_center("r")


def test_ttn_structure_comparisons():
    """same_connectivity_as / same_hierarchy_as / same_structure_as /
    same_open_dimensions_as / same_bond_dimensions_as."""
    import pytreenet_gb300 as P

    def tree(bond, phys):
        t = P.TTNS()
        t.add_root("r", np.ones((bond, 1, phys), dtype=complex))
        t.add_child_to_parent("a", np.ones((bond, phys), dtype=complex), 0, "r", 0)
        t.add_child_to_parent("b", np.ones((1, 2), dtype=complex), 0, "r", 1)
        return t
    a, b, c, d = tree(2, 2), tree(2, 2), tree(3, 2), tree(2, 3)
    assert a.same_connectivity_as(b) and a.same_hierarchy_as(b) and a.same_structure_as(b)
    assert a.same_bond_dimensions_as(b) and not a.same_bond_dimensions_as(c)
    assert a.same_structure_as(c) and not a.same_structure_as(d) and not a.same_open_dimensions_as(d)
    e = P.TTNS()
    e.add_root("a", np.ones((2, 1, 2), dtype=complex))
    e.add_child_to_parent("r", np.ones((2, 1, 2), dtype=complex), 0, "a", 0)
    e.add_child_to_parent("b", np.ones((1, 2), dtype=complex), 0, "r", 1)
    assert a.same_connectivity_as(e) and not a.same_hierarchy_as(e)   # same edges, other root


def test_ttn_parentage_and_to_complex():
    import pytreenet_gb300 as P
    t = P.TTNS()
    t.add_root("r", np.ones((1, 2)))
    t.add_child_to_parent("a", np.ones((1, 2)), 0, "r", 0)
    assert t.is_child_of("a", "r") and t.is_parent_of("r", "a") and not t.is_child_of("r", "a")
    assert t.to_complex() is t and t.tensors["a"].dtype == np.complex128
    t.to_complex(64)
    assert t.tensors["r"].dtype == np.complex64
    with pytest.raises(ValueError):
        t.to_complex(32)


@pytest.mark.parametrize("name", ["ttree3_heis_chi6_o1", "binary7_tfim_chi4_o2", "ternary2_xxz_chi4_o1"])
def test_expect_many_one_pass(monkeypatch, name):
    """DeviceNetwork.expect_many: one-site operators (several on one node, on
    the root and on leaves), products on several nodes (in one subtree and
    across the root) and the norm, against the oracle's full contraction per
    product, on a T-tree, a binary and a ternary tree; the plan is built once
    per operator layout and rebuilt when a site tensor changes shape."""
    import pytreenet_gb300 as P
    import oracle as O
    from pytreenet_gb300.engine import DeviceNetwork
    fake_ptn.install(monkeypatch)
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    ost = oracle_state(c)
    net = DeviceNetwork(st)
    rng = np.random.default_rng(3)
    ids = [nid for nid, _ in c["spec"]]

    def herm(d):
        m = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
        return m + m.conj().T
    root = ids[0]
    ops = [{root: herm(2)}, {ids[1]: Zm}, {ids[1]: herm(2)}, {ids[-1]: herm(2)}, {},
           {ids[1]: Zm, ids[2]: herm(2)}, {ids[-1]: Zm, ids[1]: herm(2), root: herm(2)},
           {ids[-2]: rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))}]
    got = net.expect_many(ops)
    want = np.array([O.expect_product(ost, op) for op in ops])
    assert np.max(np.abs(got - want)) < 1e-12 * max(1.0, np.max(np.abs(want)))
    assert abs(net.expect_local({ids[1]: Zm}) - want[1]) < 1e-12
    # the same layout with other matrices reuses the plan
    n_plans = len(net._obs_plans)
    ops2 = [{k: 2 * v for k, v in op.items()} for op in ops]
    got2 = net.expect_many(ops2)
    want2 = np.array([O.expect_product(ost, op) for op in ops2])
    assert len(net._obs_plans) == n_plans
    assert np.max(np.abs(got2 - want2)) < 1e-12 * max(1.0, np.max(np.abs(want2)))
    with pytest.raises(ValueError):
        net.expect_many([{ids[1]: np.eye(3)}])
    with pytest.raises(KeyError):
        net.expect_many([{"no-such-node": Zm}])
    # a tensor replaced by one of another shape drops the plans
    leaf = ids[-1]
    t = net.t[leaf]
    bigger = torch.zeros((t.shape[0] + 1,) + tuple(t.shape[1:]), dtype=t.dtype)
    bigger[:t.shape[0]] = t
    par = st.nodes[leaf].parent
    tp = net.t[par]
    ax = st.phys_axis(par, leaf)
    shp = list(tp.shape)
    shp[ax] += 1
    tp2 = torch.zeros(shp, dtype=tp.dtype)
    tp2.narrow(ax, 0, tp.shape[ax]).copy_(tp)
    net._set_node_tensor(leaf, bigger)
    net._set_node_tensor(par, tp2)
    got3 = net.expect_many(ops)
    assert np.max(np.abs(got3 - got)) < 1e-12 * max(1.0, np.max(np.abs(want)))


def test_run_loop_measures_in_one_pass(monkeypatch):
    """The run loop hands all one-site products to one expect_many call per
    measurement and a TTNO to expect_ttno; the values are the per-operator ones."""
    import pytreenet_gb300 as P
    fake_ptn.install(monkeypatch)
    c = load_case("ttree3_heis_chi6_o1")
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    ids = [nid for nid, _ in c["spec"]]
    ops = {f"z{n}": P.TensorProduct({n: Zm}) for n in ids}
    ops["energy"] = H
    algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], 2 * c["dt"], ops,
                                   config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                   solver_options={"krylov_tol": c["krylov_tol"]})
    calls = []
    orig = algo.net.expect_many
    monkeypatch.setattr(algo.net, "expect_many", lambda lst: calls.append(len(lst)) or orig(lst))
    algo.run(pgbar=False)
    assert calls == [len(ids)] * 3
    res = algo.results
    for n in ids:
        assert abs(res.operator_result(f"z{n}")[-1] - algo.net.expect_local({n: Zm})) < 1e-13
    assert abs(res.operator_result("energy")[-1] - algo.net.expect_ttno(H)) < 1e-12


def test_first_order_reset_reuses_unchanged_environments(monkeypatch):
    """The first-order step's closing reset keeps the environments whose side
    of the tree was not written after they were computed: some are kept on the
    T-tree, and the evolved tensors are bitwise those of a run that recomputes
    every environment."""
    import pytreenet_gb300 as P
    from pytreenet_gb300.engine import DeviceNetwork
    fake_ptn.install(monkeypatch)
    c = load_case("ttree3_heis_chi6_o1")

    def run(reuse):
        st = build_ttn(P.TTNS, c["spec"], c["init"])
        H = build_ttn(P.TTNO, c["spec"], c["ttno"])
        algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"] * c["steps"], {},
                                       config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                       solver_options={"krylov_tol": c["krylov_tol"]})
        if not reuse:
            orig = algo.net.init_cache_but_one
            algo.net.init_cache_but_one = lambda left_out, reuse=False: orig(left_out, reuse=False)
        for _ in range(c["steps"]):
            algo.run_one_time_step()
        return algo, {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    a, ta = run(True)
    b, tb = run(False)
    assert getattr(a.net, "env_reused", 0) > 0
    assert getattr(b.net, "env_reused", 0) == 0
    for nid in ta:
        assert np.array_equal(ta[nid], tb[nid]), nid
    for key, E in a.net.env.items():
        assert np.array_equal(E.numpy(), b.net.env[key].numpy()), key


def test_plan_rereads_moved_workspace_slots(monkeypatch):
    """A plan keeps its operand addresses between runs only while the
    workspace's buffers are unchanged: after a slot it uses is replaced by a
    larger one (another plan grew it), the next run reads the new address and
    still gives the right result."""
    fake_ptn.install(monkeypatch)
    from pytreenet_gb300.engine import ChainBuilder, Operand, Workspace
    rng = np.random.default_rng(0)
    ws = Workspace("cpu")
    A = torch.from_numpy(rng.normal(size=(6, 5)) + 1j * rng.normal(size=(6, 5)))
    B = torch.from_numpy(rng.normal(size=(5, 4)) + 1j * rng.normal(size=(5, 4)))
    D = torch.from_numpy(rng.normal(size=(4, 3)) + 1j * rng.normal(size=(4, 3)))
    out = torch.zeros((6, 3), dtype=torch.complex128)
    cb = ChainBuilder(ws)
    T = cb.contract(Operand.contiguous(("fixed", A), ["i", "k"], [6, 5]),
                    Operand.contiguous(("fixed", B), ["k", "j"], [5, 4]), ["k"])     # T lives in a ws slot
    cb.contract(T, Operand.contiguous(("fixed", D), ["j", "l"], [4, 3]), ["j"],
                out=Operand.contiguous(("fixed", out), ["i", "l"], [6, 3]))
    p = cb.plan()
    ref = (A @ B @ D).numpy()
    p.run()
    assert np.allclose(out.numpy(), ref)
    gen = ws.gen
    name = T.ref[1]
    old = ws.bufs[name]
    ws.get(name, old.numel() * 4)              # the slot moves
    assert ws.gen != gen and ws.bufs[name].data_ptr() != old.data_ptr()
    old.fill_(float("nan"))                    # the old buffer must not be read again
    out.zero_()
    p.run()
    assert np.allclose(out.numpy(), ref)
