"""End-to-end one-site TDVP on the GPU against the reference's golden fixtures."""
import numpy as np
import pytest

import oracle as O
from golden_util import CASES, build_ttn, load_case, oracle_state, fidelity_and_dist

pytestmark = pytest.mark.gpu
Zm = np.diag([1.0, -1.0]).astype(complex)


def _run(name, steps=None):
    import pytreenet_gb300 as P
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    cls = P.FirstOrderOneSiteTDVP if c["order"] == 1 else P.SecondOrderOneSiteTDVP
    algo = cls(st, H, c["dt"], c["dt"] * c["steps"], {},
               config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
               solver_options={"krylov_tol": c["krylov_tol"]})
    assert algo.update_path == c["update_path"]
    zerr = 0.0
    for k in range(c["steps"] if steps is None else steps):
        algo.run_one_time_step()
        z = [algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]]
        zerr = max(zerr, float(np.max(np.abs(np.array(z) - c["z"][k]))))
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    return c, O.OState(oracle_state(c).tree, out), zerr


@pytest.mark.parametrize("name", [n for n in CASES if n != "c1_binary15_tfim_chi8"])
def test_gpu_tdvp_full_rank_cases(name):
    c, got, zerr = _run(name)
    one_minus_f, dist = fidelity_and_dist(oracle_state(c, "final"), got)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12


def test_gpu_tdvp_c1_padded():
    """15-node binary TFIM from a zero-padded product state, 50 steps; bounded by the reference's own rounding floor."""
    c, got, zerr = _run("c1_binary15_tfim_chi8")
    ids = [s[0] for s in c["spec"]]
    a = O.state_vector(got, ids)
    b = O.state_vector(oracle_state(c, "final"), ids)
    assert zerr < 1e-8
    assert abs(1 - abs(np.vdot(a, b)) / np.linalg.norm(a) / np.linalg.norm(b)) < 1e-10


def test_gpu_tdvp_ttree_chi16_vs_oracle():
    """A T-tree (root + 3 arms) at reduced size against the oracle: own TTNO builder."""
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    st, spec, tensors = t_tree_state(arm_len=5, chi=16, seed=5)
    H, Wphys = t_tree_heisenberg(st, seed=6)
    algo = P.FirstOrderOneSiteTDVP(st, H, 0.01, 0.02, {}, config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                   solver_options={"krylov_tol": 1e-12})
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    ora = O.FirstOrderOneSiteTDVPOracle(O.OState(tree, tensors), Wphys, 0.01, krylov_tol=1e-12)
    for _ in range(2):
        algo.run_one_time_step()
        ora.run_one_time_step()
    got = O.OState(tree, {nid: algo.state.get_phys_numpy(nid) for nid, _ in spec})
    one_minus_f, dist = fidelity_and_dist(ora.state, got)
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", ["ttree3_heis_l2l_o1", "binary15_tfim_l2l_o2"])
def test_gpu_leaf_to_leaf_path(name):
    """TDVPConfig(main_path_mode=LeafToLeaf) on the GB300 against the reference."""
    from golden_util import run_one_site_case
    c, st, zerr = run_one_site_case(name)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", ["ttree3_heis_rk45_o1", "binary7_tfim_dop853_o2", "binary7_tfim_rk23_o1"])
def test_gpu_ode_modes(name):
    """RK45 / DOP853 / RK23 (the solve_ivp modes) on the GB300 against the
    reference: the same adaptive steps on device vectors. The exact evolution
    differs from these fixtures by 1e-9 to 1e-7 in <Z>, far above the bound."""
    from golden_util import run_one_site_case
    c, st, zerr = run_one_site_case(name)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert zerr < 1e-11
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", ["ttree3_heis_fastest_o1", "binary7_tfim_fastest_o2"])
def test_gpu_default_mode(name):
    """TDVPConfig() (FASTEST) on the GB300 against the reference's dense exponential."""
    from golden_util import run_one_site_case
    c, st, zerr = run_one_site_case(name)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert zerr < 1e-11
    assert one_minus_f < 1e-12


def test_gpu_observables_one_pass():
    """The run loop measures every <Z_i> in one pass over the tree
    (``expect_many``) after each step: the values are the reference's saved
    ones, and products across the root, several operators on one node and the
    norm match the oracle's full contraction of the device state."""
    import pytreenet_gb300 as P
    name = "ttree3_heis_chi6_o1"
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    ids = [nid for nid, _ in c["spec"]]
    ops = {nid: P.TensorProduct({nid: Zm}) for nid in ids}
    algo = P.FirstOrderOneSiteTDVP(st, H, c["dt"], c["dt"] * c["steps"], ops,
                                   config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                   solver_options={"krylov_tol": c["krylov_tol"]})
    res = algo.run(pgbar=False)
    assert np.max(np.abs(res[1:] - c["z"])) < 1e-10
    rng = np.random.default_rng(11)
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    M = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
    prods = [{ids[1]: X}, {ids[1]: M}, {ids[0]: Zm, ids[-1]: X}, {ids[1]: X, ids[2]: X}, {},
             {ids[-1]: M, ids[-2]: Zm, ids[0]: X}]
    got = algo.net.expect_many(prods)
    ost = O.OState(oracle_state(c).tree, {nid: algo.state.get_phys_numpy(nid) for nid in ids})
    want = np.array([O.expect_product(ost, p) for p in prods])
    assert np.max(np.abs(got - want)) < 1e-12
