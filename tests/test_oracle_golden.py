"""The oracle (NumPy restatement) against fixtures produced by the reference itself."""
import numpy as np
import pytest

import oracle as O
from golden_util import CASES, GOLDEN, load_case, oracle_state, fidelity_and_dist

Zm = np.diag([1.0, -1.0]).astype(complex)


def _run(c, steps=None):
    st = oracle_state(c)
    cls = O.FirstOrderOneSiteTDVPOracle if c["order"] == 1 else O.SecondOrderOneSiteTDVPOracle
    ode = None
    if c["time_evo_mode"] in ("RK45", "RK23", "DOP853"):
        ode = dict(c["solver_options"], method=c["time_evo_mode"])
    algo = cls(st, c["ttno"], c["dt"], krylov_tol=c["krylov_tol"], path_mode=c["path_mode"],
               exact=c["time_evo_mode"] != "KRYLOV", ode=ode)
    assert algo.update_path == c["update_path"]
    zerr = 0.0
    for k in range(c["steps"] if steps is None else steps):
        algo.run_one_time_step()
        z = np.array([O.expect_product(algo.state, {nid: Zm}) for nid, _ in c["spec"]])
        zerr = max(zerr, float(np.max(np.abs(z - c["z"][k]))))
    return algo, zerr


@pytest.mark.parametrize("name", [n for n in CASES if n != "c1_binary15_tfim_chi8"])
def test_oracle_full_rank_cases(name):
    c = load_case(name)
    algo, zerr = _run(c)
    one_minus_f, dist = fidelity_and_dist(oracle_state(c, "final"), algo.state)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12


def test_oracle_c1_padded_product_state():
    """15-node binary TFIM, chi=8 zero-padded product state, 50 steps.
    The reference's own result moves by ~2e-6 (state) / 5e-9 (<Z>) under a
    1e-15 relative input perturbation, because some QRs see noise-level
    rank deficiency; parity is asserted at that floor."""
    c = load_case("c1_binary15_tfim_chi8")
    algo, zerr = _run(c)
    ids = [s[0] for s in c["spec"]]
    a = O.state_vector(algo.state, ids)
    b = O.state_vector(oracle_state(c, "final"), ids)
    ph = np.vdot(a, b) / abs(np.vdot(a, b))
    rel = np.linalg.norm(a * ph - b) / np.linalg.norm(b)
    assert zerr < 1e-8
    assert rel < 1e-5
    assert abs(1 - abs(np.vdot(a, b)) / np.linalg.norm(a) / np.linalg.norm(b)) < 1e-10


def test_oracle_krylov_known_answers():
    d = np.load(f"{GOLDEN}/units.npz")
    keys = sorted({k.rsplit("/", 1)[0] for k in d.files if k.startswith("krylov/")})
    assert keys
    for k in keys:
        H = d[k + "/H"]
        ef = -1j if k.endswith("fwd") else 1j
        out = O.krylov_exp_action(d[k + "/psi"], lambda y: H @ y, 0.05, ef, krylov_tol=float(d[k + "/tol"]))
        assert np.max(np.abs(out - d[k + "/out"])) < 1e-12 * np.linalg.norm(d[k + "/out"])


def test_update_path_and_orth_paths():
    for name in CASES:
        c = load_case(name)
        st = oracle_state(c)
        assert O.leaf_to_root_path(st.tree) == c["update_path"]


# ---------------------------------------------------------------------------
# two-site TDVP and truncation
# ---------------------------------------------------------------------------
from golden_util import TWO_SITE_CASES, oracle_ode  # noqa: E402


def test_oracle_truncation_known_answers():
    d = np.load(f"{GOLDEN}/units.npz")
    n = int(d["svd/n"])
    assert n > 20
    for i in range(n):
        maxd, rel, tot, renorm, sumt = d[f"svd/{i}/params"]
        p = O.SVDParams(max_bond_dim=int(maxd), rel_tol=rel, total_tol=tot, renorm=bool(renorm),
                        sum_trunc=bool(sumt))
        keep, new_s = O.truncate_singular_values(d[f"svd/{i}/s"], p)
        ref = d[f"svd/{i}/out"]
        assert keep == len(ref), i
        np.testing.assert_allclose(new_s, ref, rtol=1e-15, atol=0)


@pytest.mark.parametrize("name", TWO_SITE_CASES)
def test_oracle_two_site_cases(name):
    c = load_case(name)
    st = oracle_state(c)
    algo = O.SecondOrderTwoSiteTDVPOracle(st, c["ttno"], c["dt"], O.SVDParams(**c["svd"]),
                                          krylov_tol=c["krylov_tol"], path_mode=c["path_mode"], ode=oracle_ode(c),
                                          exact=c["time_evo_mode"] not in ("KRYLOV", "RK45", "RK23", "DOP853"))
    assert algo.update_path == c["update_path"]
    zerr = 0.0
    for k in range(c["steps"]):
        algo.run_one_time_step()
        z = np.array([O.expect_product(algo.state, {nid: Zm}) for nid, _ in c["spec"]])
        zerr = max(zerr, float(np.max(np.abs(z - c["z"][k]))))
    fin = oracle_state(c, "final")
    for nid in fin.tensors:
        assert fin.tensors[nid].shape == algo.state.tensors[nid].shape, nid
    one_minus_f, dist = fidelity_and_dist(fin, algo.state)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12
    assert dist < 1e-8


def test_oracle_first_order_two_site_runs():
    """First-order two-site TDVP (the reference's driver raises on branching
    trees; the oracle runs the intended schedule): norm kept, energy drift small."""
    c = load_case("ternary2_xxz_neel_2tdvp")
    st = oracle_state(c)
    algo = O.FirstOrderTwoSiteTDVPOracle(st, c["ttno"], 0.01, O.SVDParams(**c["svd"]),
                                         krylov_tol=1e-12)
    for _ in range(3):
        algo.run_one_time_step()
    nrm = O.scalar_product(algo.state, algo.state).real
    assert abs(nrm - 1) < 1e-9
    # second order and first order agree to O(dt) on <Z>
    algo2 = O.SecondOrderTwoSiteTDVPOracle(oracle_state(c), c["ttno"], 0.01, O.SVDParams(**c["svd"]),
                                           krylov_tol=1e-12)
    for _ in range(3):
        algo2.run_one_time_step()
    z1 = np.array([O.expect_product(algo.state, {nid: Zm}) for nid, _ in c["spec"]])
    z2 = np.array([O.expect_product(algo2.state, {nid: Zm}) for nid, _ in c["spec"]])
    assert np.max(np.abs(z1 - z2)) < 5e-3


def test_oracle_tebd_matches_reference():
    from golden_util import TEBD_CASES
    for name in TEBD_CASES:
        c = load_case(name)
        algo = O.TEBDOracle(oracle_state(c), c["gates"], O.SVDParams(**c["svd"]))
        zerr = 0.0
        for k in range(c["steps"]):
            algo.run_one_time_step()
            z = np.array([O.expect_product(algo.state, {nid: Zm}) for nid, _ in c["spec"]])
            zerr = max(zerr, float(np.max(np.abs(z - c["z"][k]))))
        fin = oracle_state(c, "final")
        for nid in fin.tensors:
            assert fin.tensors[nid].shape == algo.state.tensors[nid].shape
        one_minus_f, dist = fidelity_and_dist(fin, algo.state)
        # the state is not normalised (TEBD keeps the norm, here ~6e4): relative <Z> error
        assert zerr < 1e-13 * np.max(np.abs(c["z"]))
        assert one_minus_f < 1e-13


@pytest.mark.parametrize("name", CASES)
def test_oracle_ttno_expectation_matches_reference(name):
    c = load_case(name)
    e = O.ttno_expectation(oracle_state(c, "final"), c["ttno"])
    assert abs(e - c["energy_final"]) < 1e-12 * max(1.0, abs(c["energy_final"]))


@pytest.mark.parametrize("name", ["binary7_tfim_driven_o1", "binary7_tfim_driven_o2"])
def test_oracle_time_dependent_hamiltonian(name):
    """A driven field g(t) through the reference's TimeDependentTTNO: the oracle
    swaps in the TTNO tensors of the next time after every step, keeping the
    environments it has (the reference does not rebuild them either)."""
    from golden_util import driven_ttno
    c = load_case(name)
    st = oracle_state(c)
    cls = O.FirstOrderOneSiteTDVPOracle if c["order"] == 1 else O.SecondOrderOneSiteTDVPOracle
    algo = cls(st, driven_ttno(c, 0.0), c["dt"], krylov_tol=c["krylov_tol"])
    static = cls(oracle_state(c), driven_ttno(c, 0.0), c["dt"], krylov_tol=c["krylov_tol"])
    zerr, zstatic = 0.0, 0.0
    for k in range(c["steps"]):
        algo.run_one_time_step()
        static.run_one_time_step()
        z = np.array([O.expect_product(algo.state, {nid: Zm}) for nid, _ in c["spec"]])
        zs = np.array([O.expect_product(static.state, {nid: Zm}) for nid, _ in c["spec"]])
        zerr = max(zerr, float(np.max(np.abs(z - c["z"][k]))))
        zstatic = max(zstatic, float(np.max(np.abs(zs - c["z"][k]))))
        algo.W = driven_ttno(c, (k + 1) * c["dt"])
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), algo.state)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12
    assert zstatic > 1e-4            # the drive matters at this resolution


@pytest.mark.parametrize("name", ["binary15_tfim_fixed_bug", "ternary2_xxz_fixed_bug",
                                  "binary15_tfim_fixed_bug_rk45"])
def test_oracle_fixed_bug_matches_reference(name):
    """Fixed-rank BUG: the oracle's step against the reference's FixedBUG
    (Krylov, or RK45 with the deeper nodes at solve_ivp's own tolerances)."""
    c = load_case(name)
    st = oracle_state(c)
    st.orth_center = c["spec"][0][0]
    zerr = 0.0
    for k in range(c["steps"]):
        st = O.fixed_bug_step(st, c["ttno"], c["dt"], krylov_tol=c["krylov_tol"], ode=oracle_ode(c))
        z = np.array([O.expect_product(st, {nid: Zm}) for nid, _ in c["spec"]])
        zerr = max(zerr, float(np.max(np.abs(z - c["z"][k]))))
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", ["binary7_tfim_bug", "ternary2_xxz_bug"])
def test_oracle_adaptive_bug_matches_reference(name):
    """Rank-adaptive BUG with SVD truncation: the oracle against the reference's
    BUG, including the bond dimensions after every step."""
    d = np.load(f"{GOLDEN}/{name}.npz")
    c = load_case(name)
    params = O.SVDParams(max_bond_dim=int(d["svd_max_bond_dim"]), rel_tol=float(d["svd_rel_tol"]),
                         total_tol=float(d["svd_total_tol"]), renorm=False)
    st = oracle_state(c)
    st.orth_center = None
    O.canonical_form(st, c["spec"][0][0])
    zerr = 0.0
    for k in range(c["steps"]):
        st = O.adaptive_bug_step(st, c["ttno"], c["dt"], params, krylov_tol=c["krylov_tol"])
        z = np.array([O.expect_product(st, {nid: Zm}) for nid, _ in c["spec"]])
        zerr = max(zerr, float(np.max(np.abs(z - c["z"][k]))))
        bonds = [st.tensors[nid].shape[0] for nid, p in c["spec"] if p is not None]
        assert bonds == list(d["bonds"][k])
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), st)
    assert zerr < 1e-9
    assert one_minus_f < 1e-11


@pytest.mark.parametrize("name", ["ttree3_heis_l2l_o1", "binary15_tfim_l2l_o2"])
def test_oracle_leaf_to_leaf_path(name):
    """One-site TDVP on PathFinderMode.LeafToLeaf: same path and results as the reference."""
    c = load_case(name)
    algo, zerr = _run(c)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), algo.state)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12


@pytest.mark.parametrize("name", ["ttree3_heis_fastest_o1", "binary7_tfim_fastest_o2"])
def test_oracle_default_mode_matches_reference(name):
    """TDVPConfig() (FASTEST, a dense exponential): the oracle's dense
    exponential reproduces the reference."""
    c = load_case(name)
    assert c["time_evo_mode"] == "FASTEST"
    algo, zerr = _run(c)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), algo.state)
    assert zerr < 1e-12
    assert one_minus_f < 1e-13


@pytest.mark.parametrize("name", ["ttree3_heis_rk45_o1", "binary7_tfim_dop853_o2", "binary7_tfim_rk23_o1"])
def test_oracle_ode_modes_match_reference(name):
    """TDVP with a solve_ivp mode: the oracle's solve_ivp on the matrix-free
    effective Hamiltonian reproduces the reference's run (DOP853 given no
    options runs at solve_ivp's rtol 1e-3 / atol 1e-6, so its result is far
    from the exact evolution but the same integration)."""
    c = load_case(name)
    algo, zerr = _run(c)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), algo.state)
    assert zerr < 1e-11
    assert one_minus_f < 1e-13


@pytest.mark.parametrize("tag", ["cap", "tol"])
def test_oracle_zipup_matches_reference(tag):
    """Non-canonical zip-up: the oracle against the reference's zipup."""
    d = np.load(f"{GOLDEN}/binary7_tfim_zipup.npz")
    ids = [str(x) for x in d["spec_ids"]]
    spec = list(zip(ids, [str(x) or None for x in d["spec_parents"]]))
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    maxd, tol = d[f"{tag}/params"]
    out = O.zipup_apply(O.OState(tree, {i: d[f"init/{i}"] for i in ids}), {i: d[f"ttno/{i}"] for i in ids},
                        O.SVDParams(max_bond_dim=int(maxd), rel_tol=tol, total_tol=tol))
    ref = O.OState(tree, {i: d[f"{tag}/final/{i}"] for i in ids})
    for i in ids:
        assert out.tensors[i].shape == ref.tensors[i].shape, i
    a, b = O.state_vector(out, ids), O.state_vector(ref, ids)
    assert np.max(np.abs(a - b)) < 1e-12 * np.max(np.abs(b))


from golden_util import CONFIG_SHAPE_CASES, CONFIG_SHAPE_TWO_SITE_CASES  # noqa: E402


@pytest.mark.parametrize("name", CONFIG_SHAPE_CASES)
def test_oracle_config_shape_one_site(name):
    """The reference's one-site runs on the 61-site T-tree (Heisenberg +
    fields) and the 31-site binary TFIM with one field per site: same update
    path, <Z_i> after every step to 1e-10, final state 1-F < 1e-12, energy."""
    c = load_case(name)
    algo, zerr = _run(c)
    one_minus_f, _ = fidelity_and_dist(oracle_state(c, "final"), algo.state)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12
    e = O.ttno_expectation(algo.state, c["ttno"])
    assert abs(e - c["energy_final"]) < 1e-10 * max(1.0, abs(c["energy_final"]))


@pytest.mark.parametrize("name", CONFIG_SHAPE_TWO_SITE_CASES)
def test_oracle_config_shape_two_site(name):
    """The reference's second-order two-site runs on the 40-site ternary tree
    (XXZ, Neel, bonds growing to 3) and the 31-site binary tree (random fields
    up to 2, Neel, bonds growing to 8 at cutoff 1e-9): same final bond
    dimensions, <Z_i> after every step to 1e-10, 1-F < 1e-12."""
    c = load_case(name)
    algo = O.SecondOrderTwoSiteTDVPOracle(oracle_state(c), c["ttno"], c["dt"], O.SVDParams(**c["svd"]),
                                          krylov_tol=c["krylov_tol"])
    assert algo.update_path == c["update_path"]
    zerr = 0.0
    for k in range(c["steps"]):
        algo.run_one_time_step()
        z = np.array([O.expect_product(algo.state, {nid: Zm}) for nid, _ in c["spec"]])
        zerr = max(zerr, float(np.max(np.abs(z - c["z"][k]))))
    fin = oracle_state(c, "final")
    for nid in fin.tensors:
        assert fin.tensors[nid].shape == algo.state.tensors[nid].shape, nid
    one_minus_f, _ = fidelity_and_dist(fin, algo.state)
    assert zerr < 1e-10
    assert one_minus_f < 1e-12
