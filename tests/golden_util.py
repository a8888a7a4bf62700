"""Load golden fixtures into the oracle's data model (shared by the tests)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_case(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    ids = [str(x) for x in d["spec_ids"]]
    parents = [str(x) or None for x in d["spec_parents"]]
    spec = list(zip(ids, parents))
    case = {
        "spec": spec,
        "init": {i: d[f"init/{i}"] for i in ids},
        "ttno": {i: d[f"ttno/{i}"] for i in ids},
        "final": {i: d[f"final/{i}"] for i in ids},
        "z": d["z"],
        "dt": float(d["dt"]),
        "steps": int(d["steps"]),
        "order": int(d["order"]),
        "krylov_tol": float(d["krylov_tol"]),
        "update_path": [str(x) for x in d["update_path"]],
        "two_site": bool(int(d["two_site"])) if "two_site" in d.files else False,
        "energy_final": complex(d["energy_final"]) if "energy_final" in d.files else None,
    }
    case["path_mode"] = str(d["path_mode"]) if "path_mode" in d.files else "LeafToRoot"
    case["time_evo_mode"] = str(d["time_evo_mode"]) if "time_evo_mode" in d.files else "KRYLOV"
    case["solver_options"] = {k.split("/", 1)[1]: float(d[k]) for k in d.files if k.startswith("solver_options/")}
    case["tebd"] = bool(int(d["tebd"])) if "tebd" in d.files else False
    case["driven"] = "amp" in d.files
    if case["driven"]:
        case["ttno_d"] = {i: d[f"ttno_d/{i}"] for i in ids}
        case["amp"], case["omega"] = float(d["amp"]), float(d["omega"])
    if case["tebd"]:
        case["gates"] = [(d[f"gate/{i}/op"], [str(x) for x in d[f"gate/{i}/ids"]]) for i in range(int(d["n_gates"]))]
    if case["two_site"] or case["tebd"]:
        case["svd"] = dict(max_bond_dim=int(d["svd_max_bond_dim"]), rel_tol=float(d["svd_rel_tol"]),
                           total_tol=float(d["svd_total_tol"]), renorm=bool(int(d["svd_renorm"])))
    return case


CASES = ["c1_binary15_tfim_chi8", "binary7_tfim_chi4_o2", "ttree3_heis_chi6_o1",
         "ttree3_heis_chi6_o2", "ternary2_xxz_chi4_o1"]
TWO_SITE_CASES = ["ternary2_xxz_neel_2tdvp", "binary7_heis_2tdvp_trunc", "binary7_heis_2tdvp_l2l",
                  "binary7_heis_2tdvp_rk45", "binary7_heis_2tdvp_fastest"]
ODE_MODES = ("RK45", "RK23", "DOP853")
# the reference on the trees and Hamiltonian families of the five benchmark
# configurations, at small bond dimensions (make_golden.py config_shape_cases)
CONFIG_SHAPE_CASES = ["c3shape_ttree20_heis_chi8_o1", "c5shape_binary31_tfim_gi_chi8_o1"]
CONFIG_SHAPE_TWO_SITE_CASES = ["c2shape_ternary3_xxz_neel_chi3", "c4shape_binary31_heis_h2_neel_chi8"]


def case_solver(c, P):
    """(TimeEvoMode, solver_options) of a fixture for the engine's drivers."""
    mode = P.TimeEvoMode[c["time_evo_mode"]]
    if mode is P.TimeEvoMode.KRYLOV:
        return mode, {"krylov_tol": c["krylov_tol"]}
    return mode, (c["solver_options"] or None)


def oracle_ode(c):
    """The oracle's ``ode`` argument for a fixture run with a solve_ivp mode."""
    if c["time_evo_mode"] not in ODE_MODES:
        return None
    return dict(c["solver_options"], method=c["time_evo_mode"])
TEBD_CASES = ["binary7_tfim_tebd", "binary7_tfim_tebd_swaps", "binary7_tfim_tebd_strang"]
DRIVEN_CASES = ["binary7_tfim_driven_o1", "binary7_tfim_driven_o2"]
BUG_CASES = ["binary15_tfim_fixed_bug", "ternary2_xxz_fixed_bug", "binary15_tfim_fixed_bug_rk45"]
ADAPTIVE_BUG_CASES = ["binary7_tfim_bug", "ternary2_xxz_bug"]
L2L_CASES = ["ttree3_heis_l2l_o1", "binary15_tfim_l2l_o2"]
DEFAULT_MODE_CASES = ["ttree3_heis_fastest_o1", "binary7_tfim_fastest_o2"]
# TDVP with the solve_ivp modes (RK45, DOP853 with solve_ivp's own tolerances, RK23)
ODE_CASES = ["ttree3_heis_rk45_o1", "binary7_tfim_dop853_o2", "binary7_tfim_rk23_o1"]


def driven_ttno(case, t):
    """TTNO tensors of a driven case at time t: base + amp sin(omega t) D."""
    import numpy as np
    f = case["amp"] * np.sin(case["omega"] * t)
    return {k: case["ttno"][k] + f * case["ttno_d"][k] for k in case["ttno"]}


def build_ttn(cls, spec, tensors):
    """Build a pytreenet_gb300 TTNS/TTNO from tensors in physical layout."""
    t = cls()
    parent = dict(spec)
    slot = {nid: 0 for nid, _ in spec}
    for nid, p in spec:
        if p is None:
            t.add_root(nid, tensors[nid])
        else:
            off = 1 if parent[p] is not None else 0
            t.add_child_to_parent(nid, tensors[nid], 0, p, off + slot[p])
            slot[p] += 1
    return t


def oracle_state(case, key="init"):
    import oracle as O
    tree = O.OTree()
    for nid, p in case["spec"]:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    return O.OState(tree, case[key])


def fidelity_and_dist(a_state, b_state):
    """1 - |<a|b>|/(|a||b|) and the phase-aligned relative distance, by oracle contractions."""
    import numpy as np
    import oracle as O
    ab = O.scalar_product(a_state, b_state)
    aa = O.scalar_product(a_state, a_state).real
    bb = O.scalar_product(b_state, b_state).real
    f = abs(ab) / np.sqrt(aa * bb)
    # ||a - e^{i phi} b||^2 / ||a||^2 with the optimal phase; guard the cancellation
    d2 = max(aa + bb - 2 * abs(ab), 0.0) / aa
    return 1 - f, np.sqrt(d2)


class FixedSplitting:
    """A Trotter splitting whose exponentiated operators are given (taken from
    a fixture): what the reference's TrotterSplitting.exponentiate_splitting
    returned for the recorded run."""

    def __init__(self, gates):
        from pytreenet_gb300 import NumericOperator
        self._ops = [NumericOperator(op, ids) for op, ids in gates]

    def exponentiate_splitting(self, delta_time, ttn=None, dim=None):
        return list(self._ops)


def run_tebd_case(name, steps=None):
    """Run the engine's TEBD on a TEBD fixture; returns (case, oracle-state of the result, <Z> per step)."""
    import numpy as np
    import oracle as O
    import pytreenet_gb300 as P
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    Zm = np.diag([1.0, -1.0]).astype(complex)
    algo = P.TEBD(st, FixedSplitting(c["gates"]), c["dt"], c["dt"] * c["steps"], {},
                  svd_parameters=P.SVDParameters(**c["svd"]))
    zs = []
    for _ in range(c["steps"] if steps is None else steps):
        algo.run_one_time_step()
        zs.append([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    return c, O.OState(oracle_state(c).tree, out), np.array(zs), algo


def run_driven_case(name, precision="plain"):
    """Run the engine's one-site driver with a TimeDependentTTNO built from a
    driven fixture through ``run()``; returns (case, oracle-state of the
    result, <Z> rows after each step)."""
    import numpy as np
    import oracle as O
    import pytreenet_gb300 as P
    from pytreenet_gb300.time_dep import FactorUpdatable, TimeDependentTTNO
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H0 = build_ttn(P.TTNO, c["spec"], {k: v.copy() for k, v in c["ttno"].items()})
    amp, om = c["amp"], c["omega"]
    ups = [FactorUpdatable(nid, tuple(slice(0, d) for d in c["ttno_d"][nid].shape), c["ttno_d"][nid],
                           lambda t: amp * np.sin(om * t)) for nid, _ in c["spec"]]
    H = TimeDependentTTNO(ups, H0)
    Zm = np.diag([1.0, -1.0]).astype(complex)
    ops = {nid: P.TensorProduct({nid: Zm}) for nid, _ in c["spec"]}
    cls = P.FirstOrderOneSiteTDVP if c["order"] == 1 else P.SecondOrderOneSiteTDVP
    algo = cls(st, H, c["dt"], c["dt"] * c["steps"], ops,
               config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV, time_dep=True),
               solver_options={"krylov_tol": c["krylov_tol"]}, precision=precision)
    res = algo.run()
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    return c, O.OState(oracle_state(c).tree, out), np.real(res[1:1 + c["steps"]])


def run_bug_case(name):
    """Run the engine's FixedBUG on a BUG fixture; returns (case, oracle-state of
    the result, <Z_i> after each step)."""
    import numpy as np
    import oracle as O
    import pytreenet_gb300 as P
    from pytreenet_gb300.bug import FixedBUG, FixedBUGConfig
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    Zm = np.diag([1.0, -1.0]).astype(complex)
    mode, opts = case_solver(c, P)
    algo = FixedBUG(st, H, c["dt"], c["dt"] * c["steps"], {}, config=FixedBUGConfig(time_evo_mode=mode),
                    solver_options=opts)
    zs = []
    for _ in range(c["steps"]):
        algo.run_one_time_step()
        zs.append([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    return c, O.OState(oracle_state(c).tree, out), np.array(zs)


def run_one_site_case(name, precision="plain"):
    """The engine's one-site driver on a fixture, honouring its path mode;
    returns (case, oracle-state of the result, max |<Z_i> - reference| over steps)."""
    import numpy as np
    import oracle as O
    import pytreenet_gb300 as P
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    cls = P.FirstOrderOneSiteTDVP if c["order"] == 1 else P.SecondOrderOneSiteTDVP
    mode = P.TimeEvoMode[c["time_evo_mode"]]
    opts = {"krylov_tol": c["krylov_tol"]} if mode is P.TimeEvoMode.KRYLOV else (c["solver_options"] or None)
    algo = cls(st, H, c["dt"], c["dt"] * c["steps"], {},
               config=P.TDVPConfig(time_evo_mode=mode, main_path_mode=P.PathFinderMode[c["path_mode"]]),
               solver_options=opts, precision=precision)
    assert algo.update_path == c["update_path"]
    Zm = np.diag([1.0, -1.0]).astype(complex)
    zerr = 0.0
    for k in range(c["steps"]):
        algo.run_one_time_step()
        z = np.array([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
        zerr = max(zerr, float(np.max(np.abs(z - c["z"][k]))))
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    return c, O.OState(oracle_state(c).tree, out), zerr


def run_adaptive_bug_case(name):
    """The engine's rank-adaptive BUG on a fixture; returns (case, oracle-state of
    the result, <Z_i> after each step, bond dimensions after each step)."""
    import numpy as np
    import oracle as O
    import pytreenet_gb300 as P
    from pytreenet_gb300.bug import BUG, BUGConfig
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    c = load_case(name)
    st = build_ttn(P.TTNS, c["spec"], c["init"])
    H = build_ttn(P.TTNO, c["spec"], c["ttno"])
    Zm = np.diag([1.0, -1.0]).astype(complex)
    cfg = BUGConfig(time_evo_mode=P.TimeEvoMode.KRYLOV, max_bond_dim=int(d["svd_max_bond_dim"]),
                    rel_tol=float(d["svd_rel_tol"]), total_tol=float(d["svd_total_tol"]))
    algo = BUG(st, H, c["dt"], c["dt"] * c["steps"], {}, config=cfg, solver_options={"krylov_tol": c["krylov_tol"]})
    zs, bonds = [], []
    for _ in range(c["steps"]):
        algo.run_one_time_step()
        zs.append([algo.evaluate_operator({nid: Zm}) for nid, _ in c["spec"]])
        bonds.append([algo.state.phys(nid).shape[0] for nid, p in c["spec"] if p is not None])
    out = {nid: algo.state.get_phys_numpy(nid) for nid, _ in c["spec"]}
    return c, O.OState(oracle_state(c).tree, out), np.array(zs), np.array(bonds), d["bonds"]


def swap_splitting(name):
    """The engine's TrotterSplitting.from_lists rebuilt from a fixture's stored
    definition (tensor products and SWAP lists)."""
    import numpy as np
    import pytreenet_gb300 as P
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    n = int(d["n_terms"])
    tps, before, after = [], [], []
    for i in range(n):
        ids = [str(x) for x in d[f"term/{i}/ids"]]
        ops = d[f"term/{i}/ops"]
        tps.append(P.TensorProduct({k: ops[j] for j, k in enumerate(ids)}))
        before.append(P.SWAPlist([tuple(str(y) for y in x) for x in d[f"term/{i}/before"]]))
        after.append(P.SWAPlist([tuple(str(y) for y in x) for x in d[f"term/{i}/after"]]))
    splitting = None
    if "splitting" in d.files:
        splitting = [(int(i), float(f)) for i, f in d["splitting"]]
    return P.TrotterSplitting.from_lists(tps, splitting=splitting, swaps_before=before, swaps_after=after)


def check_heff_fixture(tol=1e-12):
    """Dense effective site Hamiltonians of the engine against the reference's
    ``get_effective_single_site_hamiltonian`` (fixture ``ttree2_heis_heff``)."""
    import numpy as np
    import pytreenet_gb300 as P
    d = np.load(os.path.join(GOLDEN, "ttree2_heis_heff.npz"))
    ids = [str(x) for x in d["spec_ids"]]
    spec = list(zip(ids, [str(x) or None for x in d["spec_parents"]]))
    for nid in [str(x) for x in d["heff_nodes"]]:
        st = build_ttn(P.TTNS, spec, {i: d[f"init/{i}"] for i in ids})
        H = build_ttn(P.TTNO, spec, {i: d[f"ttno/{i}"] for i in ids})
        cache = P.SandwichCache.init_cache_but_one(st, H, nid)
        got = P.get_effective_single_site_hamiltonian(nid, st, H, cache)
        ref = d[f"heff/{nid}"]
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) < tol * max(1.0, np.max(np.abs(ref))), nid
        got2 = P.get_effective_single_site_hamiltonian_nodes(st.nodes[nid], H.nodes[nid], H.get_tensor(nid), cache)
        assert np.max(np.abs(got2 - ref)) < tol * max(1.0, np.max(np.abs(ref))), nid



def run_recorded_case(precision="plain"):
    """The engine's SecondOrderTwoSiteTDVP.run(evaluation_time=2) with every
    record flag, on the inputs of ``binary7_heis_2tdvp_results``; returns
    (engine Results, reference arrays by name)."""
    import numpy as np
    import pytreenet_gb300 as P
    d = np.load(os.path.join(GOLDEN, "binary7_heis_2tdvp_results.npz"))
    ids = [str(x) for x in d["spec_ids"]]
    spec = list(zip(ids, [str(x) or None for x in d["spec_parents"]]))
    st = build_ttn(P.TTNS, spec, {i: d[f"init/{i}"] for i in ids})
    H = build_ttn(P.TTNO, spec, {i: d[f"ttno/{i}"] for i in ids})
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Zm = np.diag([1.0, -1.0]).astype(complex)
    cfg = P.TwoSiteTDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV, max_bond_dim=4, rel_tol=1e-10, total_tol=1e-10,
                              record_bond_dim=True, record_max_bdim=True, record_average_bdim=True,
                              record_total_size=True, record_norm=True, record_loschmidt_amplitude=True)
    ops = {"z0": P.TensorProduct({"s0": Zm}), "x3": P.TensorProduct({"s3": X})}
    algo = P.SecondOrderTwoSiteTDVP(st, H, 0.05, 0.05 * 6, ops, config=cfg, solver_options={"krylov_tol": 1e-12},
                                    precision=precision)
    algo.run(evaluation_time=2)
    ref = {str(k): d["res/" + str(k)] for k in d["res_keys"]}
    return algo.results, ref


def check_zipup_fixture(tag, tol=1e-12):
    """The engine's zip-up against the reference's on ``binary7_tfim_zipup``."""
    import numpy as np
    import oracle as O
    import pytreenet_gb300 as P
    d = np.load(os.path.join(GOLDEN, "binary7_tfim_zipup.npz"))
    ids = [str(x) for x in d["spec_ids"]]
    spec = list(zip(ids, [str(x) or None for x in d["spec_parents"]]))
    st = build_ttn(P.TTNS, spec, {i: d[f"init/{i}"] for i in ids})
    H = build_ttn(P.TTNO, spec, {i: d[f"ttno/{i}"] for i in ids})
    maxd, t = d[f"{tag}/params"]
    out = P.apply_ttno_to_ttns(st, H, P.ApplicationMethod.ZIPUP,
                               P.SVDParameters(max_bond_dim=int(maxd), rel_tol=t, total_tol=t))
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    for i in ids:
        assert tuple(out.phys(i).shape) == d[f"{tag}/final/{i}"].shape, i
    a = O.state_vector(O.OState(tree, {i: out.get_phys_numpy(i) for i in ids}), ids)
    b = O.state_vector(O.OState(tree, {i: d[f"{tag}/final/{i}"] for i in ids}), ids)
    assert np.max(np.abs(a - b)) < tol * np.max(np.abs(b))
