"""Generate golden fixtures by running PyTreeNet's own TDVP drivers.

Run (in a container where the reference sources are available):

    python tests/golden/make_golden.py /root/reference

The reference needs ``h5py`` only for HDF5 result I/O; when it is missing, a
stand-in module whose ``File`` raises is registered before the import. Every
fixture stores the seeded inputs (state tensors and TTNO tensors in the engine's
physical leg layout: parent, children in insertion order, physical / out, in),
the reference's outputs after each time step (state tensors in the same layout,
single-site expectation values) and the reference's update path.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_reference(ref_root: str):
    try:
        import h5py  # noqa: F401
    except ImportError:
        stub = types.ModuleType("h5py")

        class File:  # noqa: D401
            def __init__(self, *a, **k):
                raise RuntimeError("h5py unavailable")
        stub.File = File
        sys.modules["h5py"] = stub
    sys.path.insert(0, ref_root)
    import pytreenet as ptn
    return ptn


X = np.array([[0, 1], [1, 0]], dtype=complex)
Y = np.array([[0, -1j], [1j, 0]], dtype=complex)
Z = np.diag([1.0, -1.0]).astype(complex)


def binary_tree(n):
    """Heap-ordered binary tree: node i has children 2i+1, 2i+2."""
    return [(f"s{i}", None if i == 0 else f"s{(i - 1) // 2}") for i in range(n)]


def t_tree(arm_len):
    """Root with three arms of ``arm_len`` sites."""
    spec = [("root", None)]
    for a in range(3):
        prev = "root"
        for k in range(arm_len):
            nid = f"a{a}_{k}"
            spec.append((nid, prev))
            prev = nid
    return spec


def ternary_tree(depth):
    spec = [("t0", None)]
    frontier = ["t0"]
    idx = 1
    for _ in range(depth):
        nxt = []
        for p in frontier:
            for _ in range(3):
                nid = f"t{idx}"
                idx += 1
                spec.append((nid, p))
                nxt.append(nid)
        frontier = nxt
    return spec


def children_of(spec):
    ch = {nid: [] for nid, _ in spec}
    for nid, p in spec:
        if p is not None:
            ch[p].append(nid)
    return ch


def build_reference_state(ptn, spec, tensors):
    """Build the reference TTNS from tensors in physical layout."""
    ch = children_of(spec)
    ttns = ptn.TreeTensorNetworkState()
    slot = {nid: 0 for nid, _ in spec}
    for nid, p in spec:
        if p is None:
            ttns.add_root(ptn.Node(identifier=nid), tensors[nid])
        else:
            off = 1 if dict(spec)[p] is not None else 0
            ttns.add_child_to_parent(ptn.Node(identifier=nid), tensors[nid], 0, p, off + slot[p])
            slot[p] += 1
    return ttns


def phys_layout(ttn_node_parent, ttn_node_children, tensor, spec_children, nopen):
    """Permute a reference tensor (parent, logical children, open...) into
    (parent, children in insertion order, open...)."""
    off = 0 if ttn_node_parent is None else 1
    perm = list(range(off))
    perm += [off + ttn_node_children.index(c) for c in spec_children]
    nv = off + len(ttn_node_children)
    perm += list(range(nv, nv + nopen))
    # a copy: the reference updates time-dependent TTNO tensors in place
    return np.array(np.transpose(tensor, perm), order="C", copy=True)


def export_state(ttns, spec):
    ch = children_of(spec)
    out = {}
    for nid, _ in spec:
        node = ttns.nodes[nid]
        out[nid] = phys_layout(node.parent, list(node.children), ttns.tensors[nid], ch[nid], 1)
    return out


def export_ttno(ttno, spec):
    ch = children_of(spec)
    out = {}
    for nid, _ in spec:
        node = ttno.nodes[nid]
        out[nid] = phys_layout(node.parent, list(node.children), ttno.tensors[nid], ch[nid], 2)
    return out


def product_state_tensors(spec, rng, bond):
    """Product state uniform on the Bloch sphere, zero-padded to ``bond``."""
    ch = children_of(spec)
    parent = dict(spec)
    out = {}
    for nid, p in spec:
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        th, ph = np.arccos(v[2]), np.arctan2(v[1], v[0])
        site = np.array([np.cos(th / 2), np.exp(1j * ph) * np.sin(th / 2)], dtype=complex)
        nv = len(ch[nid]) + (0 if p is None else 1)
        t = np.zeros([bond] * nv + [2], dtype=complex)
        t[(0,) * nv] = site
        out[nid] = t
    return out


def random_state_tensors(spec, rng, bond):
    ch = children_of(spec)
    out = {}
    for nid, p in spec:
        nv = len(ch[nid]) + (0 if p is None else 1)
        shape = [bond] * nv + [2]
        out[nid] = (rng.normal(size=shape) + 1j * rng.normal(size=shape)) / np.sqrt(2)
    return out


def tfim(ptn, spec, J=1.0, g=0.5):
    conv = {"mJZ": -J * Z, "Z": Z, "mgX": -g * X, "I2": np.eye(2, dtype=complex)}
    terms = [ptn.TensorProduct({nid: "mJZ", p: "Z"}) for nid, p in spec if p is not None]
    terms += [ptn.TensorProduct({nid: "mgX"}) for nid, _ in spec]
    return ptn.Hamiltonian(terms, conv)


def heisenberg_fields(ptn, spec, fields, jxy=None, jz=None):
    conv = {"I2": np.eye(2, dtype=complex)}
    terms = []
    for i, (nid, p) in enumerate(spec):
        conv[f"h{nid}"] = fields[i] * Z
        terms.append(ptn.TensorProduct({nid: f"h{nid}"}))
    for e, (nid, p) in enumerate([x for x in spec if x[1] is not None]):
        cxy = 1.0 if jxy is None else jxy[e]
        cz = 1.0 if jz is None else jz[e]
        conv[f"X{e}"] = cxy * X
        conv[f"Y{e}"] = cxy * Y
        conv[f"Z{e}"] = cz * Z
        conv["X"], conv["Y"], conv["Z"] = X, Y, Z
        terms.append(ptn.TensorProduct({nid: f"X{e}", p: "X"}))
        terms.append(ptn.TensorProduct({nid: f"Y{e}", p: "Y"}))
        terms.append(ptn.TensorProduct({nid: f"Z{e}", p: "Z"}))
    return ptn.Hamiltonian(terms, conv)


def run_case(ptn, name, spec, tensors, ham_fn, dt, steps, order, tol, canonical_random=False, path_mode=None,
             default_mode=False, ode_mode=None, ode_options=None):
    from pytreenet.time_evolution.time_evolution import TimeEvoMode
    from pytreenet.time_evolution.tdvp_algorithms.tdvp_algorithm import TDVPConfig
    from pytreenet.time_evolution.time_evo_util import PathFinderMode
    psi = build_reference_state(ptn, spec, tensors)
    if canonical_random:
        psi.canonical_form(spec[0][0])
        psi.normalise()
        tensors = export_state(psi, spec)
        psi = build_reference_state(ptn, spec, tensors)
    H = ptn.TTNO.from_hamiltonian(ham_fn(psi), psi)
    cls = ptn.FirstOrderOneSiteTDVP if order == 1 else ptn.SecondOrderOneSiteTDVP
    ops = {nid: ptn.TensorProduct({nid: Z}) for nid, _ in spec}
    cfg = TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV)
    if path_mode is not None:
        cfg = TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV, main_path_mode=PathFinderMode[path_mode])
    if default_mode:
        # TDVPConfig() runs the reference's default local exponential (FASTEST -> CHEBYSHEV)
        algo = cls(psi, H, dt, dt * steps, ops, config=TDVPConfig())
    elif ode_mode is not None:
        # a solve_ivp mode; ode_options None = the solver's own tolerances
        algo = cls(psi, H, dt, dt * steps, ops, config=TDVPConfig(time_evo_mode=TimeEvoMode[ode_mode]),
                   solver_options=None if ode_options is None else dict(ode_options))
    else:
        algo = cls(psi, H, dt, dt * steps, ops, config=cfg, solver_options={"krylov_tol": tol})
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": dt, "steps": steps, "order": order, "krylov_tol": tol,
           "update_path": np.array(algo.update_path)}
    if path_mode is not None:
        rec["path_mode"] = path_mode
    if default_mode or ode_mode is not None:
        rec["time_evo_mode"] = str(algo.config.time_evo_mode.name)
    for k, v in (ode_options or {}).items():
        rec[f"solver_options/{k}"] = v
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in export_ttno(H, spec).items():
        rec[f"ttno/{nid}"] = t
    zs = []
    for step in range(steps):
        algo.run_one_time_step()
        zs.append([algo.state.operator_expectation_value(ops[nid]) for nid, _ in spec])
    rec["z"] = np.array(zs)
    rec["energy_final"] = algo.state.operator_expectation_value(H)
    for nid, t in export_state(algo.state, spec).items():
        rec[f"final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "written; path", algo.update_path[:6], "...")


def neel_state_tensors(spec):
    """Neel product state by depth parity, every bond of dimension 1."""
    ch = children_of(spec)
    parent = dict(spec)
    depth = {}
    out = {}
    for nid, p in spec:
        depth[nid] = 0 if p is None else depth[p] + 1
        v = np.array([1, 0], dtype=complex) if depth[nid] % 2 == 0 else np.array([0, 1], dtype=complex)
        nv = len(ch[nid]) + (0 if p is None else 1)
        out[nid] = v.reshape([1] * nv + [2])
    return out


def run_case_two_site(ptn, name, spec, tensors, ham_fn, dt, steps, tol, svd, canonical_random=False,
                      path_mode=None, ode_mode=None, ode_options=None):
    """Second-order two-site TDVP (``secondordertwosite.py``) with truncation ``svd``
    = (max_bond_dim, rel_tol, total_tol, renorm)."""
    from pytreenet.time_evolution.time_evolution import TimeEvoMode
    from pytreenet.time_evolution.tdvp_algorithms.twositetdvp import TwoSiteTDVPConfig
    from pytreenet.time_evolution.tdvp_algorithms.secondordertwosite import SecondOrderTwoSiteTDVP
    psi = build_reference_state(ptn, spec, tensors)
    if canonical_random:
        psi.canonical_form(spec[0][0])
        psi.normalise()
        tensors = export_state(psi, spec)
        psi = build_reference_state(ptn, spec, tensors)
    H = ptn.TTNO.from_hamiltonian(ham_fn(psi), psi)
    ops = {nid: ptn.TensorProduct({nid: Z}) for nid, _ in spec}
    maxd, rel, tot, renorm = svd
    extra = {}
    if path_mode is not None:
        from pytreenet.time_evolution.time_evo_util import PathFinderMode
        extra["main_path_mode"] = PathFinderMode[path_mode]
    mode = TimeEvoMode.KRYLOV if ode_mode is None else TimeEvoMode[ode_mode]
    cfg = TwoSiteTDVPConfig(time_evo_mode=mode, max_bond_dim=maxd, rel_tol=rel,
                            total_tol=tot, renorm=renorm, **extra)
    algo = SecondOrderTwoSiteTDVP(psi, H, dt, dt * steps, ops, config=cfg,
                                  solver_options={"krylov_tol": tol} if ode_mode is None else
                                  (None if ode_options is None else dict(ode_options)))
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": dt, "steps": steps, "order": 2, "krylov_tol": tol,
           "two_site": 1, "svd_max_bond_dim": maxd, "svd_rel_tol": rel, "svd_total_tol": tot,
           "svd_renorm": int(renorm), "update_path": np.array(algo.update_path)}
    if path_mode is not None:
        rec["path_mode"] = path_mode
    if ode_mode is not None:
        rec["time_evo_mode"] = ode_mode
    for k, v in (ode_options or {}).items():
        rec[f"solver_options/{k}"] = v
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in export_ttno(H, spec).items():
        rec[f"ttno/{nid}"] = t
    zs = []
    for step in range(steps):
        algo.run_one_time_step()
        zs.append([algo.state.operator_expectation_value(ops[nid]) for nid, _ in spec])
    rec["z"] = np.array(zs)
    for nid, t in export_state(algo.state, spec).items():
        rec[f"final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "written; max bond", algo.state.max_bond_dim())


def run_case_tebd(ptn, name, spec, tensors, dt, steps, svd, J=1.0, g=0.7):
    """TEBD (``time_evolution/tebd.py``) with a first-order Trotter splitting of
    H = -J sum Z Z - g sum X: every edge term and every field term is one
    TrotterStep with factor 1, in the order: edges (spec order), then fields.
    The exponentiated gates the reference applies are stored with the result."""
    psi = build_reference_state(ptn, spec, tensors)
    steps_ = [ptn.TrotterStep(ptn.TensorProduct({p: -J * Z, nid: Z}), 1.0) for nid, p in spec if p is not None]
    steps_ += [ptn.TrotterStep(ptn.TensorProduct({nid: -g * X}), 1.0) for nid, _ in spec]
    split = ptn.TrotterSplitting(steps_)
    maxd, rel, tot, renorm = svd
    params = ptn.SVDParameters(max_bond_dim=maxd, rel_tol=rel, total_tol=tot, renorm=renorm)
    ops = {nid: ptn.TensorProduct({nid: Z}) for nid, _ in spec}
    tebd = ptn.TEBD(psi, split, dt, dt * steps, ops, svd_parameters=params)
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": dt, "steps": steps, "order": 0, "krylov_tol": 0.0, "tebd": 1,
           "svd_max_bond_dim": maxd, "svd_rel_tol": rel, "svd_total_tol": tot, "svd_renorm": int(renorm),
           "update_path": np.array([s[0] for s in spec]), "n_gates": len(tebd.exponents)}
    for i, u in enumerate(tebd.exponents):
        rec[f"gate/{i}/op"] = np.asarray(u.operator)
        rec[f"gate/{i}/ids"] = np.array(list(u.node_identifiers))
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, _ in spec:
        rec[f"ttno/{nid}"] = np.zeros(1)
    zs = []
    for step in range(steps):
        tebd.run_one_time_step()
        zs.append([tebd.state.operator_expectation_value(ops[nid]) for nid, _ in spec])
    rec["z"] = np.array(zs)
    for nid, t in export_state(tebd.state, spec).items():
        rec[f"final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "written; max bond", tebd.state.max_bond_dim())


def run_case_tebd_swaps(ptn, name, spec, tensors, dt, steps, svd, J=1.0, g=0.7, K=0.4):
    """TEBD whose splitting (``TrotterSplitting.from_lists``, ``trotter.py:218-283``)
    also carries a next-nearest-neighbour term -K Z_s3 Z_s0: s3 and s1 are
    swapped before the exponentiated (s1, s0) term and swapped back after it
    (``SWAPlist``, ``trotter.py:15-103``). The splitting's definition and the
    gates the reference applies are stored."""
    from pytreenet.time_evolution.trotter import SWAPlist
    psi = build_reference_state(ptn, spec, tensors)
    tps = [ptn.TensorProduct({p: -J * Z, nid: Z}) for nid, p in spec if p is not None]
    tps += [ptn.TensorProduct({nid: -g * X}) for nid, _ in spec]
    tps.append(ptn.TensorProduct({"s1": -K * Z, "s0": Z}))
    n = len(tps)
    before = [SWAPlist() for _ in range(n)]
    after = [SWAPlist() for _ in range(n)]
    before[-1] = SWAPlist([("s3", "s1")])
    after[-1] = SWAPlist([("s3", "s1")])
    split = ptn.TrotterSplitting.from_lists(tps, swaps_before=before, swaps_after=after)
    maxd, rel, tot, renorm = svd
    params = ptn.SVDParameters(max_bond_dim=maxd, rel_tol=rel, total_tol=tot, renorm=renorm)
    ops = {nid: ptn.TensorProduct({nid: Z}) for nid, _ in spec}
    tebd = ptn.TEBD(psi, split, dt, dt * steps, ops, svd_parameters=params)
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": dt, "steps": steps, "order": 0, "krylov_tol": 0.0, "tebd": 1,
           "svd_max_bond_dim": maxd, "svd_rel_tol": rel, "svd_total_tol": tot, "svd_renorm": int(renorm),
           "update_path": np.array([s[0] for s in spec]), "n_gates": len(tebd.exponents), "n_terms": n}
    for i, u in enumerate(tebd.exponents):
        rec[f"gate/{i}/op"] = np.asarray(u.operator)
        rec[f"gate/{i}/ids"] = np.array(list(u.node_identifiers))
    for i, tp in enumerate(tps):
        rec[f"term/{i}/ids"] = np.array(list(tp.keys()))
        rec[f"term/{i}/ops"] = np.array([tp[k] for k in tp.keys()])
        rec[f"term/{i}/before"] = np.array(list(before[i]), dtype=str).reshape(-1, 2)
        rec[f"term/{i}/after"] = np.array(list(after[i]), dtype=str).reshape(-1, 2)
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, _ in spec:
        rec[f"ttno/{nid}"] = np.zeros(1)
    zs = []
    for step in range(steps):
        tebd.run_one_time_step()
        zs.append([tebd.state.operator_expectation_value(ops[nid]) for nid, _ in spec])
    rec["z"] = np.array(zs)
    for nid, t in export_state(tebd.state, spec).items():
        rec[f"final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "written; gates", len(tebd.exponents))


def run_case_tebd_strang(ptn, name, spec, tensors, dt, steps, svd, J=1.0, g=0.7):
    """TEBD with a symmetric (Strang) splitting from ``TrotterSplitting.from_lists``:
    the field terms by dt/2, the edge terms by dt, the field terms by dt/2."""
    psi = build_reference_state(ptn, spec, tensors)
    tps = [ptn.TensorProduct({p: -J * Z, nid: Z}) for nid, p in spec if p is not None]
    ne = len(tps)
    tps += [ptn.TensorProduct({nid: -g * X}) for nid, _ in spec]
    fields = list(range(ne, len(tps)))
    splitting = [(i, 0.5) for i in fields] + [(i, 1) for i in range(ne)] + [(i, 0.5) for i in fields]
    split = ptn.TrotterSplitting.from_lists(tps, splitting=splitting)
    maxd, rel, tot, renorm = svd
    params = ptn.SVDParameters(max_bond_dim=maxd, rel_tol=rel, total_tol=tot, renorm=renorm)
    ops = {nid: ptn.TensorProduct({nid: Z}) for nid, _ in spec}
    tebd = ptn.TEBD(psi, split, dt, dt * steps, ops, svd_parameters=params)
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": dt, "steps": steps, "order": 0, "krylov_tol": 0.0, "tebd": 1,
           "svd_max_bond_dim": maxd, "svd_rel_tol": rel, "svd_total_tol": tot, "svd_renorm": int(renorm),
           "update_path": np.array([s[0] for s in spec]), "n_gates": len(tebd.exponents), "n_terms": len(tps),
           "splitting": np.array(splitting, dtype=float)}
    for i, u in enumerate(tebd.exponents):
        rec[f"gate/{i}/op"] = np.asarray(u.operator)
        rec[f"gate/{i}/ids"] = np.array(list(u.node_identifiers))
    for i, tp in enumerate(tps):
        rec[f"term/{i}/ids"] = np.array(list(tp.keys()))
        rec[f"term/{i}/ops"] = np.array([tp[k] for k in tp.keys()])
        rec[f"term/{i}/before"] = np.zeros((0, 2), dtype=str)
        rec[f"term/{i}/after"] = np.zeros((0, 2), dtype=str)
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, _ in spec:
        rec[f"ttno/{nid}"] = np.zeros(1)
    zs = []
    for step in range(steps):
        tebd.run_one_time_step()
        zs.append([tebd.state.operator_expectation_value(ops[nid]) for nid, _ in spec])
    rec["z"] = np.array(zs)
    for nid, t in export_state(tebd.state, spec).items():
        rec[f"final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "written; gates", len(tebd.exponents))


def tebd_swap_cases(ptn):
    rng = np.random.default_rng(53)
    spec = binary_tree(7)
    run_case_tebd_swaps(ptn, "binary7_tfim_tebd_swaps", spec, random_state_tensors(spec, rng, 2), 0.05, 4,
                        (6, 1e-10, 1e-10, False))
    run_case_tebd_strang(ptn, "binary7_tfim_tebd_strang", spec, random_state_tensors(spec, rng, 2), 0.05, 4,
                         (6, 1e-10, 1e-10, False))


def svd_cases():
    """Truncation known answers: the reference's own truncation of fixed spectra."""
    from pytreenet.util.tensor_splitting import SVDParameters, truncate_singular_values
    rec = {}
    spectra = [np.array([1.0, 0.5, 1e-3, 1e-9, 1e-12]), np.array([3.0, 3.0, 2.0, 1e-16]),
               np.array([1e-20, 1e-21]), np.linspace(1.0, 0.01, 40)]
    params = [(100, 1e-15, 1e-15, False, False), (2, 1e-15, 1e-15, False, False),
              (100, 1e-10, 1e-10, False, False), (100, 1e-2, 1e-15, True, False),
              (3, 1e-15, 1e-15, True, False), (100, 1e-15, 1e-3, False, True),
              (100, 1e-15, 0.1, False, True)]
    i = 0
    for s in spectra:
        for (maxd, rel, tot, renorm, sumt) in params:
            p = SVDParameters(max_bond_dim=maxd, rel_tol=rel, total_tol=tot, renorm=renorm,
                              sum_trunc=sumt)
            import warnings
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                new_s, _ = truncate_singular_values(s, p)
            rec[f"{i}/s"] = s
            rec[f"{i}/params"] = np.array([maxd, rel, tot, float(renorm), float(sumt)])
            rec[f"{i}/out"] = np.asarray(new_s)
            i += 1
    rec["n"] = i
    return rec


def unit_cases(ptn):
    """Krylov exponential and single-site matvec known answers."""
    from pytreenet.time_evolution.time_evolution import krylov_exp_action
    from pytreenet.contractions.state_operator_contraction import contract_ket_ham_with_envs
    rng = np.random.default_rng(7)
    rec = {}
    for n, tol in ((40, 1e-10), (48, 1e-12), (16, 0.0)):
        A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        Hm = (A + A.conj().T) / 2
        psi = rng.normal(size=n) + 1j * rng.normal(size=n)
        for ef, tag in ((-1j, "fwd"), (1j, "bwd")):
            out = krylov_exp_action(psi, lambda y: Hm @ y, 0.05, ef, krylov_tol=tol)
            rec[f"krylov/{n}/{tag}/H"] = Hm
            rec[f"krylov/{n}/{tag}/psi"] = psi
            rec[f"krylov/{n}/{tag}/out"] = out
            rec[f"krylov/{n}/{tag}/tol"] = tol
    for k, v in svd_cases().items():
        rec[f"svd/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "units.npz"), **rec)
    print("units written")


def run_case_time_dep(ptn, name, spec, tensors, dt, steps, order, tol, J=1.0, g0=0.5, amp=0.3, omega=5.0):
    """TFIM with a driven field g(t) = g0 + amp sin(omega t) on every site, through
    the reference's ``TimeDependentTTNO`` with one ``FactorUpdatable`` per node
    (``ttno/time_dep_ttno.py:211-342, 370-470``) and ``TDVPConfig(time_dep=True)``.
    The updatable of a node carries the difference of the TTNO tensors at
    g0 + 1 and g0 (the TTNO is affine in g). The loop is the one of
    ``TimeEvolution.run`` (``time_evolution/time_evolution.py:346-368``): step,
    measure, update the Hamiltonian."""
    from pytreenet.time_evolution.time_evolution import TimeEvoMode
    from pytreenet.time_evolution.tdvp_algorithms.tdvp_algorithm import TDVPConfig
    from pytreenet.ttno.time_dep_ttno import TimeDependentTTNO, FactorUpdatable
    psi = build_reference_state(ptn, spec, tensors)
    psi.canonical_form(spec[0][0])
    psi.normalise()
    tensors = export_state(psi, spec)
    psi = build_reference_state(ptn, spec, tensors)
    H0 = ptn.TTNO.from_hamiltonian(tfim(ptn, spec, J=J, g=g0), psi)
    H1 = ptn.TTNO.from_hamiltonian(tfim(ptn, spec, J=J, g=g0 + 1.0), psi)
    ups = []
    for nid, _ in spec:
        D = np.asarray(H1.tensors[nid]) - np.asarray(H0.tensors[nid])
        idx = tuple(slice(0, d) for d in D.shape)
        ups.append(FactorUpdatable(nid, idx, D, lambda t: amp * np.sin(omega * t)))
    H = TimeDependentTTNO(ups, H0)
    cls = ptn.FirstOrderOneSiteTDVP if order == 1 else ptn.SecondOrderOneSiteTDVP
    ops = {nid: ptn.TensorProduct({nid: Z}) for nid, _ in spec}
    algo = cls(psi, H, dt, dt * steps, ops,
               config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV, time_dep=True),
               solver_options={"krylov_tol": tol})
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": dt, "steps": steps, "order": order, "krylov_tol": tol,
           "update_path": np.array(algo.update_path), "J": J, "g0": g0, "amp": amp, "omega": omega}
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in export_ttno(H0, spec).items():
        rec[f"ttno/{nid}"] = t
    ch = children_of(spec)
    for (nid, _), u in zip(spec, ups):
        node = H0.nodes[nid]
        rec[f"ttno_d/{nid}"] = phys_layout(node.parent, list(node.children), u.initial_values, ch[nid], 2)
    zs = []
    for step in range(steps):
        algo.run_one_time_step()
        zs.append([algo.state.operator_expectation_value(ops[nid]) for nid, _ in spec])
        algo.update_hamiltonian()
    rec["z"] = np.array(zs)
    for nid, t in export_state(algo.state, spec).items():
        rec[f"final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "written")


def saved_files(ptn):
    """A TTNS and a TTNO written by the reference's ``TreeTensorNetwork.save``
    (``core/ttn.py:1747-1780``), after a canonical form and a TDVP step have
    reordered children, so the files carry non-trivial leg orders."""
    from pytreenet.time_evolution.time_evolution import TimeEvoMode
    from pytreenet.time_evolution.tdvp_algorithms.tdvp_algorithm import TDVPConfig
    rng = np.random.default_rng(5)
    spec = binary_tree(7)
    psi = build_reference_state(ptn, spec, random_state_tensors(spec, rng, 2))
    H = ptn.TTNO.from_hamiltonian(tfim(ptn, spec), psi)
    algo = ptn.FirstOrderOneSiteTDVP(psi, H, 0.05, 0.1, {}, config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV))
    algo.run_one_time_step()
    algo.state.save(os.path.join(HERE, "saved_ttns"))
    H.save(os.path.join(HERE, "saved_ttno"))
    ids = [nid for nid, _ in spec]
    rec = {"ids": np.array(ids),
           "z": np.array([algo.state.operator_expectation_value(ptn.TensorProduct({nid: Z})) for nid in ids]),
           "norm2": algo.state.scalar_product()}
    np.savez_compressed(os.path.join(HERE, "saved_ttns_values.npz"), **rec)
    print("saved files written")


def capped_state_tensors(spec, rng, chi):
    """Gaussian tensors whose bond to a subtree of s sites has dimension
    min(chi, 2^s, 2^(n-s)): every QR of a sweep is tall and of full rank."""
    ch = children_of(spec)
    n = len(spec)
    size = {}
    for nid, _ in reversed(spec):
        size[nid] = 1 + sum(size[c] for c in ch[nid])

    def bond(c):
        return int(min(chi, 2 ** size[c], 2 ** (n - size[c])))
    out = {}
    for nid, p in spec:
        shape = ([bond(nid)] if p is not None else []) + [bond(c) for c in ch[nid]] + [2]
        out[nid] = (rng.normal(size=shape) + 1j * rng.normal(size=shape)) / np.sqrt(2)
    return out


def run_case_bug(ptn, name, spec, tensors, ham_fn, dt, steps, tol, ode_mode=None, ode_options=None):
    """The reference's fixed-rank BUG (``time_evolution/fixed_bug.py``,
    ``time_evo_util/common_bug.py``) with KRYLOV local exponentials, or a
    solve_ivp mode (``ode_mode``) with ``ode_options``."""
    from pytreenet.time_evolution.time_evolution import TimeEvoMode
    from pytreenet.time_evolution.fixed_bug import FixedBUG, FixedBUGConfig
    psi = build_reference_state(ptn, spec, tensors)
    psi.canonical_form(spec[0][0])
    psi.normalise()
    tensors = export_state(psi, spec)
    psi = build_reference_state(ptn, spec, tensors)
    H = ptn.TTNO.from_hamiltonian(ham_fn(psi), psi)
    ops = {nid: ptn.TensorProduct({nid: Z}) for nid, _ in spec}
    if ode_mode is None:
        algo = FixedBUG(psi, H, dt, dt * steps, ops, config=FixedBUGConfig(time_evo_mode=TimeEvoMode.KRYLOV),
                        solver_options={"krylov_tol": tol})
    else:
        algo = FixedBUG(psi, H, dt, dt * steps, ops, config=FixedBUGConfig(time_evo_mode=TimeEvoMode[ode_mode]),
                        solver_options=None if ode_options is None else dict(ode_options))
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": dt, "steps": steps, "order": 1, "krylov_tol": tol, "bug": 1,
           "update_path": np.array([])}
    if ode_mode is not None:
        rec["time_evo_mode"] = ode_mode
    for k, v in (ode_options or {}).items():
        rec[f"solver_options/{k}"] = v
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in export_ttno(H, spec).items():
        rec[f"ttno/{nid}"] = t
    zs = []
    for step in range(steps):
        algo.run_one_time_step()
        zs.append([algo.state.operator_expectation_value(ops[nid]) for nid, _ in spec])
    rec["z"] = np.array(zs)
    for nid, t in export_state(algo.state, spec).items():
        rec[f"final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "written")


def run_case_adaptive_bug(ptn, name, spec, tensors, ham_fn, dt, steps, tol, svd):
    """The reference's rank-adaptive BUG (``time_evolution/bug.py``): bases
    augmented with the evolved tensors, then ``svd_truncation``. The bond cap
    does not bind, so the truncation keeps every singular value above the
    tolerances and its visiting order (which in the reference follows the
    node dictionary order) cannot change the result beyond them."""
    from pytreenet.time_evolution.time_evolution import TimeEvoMode
    from pytreenet.time_evolution.bug import BUG, BUGConfig
    psi = build_reference_state(ptn, spec, tensors)
    H = ptn.TTNO.from_hamiltonian(ham_fn(psi), psi)
    ops = {nid: ptn.TensorProduct({nid: Z}) for nid, _ in spec}
    maxd, rel, tot = svd
    cfg = BUGConfig(time_evo_mode=TimeEvoMode.KRYLOV, max_bond_dim=maxd, rel_tol=rel, total_tol=tot)
    algo = BUG(psi, H, dt, dt * steps, ops, config=cfg, solver_options={"krylov_tol": tol})
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": dt, "steps": steps, "order": 1, "krylov_tol": tol, "bug": 2,
           "update_path": np.array([]), "svd_max_bond_dim": maxd, "svd_rel_tol": rel, "svd_total_tol": tot,
           "svd_renorm": 0}
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in export_ttno(H, spec).items():
        rec[f"ttno/{nid}"] = t
    zs, bonds = [], []
    for step in range(steps):
        algo.run_one_time_step()
        zs.append([algo.state.operator_expectation_value(ops[nid]) for nid, _ in spec])
        bonds.append([algo.state.tensors[nid].shape[0] for nid, p in spec if p is not None])
    rec["z"] = np.array(zs)
    rec["bonds"] = np.array(bonds)
    for nid, t in export_state(algo.state, spec).items():
        rec[f"final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(name, "written; bonds", bonds[-1])


def bug_cases(ptn):
    rng = np.random.default_rng(31)
    spec = binary_tree(15)
    run_case_bug(ptn, "binary15_tfim_fixed_bug", spec, capped_state_tensors(spec, rng, 8),
                 lambda psi: tfim(ptn, spec, g=0.7), 0.05, 4, 1e-12)
    spec = ternary_tree(2)
    ne = len(spec) - 1
    jxy = rng.uniform(0.5, 1.5, size=ne)
    jz = rng.uniform(0.5, 1.5, size=ne)
    run_case_bug(ptn, "ternary2_xxz_fixed_bug", spec, capped_state_tensors(spec, rng, 4),
                 lambda psi: heisenberg_fields(ptn, spec, rng.uniform(-1, 1, size=len(spec)), jxy, jz),
                 0.05, 3, 1e-12)
    spec = binary_tree(7)
    run_case_adaptive_bug(ptn, "binary7_tfim_bug", spec, capped_state_tensors(spec, rng, 1),
                          lambda psi: tfim(ptn, spec, g=0.8), 0.05, 4, 1e-12, (100, 1e-10, 1e-10))
    spec = ternary_tree(2)
    run_case_adaptive_bug(ptn, "ternary2_xxz_bug", spec, neel_state_tensors(spec),
                          lambda psi: heisenberg_fields(ptn, spec, np.zeros(len(spec)), jxy, jz),
                          0.05, 3, 1e-12, (100, 1e-10, 1e-10))


def leaf_to_leaf_two_site_cases(ptn):
    """Second-order two-site TDVP on the leaf-to-leaf path, bonds growing
    from a Neel state."""
    rng = np.random.default_rng(107)
    spec = binary_tree(7)
    h = rng.uniform(-1, 1, size=len(spec))
    run_case_two_site(ptn, "binary7_heis_2tdvp_l2l", spec, neel_state_tensors(spec),
                      lambda psi: heisenberg_fields(ptn, spec, h), 0.05, 3, 1e-12, (6, 1e-10, 1e-10, False),
                      path_mode="LeafToLeaf")


def leaf_to_leaf_cases(ptn):
    """One-site TDVP on the leaf-to-leaf update path
    (``PathFinderMode.LeafToLeaf``, ``update_path.py:255-396``)."""
    rng = np.random.default_rng(41)
    spec = t_tree(3)
    h = rng.uniform(-1, 1, size=len(spec))
    run_case(ptn, "ttree3_heis_l2l_o1", spec, capped_state_tensors(spec, rng, 6),
             lambda psi: heisenberg_fields(ptn, spec, h), 0.02, 3, 1, 1e-12, canonical_random=True,
             path_mode="LeafToLeaf")
    spec = binary_tree(15)
    run_case(ptn, "binary15_tfim_l2l_o2", spec, capped_state_tensors(spec, rng, 6),
             lambda psi: tfim(ptn, spec, g=0.6), 0.02, 3, 2, 1e-12, canonical_random=True,
             path_mode="LeafToLeaf")


def default_mode_cases(ptn):
    """TDVP with the reference's default configuration (time_evo_mode FASTEST,
    a dense exponential of the effective Hamiltonian)."""
    rng = np.random.default_rng(61)
    spec = t_tree(3)
    h = rng.uniform(-1, 1, size=len(spec))
    run_case(ptn, "ttree3_heis_fastest_o1", spec, capped_state_tensors(spec, rng, 6),
             lambda psi: heisenberg_fields(ptn, spec, h), 0.05, 3, 1, 0.0, canonical_random=True,
             default_mode=True)
    spec = binary_tree(7)
    run_case(ptn, "binary7_tfim_fastest_o2", spec, capped_state_tensors(spec, rng, 4),
             lambda psi: tfim(ptn, spec, g=0.9), 0.05, 3, 2, 0.0, canonical_random=True, default_mode=True)


def ode_cases(ptn):
    """TDVP with the solve_ivp modes of ``TimeEvoMode`` (``time_evolution.py:595-615``):
    RK45 at tight tolerances, DOP853 with no options (solve_ivp's rtol 1e-3,
    atol 1e-6), RK23 at 1e-8."""
    rng = np.random.default_rng(67)
    spec = t_tree(3)
    h = rng.uniform(-1, 1, size=len(spec))
    run_case(ptn, "ttree3_heis_rk45_o1", spec, capped_state_tensors(spec, rng, 6),
             lambda psi: heisenberg_fields(ptn, spec, h), 0.05, 3, 1, 0.0, canonical_random=True,
             ode_mode="RK45", ode_options={"atol": 1e-10, "rtol": 1e-10})
    spec = binary_tree(7)
    run_case(ptn, "binary7_tfim_dop853_o2", spec, capped_state_tensors(spec, rng, 4),
             lambda psi: tfim(ptn, spec, g=0.9), 0.3, 2, 2, 0.0, canonical_random=True, ode_mode="DOP853")
    run_case(ptn, "binary7_tfim_rk23_o1", spec, capped_state_tensors(spec, rng, 4),
             lambda psi: tfim(ptn, spec, g=0.7), 0.04, 2, 1, 0.0, canonical_random=True, ode_mode="RK23",
             ode_options={"atol": 1e-8, "rtol": 1e-8})
    # second-order two-site TDVP with RK45 and bond growth under truncation
    h = rng.uniform(-1, 1, size=len(spec))
    run_case_two_site(ptn, "binary7_heis_2tdvp_rk45", spec, random_state_tensors(spec, rng, 2),
                      lambda psi: heisenberg_fields(ptn, spec, h), 0.05, 2, 0.0, (6, 1e-10, 1e-10, False),
                      canonical_random=True, ode_mode="RK45", ode_options={"atol": 1e-10, "rtol": 1e-10})
    # fixed-rank BUG with RK45: the root and its children at 1e-10, deeper
    # nodes at solve_ivp's own tolerances (the reference passes no options there)
    spec = binary_tree(15)
    run_case_bug(ptn, "binary15_tfim_fixed_bug_rk45", spec, capped_state_tensors(spec, rng, 4),
                 lambda psi: tfim(ptn, spec, g=0.6), 0.1, 2, 0.0, ode_mode="RK45",
                 ode_options={"atol": 1e-10, "rtol": 1e-10})
    # second-order two-site TDVP with the default mode (FASTEST: dense two-site
    # effective Hamiltonians in the reference)
    spec = binary_tree(7)
    h = rng.uniform(-1, 1, size=len(spec))
    run_case_two_site(ptn, "binary7_heis_2tdvp_fastest", spec, random_state_tensors(spec, rng, 2),
                      lambda psi: heisenberg_fields(ptn, spec, h), 0.05, 2, 0.0, (5, 1e-10, 1e-10, False),
                      canonical_random=True, ode_mode="FASTEST")


def from_tensor_cases(ptn):
    """``TTNO.from_tensor`` (``ttno/ttno_class.py:163-298``, QR mode) on a
    4-node tree and a 6-node tree with mixed physical dimensions: the input
    operator tensor, its leg dictionary and the reference's node tensors in
    the reference's node leg order."""
    rng = np.random.default_rng(83)
    rec = {}
    cases = [("t4", [("root", None), ("a", "root"), ("b", "root"), ("c", "a")],
              {"root": 2, "a": 0, "b": 3, "c": 1}, {"root": 2, "a": 2, "b": 2, "c": 2}),
             ("t6", [("r", None), ("x", "r"), ("y", "r"), ("z", "r"), ("u", "y"), ("v", "y")],
              {"r": 5, "x": 0, "y": 1, "z": 4, "u": 2, "v": 3}, {"r": 2, "x": 3, "y": 2, "z": 2, "u": 2, "v": 3})]
    for tag, spec, leg_dict, dims in cases:
        ch = children_of(spec)
        tensors = {}
        for nid, p in spec:
            nv = len(ch[nid]) + (0 if p is None else 1)
            tensors[nid] = np.ones([1] * nv + [dims[nid]], dtype=complex)
        psi = build_reference_state(ptn, spec, tensors)
        out_dims = [0] * len(spec)
        for nid, leg in leg_dict.items():
            out_dims[leg] = dims[nid]
        shape = out_dims + out_dims
        op = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        ttno = ptn.TTNO.from_tensor(psi, op, leg_dict)
        rec[f"{tag}/spec_ids"] = np.array([x[0] for x in spec])
        rec[f"{tag}/spec_parents"] = np.array(["" if x[1] is None else x[1] for x in spec])
        rec[f"{tag}/op"] = op
        for nid, _ in spec:
            rec[f"{tag}/init/{nid}"] = tensors[nid]
            rec[f"{tag}/leg/{nid}"] = leg_dict[nid]
            rec[f"{tag}/ttno/{nid}"] = np.asarray(ttno.tensors[nid])
            rec[f"{tag}/children/{nid}"] = np.array(list(ttno.nodes[nid].children), dtype=str)
    np.savez_compressed(os.path.join(HERE, "ttno_from_tensor.npz"), **rec)
    print("ttno_from_tensor written")


PATH_TREES = {
    "rootleaf7": ("node4", [("node0", "node4", 0), ("node1", "node0", 1), ("node2", "node1", 1),
                            ("node3", "node1", 2), ("node5", "node0", 2), ("node6", "node5", 1)]),
    "chainroot": ("r", [("a", "r", 0), ("b", "a", 1), ("c", "b", 1)]),
    "rootleafT": ("r", [("a", "r", 0), ("b", "a", 1), ("c", "a", 2), ("d", "b", 1), ("e", "c", 1)]),
    "wide": ("r", [("a", "r", 0), ("b", "r", 1), ("c", "r", 2), ("d", "a", 1), ("e", "a", 2), ("f", "c", 1),
                   ("g", "f", 1)]),
}


def path_cases(ptn):
    """Update paths of ``TDVPUpdatePathFinder`` (both modes) on trees built
    with ``add_child_to_parent`` on chosen legs, roots with one child included."""
    from pytreenet.time_evolution.time_evo_util.update_path import TDVPUpdatePathFinder, PathFinderMode
    from pytreenet.core.node import Node as RNode
    rec = {}
    for name, (root, edges) in PATH_TREES.items():
        nch = {root: 0}
        for c, p, _ in edges:
            nch[p] = nch.get(p, 0) + 1
            nch.setdefault(c, 0)

        def ones(n, is_root):
            return np.ones([1] * (nch[n] + (0 if is_root else 1)) + [2], dtype=complex)
        t = ptn.TreeTensorNetworkState()
        t.add_root(RNode(identifier=root), ones(root, True))
        for c, p, leg in edges:
            t.add_child_to_parent(RNode(identifier=c), ones(c, False), 0, p, leg)
        rec[f"{name}/edges"] = np.array([[c, p, str(leg)] for c, p, leg in edges])
        rec[f"{name}/root"] = root
        for mode in ("LeafToRoot", "LeafToLeaf"):
            rec[f"{name}/{mode}"] = np.array(TDVPUpdatePathFinder(t, PathFinderMode[mode]).find_path())
    np.savez_compressed(os.path.join(HERE, "update_paths.npz"), **rec)
    print("update_paths written")


def heff_cases(ptn):
    """Dense effective site Hamiltonians from the reference's
    ``get_effective_single_site_hamiltonian`` (``contractions/effective_hamiltonians.py:133-157``)
    with ``SandwichCache.init_cache_but_one`` environments, on a T-tree state."""
    from pytreenet.contractions.sandwich_caching import SandwichCache
    from pytreenet.contractions.effective_hamiltonians import get_effective_single_site_hamiltonian
    rng = np.random.default_rng(71)
    spec = t_tree(2)
    h = rng.uniform(-1, 1, size=len(spec))
    tensors = random_state_tensors(spec, rng, 3)
    psi = build_reference_state(ptn, spec, tensors)
    H = ptn.TTNO.from_hamiltonian(heisenberg_fields(ptn, spec, h), psi)
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec])}
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in export_ttno(H, spec).items():
        rec[f"ttno/{nid}"] = t
    nodes = ["root", "a0_0", "a1_1"]
    for nid in nodes:
        cache = SandwichCache.init_cache_but_one(psi, H, nid)
        rec[f"heff/{nid}"] = get_effective_single_site_hamiltonian(nid, psi, H, cache)
    rec["heff_nodes"] = np.array(nodes)
    np.savez_compressed(os.path.join(HERE, "ttree2_heis_heff.npz"), **rec)
    print("heff written", {n: rec[f"heff/{n}"].shape for n in nodes})


def exact_cases(ptn):
    """``ExactTimeEvolution`` (``time_evolution/exact_time_evolution.py``) on a
    random 6-site Hermitian H: a closed run (state vector) and an open one (a
    vectorised density matrix under a 64 x 64 generator)."""
    from pytreenet.time_evolution.exact_time_evolution import ExactTimeEvolution, ExactTimeEvolutionConfig
    rng = np.random.default_rng(83)
    n = 64
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    H = (a + a.conj().T) / 4
    psi = rng.normal(size=n) + 1j * rng.normal(size=n)
    psi /= np.linalg.norm(psi)
    ops = [np.diag(rng.normal(size=n)).astype(complex), (lambda b: (b + b.conj().T) / 2)(rng.normal(size=(n, n)) + 0j)]
    rec = {"H": H, "psi": psi, "op0": ops[0], "op1": ops[1], "dt": 0.05, "final": 0.2}
    m = 8
    L = rng.normal(size=(m * m, m * m)) + 1j * rng.normal(size=(m * m, m * m))
    L = (L + L.conj().T) / 8
    rho = np.eye(m, dtype=complex).reshape(-1) / m
    O = np.diag(np.arange(m)).astype(complex)
    ev2 = ExactTimeEvolution(rho, L, 0.05, 0.2, [O], config=ExactTimeEvolutionConfig(open=True))
    for _ in range(4):
        ev2.run_one_time_step()
    rec.update(L=L, rho=rho, O=O, open_final=ev2.evaluate_operator(O))
    ev3 = ExactTimeEvolution(psi, H, 0.05, 0.2, ops)
    vals = []
    for _ in range(4):
        ev3.run_one_time_step()
        vals.append([ev3.evaluate_operator(o) for o in ops])
    rec["closed_values"] = np.array(vals)
    np.savez_compressed(os.path.join(HERE, "exact_evolution.npz"), **rec)
    print("exact written")


def run_results_case(ptn):
    """``run(evaluation_time=2)`` of the reference's two-site TDVP with every
    ``record_*`` flag set (``time_evolution.py:346-368``,
    ``ttn_time_evolution.py:88-211``): the whole Results content is stored."""
    from pytreenet.time_evolution.time_evolution import TimeEvoMode
    from pytreenet.time_evolution.tdvp_algorithms.twositetdvp import TwoSiteTDVPConfig
    rng = np.random.default_rng(97)
    spec = binary_tree(7)
    tensors = neel_state_tensors(spec)
    psi = build_reference_state(ptn, spec, tensors)
    h = rng.uniform(-1, 1, size=len(spec))
    H = ptn.TTNO.from_hamiltonian(heisenberg_fields(ptn, spec, h), psi)
    cfg = TwoSiteTDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV, max_bond_dim=4, rel_tol=1e-10, total_tol=1e-10,
                            record_bond_dim=True, record_max_bdim=True, record_average_bdim=True,
                            record_total_size=True, record_norm=True, record_loschmidt_amplitude=True)
    ops = {"z0": ptn.TensorProduct({"s0": Z}), "x3": ptn.TensorProduct({"s3": X})}
    algo = ptn.SecondOrderTwoSiteTDVP(psi, H, 0.05, 0.05 * 6, ops, config=cfg, solver_options={"krylov_tol": 1e-12})
    algo.run(evaluation_time=2, pgbar=False)
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]), "h": h}
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in export_ttno(H, spec).items():
        rec[f"ttno/{nid}"] = t
    keys = []
    for k, v in algo.results.results.items():
        name = "bond/" + "/".join(k) if isinstance(k, tuple) else str(k)
        rec["res/" + name] = np.asarray(v)
        keys.append(name)
    rec["res_keys"] = np.array(keys)
    np.savez_compressed(os.path.join(HERE, "binary7_heis_2tdvp_results.npz"), **rec)
    print("results written", keys)


def zipup_cases(ptn):
    """The reference's non-canonical zip-up application of a TTNO
    (``ttns/ttns_ttno/zipup.py:22-105``) with a bond cap that binds and with
    tolerances only."""
    from pytreenet.ttns.ttns_ttno.zipup import zipup
    rng = np.random.default_rng(101)
    spec = binary_tree(7)
    tensors = capped_state_tensors(spec, rng, 3)
    psi = build_reference_state(ptn, spec, tensors)
    H = ptn.TTNO.from_hamiltonian(tfim(ptn, spec, g=0.6), psi)
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec])}
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in export_ttno(H, spec).items():
        rec[f"ttno/{nid}"] = t
    for tag, (maxd, tol) in {"cap": (4, 1e-10), "tol": (100, 1e-12)}.items():
        out = zipup(H, build_reference_state(ptn, spec, tensors),
                    svd_params=ptn.SVDParameters(max_bond_dim=maxd, rel_tol=tol, total_tol=tol))
        rec[f"{tag}/params"] = np.array([maxd, tol])
        for nid, t in export_state(out, spec).items():
            rec[f"{tag}/final/{nid}"] = t
    np.savez_compressed(os.path.join(HERE, "binary7_tfim_zipup.npz"), **rec)
    print("zipup written")


def time_dep_cases(ptn):
    rng = np.random.default_rng(77)
    spec = binary_tree(7)
    run_case_time_dep(ptn, "binary7_tfim_driven_o1", spec, random_state_tensors(spec, rng, 3), 0.05, 6, 1, 1e-12)
    run_case_time_dep(ptn, "binary7_tfim_driven_o2", spec, random_state_tensors(spec, rng, 3), 0.05, 5, 2, 1e-12)


def tfim_fields(ptn, spec, J, gs):
    """H = -J sum Z_i Z_j - sum g_i X_i with one field per site."""
    conv = {"mJZ": -J * Z, "Z": Z, "I2": np.eye(2, dtype=complex)}
    terms = [ptn.TensorProduct({nid: "mJZ", p: "Z"}) for nid, p in spec if p is not None]
    for i, (nid, _) in enumerate(spec):
        conv[f"mgX{nid}"] = -gs[i] * X
        terms.append(ptn.TensorProduct({nid: f"mgX{nid}"}))
    return ptn.Hamiltonian(terms, conv)


def config_shape_cases(ptn):
    """The reference on the exact trees and Hamiltonian families of the five
    benchmark configurations, at bond dimensions it runs in seconds (its
    two-site contraction order needs chi^6 w^6 d^2 entries on the ternary tree,
    so chi_max stays at 3 there):

    * c2shape_ternary3_xxz_neel_chi3: ternary depth 3 (40 sites), XXZ with
      per-edge Jxy, Jz ~ U[0.5, 1.5], Neel, second-order two-site TDVP,
      max_bond_dim 3, cutoff 1e-10, dt 0.02, 4 steps;
    * c3shape_ttree20_heis_chi8_o1: T-tree root + 3 x 20 (61 sites),
      Heisenberg + fields h ~ U[-1, 1], capped random state (chi 8),
      canonicalised, first-order one-site TDVP, dt 0.01, 2 sweeps;
    * c4shape_binary31_heis_h2_neel_chi8: 31-site binary tree, Heisenberg +
      fields h ~ U[-2, 2], Neel, second-order two-site TDVP, max_bond_dim 8,
      cutoff 1e-9, dt 0.05, 2 steps;
    * c5shape_binary31_tfim_gi_chi8_o1: 31-site binary TFIM, J = 1,
      g_i ~ U[0.3, 0.7], capped random state (chi 8), canonicalised,
      first-order one-site TDVP, dt 0.02, 5 steps.
    """
    rng = np.random.default_rng(2718)
    spec = ternary_tree(3)
    ne = len(spec) - 1
    jxy = rng.uniform(0.5, 1.5, size=ne)
    jz = rng.uniform(0.5, 1.5, size=ne)
    run_case_two_site(ptn, "c2shape_ternary3_xxz_neel_chi3", spec, neel_state_tensors(spec),
                      lambda psi: heisenberg_fields(ptn, spec, np.zeros(len(spec)), jxy, jz),
                      0.02, 4, 1e-12, (3, 1e-10, 1e-10, False))
    spec = t_tree(20)
    h = rng.uniform(-1, 1, size=len(spec))
    run_case(ptn, "c3shape_ttree20_heis_chi8_o1", spec, capped_state_tensors(spec, rng, 8),
             lambda psi: heisenberg_fields(ptn, spec, h), 0.01, 2, 1, 1e-12, canonical_random=True)
    spec = binary_tree(31)
    h = rng.uniform(-2, 2, size=len(spec))
    run_case_two_site(ptn, "c4shape_binary31_heis_h2_neel_chi8", spec, neel_state_tensors(spec),
                      lambda psi: heisenberg_fields(ptn, spec, h), 0.05, 2, 1e-12, (8, 1e-9, 1e-9, False))
    spec = binary_tree(31)
    gs = rng.uniform(0.3, 0.7, size=len(spec))
    run_case(ptn, "c5shape_binary31_tfim_gi_chi8_o1", spec, capped_state_tensors(spec, rng, 8),
             lambda psi: tfim_fields(ptn, spec, 1.0, gs), 0.02, 5, 1, 1e-12, canonical_random=True)


def main(ref_root):
    ptn = _import_reference(ref_root)
    rng = np.random.default_rng(1234)
    # 15-node binary TFIM, Bloch-sphere product state zero-padded to chi=8, 50 steps.
    spec = binary_tree(15)
    run_case(ptn, "c1_binary15_tfim_chi8", spec, product_state_tensors(spec, rng, 8),
             lambda psi: tfim(ptn, spec), 0.01, 50, 1, 1e-12)
    # Small padded case, second order.
    spec = binary_tree(7)
    run_case(ptn, "binary7_tfim_chi4_o2", spec, product_state_tensors(spec, rng, 4),
             lambda psi: tfim(ptn, spec), 0.02, 8, 2, 1e-12)
    # T-tree, random canonicalised state, Heisenberg + fields (root + three arms, small).
    spec = t_tree(3)
    h = rng.uniform(-1, 1, size=len(spec))
    run_case(ptn, "ttree3_heis_chi6_o1", spec, random_state_tensors(spec, rng, 6),
             lambda psi: heisenberg_fields(ptn, spec, h), 0.01, 4, 1, 1e-12,
             canonical_random=True)
    run_case(ptn, "ttree3_heis_chi6_o2", spec, random_state_tensors(spec, rng, 6),
             lambda psi: heisenberg_fields(ptn, spec, h), 0.01, 3, 2, 1e-12,
             canonical_random=True)
    # Ternary depth 2, XXZ with random couplings, random chi=4 state.
    spec = ternary_tree(2)
    ne = len(spec) - 1
    jxy = rng.uniform(0.5, 1.5, size=ne)
    jz = rng.uniform(0.5, 1.5, size=ne)
    run_case(ptn, "ternary2_xxz_chi4_o1", spec, random_state_tensors(spec, rng, 4),
             lambda psi: heisenberg_fields(ptn, spec, np.zeros(len(spec)), jxy, jz),
             0.02, 4, 1, 1e-12, canonical_random=True)
    # Two-site TDVP (second order): ternary depth 2 from a Neel product state
    # (bond dimensions grow from 1), and a random binary tree truncated by
    # max_bond_dim with renormalisation.
    spec = ternary_tree(2)
    ne = len(spec) - 1
    jxy = rng.uniform(0.5, 1.5, size=ne)
    jz = rng.uniform(0.5, 1.5, size=ne)
    run_case_two_site(ptn, "ternary2_xxz_neel_2tdvp", spec, neel_state_tensors(spec),
                      lambda psi: heisenberg_fields(ptn, spec, np.zeros(len(spec)), jxy, jz),
                      0.02, 6, 1e-12, (8, 1e-10, 1e-10, False))
    spec = binary_tree(7)
    h = rng.uniform(-1, 1, size=len(spec))
    run_case_two_site(ptn, "binary7_heis_2tdvp_trunc", spec, random_state_tensors(spec, rng, 4),
                      lambda psi: heisenberg_fields(ptn, spec, h), 0.05, 3, 1e-12,
                      (3, 1e-10, 1e-10, True), canonical_random=True)
    # TEBD on the 7-node binary tree (random chi=3 state, truncation to 4)
    spec = binary_tree(7)
    run_case_tebd(ptn, "binary7_tfim_tebd", spec, random_state_tensors(spec, rng, 3), 0.05, 4,
                  (4, 1e-10, 1e-10, False))
    unit_cases(ptn)
    time_dep_cases(ptn)
    saved_files(ptn)
    bug_cases(ptn)
    leaf_to_leaf_cases(ptn)
    tebd_swap_cases(ptn)
    default_mode_cases(ptn)
    heff_cases(ptn)
    exact_cases(ptn)
    run_results_case(ptn)
    zipup_cases(ptn)
    leaf_to_leaf_two_site_cases(ptn)
    ode_cases(ptn)
    from_tensor_cases(ptn)
    path_cases(ptn)


if __name__ == "__main__":
    # python make_golden.py REF_ROOT [group ...]: all fixtures, or only the
    # named generator groups (e.g. config_shape_cases)
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    if len(sys.argv) > 2:
        mod = _import_reference(ref)
        for group in sys.argv[2:]:
            globals()[group](mod)
    else:
        main(ref)
