"""Fixtures at sizes the reference cannot run, generated by the CPU oracle.

    python tests/golden/make_oracle_fixtures.py [name ...]

PyTreeNet's two-site TDVP contracts every environment of a merged pair before
its TTNO tensors; on the depth-3 ternary tree at max_bond_dim 16 that
intermediate is ~1e10 complex entries, so the reference cannot produce these
outputs. The oracle (oracle/ptn_oracle.py, pinned on the reference's own runs
of the depth-2 ternary tree and the binary trees in tests/test_oracle_golden.py)
produces them instead; the file layout is that of make_golden.py, plus the
bond-dimension history of the two-site splits.

c2_ternary3_xxz_neel_chi16: second-order two-site TDVP on the ternary tree of
depth 3 (40 sites), XXZ with per-edge Jxy, Jz ~ U[0.5, 1.5] (seed 7), Neel
product state by depth parity, max_bond_dim 16, rel_tol = total_tol = 1e-10,
dt = 0.02, 10 steps, Krylov tolerance 1e-12.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

Z = np.diag([1.0, -1.0]).astype(complex)


def c2_ternary3_xxz_neel_chi16(steps=10, chi=16, tol=1e-12):
    import oracle as O
    from pytreenet_gb300.workloads import ternary_neel_state, ternary_xxz
    st, spec, tensors = ternary_neel_state(depth=3)
    H, W = ternary_xxz(st, seed=7)
    W = {k: np.asarray(v) for k, v in W.items()}
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    params = O.SVDParams(max_bond_dim=chi, rel_tol=1e-10, total_tol=1e-10)
    algo = O.SecondOrderTwoSiteTDVPOracle(O.OState(tree, tensors), W, 0.02, params, krylov_tol=tol)
    rec = {"spec_ids": np.array([s[0] for s in spec]),
           "spec_parents": np.array(["" if s[1] is None else s[1] for s in spec]),
           "dt": 0.02, "steps": steps, "order": 2, "krylov_tol": tol, "two_site": 1,
           "svd_max_bond_dim": chi, "svd_rel_tol": 1e-10, "svd_total_tol": 1e-10, "svd_renorm": 0,
           "update_path": np.array(algo.update_path)}
    for nid, t in tensors.items():
        rec[f"init/{nid}"] = t
    for nid, t in W.items():
        rec[f"ttno/{nid}"] = t
    zs = []
    for k in range(steps):
        t0 = time.time()
        algo.run_one_time_step()
        zs.append([O.expect_product(algo.state, {nid: Z}) for nid, _ in spec])
        print(f"step {k}: {time.time() - t0:.1f} s, bonds so far {len(algo.bond_history)}", flush=True)
    rec["z"] = np.array(zs)
    rec["bond_history"] = np.array(algo.bond_history)
    for nid in algo.state.tensors:
        rec[f"final/{nid}"] = algo.state.tensors[nid]
    return rec


CASES = {"c2_ternary3_xxz_neel_chi16": c2_ternary3_xxz_neel_chi16}

if __name__ == "__main__":
    for name in (sys.argv[1:] or list(CASES)):
        rec = CASES[name]()
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        print(name, "written")
