"""Per-operation time of one TDVP time step (CUDA-synchronised wall time).

    python -m pytreenet_gb300.profile_sweep [--chi 256] [--arm 20] [--precision mixed]
    python -m pytreenet_gb300.profile_sweep --workload ternary [--chi 64]

ttree: one-site TDVP on the T-tree; ternary: second-order two-site TDVP on the
depth-3 ternary tree (XXZ) starting at the saturated bond dimensions with
max_bond_dim = chi. Runs two warm steps (plans built, QR graphs captured),
then one step in which every site update, two-site update, SVD split, link
update, QR split, environment update and absorption is bracketed by device
synchronisations and timed; prints the totals per operation and node class.
"""
from __future__ import annotations

import argparse
import time
from collections import defaultdict

import torch

from . import engine as E
from .tdvp import (FirstOrderOneSiteTDVP, SecondOrderTwoSiteTDVP, TDVPConfig, TimeEvoMode,
                   TwoSiteTDVPConfig)
from .workloads import t_tree_heisenberg, t_tree_state, ternary_saturated_state, ternary_xxz


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--chi", type=int, default=256)
    ap.add_argument("--arm", type=int, default=20)
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--workload", default="ttree", choices=["ttree", "ternary"])
    a = ap.parse_args()
    acc, cnt = defaultdict(float), defaultdict(int)
    if a.workload == "ttree":
        st, _, _ = t_tree_state(arm_len=a.arm, chi=a.chi, seed=0)
        H, _ = t_tree_heisenberg(st, seed=1)
        algo = FirstOrderOneSiteTDVP(st, H, 0.01, 1.0, {}, config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV),
                                     solver_options={"krylov_tol": 1e-10}, precision=a.precision)
        last = f"_{a.arm - 1}"

        def cls(nid):
            return "root" if nid == "root" else ("leaf" if nid.endswith(last) else "arm")
    else:
        st, spec, _ = ternary_saturated_state(depth=3, chi=a.chi, seed=0)
        H, _ = ternary_xxz(st, seed=7)
        cfg = TwoSiteTDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV, max_bond_dim=a.chi, rel_tol=1e-10,
                                total_tol=1e-10)
        algo = SecondOrderTwoSiteTDVP(st, H, 0.02, 1.0, {}, config=cfg, solver_options={"krylov_tol": 1e-10},
                                      precision=a.precision)
        depth = {}
        for nid, p in spec:
            depth[nid] = 0 if p is None else depth[p] + 1

        def cls(nid):
            return f"depth{depth[nid]}"
    algo.net.normalise_center()

    def wrap(name, key):
        orig = getattr(E.DeviceNetwork, name)

        def timed(self, *args, **kw):
            torch.cuda.synchronize()
            t = time.perf_counter()
            r = orig(self, *args, **kw)
            torch.cuda.synchronize()
            k = f"{name}:{key(*args)}"
            acc[k] += time.perf_counter() - t
            cnt[k] += 1
            return r
        setattr(E.DeviceNetwork, name, timed)
    wrap("evolve_site", lambda nid, *r: cls(nid))
    wrap("evolve_bond", lambda r, nid, *x: cls(nid))
    wrap("update_env", lambda nid, *x: cls(nid))
    wrap("qr_split", lambda nid, *x: cls(nid))
    wrap("absorb", lambda R, src, dst, *x: cls(dst))
    wrap("evolve_two_site", lambda u, v, *x: cls(u) + "-" + cls(v))
    wrap("svd_split", lambda u, v, *x: cls(u) + "-" + cls(v))
    wrap("merge_plan", lambda u, v, *x: cls(u) + "-" + cls(v))
    wrap("_subspace_factor", lambda *x: "")
    wrap("_jacobi", lambda src, m, n, *x: f"{m}x{n}")
    algo.run_one_time_step()
    algo.run_one_time_step()
    acc.clear()
    cnt.clear()
    torch.cuda.synchronize()
    t = time.perf_counter()
    algo.run_one_time_step()
    torch.cuda.synchronize()
    total = time.perf_counter() - t
    print(f"step {total * 1e3:.1f} ms ({a.workload}, chi={a.chi}, {a.precision})")
    for k in sorted(acc, key=lambda k: -acc[k]):
        print(f"{k:24s} {acc[k] * 1e3:9.1f} ms  {100 * acc[k] / total:5.1f} %  n={cnt[k]:4d}  "
              f"{acc[k] * 1e3 / max(cnt[k], 1):8.3f} ms each")


if __name__ == "__main__":
    main()
