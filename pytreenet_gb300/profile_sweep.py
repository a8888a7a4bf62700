"""Per-operation time of one one-site TDVP sweep (CUDA-synchronised wall time).

    python -m pytreenet_gb300.profile_sweep [--chi 256] [--arm 20] [--precision mixed]

Builds the T-tree workload, runs two warm sweeps (plans built, QR graphs
captured), then one sweep in which every site update, link update, QR split,
environment update and absorption is bracketed by device synchronisations and
timed; prints the totals per operation and node class (root / arm / leaf).
"""
from __future__ import annotations

import argparse
import time
from collections import defaultdict

import torch

from . import engine as E
from .tdvp import FirstOrderOneSiteTDVP, TDVPConfig, TimeEvoMode
from .workloads import t_tree_heisenberg, t_tree_state


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--chi", type=int, default=256)
    ap.add_argument("--arm", type=int, default=20)
    ap.add_argument("--precision", default="mixed")
    a = ap.parse_args()
    st, _, _ = t_tree_state(arm_len=a.arm, chi=a.chi, seed=0)
    H, _ = t_tree_heisenberg(st, seed=1)
    algo = FirstOrderOneSiteTDVP(st, H, 0.01, 1.0, {}, config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV),
                                 solver_options={"krylov_tol": 1e-10}, precision=a.precision)
    algo.net.normalise_center()
    last = f"_{a.arm - 1}"
    acc, cnt = defaultdict(float), defaultdict(int)

    def cls(nid):
        return "root" if nid == "root" else ("leaf" if nid.endswith(last) else "arm")

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
    algo.run_one_time_step()
    algo.run_one_time_step()
    acc.clear()
    cnt.clear()
    torch.cuda.synchronize()
    t = time.perf_counter()
    algo.run_one_time_step()
    torch.cuda.synchronize()
    total = time.perf_counter() - t
    print(f"sweep {total * 1e3:.1f} ms (chi={a.chi}, arm={a.arm}, {a.precision})")
    for k in sorted(acc, key=lambda k: -acc[k]):
        print(f"{k:24s} {acc[k] * 1e3:9.1f} ms  {100 * acc[k] / total:5.1f} %  n={cnt[k]:4d}  "
              f"{acc[k] * 1e3 / max(cnt[k], 1):8.3f} ms each")


if __name__ == "__main__":
    main()
