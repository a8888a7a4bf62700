"""Run one node's effective-Hamiltonian matvec repeatedly (for profilers).

    python -m pytreenet_gb300.profile_matvec [--chi 128] [--arm 2] [--node root]
                                             [--precision mixed] [--reps 3]

Builds the T-tree workload (root + 3 arms, Heisenberg + fields), puts it in
canonical form, builds the environments around ``--node`` and applies that
node's matvec ``--reps`` times, printing the time per application.
"""
from __future__ import annotations

import argparse
import time

import torch

from .engine import DeviceNetwork
from .workloads import t_tree_heisenberg, t_tree_state


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--chi", type=int, default=128)
    ap.add_argument("--arm", type=int, default=2)
    ap.add_argument("--node", default="root")
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    st, _, _ = t_tree_state(arm_len=a.arm, chi=a.chi, seed=0)
    H, _ = t_tree_heisenberg(st, seed=1)
    net = DeviceNetwork(st, H, precision=a.precision)
    net.canonical_form(a.node)
    net.normalise_center()
    net.init_cache_but_one(a.node)
    x = net.t[a.node].clone()
    y = torch.zeros_like(x)
    plan = net.heff_plan(a.node)
    plan.run(x.data_ptr(), y.data_ptr())
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("matvec")
    t0 = time.perf_counter()
    for _ in range(a.reps):
        plan.run(x.data_ptr(), y.data_ptr())
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    dt = (time.perf_counter() - t0) / a.reps
    print(f"{a.node} matvec chi={a.chi} {a.precision}: {dt * 1e3:.3f} ms, "
          f"{plan.flops / dt / 1e12:.1f} TFLOP/s algorithmic")


if __name__ == "__main__":
    main()
