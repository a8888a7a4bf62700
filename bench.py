"""Benchmark: one-site TDVP sweeps/sec on the T-tree at chi=256 (GB300 engine).

Workload (seeded, synthetic): root + 3 arms of 20 sites (61 sites, d=2),
Heisenberg couplings + random fields h_i ~ U[-1, 1] (TTNO bond 5), Gaussian
complex TTNS at chi=256 on every bond, canonicalised and normalised; first-order
one-site TDVP, dt=0.01, Krylov exponential with krylov_tol=1e-10. One step =
one sweep (run_one_time_step). Inputs are larger than L2 (the root tensor alone
is 537 MB in complex128), so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--chi 256] [--arm 20]

Multi-GPU: replicas only (a sweep is sequential); each rank advances its own
realisation and ``value`` is the sum of sweeps over ranks / max time.
The reference arm (--impl reference) times the NumPy oracle (the reference's
algorithm restated; PyTreeNet itself is a Python package that cannot run at
chi=256 -- its contraction order needs a 67 GB intermediate) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

def metric_name(args) -> str:
    return (f"TDVP sweeps/sec at chi={args.chi} (one-site, {3 * args.arm + 1}-site T-tree, "
            "Heisenberg+fields)")
FP64_NOMINAL_TFLOPS = 1.25


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--chi", type=int, default=256)
    ap.add_argument("--arm", type=int, default=20)
    ap.add_argument("--dt", type=float, default=0.01)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "plain"])
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison sweep")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch the QR sequences eagerly instead of replaying CUDA graphs")
    ap.add_argument("--workload", default="ttree", choices=["ttree", "ternary", "disorder", "gradient"],
                    help="ttree: one-site TDVP on the T-tree (headline); ternary: second-order "
                         "two-site TDVP on the depth-3 ternary tree (40 sites, XXZ) with truncation; "
                         "disorder: many independent random-field realisations (binary tree, 31 sites); "
                         "gradient: d<Z_root>/d(g_i, J) after 30 one-site TDVP steps by the adjoint "
                         "(binary tree, 31 sites, TFIM)")
    ap.add_argument("--fd-params", type=int, default=3,
                    help="gradient: parameters checked against central differences of the driver")
    ap.add_argument("--realisations", type=int, default=32, help="disorder: number of realisations")
    ap.add_argument("--workers", type=int, default=8, help="disorder: concurrent worker streams")
    ap.add_argument("--chi-max", type=int, default=64, help="ternary: max_bond_dim of the SVD split")
    return ap.parse_args()


def config(args, precision):
    return {"workload": f"T-tree root+3x{args.arm} ({3 * args.arm + 1} sites), chi={args.chi}, d=2, "
                        f"TTNO bond 5, Heisenberg+fields, first-order 1TDVP, dt={args.dt}, "
                        f"krylov_tol={args.tol}",
            "precision": precision, "l2": "inputs larger than L2 (root tensor > 129 MB); no flush",
            "parallelism": "replicas"}


# ----------------------------------------------------------------------------
# CPU baseline: the NumPy oracle on a bounded sample, extrapolated to a sweep
# ----------------------------------------------------------------------------
def oracle_schedule_counts(arm, tol, dt):
    """Operation counts of one sweep, from a dry run of the oracle driver at chi=8
    (the schedule and Krylov depths do not depend on chi in any material way)."""
    import oracle as O
    import oracle.ptn_oracle as OP
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg, t_tree_spec
    st, spec, tensors = t_tree_state(arm_len=arm, chi=8, seed=0)
    H, W = t_tree_heisenberg(st, seed=1)
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    counts = {}
    deg = {nid: len(tree.neighbours(nid)) for nid, _ in spec}

    def wrap(name, fn, key):
        def w(*a, **k):
            nid = key(*a)
            counts[(name, deg[nid])] = counts.get((name, deg[nid]), 0) + 1
            return fn(*a, **k)
        return w
    saved = (OP.heff_apply, OP.env_update, OP.qr_keep_split)
    OP.heff_apply = wrap("heff", OP.heff_apply, lambda x, tree, nid, *r: nid)
    OP.env_update = wrap("env", OP.env_update, lambda tree, nid, *r: nid)
    OP.qr_keep_split = wrap("qr", OP.qr_keep_split, lambda state, nid, *r: nid)
    try:
        algo = O.FirstOrderOneSiteTDVPOracle(O.OState(tree, tensors), W, dt, krylov_tol=tol)
        c0 = algo.state.orth_center
        algo.state.tensors[c0] = algo.state.tensors[c0] / np.linalg.norm(algo.state.tensors[c0])
        counts.clear()
        algo.run_one_time_step()
    finally:
        OP.heff_apply, OP.env_update, OP.qr_keep_split = saved
    return counts


def oracle_op_times(chi, reps=1):
    """Seconds per oracle operation at this chi, by node degree (bounded sample)."""
    import oracle as O
    rng = np.random.default_rng(0)
    w, d = 5, 2

    def c(*s):
        return (rng.standard_normal(s) + 1j * rng.standard_normal(s)) / np.sqrt(2)
    times = {}
    for degn in (1, 2, 3):
        tree = O.OTree()
        tree.add_root("v")
        for i in range(degn):
            tree.add_child(f"u{i}", "v")
        shape = [chi] * degn + [d]
        x = c(*shape)
        W = c(*([w] * degn + [d, d]))
        envs = {(f"u{i}", "v"): c(chi, w, chi) for i in range(degn)}
        t0 = time.perf_counter()
        for _ in range(reps):
            O.heff_apply(x, tree, "v", W, envs)
        times[("heff", degn)] = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            O.env_update(tree, "v", "u0", x, W, envs)
        times[("env", degn)] = (time.perf_counter() - t0) / reps
        mat = x.reshape(-1, chi)
        t0 = time.perf_counter()
        for _ in range(reps):
            np.linalg.qr(mat)
        times[("qr", degn)] = (time.perf_counter() - t0) / reps
    return times


def cpu_sweeps_per_s(args):
    t0 = time.perf_counter()
    counts = oracle_schedule_counts(args.arm, args.tol, args.dt)
    times = oracle_op_times(args.chi)
    sweep = sum(n * times.get(k, 0.0) for k, n in counts.items())
    wall = time.perf_counter() - t0
    return 1.0 / sweep, {"counts": {f"{a}/deg{b}": n for (a, b), n in sorted(counts.items())},
                         "sample_seconds": round(wall, 2)}


def cpu_baseline_obj(args):
    v, info = cpu_sweeps_per_s(args)
    return {"value": v, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": (f"NumPy oracle (OpenBLAS, all host threads): one heff matvec, env update and QR per "
                       f"node degree at chi={args.chi}, weighted by the operation counts of one oracle sweep "
                       f"(from a chi=8 dry run); {info['sample_seconds']} s of CPU work"),
            "detail": info}


# ----------------------------------------------------------------------------
# clocks
# ----------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------
# replicas: whole-job rate over ranks
# ----------------------------------------------------------------------------
def aggregate_over_ranks(local_ms: float, steps: int, world: int, dist=None, device=None):
    """Rate of N independent replicas (a TDVP sweep does not shard): every rank
    advanced ``steps`` sweeps of its own realisation; the job took as long as
    the slowest rank (all-reduce MAX). Returns (sweeps/s over all ranks, max ms)."""
    import torch
    t_max = float(local_ms)
    if dist is not None and world > 1:
        t = torch.tensor([t_max], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    return world * steps / (t_max / 1000.0), t_max


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def run_gb300(args, rank, world):
    import torch
    import pytreenet_gb300 as P
    from pytreenet_gb300 import _lib
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    dist = None
    if world > 1:
        import torch.distributed as dist
    lib = _lib.load()
    def make(precision):
        st, spec, _ = t_tree_state(arm_len=args.arm, chi=args.chi, seed=rank)
        H, _ = t_tree_heisenberg(st, seed=1000 + rank)
        total = args.warmup + 2 * args.steps + 1
        a = P.FirstOrderOneSiteTDVP(st, H, args.dt, args.dt * total, {},
                                    config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                    solver_options={"krylov_tol": args.tol}, precision=precision)
        a.net.normalise_center()
        return a
    algo = make(args.precision)
    net = algo.net
    net.use_graphs = not args.no_graphs
    for _ in range(args.warmup):
        algo.run_one_time_step()
    torch.cuda.synchronize()

    # -- timed region: K sweeps, device-resident ---------------------------------
    heff_events = []
    orig = net.evolve_site

    def timed_evolve(nid, *a, **k):
        p = net.heff_plan(nid)
        run = p.run

        def run_timed(xp=0, yp=0):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            run(xp, yp)
            e1.record()
            heff_events.append((e0, e1, p.flops))
        p.run = run_timed
        try:
            return orig(nid, *a, **k)
        finally:
            p.run = run
    net.evolve_site = timed_evolve
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = lib.ptn_launch_counter() + net.graph_launches
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(torch.cuda.current_device()) as clk:
        torch.cuda.nvtx.range_push("timed_region")
        start.record()
        for _ in range(args.steps):
            algo.run_one_time_step()
        stop.record()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    if dist:
        dist.barrier()
    launches = int(lib.ptn_launch_counter() + net.graph_launches - l0)
    net.evolve_site = orig
    ms = start.elapsed_time(stop)
    heff_ms = sum(a.elapsed_time(b) for a, b, _ in heff_events)
    heff_flops = sum(f for _, _, f in heff_events)
    n_heff = len(heff_events)
    value, t_max = aggregate_over_ranks(ms, args.steps, world, dist, "cuda")

    # -- end to end: state uploaded from pinned host memory, sweep, state read back
    e2e = None
    if not args.no_e2e:
        pinned = {nid: torch.empty(net.t[nid].shape, dtype=net.t[nid].dtype, pin_memory=True)
                  for nid in net.t}
        for nid, t in net.t.items():
            pinned[nid].copy_(t)
        nbytes = sum(t.numel() * t.element_size() for t in net.t.values())
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            for nid, t in net.t.items():
                t.copy_(pinned[nid], non_blocking=True)
            algo.run_one_time_step()
            for nid, t in net.t.items():
                pinned[nid].copy_(t, non_blocking=True)
            torch.cuda.synchronize()
        w1 = time.perf_counter()
        e2e_value, _ = aggregate_over_ranks((w1 - w0) * 1000.0, args.steps, world, dist, "cuda")
        e2e = {"value": e2e_value, "unit": "sweeps/s",
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes}

    achieved = heff_flops / (heff_ms / 1000.0) / 1e12 if heff_ms > 0 else None
    if args.precision == "mixed":
        peak, peak_src = _measured_bf16_peak()
        # algorithmic complex flops (8 per complex MAC); the BF16x3 split issues 3x that on the pipe
        roof = {"bound": "tensor", "kernel": "ptn_cgemm_bf16x3 (heff matvec chain, tcgen05, 3 split levels)",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if achieved else None,
                "peak_source": peak_src + "; achieved counts algorithmic complex flops, the BF16x6 "
                               "split issues 6x as many tensor flops",
                "traffic": None}
    else:
        roof = {"bound": "tensor", "kernel": "ptn_zcontract (heff matvec chain, FP64)",
                "achieved": achieved, "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                "frac": (achieved / FP64_NOMINAL_TFLOPS) if achieved else None,
                "peak_source": "nominal GB300 FP64 (1.25 TFLOP/s); FP64 is not in MEASURED_PEAKS.json",
                "traffic": None}
    roof.update({
            "algorithmic_flops_per_matvec": heff_flops / max(n_heff, 1),
            "matvecs_timed": n_heff, "matvec_ms_total": heff_ms, "share_of_step": heff_ms / ms})
    plain = None
    if args.precision == "mixed" and not args.no_plain and rank == 0:
        plain = compare_with_plain(args, make)
        plain["speedup_mixed_over_plain"] = value / plain["sweeps_per_s"]
    line = {"metric": metric_name(args), "value": value, "unit": "sweeps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x6 split (tcgen05, fp32 accumulate) contractions / f64 Krylov+QR" if args.precision == "mixed" else "c128 (fp64)",
            "data": "synthetic",
            "config": config(args, "mixed: BF16x6 (3-level split) tcgen05 contractions, FP32 accumulate, FP64 Krylov/QR/norm"
                             if args.precision == "mixed" else "plain complex128"),
            "roofline": roof, "e2e": e2e, "plain_fp64": plain,
            "gpu_launches": launches, "clocks": clk.summary(),
            "krylov_depth_mean": float(np.mean(net.krylov.depths[-n_heff:])) if n_heff else None}
    return line


def _measured_bf16_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS), of measured"
    except Exception:
        return 1900.0, "fallback 1.9 PFLOP/s bf16 (MEASURED_PEAKS.json absent), of fallback"


def compare_with_plain(args, make):
    """One sweep on the plain complex128 path from the same initial state as one
    sweep on the mixed path: plain sweep time and the fidelity error of the
    mixed result (1 - |<mixed|plain>| / (|mixed| |plain|))."""
    import torch
    a_m = make("mixed")
    a_m.run_one_time_step()
    a_p = make("plain")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    a_p.run_one_time_step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ov = a_m.net.overlap(a_p.net)
    nm = a_m.net.overlap(a_m.net).real
    npl = a_p.net.overlap(a_p.net).real
    err = 1.0 - abs(ov) / np.sqrt(nm * npl)
    t = args.dt
    return {"sweeps_per_s": 1000.0 / ms, "ms_per_sweep": ms, "fidelity_error_one_sweep": err,
            "fidelity_error_per_unit_time": err / t, "sweeps_compared": 1}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    samples = []
    for i in range(args.warmup + args.steps):
        v, info = cpu_sweeps_per_s(args)
        if i >= args.warmup:
            samples.append(1.0 / v)
    v = 1.0 / float(np.mean(samples))
    cb = {"value": v, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
          "sample": (f"NumPy oracle restatement of the reference algorithm; each step times one heff "
                     f"matvec, env update and QR per node degree at chi={args.chi} and weights them by "
                     f"one sweep's operation counts")}
    return {"metric": metric_name(args), "value": v, "unit": "sweeps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128 (fp64)", "data": "synthetic",
            "config": config(args, "plain complex128 (CPU)"), "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_two_site(args):
    """Second-order two-site TDVP on the depth-3 ternary tree (40 sites), XXZ with
    per-edge couplings U[0.5, 1.5], truncation max_bond_dim=chi_max with
    rel_tol = total_tol = 1e-10, dt = 0.02. The state starts at the bond
    dimensions such a run saturates at (random, canonicalised, normalised), so
    every step does full-size work. One step = run_one_time_step (forward and
    backward sweep)."""
    import torch
    import pytreenet_gb300 as P
    from pytreenet_gb300 import _lib
    from pytreenet_gb300.workloads import ternary_saturated_state, ternary_xxz
    lib = _lib.load()

    def make(precision):
        st, spec, _ = ternary_saturated_state(depth=3, chi=args.chi_max, seed=0)
        H, _ = ternary_xxz(st, seed=7)
        cfg = P.TwoSiteTDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV, max_bond_dim=args.chi_max,
                                  rel_tol=1e-10, total_tol=1e-10)
        a = P.SecondOrderTwoSiteTDVP(st, H, 0.02, 0.02 * 1000, {}, config=cfg,
                                     solver_options={"krylov_tol": args.tol}, precision=precision)
        a.net.normalise_center()
        return a
    algo = make(args.precision)
    for _ in range(args.warmup):
        algo.run_one_time_step()
    torch.cuda.synchronize()
    l0 = lib.ptn_launch_counter() + algo.net.graph_launches
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(torch.cuda.current_device()) as clk:
        start.record()
        for _ in range(args.steps):
            algo.run_one_time_step()
        stop.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    launches = int(lib.ptn_launch_counter() + algo.net.graph_launches - l0)
    bonds = sorted({int(x) for x in algo.bond_dims_history[-20:]})
    return {"metric": f"two-site TDVP steps/sec (ternary depth 3, 40 sites, XXZ, chi_max={args.chi_max})",
            "value": args.steps / (ms / 1000.0), "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x6 split contractions / f64 Krylov+QR+SVD" if args.precision == "mixed" else "c128 (fp64)",
            "data": "synthetic",
            "config": {"workload": "ternary depth 3 (40 sites), XXZ Jxy,Jz~U[0.5,1.5], second-order 2TDVP, "
                                   f"dt=0.02, max_bond_dim={args.chi_max}, rel_tol=total_tol=1e-10, "
                                   f"krylov_tol={args.tol}", "precision": args.precision,
                       "start": "random state at the saturated bond dimensions"},
            "gpu_launches": launches, "clocks": clk.summary(), "recent_bond_dims": bonds,
            "krylov_depth_mean": float(np.mean(algo.net.krylov.depths)) if algo.net.krylov.depths else None}


def run_disorder(args):
    """Independent realisations of second-order two-site TDVP on the 31-site
    binary tree (Heisenberg + random fields h_i ~ U[-2, 2], Neel start),
    max_bond_dim cycling through 8, 16, 32, 64 over the realisations,
    cutoff 1e-9, dt = 0.05; ``--steps`` time steps each (one step = a forward
    and a backward sweep). Runs them one worker at a time, then with
    ``--workers`` concurrent streams, and reports realisation-steps/s."""
    import torch
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import binary_neel_random_field
    caps = [8, 16, 32, 64]

    def make(i):
        st, H, _, _, _ = binary_neel_random_field(n=31, seed=i)
        cfg = P.TwoSiteTDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV, max_bond_dim=caps[i % len(caps)],
                                  rel_tol=1e-9, total_tol=1e-9)
        return P.SecondOrderTwoSiteTDVP(st, H, 0.05, 100.0, {}, config=cfg, solver_options={"krylov_tol": 1e-10},
                                        precision=args.precision)
    out = {}
    for w in (1, args.workers):
        P.run_realisations(make, min(w, args.realisations), 1, workers=w)      # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        P.run_realisations(make, args.realisations, args.steps, workers=w)
        torch.cuda.synchronize()
        out[w] = args.realisations * args.steps / (time.perf_counter() - t0)
    return {"metric": "two-site TDVP realisation-steps/sec (31-site binary tree, random fields, chi_max 8..64)",
            "value": out[args.workers], "unit": "realisation-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x6 split contractions / f64 Krylov+QR+SVD" if args.precision == "mixed" else "c128 (fp64)",
            "data": "synthetic",
            "config": {"workload": f"{args.realisations} realisations x 31-site binary tree, Heisenberg + "
                                   "h_i~U[-2,2], Neel start, second-order 2TDVP, dt=0.05, cutoff 1e-9, "
                                   "max_bond_dim 8/16/32/64", "workers": args.workers,
                       "timing": "wall clock over all realisations, includes building each driver"},
            "one_worker": out[1], "speedup_over_one_worker": out[args.workers] / out[1]}


def run_gradient(args):
    """Gradient of <Z_root>(T) after 30 first-order one-site TDVP steps (dt=0.02)
    with respect to the 31 transverse fields g_i ~ U[0.3, 0.7] and J = 1 on the
    31-site binary tree, bonds min(chi, subtree dimensions), random state scaled
    to unit norm, complex128. One step
    = one gradient evaluation (forward sweep, checkpointed backward sweep).
    Also times one forward evolution through the driver and checks
    ``--fd-params`` components against central differences (step 1e-5)."""
    import torch
    from pytreenet_gb300 import _lib
    from pytreenet_gb300.adjoint import OneSiteTDVPAdjoint, coupling_gradient
    from pytreenet_gb300.operators import tfim_ttno
    from pytreenet_gb300.tdvp import FirstOrderOneSiteTDVP, TDVPConfig, TimeEvoMode, TensorProduct
    from pytreenet_gb300.workloads import binary_tfim_random_state
    lib = _lib.load()
    chi, nsteps, dt, tol = args.chi, 30, 0.02, args.tol
    st, spec, tensors, g, J = binary_tfim_random_state(n=31, chi=chi, seed=0)
    theta = np.array([g[nid] for nid, _ in spec] + [J])
    ops = {"s0": np.diag([1.0, -1.0]).astype(complex)}

    def ham(th):
        return tfim_ttno(st, J=float(th[-1]), g={nid: float(th[i]) for i, (nid, _) in enumerate(spec)})
    adj = OneSiteTDVPAdjoint(st, ham(theta), dt, nsteps, krylov_tol=tol, normalise=True)
    for _ in range(args.warmup):
        coupling_gradient(adj, ham, theta, ops)
    torch.cuda.synchronize()
    l0 = lib.ptn_launch_counter()
    t0 = time.perf_counter()
    with Clocks(torch.cuda.current_device()) as clk:
        for _ in range(args.steps):
            val, grad = coupling_gradient(adj, ham, theta, ops)
        torch.cuda.synchronize()
    sec = (time.perf_counter() - t0) / args.steps
    launches = int(lib.ptn_launch_counter() - l0) // args.steps

    def run(th_):
        s = st.copy_structure()
        s._phys = {k: np.array(v, copy=True) for k, v in tensors.items()}
        algo = FirstOrderOneSiteTDVP(s, ham(th_), dt, dt * nsteps, {},
                                     config=TDVPConfig(time_evo_mode=TimeEvoMode.KRYLOV),
                                     solver_options={"krylov_tol": tol})
        algo.net.normalise_center()
        for _ in range(nsteps):
            algo.run_one_time_step()
        return float(np.real(algo.evaluate_operator(TensorProduct(ops))))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    v0 = run(theta)
    torch.cuda.synchronize()
    fwd = time.perf_counter() - t1
    idx = [0, theta.size - 1, theta.size - 2][:max(0, args.fd_params)]
    h = 1e-5
    fd = {j: (run(theta + h * np.eye(theta.size)[j]) - run(theta - h * np.eye(theta.size)[j])) / (2 * h) for j in idx}
    err = max((abs(grad[j] - fd[j]) for j in idx), default=None)
    return {"metric": "gradient evaluations/sec (d<Z_root>/d(g_1..g_31, J), 30 one-site TDVP steps, "
                      f"31-site binary tree, chi={chi})",
            "value": 1.0 / sec, "unit": "gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * sec, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128 (fp64)", "data": "synthetic",
            "config": {"workload": f"binary tree 31 sites, TFIM g_i~U[0.3,0.7], J=1, chi={chi} (bonds capped at the "
                                   f"subtree dimensions), first-order 1TDVP, dt={dt}, {nsteps} steps, "
                                   f"krylov_tol={tol}", "timing": "wall clock per gradient, forward + backward"},
            "gpu_launches": launches, "clocks": clk.summary(), "value_Z_root": val,
            "forward_seconds": fwd, "central_difference_seconds_estimate": 2 * theta.size * fwd,
            "forward_matches_driver": abs(v0 - val),
            "fd_check": {"params": idx, "adjoint": [float(grad[j]) for j in idx], "central": [fd[j] for j in idx],
                         "max_abs_err": err, "grad_norm": float(np.linalg.norm(grad))}}


def main():
    args = parse()
    if args.workload == "gradient":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        if args.chi == 256:
            args.chi = 64
        print(json.dumps(run_gradient(args)), flush=True)
        return
    if args.workload == "disorder":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        print(json.dumps(run_disorder(args)), flush=True)
        return
    if args.workload == "ternary":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        print(json.dumps(run_two_site(args)), flush=True)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    line = run_gb300(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_obj(args)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
