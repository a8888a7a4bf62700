"""Benchmark: one-site TDVP sweeps/sec on the T-tree at chi=256 (GB300 engine).

Workload (seeded, synthetic): root + 3 arms of 20 sites (61 sites, d=2),
Heisenberg couplings + random fields h_i ~ U[-1, 1] (TTNO bond 5), Gaussian
complex TTNS at chi=256 on every bond, canonicalised and normalised; first-order
one-site TDVP, dt=0.01, Krylov exponential with krylov_tol=1e-10. One step =
one sweep (run_one_time_step). Inputs are larger than L2 (the root tensor alone
is 537 MB in complex128), so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--chi 256] [--arm 20] [--precision mixed|plain]
  python bench.py --breakdown            # time per engine operation of one sweep
  python bench.py --fidelity-sweeps 20   # mixed vs plain complex128 over 20 sweeps
  python bench.py --impl reference --full-sweep   # one complete CPU oracle sweep
  python bench.py --workload c1|ternary|disorder|gradient   # the other configurations
  python bench.py --workload matvec --arm 2   # root H_eff matvec + Gram-Schmidt step (ncu target)

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
    ap.add_argument("--breakdown", action="store_true",
                    help="time every engine operation of one sweep (synchronised) instead of the bench")
    ap.add_argument("--fidelity-sweeps", type=int, default=0,
                    help="run this many sweeps on the mixed and the plain path from one state and "
                         "report fidelity and energy error after each")
    ap.add_argument("--full-sweep", action="store_true",
                    help="reference arm: time one complete oracle sweep and compare the per-operation model")
    ap.add_argument("--entries", type=int, default=1 << 24, help="gram_schmidt: vector length")
    ap.add_argument("--qr-m", type=int, default=512, help="qr: rows")
    ap.add_argument("--qr-k", type=int, default=256, help="qr: columns")
    ap.add_argument("--workload", default="ttree",
                    choices=["ttree", "c1", "qr", "ternary", "disorder", "gradient", "matvec", "gram_schmidt"],
                    help="ttree: one-site TDVP on the T-tree (headline); c1: one-site TDVP on the "
                         "15-node binary tree with <Z_i> at every site each step; ternary: second-order "
                         "two-site TDVP on the depth-3 ternary tree (40 sites, XXZ) with truncation; "
                         "disorder: many independent random-field realisations (binary tree, 31 sites); "
                         "gradient: d<Z_root>/d(g_i, J) after 30 one-site TDVP steps by the adjoint "
                         "(binary tree, 31 sites, TFIM)")
    ap.add_argument("--fd-params", type=int, default=3,
                    help="gradient: parameters checked against central differences of the driver")
    ap.add_argument("--realisations", type=int, default=32, help="disorder: number of realisations")
    ap.add_argument("--workers", type=int, default=8, help="disorder: concurrent worker streams")
    ap.add_argument("--processes", type=int, default=8, help="disorder: worker processes on the GPU")
    ap.add_argument("--chi-max", type=int, default=64, help="ternary: max_bond_dim of the SVD split")
    return ap.parse_args()


def config(args, precision):
    return {"workload": f"T-tree root+3x{args.arm} ({3 * args.arm + 1} sites), chi={args.chi}, d=2, "
                        f"TTNO bond 5, Heisenberg+fields, first-order 1TDVP, dt={args.dt}, "
                        f"krylov_tol={args.tol}",
            "precision": precision, "l2": "inputs larger than L2 (root tensor > 129 MB); no flush",
            "parallelism": "replicas"}


# ----------------------------------------------------------------------------
# CPU baseline: the NumPy oracle, per-operation model of one sweep
# ----------------------------------------------------------------------------
# Operation classes of one oracle sweep: H_eff matvecs, environment updates, QR
# splits and R absorptions by node degree, bond matvecs, and the Krylov vector
# work (Gram-Schmidt step) by vector length. Counted in a dry run of the oracle
# driver at chi=8 (the schedule and the Krylov depths do not depend on chi in
# any material way), timed at the bench's chi.
def oracle_schedule_counts(arm, tol, dt, chi=8, seconds=None, seed=0):
    """Operation counts of one oracle sweep (a dry run at ``chi``). With a dict
    ``seconds``, also the wall time spent in each operation class (the Krylov
    class "gs" then holds the whole exponential minus its matvecs)."""
    import oracle as O
    import oracle.ptn_oracle as OP
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    st, spec, tensors = t_tree_state(arm_len=arm, chi=chi, seed=seed)
    H, W = t_tree_heisenberg(st, seed=1 if seconds is None else 1000)
    tree = O.OTree()
    for nid, p in spec:
        tree.add_root(nid) if p is None else tree.add_child(nid, p)
    counts = {}
    deg = {nid: len(tree.neighbours(nid)) for nid, _ in spec}

    def bump(key):
        counts[key] = counts.get(key, 0) + 1

    def wrap(fn, key):
        def w(*a, **k):
            kk = key(*a)
            bump(kk)
            if seconds is None:
                return fn(*a, **k)
            t0 = time.perf_counter()
            try:
                return fn(*a, **k)
            finally:
                seconds[kk] = seconds.get(kk, 0.0) + time.perf_counter() - t0
        return w
    saved = (OP.heff_apply, OP.env_update, OP.qr_keep_split, OP.bond_apply, OP.absorb_r, OP.krylov_exp_action)
    OP.heff_apply = wrap(OP.heff_apply, lambda x, tree, nid, *r: ("heff", deg[nid]))
    OP.env_update = wrap(OP.env_update, lambda tree, nid, *r: ("env", deg[nid]))
    OP.qr_keep_split = wrap(OP.qr_keep_split, lambda state, nid, *r: ("qr", deg[nid]))
    OP.bond_apply = wrap(OP.bond_apply, lambda *r: ("bond", 0))
    OP.absorb_r = wrap(OP.absorb_r, lambda state, r, src, dst, *x: ("absorb", deg[dst]))
    orig_kry = OP.krylov_exp_action

    def kry(psi, action, *a, stats=None, **k):
        # one Gram-Schmidt step per matvec; keyed by the vector's node class
        n = psi.size
        cls = 0 if psi.ndim == 2 and psi.shape[0] == psi.shape[1] and psi.shape[0] > 2 else psi.ndim - 1
        local = []
        if seconds is not None:
            inner = sum(seconds.values())
            t0 = time.perf_counter()
        out = orig_kry(psi, action, *a, stats=local, **k)
        if seconds is not None:
            own = time.perf_counter() - t0 - (sum(seconds.values()) - inner)
            seconds[("gs", cls)] = seconds.get(("gs", cls), 0.0) + own
        for m in local:
            counts[("gs", cls)] = counts.get(("gs", cls), 0) + int(m)
        if stats is not None:
            stats.extend(local)
        return out
    OP.krylov_exp_action = kry
    try:
        algo = O.FirstOrderOneSiteTDVPOracle(O.OState(tree, tensors), W, dt, krylov_tol=tol)
        c0 = algo.state.orth_center
        algo.state.tensors[c0] = algo.state.tensors[c0] / np.linalg.norm(algo.state.tensors[c0])
        counts.clear()
        if seconds is not None:
            seconds.clear()
            t0 = time.perf_counter()
        algo.run_one_time_step()
        if seconds is not None:
            seconds["sweep"] = time.perf_counter() - t0
            seconds["krylov_depth_mean"] = float(np.mean(algo.krylov_dims)) if algo.krylov_dims else None
    finally:
        (OP.heff_apply, OP.env_update, OP.qr_keep_split, OP.bond_apply, OP.absorb_r,
         OP.krylov_exp_action) = saved
    return counts


# classes timed in one sample: node degree 1, 2, 3, and the bond (0)
OP_CLASSES = (1, 2, 3, 0)

# The per-operation model checked against one complete oracle sweep at the
# headline size (chi=256, arms of 20) on a Grace host with 16 Arm cores
# (``bench.py --impl reference --full-sweep``): recorded figures.
MODEL_CHECK = {"command": "python bench.py --impl reference --full-sweep",
               "full_sweep_seconds": 153.80, "model_seconds": 148.39, "model_error_relative": -0.0352,
               "cores": 16, "host": "Grace (aarch64)"}

# The mixed path against the plain complex128 path over the 20 sweeps of the
# headline workload (``bench.py --fidelity-sweeps 20``, one GB300): recorded
# figures. The default run compares one sweep; 20 plain sweeps take ~11 min.
FIDELITY_20_SWEEPS = {"command": "python bench.py --fidelity-sweeps 20", "sweeps_compared": 20, "t": 0.2,
                      "fidelity_error": 2.318e-09, "fidelity_error_per_unit_time": 1.159e-08,
                      "fidelity_error_at_sweeps_1_10_17_20": [6.99e-12, 6.15e-10, 1.69e-09, 2.318e-09],
                      "energy_error": 5.70e-06, "energy_error_relative": 1.96e-05}


def oracle_op_times(chi, classes=OP_CLASSES, depth=4):
    """Seconds per oracle operation at this chi for the given classes (one
    timing each). ``gs`` is one Gram-Schmidt step of the oracle's Krylov
    loop (norms, two passes over ``depth`` basis vectors: the mean over the
    steps of a solve of depth ~7) at that vector length."""
    import oracle as O
    import oracle.ptn_oracle as OP
    rng = np.random.default_rng(0)
    w, d = 5, 2

    def c(*s):
        return (rng.standard_normal(s) + 1j * rng.standard_normal(s)) / np.sqrt(2)

    def timed(fn, *a):
        t0 = time.perf_counter()
        fn(*a)
        return time.perf_counter() - t0

    def gs_step(n):
        Q = [c(n) for _ in range(depth)]
        wv = c(n)

        def run():
            x = wv
            np.linalg.norm(x)
            for _ in range(2):
                for q in Q:
                    h = np.vdot(q, x)
                    x = x - h * q
            np.linalg.norm(x)
        return timed(run)
    times = {}
    for degn in classes:
        if degn == 0:
            r, eq, en = c(chi, chi), c(chi, w, chi), c(chi, w, chi)
            times[("bond", 0)] = timed(OP.bond_apply, r, eq, en)
            times[("gs", 0)] = gs_step(chi * chi)
            continue
        tree = O.OTree()
        tree.add_root("v")
        for i in range(degn):
            tree.add_child(f"u{i}", "v")
        shape = [chi] * degn + [d]
        x = c(*shape)
        W = c(*([w] * degn + [d, d]))
        envs = {(f"u{i}", "v"): c(chi, w, chi) for i in range(degn)}
        times[("heff", degn)] = timed(O.heff_apply, x, tree, "v", W, envs)
        times[("env", degn)] = timed(O.env_update, tree, "v", "u0", x, W, envs)
        state = O.OState(tree, {"v": x.copy(), **{f"u{i}": c(chi, d) for i in range(degn)}})
        times[("qr", degn)] = timed(OP.qr_keep_split, state, "v", "u0")
        times[("absorb", degn)] = timed(OP.absorb_r, state, c(chi, chi), "u0", "v", True)
        times[("gs", degn)] = gs_step(x.size)
    return times


def model_sweep_seconds(counts, times):
    missing = sorted({k for k in counts if k not in times})
    if missing:
        raise KeyError(f"no timing for {missing}")
    return sum(n * times[k] for k, n in counts.items())


def cpu_baseline_obj(args):
    t0 = time.perf_counter()
    counts = oracle_schedule_counts(args.arm, args.tol, args.dt)
    times = oracle_op_times(args.chi)
    sweep = model_sweep_seconds(counts, times)
    wall = time.perf_counter() - t0
    return {"value": 1.0 / sweep, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": (f"NumPy oracle (OpenBLAS, all host threads): one H_eff matvec, environment update, "
                       f"QR split and R absorption per node degree, one bond matvec and one Gram-Schmidt "
                       f"step per vector length, at chi={args.chi}, weighted by the operation counts of "
                       f"one oracle sweep (chi=8 dry run); {wall:.1f} s of CPU work"),
            "detail": {"counts": {f"{a}/{b}": n for (a, b), n in sorted(counts.items())},
                       "seconds_each": {f"{a}/{b}": t for (a, b), t in sorted(times.items())}}}


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
def _make_ttree(args, precision, seed, steps_total):
    import pytreenet_gb300 as P
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    st, spec, _ = t_tree_state(arm_len=args.arm, chi=args.chi, seed=seed)
    H, _ = t_tree_heisenberg(st, seed=1000 + seed)
    a = P.FirstOrderOneSiteTDVP(st, H, args.dt, args.dt * steps_total, {},
                                config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                solver_options={"krylov_tol": args.tol}, precision=precision)
    a.net.normalise_center()
    a.net.use_graphs = not args.no_graphs
    return a, H


def _measured_peak(kind: str):
    """Roofline denominator from MEASURED_PEAKS.json. The heff chain is timed
    inside a sweep of about a second, so the sustained tensor figure applies."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        if kind == "tensor":
            return float(d["bf16_tflops_sustained"]), "MEASURED_PEAKS.json bf16_tflops_sustained (cuBLAS, of measured)"
        return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (copy, of measured)"
    except Exception:
        if kind == "tensor":
            return 1700.0, "fallback 1.7 PFLOP/s bf16 sustained (MEASURED_PEAKS.json absent), of fallback"
        return 6800.0, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent), of fallback"


# DRAM bytes per root matvec at chi=256 of its three tensor-core steps (E0, E1,
# E2: dram__bytes_read.sum + dram__bytes_write.sum from one ncu capture,
# profiles/cgemm_bf16x6_root_matvec_chi256.md); the W step and the operand
# conversions are not included.
ROOT_MATVEC_DRAM_BYTES = 17.60e9


def run_gb300(args, rank, world):
    import torch
    from pytreenet_gb300 import _lib
    dist = None
    if world > 1:
        import torch.distributed as dist
    lib = _lib.load()
    total = args.warmup + 2 * args.steps + 1
    algo, H = _make_ttree(args, args.precision, rank, total)
    net = algo.net
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
            heff_events.append((e0, e1, p.flops, nid))
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
    c0 = (net.cholqr_count, net.householder_count, net.qr_rows_skipped, len(net.krylov.depths))
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
    heff_ms = sum(a.elapsed_time(b) for a, b, _, _ in heff_events)
    heff_flops = sum(f for _, _, f, _ in heff_events)
    root_ev = [(a.elapsed_time(b), f) for a, b, f, nid in heff_events if nid == "root"]
    n_heff = len(heff_events)
    value, t_max = aggregate_over_ranks(ms, args.steps, world, dist, "cuda")
    qr_stats = {"cholqr2_splits": (net.cholqr_count - c0[0]) / args.steps,
                "householder_splits": (net.householder_count - c0[1]) / args.steps,
                "zero_rows_skipped": (net.qr_rows_skipped - c0[2]) / args.steps,
                "cholqr2_rejected_keys": len(net.cholqr_fails), "per": "sweep"}
    depths = net.krylov.depths[c0[3]:]

    # -- end to end through the public API: every sweep the caller's state goes
    # up from host memory (TTNS.tensors[node] = array, written into the running
    # driver's device buffers) and comes back (TTNS.tensors[node] -> NumPy)
    e2e = None
    if not args.no_e2e:
        st = algo.state
        host = {nid: np.array(st.tensors[nid]) for nid in st._order}
        nbytes = sum(a.nbytes for a in host.values())
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            for nid, a in host.items():
                st.tensors[nid] = a
            algo.run_one_time_step()
            host = {nid: st.tensors[nid] for nid in st._order}
        torch.cuda.synchronize()
        w1 = time.perf_counter()
        e2e_value, _ = aggregate_over_ranks((w1 - w0) * 1000.0, args.steps, world, dist, "cuda")
        e2e = {"value": e2e_value, "unit": "sweeps/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "how": "TTNS.tensors[node] = host array before each sweep, TTNS.tensors[node] after it "
                      "(run_one_time_step on the public driver)"}

    achieved = heff_flops / (heff_ms / 1000.0) / 1e12 if heff_ms > 0 else None
    if args.precision == "mixed":
        peak, peak_src = _measured_peak("tensor")
        roof = {"bound": "tensor", "kernel": "H_eff matvec chain: cgemm_bf16_kernel<3> (tcgen05, BF16x6) + "
                                             "operand conversions",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if achieved else None,
                "peak_source": peak_src + "; achieved counts algorithmic complex flops (8 per complex MAC); "
                               "the BF16x6 split issues 6x as many tensor flops",
                "traffic": ROOT_MATVEC_DRAM_BYTES if args.chi == 256 else None,
                "traffic_scope": "DRAM bytes of the three tensor-core steps of one root matvec at chi=256 "
                                 "(ncu, one capture); achieved is per matvec as well"}
    else:
        roof = {"bound": "tensor", "kernel": "H_eff matvec chain: zcontract_kernel (FP64)",
                "achieved": achieved, "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                "frac": (achieved / FP64_NOMINAL_TFLOPS) if achieved else None,
                "peak_source": "nominal GB300 FP64 (1.25 TFLOP/s); FP64 is not in MEASURED_PEAKS.json",
                "traffic": None}
    roof.update({
        "algorithmic_flops_per_matvec": heff_flops / max(n_heff, 1),
        "matvecs_timed": n_heff, "matvec_ms_total": heff_ms, "share_of_step": heff_ms / ms})
    if root_ev:
        rt = sum(t for t, _ in root_ev)
        roof["root_matvec"] = {"count": len(root_ev), "ms_each": rt / len(root_ev),
                               "tflops_algorithmic": sum(f for _, f in root_ev) / (rt / 1000.0) / 1e12}
    plain = None
    if args.precision == "mixed" and not args.no_plain and rank == 0:
        plain = compare_with_plain(args, 1)
        plain["speedup_mixed_over_plain"] = value / plain["sweeps_per_s"]
        plain["recorded_20_sweeps"] = FIDELITY_20_SWEEPS if (args.chi == 256 and args.arm == 20) else None
    line = {"metric": metric_name(args), "value": value, "unit": "sweeps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x6 split (tcgen05, fp32 accumulate) contractions / f64 Krylov+QR" if args.precision == "mixed" else "c128 (fp64)",
            "data": "synthetic",
            "config": config(args, "mixed: BF16x6 (3-level split) tcgen05 contractions, FP32 accumulate, FP64 Krylov; "
                                   "CholeskyQR2 (tensor-core Gram, FP32 device Cholesky) for full-rank splits, "
                                   "FP64 Householder otherwise"
                             if args.precision == "mixed" else "plain complex128"),
            "roofline": roof, "e2e": e2e, "plain_fp64": plain, "qr": qr_stats,
            "gpu_launches": launches, "clocks": clk.summary(),
            "krylov_depth_mean": float(np.mean(depths)) if depths else None}
    return line


def compare_with_plain(args, sweeps: int):
    """``sweeps`` sweeps on the plain complex128 path and on the mixed path
    from the same initial state: plain sweep time, the fidelity error
    1 - |<mixed|plain>| / (|mixed| |plain|) after each sweep, and (last sweep)
    the energy <H> of both states evaluated in complex128."""
    import torch
    a_m, H = _make_ttree(args, "mixed", 0, sweeps + 2)
    a_p, _ = _make_ttree(args, "plain", 0, sweeps + 2)
    hist = []
    ms_p = 0.0
    for i in range(sweeps):
        a_m.run_one_time_step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a_p.run_one_time_step()
        e1.record()
        torch.cuda.synchronize()
        ms_p += e0.elapsed_time(e1)
        ov = a_m.net.overlap(a_p.net)
        nm = a_m.net.overlap(a_m.net).real
        npl = a_p.net.overlap(a_p.net).real
        hist.append(float(1.0 - abs(ov) / np.sqrt(nm * npl)))
    e_m = a_m.net.expect_ttno(H).real / a_m.net.overlap(a_m.net).real
    e_p = a_p.net.expect_ttno(H).real / a_p.net.overlap(a_p.net).real
    t = args.dt * sweeps
    return {"sweeps_per_s": 1000.0 * sweeps / ms_p, "ms_per_sweep": ms_p / sweeps,
            "sweeps_compared": sweeps, "fidelity_error": hist[-1], "fidelity_error_history": hist,
            "fidelity_error_per_unit_time": hist[-1] / t, "energy_mixed": e_m, "energy_plain": e_p,
            "energy_error": abs(e_m - e_p), "energy_error_relative": abs(e_m - e_p) / abs(e_p),
            "reference": "the plain complex128 GPU path (FP64 contractions, Householder QR), "
                         "from the same initial state"}


def run_breakdown(args):
    """Time of every engine operation of one sweep, each bracketed by device
    synchronisations (two warm sweeps first: plans built, QR graphs captured)."""
    import torch
    from collections import defaultdict
    from pytreenet_gb300 import engine as E
    acc, cnt = defaultdict(float), defaultdict(int)
    algo, _ = _make_ttree(args, args.precision, 0, 10)
    last = f"_{args.arm - 1}"

    def cls(nid):
        return "root" if nid == "root" else ("leaf" if nid.endswith(last) else "arm")
    saved = {}

    def wrap(name, key):
        orig = getattr(E.DeviceNetwork, name)
        saved[name] = orig

        def timed(self, *a, **kw):
            k = f"{name}:{key(*a)}"
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push(k)      # ncu --nvtx-include "<name>:<class>/" selects one class
            t = time.perf_counter()
            r = orig(self, *a, **kw)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
            acc[k] += time.perf_counter() - t
            cnt[k] += 1
            return r
        setattr(E.DeviceNetwork, name, timed)
    wrap("evolve_site", lambda nid, *r: cls(nid))
    wrap("evolve_bond", lambda r, nid, *x: cls(nid))
    wrap("update_env", lambda nid, *x: cls(nid))
    wrap("qr_split", lambda nid, *x: cls(nid))
    wrap("absorb", lambda R, src, dst, *x: cls(dst))
    try:
        for _ in range(2):
            algo.run_one_time_step()
        acc.clear()
        cnt.clear()
        torch.cuda.synchronize()
        t = time.perf_counter()
        algo.run_one_time_step()
        torch.cuda.synchronize()
        total = time.perf_counter() - t
    finally:
        for name, orig in saved.items():
            setattr(E.DeviceNetwork, name, orig)
    rows = {k: {"ms": acc[k] * 1e3, "share": acc[k] / total, "calls": cnt[k],
                "ms_each": acc[k] * 1e3 / max(cnt[k], 1)} for k in sorted(acc, key=lambda k: -acc[k])}
    for k, r in rows.items():
        print(f"{k:24s} {r['ms']:9.1f} ms  {100 * r['share']:5.1f} %  n={r['calls']:4d}  {r['ms_each']:8.3f} ms each",
              file=sys.stderr)
    return {"metric": "per-operation time of one sweep (synchronised)", "workload": config(args, args.precision),
            "sweep_ms": total * 1e3, "operations": rows,
            "qr": {"cholqr2": algo.net.cholqr_count, "householder": algo.net.householder_count}}


def run_reference(args, rank, world):
    """The reference arm: the NumPy oracle's per-operation model of one sweep
    (see oracle_op_times), each step re-timing one operation class in turn
    (degree 1, 2, 3 nodes, the bond) so the run ends in minutes; the warm-up
    steps time every class once."""
    if rank != 0:
        return None
    counts = oracle_schedule_counts(args.arm, args.tol, args.dt)
    times = {}
    samples = []
    timed_wall = 0.0
    for i in range(args.warmup + args.steps):
        classes = OP_CLASSES if i == 0 else (OP_CLASSES[i % len(OP_CLASSES)],)
        t0 = time.perf_counter()
        times.update(oracle_op_times(args.chi, classes))
        if i >= args.warmup:
            timed_wall += time.perf_counter() - t0
            samples.append(model_sweep_seconds(counts, times))
    v = 1.0 / float(np.mean(samples))
    cb = {"value": v, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
          "sample": (f"NumPy oracle restatement of the reference algorithm, all host threads: per-operation "
                     f"model of one sweep at chi={args.chi} (H_eff matvecs, environment updates, QR splits, R "
                     f"absorptions, bond matvecs, Gram-Schmidt steps, weighted by one oracle sweep's counts); "
                     f"each step re-times one operation class")}
    return {"metric": metric_name(args), "value": v, "unit": "sweeps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128 (fp64)", "data": "synthetic",
            "config": config(args, "plain complex128 (CPU)"), "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "timing": {"ms_per_step": "modelled time of one complete sweep (not wall time of this run)",
                       "sampled_wall_seconds": timed_wall,
                       "model_check": MODEL_CHECK if args.chi == 256 and args.arm == 20 else None}}


def run_reference_full_sweep(args):
    """One complete sweep of the NumPy oracle at the bench's config (canonical
    form and initial environments untimed), with the time of every operation
    class, beside the per-operation model's prediction for the same sweep
    (counts from the chi=8 dry run times the isolated timings)."""
    seconds = {}
    full_counts = oracle_schedule_counts(args.arm, args.tol, args.dt, chi=args.chi, seconds=seconds)
    sweep = seconds.pop("sweep")
    depth = seconds.pop("krylov_depth_mean")
    counts = oracle_schedule_counts(args.arm, args.tol, args.dt)
    times = oracle_op_times(args.chi)
    model = model_sweep_seconds(counts, times)
    per_class = {}
    for key in sorted(set(full_counts) | set(counts), key=str):
        per_class[f"{key[0]}/{key[1]}"] = {
            "measured_s": seconds.get(key, 0.0), "count": full_counts.get(key, 0),
            "model_s": counts.get(key, 0) * times.get(key, 0.0), "model_count": counts.get(key, 0)}
    return {"metric": metric_name(args) + " -- one complete oracle sweep", "value": 1.0 / sweep,
            "unit": "sweeps/s", "seconds": sweep, "model_seconds": model,
            "model_error_relative": (model - sweep) / sweep, "cores": os.cpu_count(),
            "seconds_in_classes": sum(v for v in seconds.values()), "per_class": per_class,
            "krylov_depth_mean": depth, "impl": "reference", "config": config(args, "plain complex128 (CPU)")}


def run_fidelity(args):
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    r = compare_with_plain(args, args.fidelity_sweeps)
    r.update({"metric": f"mixed vs plain complex128 over {args.fidelity_sweeps} sweeps",
              "config": config(args, "mixed (BF16x6) vs plain (complex128)")})
    return r


def run_matvec(args):
    """The root's H_eff matvec of the T-tree at --chi (arms of --arm sites,
    canonical form, environments toward the root), and the Gram-Schmidt step
    of the Krylov loop on vectors of the root's size: achieved algorithmic
    TFLOP/s of the matvec (8 flop per complex MAC), achieved GB/s of the
    Gram-Schmidt kernels ((3 nq + 5) vector passes of 16 bytes per entry:
    three passes over w and nq basis vectors, two of them writing w). The
    target of the ncu captures in profiles/."""
    import torch
    from pytreenet_gb300 import _lib
    from pytreenet_gb300.engine import DeviceNetwork, _stream_ptr
    from pytreenet_gb300.workloads import t_tree_state, t_tree_heisenberg
    lib = _lib.load()
    st, spec, _ = t_tree_state(arm_len=args.arm, chi=args.chi, seed=0)
    H, _ = t_tree_heisenberg(st, seed=1000)
    net = DeviceNetwork(st, H, precision=args.precision)
    net.canonical_form("root")
    net.normalise_center()
    net.init_cache_but_one("root")
    p = net.heff_plan("root")
    x = net.t["root"]
    y = torch.empty_like(x)
    reps = max(args.steps, 1)

    def timed(fn, n):
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n
    torch.cuda.nvtx.range_push("matvec")
    ms = net._held(p, lambda: timed(lambda: p.run(x.data_ptr(), y.data_ptr()), reps))
    torch.cuda.nvtx.range_pop()
    n = x.numel()
    gs = {}
    torch.cuda.nvtx.range_push("gram_schmidt")
    for nq in (4, 8):
        Q = torch.randn((nq, n), dtype=torch.complex128, device="cuda")
        w = torch.randn(n, dtype=torch.complex128, device="cuda")
        h = torch.zeros(2 * nq + 8, dtype=torch.complex128, device="cuda")
        part = torch.zeros(int(lib.ptn_krylov_partials(n)) * (nq + 2) + 64, dtype=torch.complex128, device="cuda")
        norms = torch.zeros(4, dtype=torch.float64, device="cuda")

        def step():
            lib.ptn_krylov_gs_step(Q.data_ptr(), n, nq, w.data_ptr(), n, h.data_ptr(), part.data_ptr(),
                                   norms.data_ptr(), None, _stream_ptr())
        t = timed(step, reps)
        nbytes = (3 * nq + 5) * n * 16
        gs[nq] = {"ms": t, "bytes": nbytes, "GB_s": nbytes / (t / 1000.0) / 1e9}
        del Q, w
    torch.cuda.nvtx.range_pop()
    peak_t, src_t = _measured_peak("tensor")
    peak_h, src_h = _measured_peak("hbm")
    tf = p.flops / (ms / 1000.0) / 1e12
    return {"metric": f"root H_eff matvec and Gram-Schmidt step at chi={args.chi}", "precision": args.precision,
            "matvec_ms": ms, "matvec_algorithmic_flops": p.flops, "matvec_tflops": tf,
            "matvec_frac_of_bf16_sustained": tf / peak_t, "peak_tensor_source": src_t,
            "gram_schmidt": {str(k): dict(v, frac_of_hbm=v["GB_s"] / peak_h) for k, v in gs.items()},
            "peak_hbm_source": src_h, "vector_entries": n}


def run_gram_schmidt(args):
    """The Gram-Schmidt step of the Krylov loop (ptn_krylov_gs_step: |w|, two
    passes of h = Q^H w, w -= Q h, |w|) on --entries complex128 entries with
    nq = 4 and 8 basis vectors: achieved GB/s against MEASURED_PEAKS.json
    hbm_gbs, algorithmic bytes (3 nq + 5) x entries x 16 per step."""
    import torch
    from pytreenet_gb300 import _lib
    from pytreenet_gb300.engine import _stream_ptr
    lib = _lib.load()
    n = args.entries
    peak_h, src_h = _measured_peak("hbm")
    out = {}
    for nq in (4, 8):
        Q = torch.randn((nq, n), dtype=torch.complex128, device="cuda")
        w = torch.randn(n, dtype=torch.complex128, device="cuda")
        h = torch.zeros(2 * nq + 8, dtype=torch.complex128, device="cuda")
        part = torch.zeros(int(lib.ptn_krylov_partials(n)) * (nq + 2) + 64, dtype=torch.complex128, device="cuda")
        norms = torch.zeros(4, dtype=torch.float64, device="cuda")

        def step():
            lib.ptn_krylov_gs_step(Q.data_ptr(), n, nq, w.data_ptr(), n, h.data_ptr(), part.data_ptr(),
                                   norms.data_ptr(), None, _stream_ptr())
        for _ in range(max(args.warmup, 1)):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(max(args.steps, 1)):
            step()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / max(args.steps, 1)
        nbytes = (3 * nq + 5) * n * 16
        out[str(nq)] = {"ms": ms, "bytes": nbytes, "GB_s": nbytes / (ms / 1000.0) / 1e9,
                        "frac_of_hbm": nbytes / (ms / 1000.0) / 1e9 / peak_h}
        del Q, w
    return {"metric": f"Gram-Schmidt step GB/s ({n} complex128 entries per vector)", "results": out,
            "peak_source": src_h, "kernels": "gs_pass_kernel (3 passes) + partial-sum finish in the last CTA"}


def run_qr(args):
    """One Householder QR (LAPACK conventions, Q kept in place) of a seeded
    random --qr-m x --qr-k complex128 matrix, the shape of the T-tree arm split
    by default (512 x 256): the one-launch kernel (ptn_zqr_keep) and the launch
    sequence (ptn_zqr_keep_steps), each timed with CUDA events around the call
    only (the input is restored before each call), and the FP64 work
    8 (m k^2 - k^3 / 3) flops of the factorisation plus as much for forming Q."""
    import torch
    from pytreenet_gb300 import _lib
    from pytreenet_gb300.engine import _stream_ptr
    lib = _lib.load()
    m, k = args.qr_m, args.qr_k
    g = torch.Generator().manual_seed(0)
    A0 = torch.complex(torch.randn(m * k, generator=g, dtype=torch.float64),
                       torch.randn(m * k, generator=g, dtype=torch.float64)).cuda()
    A = torch.empty_like(A0)
    rowoff = torch.arange(m, dtype=torch.int64, device="cuda")
    R = torch.zeros(k * k, dtype=torch.complex128, device="cuda")
    work = torch.zeros((int(lib.ptn_zqr_work_bytes(m, k)) + 15) // 16, dtype=torch.complex128, device="cuda")
    out, res = {}, {}
    for name, fn in (("one_launch", lib.ptn_zqr_keep), ("launch_sequence", lib.ptn_zqr_keep_steps)):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(max(args.steps, 1))]
        for i in range(max(args.warmup, 1) + len(ev)):
            A.copy_(A0)
            if i >= max(args.warmup, 1):
                ev[i - max(args.warmup, 1)][0].record()
            st = fn(A.data_ptr(), rowoff.data_ptr(), m, k, m, R.data_ptr(), work.data_ptr(), _stream_ptr())
            if st != 0:
                raise RuntimeError(f"QR status {st}")
            if i >= max(args.warmup, 1):
                ev[i - max(args.warmup, 1)][1].record()
        torch.cuda.synchronize()
        ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        out[name] = {"ms": ms}
        res[name] = (A.clone(), R.clone())
    flops = 2 * 8 * (m * k * k - k ** 3 / 3)
    return {"metric": f"Householder QR ms ({m} x {k} complex128, Q kept)", "results": out,
            "fp64_gflop": flops / 1e9,
            "fp64_tflops_one_launch": flops / (out["one_launch"]["ms"] / 1000.0) / 1e12,
            "fp64_nominal_tflops": FP64_NOMINAL_TFLOPS,
            "path": "one launch" if int(lib.ptn_zqr_path(m, k)) == 1 else "launch sequence",
            "same_bits": all(torch.equal(x, y) for x, y in zip(res["one_launch"], res["launch_sequence"]))}


def run_c1(args):
    """First-order one-site TDVP (Krylov) on the 15-node binary tree, TFIM J=1,
    g=0.5, seeded random product state padded to chi=8, dt=0.01, with <Z_i> at
    all 15 sites after every step. One step = run_one_time_step plus the 15
    values read back to the host (``evaluate_operator_values``: one pass over
    the tree). Also timed: the 15 values one operator at a time (the
    reference's pattern), a whole 50-step ``run`` through the public API from
    host tensors, and the NumPy oracle doing the same steps on the host."""
    import torch
    import pytreenet_gb300 as P
    from pytreenet_gb300 import _lib
    from pytreenet_gb300.engine import ttno_site_tensors
    from pytreenet_gb300.workloads import binary_tfim_product_state
    lib = _lib.load()
    Z = np.diag([1.0, -1.0]).astype(complex)
    dt, total = 0.01, 50

    def make(seed=0):
        st, H, spec, tensors = binary_tfim_product_state(n=15, chi=8, seed=seed)
        ids = [nid for nid, _ in spec]
        ops = {f"Z_{nid}": P.TensorProduct({nid: Z}) for nid in ids}
        algo = P.FirstOrderOneSiteTDVP(st, H, dt, dt * total, ops,
                                       config=P.TDVPConfig(time_evo_mode=P.TimeEvoMode.KRYLOV),
                                       solver_options={"krylov_tol": args.tol})
        return algo, st, H, spec, tensors, ids
    algo, st, H, spec, tensors, ids = make()

    def step():
        algo.run_one_time_step()
        return algo.evaluate_operator_values()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    l0 = lib.ptn_launch_counter() + algo.net.graph_launches
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(torch.cuda.current_device()) as clk:
        start.record()
        for _ in range(args.steps):
            step()
        stop.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop) / args.steps
    launches = int(lib.ptn_launch_counter() + algo.net.graph_launches - l0) // args.steps

    def timed(fn, reps=20):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return 1000.0 * (time.perf_counter() - t0) / reps
    obs_pass = timed(algo.evaluate_operator_values)
    obs_each = timed(lambda: [algo.net.expect_local({nid: Z}) for nid in ids])
    vals = np.array(algo.evaluate_operator_values())
    each = np.array([algo.net.expect_local({nid: Z}) for nid in ids])
    # the public API end to end: a fresh driver on host tensors, 50 steps with
    # the measurements, results on the host
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    a2 = make()[0]
    res = a2.run(pgbar=False)
    torch.cuda.synchronize()
    run_s = time.perf_counter() - t0
    line = {"metric": "one-site TDVP steps/sec with <Z_i> at all 15 sites per step (15-node binary tree, TFIM, chi=8)",
            "value": 1000.0 / ms, "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128 (fp64)", "data": "synthetic",
            "config": {"workload": "binary tree 15 sites, TFIM J=1 g=0.5, random product state padded to chi=8, "
                                   f"first-order 1TDVP, dt={dt}, krylov_tol={args.tol}, <Z_i> every step",
                       "l2": "state fits in L2 (launch-bound workload); no flush"},
            "gpu_launches": launches, "clocks": clk.summary(),
            "observables": {"one_pass_ms": obs_pass, "per_operator_ms": obs_each,
                            "max_abs_difference": float(np.max(np.abs(vals - each)))},
            "e2e": {"value": total / run_s, "unit": "steps/s", "what": f"{total}-step run() from host tensors "
                    "with <Z_i> recorded every step, driver construction included",
                    "h2d_bytes_per_step": int(sum(t.size for t in tensors.values()) * 16 // total),
                    "d2h_bytes_per_step": 16 * len(ids), "seconds": run_s, "z_final": res[-1].real.tolist()}}
    if not args.no_cpu_baseline:
        import oracle as O
        tree = O.OTree()
        for nid, p in spec:
            tree.add_root(nid) if p is None else tree.add_child(nid, p)
        _, st2, H2, _, tensors2, _ = make()
        W = ttno_site_tensors(st2, H2)
        ora = O.FirstOrderOneSiteTDVPOracle(O.OState(tree, {k: np.array(v) for k, v in tensors2.items()}), W, dt,
                                            krylov_tol=args.tol)
        n_cpu = 10
        t0 = time.perf_counter()
        for _ in range(n_cpu):
            ora.run_one_time_step()
            [O.expect_product(ora.state, {nid: Z}) for nid in ids]
        cpu = (time.perf_counter() - t0) / n_cpu
        line["cpu_baseline"] = {"value": 1.0 / cpu, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"NumPy oracle: {n_cpu} steps of the same run, each with the 15 "
                                          "<Z_i> by a full contraction per operator"}
    return line


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
    line = {"metric": f"two-site TDVP steps/sec (ternary depth 3, 40 sites, XXZ, chi_max={args.chi_max})",
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
    if args.precision == "mixed" and not args.no_plain:
        # the same number of steps on the plain path from the same state; the
        # timed driver is released first (at max_bond_dim 64 the complex128
        # root-pair chain alone needs ~125 GB of intermediates)
        del algo
        import gc
        gc.collect()
        torch.cuda.empty_cache()
        try:
            ref = make("plain")
            for _ in range(args.steps):
                ref.run_one_time_step()
            other = make("mixed")
            for _ in range(args.steps):
                other.run_one_time_step()
            ov = other.net.overlap(ref.net)
            f = 1.0 - abs(ov) / np.sqrt(other.net.overlap(other.net).real * ref.net.overlap(ref.net).real)
            line["plain_fp64"] = {"steps_compared": args.steps, "fidelity_error": float(f),
                                  "fidelity_error_per_unit_time": float(f) / (0.02 * args.steps),
                                  "same_bond_dims": list(ref.bond_dims_history) == list(other.bond_dims_history)}
        except torch.OutOfMemoryError as exc:
            line["plain_fp64"] = {"skipped": f"device memory: {str(exc).splitlines()[0][:160]}"}
    return line


def run_disorder(args):
    """Independent realisations of second-order two-site TDVP on the 31-site
    binary tree (Heisenberg + random fields h_i ~ U[-2, 2], Neel start),
    max_bond_dim cycling through 8, 16, 32, 64, 128 over the realisations,
    cutoff 1e-9, dt = 0.05; ``--steps`` time steps each (one step = a forward
    and a backward sweep), each realisation's driver built inside the timed
    region. Timed three ways: one worker thread, ``--workers`` threads on their
    own streams, and ``--processes`` spawned worker processes on the same GPU
    (pool started and warmed before the timed region). value = the fastest."""
    import functools
    import torch
    import pytreenet_gb300 as P
    from pytreenet_gb300.batch import realisation_pool
    from pytreenet_gb300.workloads import disorder_realisation, realisation_bond_dims
    caps = (8, 16, 32, 64, 128)
    make = functools.partial(disorder_realisation, caps=caps, precision=args.precision)
    out = {}
    for w in (1, args.workers):
        P.run_realisations(make, min(w, args.realisations), 1, workers=w)      # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        P.run_realisations(make, args.realisations, args.steps, workers=w)
        torch.cuda.synchronize()
        out[f"threads_{w}"] = args.realisations * args.steps / (time.perf_counter() - t0)
    if args.processes > 1:
        pool = realisation_pool(args.processes)
        try:
            P.run_realisations(make, args.processes, 1, workers=1, on_done=realisation_bond_dims, pool=pool)
            t0 = time.perf_counter()
            P.run_realisations(make, args.realisations, args.steps, workers=1, on_done=realisation_bond_dims,
                               pool=pool)
            out[f"processes_{args.processes}"] = args.realisations * args.steps / (time.perf_counter() - t0)
        finally:
            pool.close()
            pool.join()
    best = max(out, key=out.get)
    return {"metric": "two-site TDVP realisation-steps/sec (31-site binary tree, random fields, chi_max 8..128)",
            "value": out[best], "unit": "realisation-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x6 split contractions / f64 Krylov+QR+SVD" if args.precision == "mixed" else "c128 (fp64)",
            "data": "synthetic",
            "config": {"workload": f"{args.realisations} realisations x 31-site binary tree, Heisenberg + "
                                   "h_i~U[-2,2], Neel start, second-order 2TDVP, dt=0.05, cutoff 1e-9, "
                                   "max_bond_dim 8/16/32/64/128", "workers": args.workers,
                       "processes": args.processes, "best": best,
                       "timing": "wall clock over all realisations, includes building each driver"},
            "rates": out, "speedup_over_one_thread": out[best] / out["threads_1"]}


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
    adj = OneSiteTDVPAdjoint(st, ham(theta), dt, nsteps, krylov_tol=tol, normalise=True,
                             precision=args.precision)
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
    plain = None
    if args.precision == "mixed" and not args.no_plain:
        # the complex128 adjoint on the same workload, timed the same way
        adj64 = OneSiteTDVPAdjoint(st, ham(theta), dt, nsteps, krylov_tol=tol, normalise=True)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        v64, g64 = coupling_gradient(adj64, ham, theta, ops)
        torch.cuda.synchronize()
        plain = {"seconds": time.perf_counter() - t2, "value_difference": abs(val - v64),
                 "gradient_difference_relative": float(np.linalg.norm(grad - g64) / np.linalg.norm(g64))}
    return {"metric": "gradient evaluations/sec (d<Z_root>/d(g_1..g_31, J), 30 one-site TDVP steps, "
                      f"31-site binary tree, chi={chi})",
            "value": 1.0 / sec, "unit": "gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * sec, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": ("bf16x6 split contractions / f64 Krylov+QR+phi-integral" if args.precision == "mixed"
                      else "c128 (fp64)"), "data": "synthetic",
            "config": {"workload": f"binary tree 31 sites, TFIM g_i~U[0.3,0.7], J=1, chi={chi} (bonds capped at the "
                                   f"subtree dimensions), first-order 1TDVP, dt={dt}, {nsteps} steps, "
                                   f"krylov_tol={tol}", "timing": "wall clock per gradient, forward + backward",
                       "precision": args.precision},
            "gpu_launches": launches, "clocks": clk.summary(), "value_Z_root": val,
            "forward_seconds": fwd, "central_difference_seconds_estimate": 2 * theta.size * fwd,
            "forward_matches_driver": abs(v0 - val),
            "plain_fp64_adjoint": plain,
            "fd_check": {"params": idx, "adjoint": [float(grad[j]) for j in idx], "central": [fd[j] for j in idx],
                         "max_abs_err": err, "grad_norm": float(np.linalg.norm(grad))}}


def main():
    args = parse()
    if args.impl == "reference" and args.full_sweep:
        print(json.dumps(run_reference_full_sweep(args)), flush=True)
        return
    single = {"qr": run_qr, "c1": run_c1, "gradient": run_gradient, "disorder": run_disorder, "ternary": run_two_site, "matvec": run_matvec,
              "gram_schmidt": run_gram_schmidt}
    if args.impl == "gb300" and (args.workload in single or args.breakdown or args.fidelity_sweeps):
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        if args.workload == "gradient" and args.chi == 256:
            args.chi = 64
        if args.breakdown:
            fn = run_breakdown
        elif args.fidelity_sweeps:
            fn = run_fidelity
        else:
            fn = single[args.workload]
        print(json.dumps(fn(args)), flush=True)
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
