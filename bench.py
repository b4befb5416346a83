#!/usr/bin/env python3
"""Benchmark of the elliptic-solve path on one GB300.

Workload (default): 3D Poisson, P1 on a 64^3 Kuhn-split unit cube
(1,572,864 tetrahedra, 274,625 DOFs), jitter 0.15h seed 1, f = sum of 8
Gaussians, zero Dirichlet data, b = M f.  Seeded synthetic input; no public
data set is involved.

The operator and its AMG hierarchy are set up once and stay resident.  A
step is one batched solve of `--width` (64) requests -- right-hand sides
b_j = M f_j, f_j a sum of 8 Gaussians drawn per request like the workload's
f -- by CG preconditioned with one mixed-precision V-cycle per iteration
(FP32 V-cycle with a double-float dense tail, FP64 CG recurrences) to
||b - A x||_2 <= tol ||b||_2 (1e-10) per request.  `value` is those solves/s
with the inputs resident on the device; `e2e` is the same requests served
through the C ABI batch server (afp_batch_server_*: continuous batching,
requests join free columns between CG iterations) with host buffers in and
out, all submitted at once; `served` adds Poisson arrivals at 60% of that
rate with p50/p99 latency.  Beside them: the plain FP64 GPU drop-in
(`fp64`, one solve at a time) and single mixed solves (`mixed_single`).
Assembly, Dirichlet elimination and AMG setup are timed once (`setup`).  L2
is flushed (a 512 MB write) before every timed step.

    python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl ours|reference]
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

METRIC = "Poisson solves/s, p50/p99 latency @1e-8 rel err: mixed-prec served vs FP64 GPU"
WORKLOADS = {
    "poisson3d_p1_64": lambda W: W.poisson3d_p1(64),
    "poisson3d_p1_32": lambda W: W.poisson3d_p1(32),
    "poisson2d_p1_256": lambda W: W.poisson2d_p1(256),
    "elliptic2d_p2_512": lambda W: W.elliptic2d_p2(512),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="poisson3d_p1_64", choices=sorted(WORKLOADS))
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--width", type=int, default=64, help="requests per batched step / batch-server columns")
    ap.add_argument("--served", type=int, default=256, help="requests sent through the batch server")
    ap.add_argument("--stream", action="store_true", help="served request stream instead of one workload")
    ap.add_argument("--stream-sample", type=int, default=200)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--multi", action="store_true", help="batched multi-RHS workload (3D P2, 64 RHS)")
    ap.add_argument("--multi-n", type=int, default=48)
    # lazy: the reference's lazyProject hierarchy (AMGPreconditioner's); the
    # classical C/F hierarchy of 3D P2 at 48^3 fills in (a 75,511-row level
    # with 80M entries) and its setup does not finish in minutes
    ap.add_argument("--multi-hierarchy", default="lazy", choices=["lazy", "classical"])
    ap.add_argument("--nrhs", type=int, default=64)
    ap.add_argument("--tol-multi", type=float, default=1e-10)
    return ap.parse_args()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9 or p[0] != os.environ.get("BENCH_GPU_INDEX", p[0]):
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


_CLOCK = [time.perf_counter()]


def phase(name):
    """Wall time of each part of a run, on stderr (the JSON line is stdout)."""
    now = time.perf_counter()
    print(f"[bench] {name}: {now - _CLOCK[0]:.1f} s", file=sys.stderr, flush=True)
    _CLOCK[0] = now


def world_size():
    return int(os.environ.get("WORLD_SIZE", "1"))


def local_device():
    return int(os.environ.get("LOCAL_RANK", "0"))


def dist_init():
    """N > 1 (torchrun): one rank per GPU, each an independent replica of the
    whole workload (the solve path does not shard); NCCL on GPUs, gloo else."""
    import torch
    import torch.distributed as dist
    if world_size() > 1 and not dist.is_initialized():
        if torch.cuda.is_available():
            torch.cuda.set_device(local_device())
        dist.init_process_group(backend="nccl" if torch.cuda.is_available() else "gloo")


def barrier():
    if world_size() > 1:
        import torch.distributed as dist
        dist.barrier()


def combine_replicas(line):
    """Whole-job line for N replicas (called on every rank; rank 0's return
    value is printed): every rank processed `steps` solves, so value = N solves
    per step over the slowest rank's time per step (max over ranks), and the
    same for the end-to-end figure; latencies are the slowest rank's."""
    n = world_size()
    if n == 1:
        return line
    import torch.distributed as dist
    lines = [None] * n
    dist.all_gather_object(lines, line)
    out = dict(lines[0])
    out["n_gpus"] = n
    out["per_rank_value"] = [l["value"] for l in lines]
    if any(l.get("ms_per_step") is None for l in lines):  # served stream: throughputs add up
        out["value"] = round(sum(l["value"] for l in lines), 3)
        return out
    worst = max(lines, key=lambda l: l["ms_per_step"])
    out["ms_per_step"] = worst["ms_per_step"]
    out["value"] = round(n * 1e3 / worst["ms_per_step"], 3)
    for key in ("p50_ms", "p99_ms"):
        if key in worst:
            out[key] = worst[key]
    if isinstance(out.get("e2e"), dict):
        e2e = dict(out["e2e"])
        e2e["value"] = round(n * min(l["e2e"]["value"] for l in lines), 3)
        out["e2e"] = e2e
    out["cpu_baseline"] = None  # the CPU sample is taken at N = 1 only
    out["config"] = dict(out["config"], parallelism=f"replicas only ({n} independent replicas, one per GPU)")
    return out


def profiled_ratio(workload, kernel):
    """DRAM bytes over algorithmic bytes of one launch of `kernel`, from the
    committed ncu summary of this workload (None without one); the traffic is
    reported as that ratio times the launch's algorithmic bytes."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        for line in open(path):
            if line.startswith("dram_over_algorithmic:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def run_ours(args):
    import torch
    from afepack_gb300 import build as B
    from afepack_gb300 import workloads as W
    from afepack_gb300.amg import FP64, MIXED, AMGSolver
    from afepack_gb300.fem import BoundaryConditionAdmin, Context, Space, assemble

    B.build()
    torch.cuda.init()
    dev = torch.device(f"cuda:{local_device()}")
    ctx = Context(local_device())
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    wl = WORKLOADS[args.workload](W)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # ---- setup (timed once): assembly, b = M f, Dirichlet, AMG
    setup = {}
    e = [ev() for _ in range(6)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e[0].record(stream)
    space = Space(ctx, wl.space)
    K, M = assemble(space, wl.acc_stiff, wl.acc_mass, wl.coef)
    e[1].record(stream)
    f_dev = torch.from_numpy(np.ascontiguousarray(wl.f)).to(dev)
    torch.cuda.synchronize()
    b = M.vmult(f_dev)
    bca = BoundaryConditionAdmin(wl.space)
    bca.add(1, 0.0)
    bca.apply(K, b)
    e[2].record(stream)
    t1 = time.perf_counter()
    amg64 = AMGSolver(K, precision=FP64)
    e[3].record(stream)
    t2 = time.perf_counter()
    torch.cuda.nvtx.range_push("setup_mixed")  # the setup's launches, for the profiler's launch list
    amg32 = AMGSolver(K, precision=MIXED)
    torch.cuda.nvtx.range_pop()
    e[4].record(stream)
    t3 = time.perf_counter()
    torch.cuda.synchronize()
    setup["assembly_ms"] = e[0].elapsed_time(e[1])
    setup["rhs_dirichlet_ms"] = e[1].elapsed_time(e[2])
    setup["amg_setup_fp64_ms"] = (t2 - t1) * 1e3
    setup["amg_setup_mixed_ms"] = (t3 - t2) * 1e3
    setup["assembly_wall_ms"] = (t1 - t0) * 1e3
    levels = [amg64.level_info(l) for l in range(amg64.solve_levels())]

    # ---- FP64 reference solution (tight) for the error of the timed solves
    phase("setup")
    x_ref, info_ref = amg64.pcg(b, 1e-14, 1000)
    torch.cuda.synchronize()

    def solve(amg, tol):
        x = torch.zeros_like(b)
        return x, amg.pcg(b, tol, 1000, x)[1]

    phase("fp64 reference solution")
    results = {}
    clocks = Clocks()
    for name, amg in (("fp64", amg64), ("mixed", amg32)):
        for _ in range(max(args.warmup, 3)):
            solve(amg, args.tol)
        times, iters = [], []
        # named range of the timed solves ("timed_fp64" / "timed_mixed"), so a
        # profiler's launch list can be limited to them (ncu --nvtx-include)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.nvtx.range_push(f"timed_{name}")
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            s0, s1 = ev(), ev()
            s0.record(stream)
            x, info = solve(amg, args.tol)
            s1.record(stream)
            torch.cuda.synchronize()
            times.append(s0.elapsed_time(s1))
            iters.append(info["iterations"])
        torch.cuda.nvtx.range_pop()
        barrier()
        err = float(torch.linalg.norm(x - x_ref) / torch.linalg.norm(x_ref))
        t = np.array(times)
        results[name] = {"solves_per_s": 1e3 * len(t) / t.sum(), "ms_mean": float(t.mean()),
                         "p50_ms": float(np.percentile(t, 50)), "p99_ms": float(np.percentile(t, 99)),
                         "pcg_iterations": int(np.median(iters)), "rel_err_vs_fp64": err}

    phase("timed single solves")
    # ---- served: many right-hand sides against the resident hierarchy.
    # Requests: f_j drawn like the workload's f (sums of 8 Gaussians), b_j = M f_j
    # with the Dirichlet rows zeroed (zero boundary data).
    from afepack_gb300.serve import BatchServer
    Wd = args.width
    nreq_dev = Wd * (max(args.warmup, 3) + args.steps)
    F = W.gaussian_sources(wl.space, nreq_dev + args.served, seed=5, device=dev)
    dmask = torch.from_numpy((wl.space.dof_bmark != 0)).to(dev)
    Bcols = []
    for j in range(F.shape[1]):
        bj = M.vmult(F[:, j].contiguous())
        bj[dmask] = 0.0
        Bcols.append(bj)
    blocks = [torch.stack(Bcols[i * Wd:(i + 1) * Wd], dim=1).contiguous() for i in range(nreq_dev // Wd)]
    served_b = [c.cpu().numpy() for c in Bcols[nreq_dev:]]
    del Bcols
    phase("request generation")
    # device-resident batches (value): one step = one batched solve of Wd requests
    for i in range(max(args.warmup, 3)):
        amg32.pcg_multi(blocks[i], args.tol, 1000)
    bt, bit = [], []
    clocks.start()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.nvtx.range_push("timed_batched")
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        s0, s1 = ev(), ev()
        s0.record(stream)
        Xb, infos = amg32.pcg_multi(blocks[max(args.warmup, 3) + i], args.tol, 1000)
        s1.record(stream)
        torch.cuda.synchronize()
        bt.append(s0.elapsed_time(s1))
        bit.append(max(inf["iterations"] for inf in infos))
    torch.cuda.nvtx.range_pop()
    barrier()
    clk = clocks.stop()
    bt = np.array(bt)
    # error of a served (batched) solution against the FP64 GPU solve to 1e-14
    j_last = blocks[-1][:, 0].contiguous()
    xr_last, _ = amg64.pcg(j_last, 1e-14, 1000)
    err_b = float(torch.linalg.norm(Xb[:, 0] - xr_last) / torch.linalg.norm(xr_last))
    phase("timed batched solves")
    # end to end through the C ABI batch server with host buffers: saturation
    # (every request submitted at once), then Poisson arrivals at 60% of it
    served = {}
    with BatchServer(amg32, width=Wd, tol=args.tol, maxit=1000) as srv:
        for t in [srv.submit(v) for v in served_b[:Wd]]:
            srv.wait(t)
        srv.reset_stats()
        t0 = time.perf_counter()
        tickets = [srv.submit(v) for v in served_b]
        res = [srv.wait(t)[1] for t in tickets]
        wall = time.perf_counter() - t0
        lat = np.array([r["latency_seconds"] for r in res])
        sat = len(res) / wall
        served["saturation"] = {"requests": len(res), "solves_per_s": round(sat, 2),
                                "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
                                "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 2),
                                "failed": int(sum(r["status"] != 0 for r in res))}
        rate = 0.6 * sat
        gaps = np.random.default_rng(7).exponential(1.0 / rate, len(served_b))
        srv.reset_stats()
        t0 = time.perf_counter()
        due = t0
        tickets = []
        for v, g in zip(served_b, gaps):
            due += g
            while time.perf_counter() < due:
                time.sleep(0.0002)
            tickets.append(srv.submit(v))
        res = [srv.wait(t)[1] for t in tickets]
        wall = time.perf_counter() - t0
        lat = np.array([r["latency_seconds"] for r in res])
        served["poisson_60pct"] = {"requests": len(res), "arrival_rate_per_s": round(rate, 2),
                                   "solves_per_s": round(len(res) / wall, 2),
                                   "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
                                   "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 2),
                                   "failed": int(sum(r["status"] != 0 for r in res))}
    phase("served through the batch server")
    # ---- roofline: kernels timed live with CUDA events on the library stream
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    n0, nnz0, _ = levels[0]
    kernels = {}
    amg32.pcg_multi(blocks[0], args.tol, 1000)  # the batched state at width Wd
    units = [("batched_vcycle_mixed", amg32, 4, 0)]
    units += [(f"batched_gs_sweep_level{l}_mixed", amg32, 5, l) for l in range(len(levels) - 1)]
    units += [("vcycle_mixed", amg32, 2, 0), ("residual_level0_mixed", amg32, 1, 0)]
    units += [(f"gs_sweep_level{l}_mixed", amg32, 0, l) for l in range(len(levels) - 1)]
    units += [("vcycle_fp64", amg64, 2, 0), ("gs_sweep_level0_fp64", amg64, 0, 0), ("spmv_fine_fp64", amg64, 3, 0)]
    reps = 10
    for label, amg, kind, lev in units:
        c0 = ctx.launch_count()
        ms, nbytes = amg.time_kernel(kind, lev, reps)
        per_unit = (ctx.launch_count() - c0) / (reps + 1)  # the timer runs one warm-up unit first
        kernels[label] = {"ms": round(ms, 5), "bytes": int(nbytes), "GBps": round(nbytes / ms / 1e6, 1),
                          "frac": round(nbytes / ms / 1e6 / hbm, 4), "launches": round(per_unit, 2)}
    # the dominant kernel of the served path: the batched Gauss-Seidel sweep
    # of the level that takes longest (k_rows_m, one launch per colour class)
    lev = max(range(len(levels) - 1), key=lambda l: kernels[f"batched_gs_sweep_level{l}_mixed"]["ms"])
    dom = kernels[f"batched_gs_sweep_level{lev}_mixed"]
    name = (f"k_rows_m<float> Gauss-Seidel classes (+ l1-Jacobi overflow class): one batched sweep of level {lev} "
            f"({levels[lev][0]} rows x {Wd} right-hand sides, {dom['launches']:.0f} launches)")
    ratio = profiled_ratio(args.workload, "rows_m_gs_batched")
    traffic = int(ratio * dom["bytes"]) if ratio else None
    roof = {"bound": "hbm", "kernel": name, "achieved": dom["GBps"], "peak": hbm, "unit": "GB/s",
            "frac": dom["frac"], "traffic": traffic,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6800 GB/s",
            "kernels": kernels}

    phase("kernel timings")
    launches = ctx.launch_count()
    # CPU baseline (rank 0, N=1): the reference algorithm's solve on one core
    cpu = (cpu_baseline_sample(amg64, b.cpu().numpy().copy(), args.tol, results["fp64"]["pcg_iterations"])
           if world_size() == 1 else None)
    phase("CPU sample")
    nb = int(blocks[0].shape[0])
    line = {
        "metric": METRIC, "value": round(Wd * 1e3 * len(bt) / bt.sum(), 3), "unit": "solves/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(float(bt.mean()), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 V-cycle + fp64 CG", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "n_dof": int(n0), "nnz": int(nnz0), "tol": args.tol,
                   "requests_per_step": Wd, "levels": [list(map(int, l)) for l in levels],
                   "step": f"one batched CG solve of {Wd} requests (different right-hand sides) against the resident "
                           f"operator and hierarchy, inputs resident on the device",
                   "l2": "flushed before every step (512 MB write)", "parallelism": "replicas only"},
        "p50_ms": served["poisson_60pct"]["p50_ms"], "p99_ms": served["poisson_60pct"]["p99_ms"],
        "served": served, "rel_err_vs_fp64": err_b, "pcg_iterations_max": int(max(bit)),
        "fp64": results["fp64"], "mixed_single": results["mixed"],
        "mixed_over_fp64": round(Wd * 1e3 * len(bt) / bt.sum() / results["fp64"]["solves_per_s"], 3),
        "served_over_fp64": round(served["saturation"]["solves_per_s"] / results["fp64"]["solves_per_s"], 3),
        "setup": {k: round(v, 3) for k, v in setup.items()},
        "e2e": {"value": served["saturation"]["solves_per_s"], "unit": "solves/s",
                "h2d_bytes_per_step": int(Wd * nb * 8), "d2h_bytes_per_step": int(Wd * nb * 8),
                "p50_ms": served["saturation"]["p50_ms"], "p99_ms": served["saturation"]["p99_ms"],
                "how": f"the batch server through the C ABI (afp_batch_server_*), {Wd} columns, host buffers in and out, "
                       f"{served['saturation']['requests']} requests submitted at once; a step = {Wd} requests"},
        "roofline": roof, "clocks": clk, "gpu_launches": int(launches), "cpu_baseline": cpu,
    }
    return line


def run_multi(args):
    """3D Poisson P2 on an n^3 Kuhn cube (default 48^3, 912,673 DOFs), one
    matrix and hierarchy (by default the reference's lazyProject hierarchy),
    64 right-hand sides: one batched multi-RHS CG (FP32 V-cycle, FP64
    recurrences) per step, against sequential FP64 CG solves."""
    import torch
    from afepack_gb300 import build as B
    from afepack_gb300 import workloads as W
    from afepack_gb300.amg import FP64, MIXED, AMGSolver
    from afepack_gb300.fem import BoundaryConditionAdmin, Context, Space, assemble
    B.build()
    dev = torch.device(f"cuda:{local_device()}")
    ctx = Context(local_device())
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    wl = W.poisson3d_p2_multi(args.multi_n, args.nrhs)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    t0 = time.perf_counter()
    space = Space(ctx, wl.space)
    K, M = assemble(space, wl.acc_stiff, wl.acc_mass)
    Bm = np.stack([M.vmult(np.ascontiguousarray(wl.f[:, c])) for c in range(wl.f.shape[1])], axis=1)
    bca = BoundaryConditionAdmin(wl.space)
    bca.add(1, 0.0)
    d, _ = bca.arrays()
    bca.apply(K, np.ascontiguousarray(Bm[:, 0]).copy())
    Bm[d != 0] = 0.0
    t1 = time.perf_counter()
    phase("multi: assembly and right-hand sides")
    def hierarchy(precision):
        if args.multi_hierarchy == "classical":
            return AMGSolver(K, precision=precision)
        amg = AMGSolver(precision=precision)
        amg.lazyReinit(K)
        return amg

    amg32 = hierarchy(MIXED)
    t2 = time.perf_counter()
    phase("multi: mixed setup")
    amg64 = hierarchy(FP64)
    phase("multi: fp64 setup")
    Bd = torch.from_numpy(np.ascontiguousarray(Bm)).to(dev)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # FP64 references for the error: FP64 CG to 1e-13 on a few columns
    refs = {c: amg64.pcg(np.ascontiguousarray(Bm[:, c]), 1e-13, 1000)[0] for c in (0, args.nrhs - 1)}
    phase("multi: fp64 references")
    for _ in range(max(args.warmup, 3)):
        amg32.pcg_multi(Bd, args.tol_multi, 500)
    phase("multi: warm-up")
    times = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        s0, s1 = ev(), ev()
        s0.record(stream)
        X, infos = amg32.pcg_multi(Bd, args.tol_multi, 500)
        s1.record(stream)
        torch.cuda.synchronize()
        times.append(s0.elapsed_time(s1))
    phase("multi: timed batches")
    Xh = X.cpu().numpy()
    err = max(np.linalg.norm(Xh[:, c] - r) / np.linalg.norm(r) for c, r in refs.items())
    # drop-in: sequential FP64 single solves (a bounded sample of the 64)
    # (device time of each call, measured by the library on its own stream)
    seq, seq_it = [], []
    for c in range(min(4, args.nrhs)):
        bc = np.ascontiguousarray(Bm[:, c])
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        torch.cuda.synchronize()
        _, info = amg64.pcg(bc, args.tol_multi, 500)
        seq.append(1e3 * info["seconds"])
        seq_it.append(int(info["iterations"]))
    t = np.array(times)
    value = args.nrhs * 1e3 / t.mean()
    fp64_seq = 1e3 / np.mean(seq)
    return {
        "metric": METRIC, "value": round(value, 3), "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(float(t.mean()), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 V-cycle + fp64 CG", "data": "synthetic (seeded)",
        "config": {"workload": f"poisson3d_p2_{args.multi_n}_x{args.nrhs}", "hierarchy": args.multi_hierarchy,
                   "n_dof": int(wl.space.n_dof),
                   "nnz": int(K.n_nonzero_elements()), "nrhs": args.nrhs, "tol": args.tol_multi,
                   "l2": "flushed before every step (512 MB write)"},
        "rel_err_vs_fp64": err, "pcg_iterations_max": int(max(i["iterations"] for i in infos)),
        "fp64_sequential_solves_per_s": round(fp64_seq, 3), "fp64_sequential_iterations": seq_it,
        "batched_over_sequential_fp64": round(value / fp64_seq, 2),
        "setup": {"assembly_rhs_s": round(t1 - t0, 3), "amg_setup_s": round(t2 - t1, 3)},
    }


def run_stream(args):
    """Served stream of independent meshes (2D P1, n log-uniform in
    [32, 1024], half variable-coefficient, seed 4): every 10th of the 2000
    requests (200, a stratified sample of the stream) through the solve
    server (afp_server_*: 8 execution slots, HBM admission, each request's
    whole path -- assembly, AMG setup, CG -- on the GPU), first all at once
    (saturation), then with Poisson arrivals at 50% of that rate; mixed
    precision and FP64."""
    from afepack_gb300 import workloads as W
    from afepack_gb300 import build as B
    from afepack_gb300.serve import Server
    B.build()
    reqs = W.request_stream(2000, seed=4)[:: max(1, 2000 // args.stream_sample)]
    t0 = time.perf_counter()
    wls = [W.request_workload(r) for r in reqs]
    gen_s = time.perf_counter() - t0
    phase("stream: request generation")

    def run(srv, arrivals):
        srv.reset_stats()
        t0 = time.perf_counter()
        due, tickets = t0, []
        for wl, g in zip(wls, arrivals):
            due += g
            while time.perf_counter() < due:
                time.sleep(0.0005)
            tickets.append(srv.submit(wl))
        res = [srv.wait(t)[1] for t in tickets]
        wall = time.perf_counter() - t0
        lat = np.array([r["latency_seconds"] for r in res])
        return {"requests": len(res), "solves_per_s": round(len(res) / wall, 3),
                "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 1),
                "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 1),
                "failed": int(sum(r["status"] != 0 for r in res)),
                "iterations_median": int(np.median([r["iterations"] for r in res])),
                # where a request's time goes: admission -> hierarchy ready, and the CG on the device
                "setup_s_total": round(float(sum(r["setup_seconds"] for r in res)), 2),
                "cg_device_s_total": round(float(sum(r["device_seconds"] for r in res)), 2)}

    out = {}
    for name, prec in (("mixed", 1), ("fp64", 0)):
        # independent small requests: a dense tail of at most 2048 rows keeps each setup cheap
        with Server(workers=args.workers, precision=prec, tol=args.tol, dense_tail=2048) as srv:
            for t in [srv.submit(wl) for wl in wls[: min(4, len(wls))]]:
                srv.wait(t)
            sat = run(srv, np.zeros(len(wls)))
            rate = 0.5 * sat["solves_per_s"]
            paced = run(srv, np.random.default_rng(11).exponential(1.0 / rate, len(wls)))
            paced["arrival_rate_per_s"] = round(rate, 3)
        out[name] = {"saturation": sat, "poisson_50pct": paced}
        phase(f"stream: {name} server runs")
    ndofs = [int(w.space.n_dof) for w in wls]
    m = out["mixed"]
    return {
        "metric": METRIC, "value": m["saturation"]["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
        "steps": 1, "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 V-cycle + fp64 CG", "data": "synthetic (seeded)",
        "config": {"workload": "request_stream", "requests": len(wls), "sample": "every 10th of the 2000-request stream",
                   "workers": args.workers, "n_dof_min": min(ndofs), "n_dof_max": max(ndofs),
                   "n_dof_total": sum(ndofs), "tol": args.tol, "generation_s": round(gen_s, 2), "dense_tail": 2048,
                   "arrival": "saturation (all at once), then Poisson at 50% of the saturated rate"},
        "p50_ms": m["poisson_50pct"]["p50_ms"], "p99_ms": m["poisson_50pct"]["p99_ms"],
        "mixed": m, "fp64": out["fp64"],
        "mixed_over_fp64": round(m["saturation"]["solves_per_s"] / out["fp64"]["saturation"]["solves_per_s"], 3),
    }


def _oracle_system(wl):
    """The workload's system built by the CPU oracle (the reference algorithm):
    assembly, b = M f, Dirichlet elimination."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    K, mass = O.assemble(wl.space, wl.acc_stiff, wl.acc_mass, wl.coef)
    b = O.CSR(K.rowptr, K.cols, mass, K.shape).matvec(wl.f)
    O.apply_dirichlet(K, b, wl.space.dof_bmark)
    return K, b


def _ref_worker(conn, steps, warmup, tol):
    """Forked reference worker: times single-threaded oracle CG solves
    (one reference V-cycle per iteration) on the hierarchy of its parent."""
    import oracle as O  # noqa: F401  (already loaded in the parent)
    amg, b = _REF_STATE["amg"], _REF_STATE["b"]
    for i in range(warmup + steps):
        conn.recv()  # start signal for this step
        t0 = time.perf_counter()
        x, it, rel = amg.pcg(b, tol, 1000)
        conn.send((time.perf_counter() - t0, it, rel))
    conn.close()


_REF_STATE = {}


def run_reference(args):
    """The reference's CPU implementation of the path, timed on the host cores:
    the oracle port of AFEPack (bit-identical to AFEPack compiled from its
    sources on every fixture) builds the system and hierarchy once, then W
    forked single-threaded processes (W = host cores) each run one CG solve
    per step; value = W / (wall time of the step)."""
    import multiprocessing as mp
    from afepack_gb300 import workloads as W
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    wl = WORKLOADS[args.workload](W)
    t0 = time.perf_counter()
    K, b = _oracle_system(wl)
    t1 = time.perf_counter()
    amg = O.AMG(K)  # AMGSolver::reinit restated (rows of the Galerkin product on all cores)
    t2 = time.perf_counter()
    _REF_STATE.update(amg=amg, b=b)
    ctx = mp.get_context("fork")  # no GPU is touched in this process
    pipes, procs = [], []
    for _ in range(cores):
        a, c = ctx.Pipe()
        p = ctx.Process(target=_ref_worker, args=(c, args.steps, args.warmup, args.tol))
        p.start()
        pipes.append(a)
        procs.append(p)
    os.environ["OMP_NUM_THREADS"] = "1"
    walls, iters, lat = [], [], []
    for i in range(args.warmup + args.steps):
        s0 = time.perf_counter()
        for a in pipes:
            a.send(i)
        res = [a.recv() for a in pipes]
        wall = time.perf_counter() - s0
        if i >= args.warmup:
            walls.append(wall)
            iters.append(res[0][1])
            lat.extend(r[0] for r in res)  # each worker's own solve time
    for p in procs:
        p.join()
    walls = np.array(walls)
    value = cores * len(walls) / walls.sum()
    n0 = K.shape[0]
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * walls.mean(), 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "n_dof": int(n0), "nnz": int(K.nnz), "tol": args.tol,
                   "levels": [list(map(int, (amg.level(l).shape[0], amg.level(l).nnz))) for l in range(amg.n_level + 1)],
                   "parallelism": f"{cores} single-threaded processes, one solve each per step"},
        "pcg_iterations": int(np.median(iters)),
        "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 1), "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 1),
        "setup": {"assembly_dirichlet_s": round(t1 - t0, 2), "amg_reinit_s": round(t2 - t1, 2),
                  "amg_reinit_threads": cores},
        "cpu_baseline": {"value": round(value, 4), "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} concurrent CG solves (one reference V-cycle per iteration) per step"},
        "e2e": {"value": round(value, 4), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def cpu_baseline_sample(amg_gpu, b_host, tol, iterations, budget_s=20.0):
    """Single-threaded oracle CG (the reference's CG shape, one reference
    V-cycle per iteration: lexicographic Gauss-Seidel, restriction,
    prolongation) on the hierarchy the GPU built -- levels bitwise the
    reference's down to the dense tail -- with the reference's coarsest
    treatment, an explicit inverse, applied at that tail level (inverted here
    with LAPACK; the reference would keep coarsening it on the host for
    minutes).  Bounded by time: one iteration is timed first; when the whole
    solve (`iterations`, the GPU FP64 solve's count) would take longer than
    `budget_s`, as many iterations as fit are timed and the solve time is
    extrapolated linearly from them."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    nl = amg_gpu.n_project()
    A = [O.CSR(*amg_gpu.level_matrix(l), (amg_gpu.level_info(l)[0],) * 2) for l in range(nl + 1)]
    P = [O.CSR(*amg_gpu.projection(l), (amg_gpu.level_info(l + 1)[0], amg_gpu.level_info(l)[0])) for l in range(nl)]
    inv = np.linalg.inv(A[-1].to_scipy().toarray())
    amg = O.AMG.from_levels(A, P, coarse_inv=inv)
    t0 = time.perf_counter()
    amg.pcg(b_host, 0.0, 1)
    t1 = time.perf_counter() - t0
    k = int(max(1, min(iterations, budget_s // max(t1, 1e-9))))
    t0 = time.perf_counter()
    x, it, rel = amg.pcg(b_host, tol if k >= iterations else 0.0, k)
    dt = time.perf_counter() - t0
    solve_s = dt if k >= iterations else dt / it * iterations
    how = (f"one whole CG solve ({it} iterations)" if k >= iterations else
           f"{it} of {iterations} CG iterations timed ({dt:.1f} s), the solve extrapolated linearly")
    return {"value": round(1.0 / solve_s, 4), "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": f"{how} of the same system on 1 core, one oracle V-cycle per iteration: lexicographic "
                      f"Gauss-Seidel on the GPU-built levels, bitwise the reference's, and an explicit inverse "
                      f"of the {A[-1].shape[0]}-row coarsest level"}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    dist_init()
    line = run_stream(args) if args.stream else run_multi(args) if args.multi else run_ours(args)
    line = combine_replicas(line)
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
