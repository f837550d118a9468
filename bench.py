#!/usr/bin/env python
"""Benchmark of the hackcode1 hot path on GB300.

A step is one force evaluation of a Plummer sphere of N = 1,048,576 bodies
(mkplummer seed=1) at tol=0.5, eps=0.01 with quadrupole moments: octree
build (expandbox replay, keys, sort, cells, moments) plus the force walk of
every body.  The opening criterion is the reference's fixed-theta rule.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun (N > 1) each rank runs an
independent replica of the workload on its own GPU (the path does not shard
across GPUs); the value is the whole-job throughput.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tree-force bodies/s at N=1M, learned vs fixed-θ GPU at equal RMS force error"
UNIT = "bodies/s"
N_DEFAULT = 1048576
SEED, TOL, EPS, USEQUAD = 1, 0.5, 0.01, True
FLOPS_MONO, FLOPS_QUAD = 20, 59          # per interaction, as counted in hc_walk.cu
L2_FLUSH_BYTES = 512 << 20


def workload_config(n):
    return {"workload": f"plummer N={n} seed={SEED}: one force evaluation (octree build + walk of all bodies)",
            "n": n, "tol": TOL, "eps": EPS, "usequad": USEQUAD, "criterion": "fixed-theta (grav.c subdivp)",
            "l2": "flushed between steps (512 MiB write, outside the per-step device timing)",
            "parallelism": "replicas (one independent system per GPU)"}


# ---------------------------------------------------------------- distributed helpers

def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(n: int, my_ms: float, world: int):
    """Whole-job bodies/s of `world` replicas: every rank evaluates n bodies
    per step; the job's step time is the slowest rank's."""
    ms = reduce_max(my_ms, world)
    return world * n / (ms * 1e-3), ms


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"hc_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- CPU (oracle) legs

def _cpu_worker(args):
    path, n, nsample, seed = args
    from oracle import oracle as O
    d = np.load(path)
    m, pos = d["mass"], d["pos"]
    t0 = time.perf_counter()
    T = O.Tree(n, 1.0)
    T.set_box([-2.0, -2.0, -2.0], 4.0)
    assert T.build(m, pos, USEQUAD) == 0
    t1 = time.perf_counter()
    rng = np.random.default_rng(seed)
    idx = rng.choice(n, size=nsample, replace=False)
    T.forces(TOL, EPS, USEQUAD, test_pos=pos[idx])     # test points: same walk, self not skipped
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1, nsample


def cpu_leg(n: int, m, pos, procs: int, nsample_per_proc: int, seed: int = 0):
    """Oracle port timed on host cores: every process builds the full tree
    (the reference's build is serial) and walks its own sample of bodies.
    Returns (bodies/s extrapolated to one full evaluation on `procs` cores,
    build seconds, walk bodies/s per core)."""
    import multiprocessing as mp
    from oracle import oracle as O
    O.build(ref=False)
    fd, path = tempfile.mkstemp(suffix=".npz")
    os.close(fd)
    np.savez(path, mass=m, pos=pos)
    try:
        ctxp = mp.get_context("spawn")
        with ctxp.Pool(procs) as pool:
            res = pool.map(_cpu_worker, [(path, n, nsample_per_proc, seed + i) for i in range(procs)])
    finally:
        os.remove(path)
    t_build = statistics.mean(r[0] for r in res)
    rate = statistics.mean(r[2] / r[1] for r in res)          # bodies/s per core
    full = t_build + n / (procs * rate)
    return n / full, t_build, rate


# ---------------------------------------------------------------- GPU leg

def run_ours(args, world, rank, local):
    import torch
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode as hc
    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (the CUDA path has no CPU fallback)")
    torch.cuda.set_device(local)
    n = args.n
    m, ph = hc.mkplummer(n, SEED)
    ctx = hc.Context(n, tol=TOL, eps=EPS, fcells=1.0, usequad=USEQUAD)
    ctx.upload(m, ph)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def step():
        ctx.evaluate()          # build + walk, replayed from a captured CUDA graph

    for _ in range(args.warmup):
        step()
    peak = ctx.fp32_peak_tflops()

    # ---- device-resident throughput ----
    step_ms, build_ms, walk_ms, launches = [], [], [], 0
    barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ctx.timer_start()
            step()
            step_ms.append(ctx.timer_stop())
            b, w, nl = ctx.timing()
            build_ms.append(b)
            walk_ms.append(w)
            launches += nl
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - wall0
    d = ctx.diagnostics()
    n2b, nbc = int(d.n2b), int(d.nbc)
    ws = ctx.walk_stats()
    ws["mask_fill"] = (n2b + nbc) / max(1, 32 * (ws["entries_body"] + ws["entries_cell"]))
    value, mean_ms = job_throughput(n, statistics.mean(step_ms), world)

    # ---- end to end through the public API, host buffers (pinned) ----
    hm = torch.from_numpy(m).pin_memory()
    hph = torch.from_numpy(ph.reshape(-1)).pin_memory()
    hacc = torch.empty(3 * n, dtype=torch.float64).pin_memory()
    hphi = torch.empty(n, dtype=torch.float64).pin_memory()
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ctx.timer_start()
        ctx.upload_ptr(hm.data_ptr(), hph.data_ptr())
        ctx.evaluate()
        ctx.download_ptr(None, hacc.data_ptr(), hphi.data_ptr())
        t = ctx.timer_stop()
        if i >= args.warmup:
            e2e_ms.append(t)
    e2e_value, e2e_mean = job_throughput(n, statistics.mean(e2e_ms), world)

    # ---- roofline of the walk kernel ----
    flops = FLOPS_MONO * n2b + (FLOPS_QUAD if USEQUAD else FLOPS_MONO) * nbc
    walk_mean = statistics.mean(walk_ms)
    achieved = flops / (walk_mean * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "walk_traffic.json")
    if os.path.exists(tpath):
        try:
            t = json.load(open(tpath))
            if int(t.get("n", 0)) == n:
                traffic = t.get("bytes_per_launch")
        except (OSError, ValueError):
            traffic = None

    # ---- force error against the FP64 direct sum on a sample ----
    ferr = None
    if args.sample > 0 and rank == 0:
        rng = np.random.default_rng(12345)
        idx = np.sort(rng.choice(n, size=min(args.sample, n), replace=False)).astype(np.int64)
        ea, _ = ctx.direct_sample(idx)
        _, acc, _ = ctx.download(phase=False, phi=False)
        rel = np.linalg.norm(acc[idx] - ea, axis=1) / np.linalg.norm(ea, axis=1)
        ferr = {"rms": float(np.sqrt(np.mean(rel ** 2))), "p99": float(np.percentile(rel, 99)),
                "max": float(rel.max()), "sample": int(len(idx)), "against": "FP64 direct sum (GPU)"}

    if args.stats:
        sctx = hc.Context(n, tol=TOL, eps=EPS, fcells=1.0, usequad=USEQUAD, count_per_body=True)
        sctx.upload(m, ph)
        sctx.evaluate()
        ws["count_walk"] = sctx.walk_stats()
        sctx.close()
    clocks = clk.summary()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: Plummer sphere drawn as mkplummer does (ran3, seed=1)",
        "config": workload_config(n),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 56 * n,
                "d2h_bytes_per_step": 32 * n},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": "k_walk<quad>",
                     "peak_source": "measured live: FP32 FMA chain kernel (hc_fp32_peak), FMA = 2 flops",
                     "flops_per_launch": flops},
        "interactions_per_s": world * (n2b + nbc) / (mean_ms * 1e-3),
        "interactions": {"n2b": n2b, "nbc": nbc, "per_body": (n2b + nbc) / n},
        "phase_ms": {"build": statistics.mean(build_ms), "walk": walk_mean},
        "walk_stats": ws,
        "wall_s_timed_loop": wall,
        "force_error": ferr,
        "clocks": clocks,
    }
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        pos = np.ascontiguousarray(ph[:, 0])
        v, tb, rate = cpu_leg(n, m, pos, procs=1, nsample_per_proc=args.cpu_sample)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"oracle port (C, FP64): full tree build of {n} bodies "
                                         f"({tb:.2f} s) + walks of {args.cpu_sample} sampled bodies "
                                         f"({rate:.0f} bodies/s), extrapolated to one full evaluation"}
    ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


# ---------------------------------------------------------------- reference arm

def run_reference(args, world, rank):
    if rank != 0:
        return
    from oracle import oracle as O
    O.build(ref=False)
    n = args.n
    m, ph = O.mkplummer(n, SEED)
    pos = np.ascontiguousarray(ph[:, 0])
    procs = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        v, tb, rate = cpu_leg(n, m, pos, procs=procs, nsample_per_proc=args.ref_sample, seed=100 * i)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    sample = (f"oracle port of hackcode1's maketree/hackgrav (the reference's C cannot be built on this host: "
              f"its sources are absent here), {procs} processes: each builds the full {n}-body tree and walks "
              f"{args.ref_sample} sampled bodies; throughput = N / (build + N / (procs x walk rate))")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": n / value * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic: Plummer (ran3, seed=1)",
           "config": workload_config(n),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--sample", type=int, default=16384, help="bodies for the FP64 force-error sample")
    ap.add_argument("--cpu-sample", type=int, default=2048)
    ap.add_argument("--ref-sample", type=int, default=512)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--stats", action="store_true", help="one extra counting walk: mask popcount histogram")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
