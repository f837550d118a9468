#!/usr/bin/env python
"""Benchmark of the hackcode1 hot path on GB300.

A step is one force evaluation of a Plummer sphere of N = 1,048,576 bodies
(mkplummer seed=1) at eps=0.01 with quadrupole moments: octree build
(expandbox replay, keys, sort, cells, moments) plus the force walk of every
body.  The headline is the learned opening criterion (network trained on
labels from this system, guard on) at the RMS force error of the
reference's fixed-theta rule at tol=0.5, against that rule on the GPU; the
error-bound rule (the method without its network) and the comparison at RMS
1e-3 are reported beside it.  Errors are measured against an FP64 direct sum
on a seeded sample of 16,384 bodies.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun (N > 1) each rank runs an
independent replica of the workload on its own GPU (the path does not shard
across GPUs); the value is the whole-job throughput.  A single-GPU default
run also runs the other configurations briefly in child processes (the
one-evaluation + 100-step run, the Hernquist sphere, the ensemble, 100 steps
of the composite galaxy) and summarises their lines under "workloads"
(--no-cpu-baseline skips them and the CPU baseline).
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


WORKLOADS = {
    "plummer": {"n": N_DEFAULT, "seed": SEED, "eps": EPS,
                "what": "plummer N={n} seed={seed} (mkplummer)"},
    "hernquist": {"n": 4194304, "seed": 7, "eps": 0.005,
                  "what": "hernquist N={n} seed={seed} (M=1, a=1, truncated at 100a, Eddington-inverted DF)"},
}


def generate(hc, wl, n):
    if wl == "hernquist":
        return hc.mkhernquist(n, WORKLOADS[wl]["seed"], 100.0)
    return hc.mkplummer(n, WORKLOADS[wl]["seed"])


def workload_config(n, mode=("body", TOL), wl="plummer"):
    crit = {"body": "fixed-theta (grav.c subdivp)", "error": "error-bound group rule",
            "barnes": "treecode1 critical radius in a group walk",
            "learned": "learned opening criterion (guarded)"}[mode[0]]
    w = WORKLOADS[wl]
    what = w["what"].format(n=n, seed=w["seed"])
    return {"workload": f"{what}: one force evaluation (octree build + walk of all bodies)",
            "n": n, "tol": TOL, "eps": w["eps"], "usequad": USEQUAD, "criterion": crit,
            "criterion_setting": list(mode),
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


# ---------------------------------------------------------------- CPU legs (reference code)

def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "Model name" and v.strip():
                return f"{v.strip()} ({os.uname().machine})"
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            k, _, v = line.partition(":")
            if k.strip() in ("model name", "Model"):
                return v.strip()
    except OSError:
        pass
    return os.uname().machine


class RefWalker:
    """The CPU implementation of the path that the baselines time: the
    reference's own load.c / grav.c (oracle/_ref, compiled from the NEMO
    sources with NEMO's compiler flags) when those sources are present, else
    the oracle's restatement of them (bit-identical where both exist)."""

    def __init__(self, n: int):
        from oracle import oracle as O
        try:
            O.build(ref=None)
        except Exception as e:             # a failed ref build leaves the port
            print(f"bench.py: reference build failed ({e}); timing the oracle port", file=sys.stderr)
        self.kind = "reference" if O.Reference.available(nemo_flags=True) else "port"
        if self.kind == "reference":
            self.R = O.Reference.get(True, n, nemo_flags=True)
            self.what = ("the reference's own hackcode1 load.c/grav.c (-DQUADPOLE, built from the NEMO sources "
                         "with NEMO's flags -g -O2)")
        else:
            self.T = O.Tree(n, 1.0)
            self.what = "the oracle's C restatement of hackcode1's load.c/grav.c (NEMO sources absent)"

    def build(self, m, pos):
        if self.kind == "reference":
            self.R.build(m, pos)
        else:
            self.T.set_box([-2.0, -2.0, -2.0], 4.0)
            assert self.T.build(m, pos, USEQUAD) == 0

    def walk(self, idx, eps):
        """Counts (n2b, nbc) of hackgrav at bodies idx, each skipping itself."""
        if self.kind == "reference":
            _, _, b, c = self.R.forces_idx(TOL, eps, idx)
        else:
            _, _, b, c = self.T.forces(TOL, eps, USEQUAD, idx=idx)
        return b, c


def full_evaluation(w: RefWalker, m, pos, eps, procs: int):
    """One complete force evaluation on `procs` host cores, as hackforce does
    it (hackforce.c:177-215): maketree + hackcofm once (serial, as in the
    reference), then hackgrav for every body, the bodies split into `procs`
    contiguous shares walked by forked worker processes that share the tree.
    Returns (seconds, n2b total, nbc total)."""
    n = len(m)
    t0 = time.perf_counter()
    w.build(m, pos)
    edges = np.linspace(0, n, procs + 1).astype(np.int64)
    kids = []
    for k in range(procs):
        r, wfd = os.pipe()
        pid = os.fork()
        if pid == 0:                       # worker: walk its share, report the totals
            os.close(r)
            try:
                b, c = w.walk(np.arange(edges[k], edges[k + 1], dtype=np.int32), eps)
                os.write(wfd, np.array([b.sum(), c.sum()], dtype=np.int64).tobytes())
            finally:
                os._exit(0)
        os.close(wfd)
        kids.append((pid, r))
    n2b = nbc = 0
    for pid, r in kids:
        buf = b""
        while len(buf) < 16:
            chunk = os.read(r, 16 - len(buf))
            if not chunk:
                break
            buf += chunk
        os.close(r)
        os.waitpid(pid, 0)
        if len(buf) != 16:
            raise RuntimeError("bench.py: a reference worker failed")
        b, c = np.frombuffer(buf, dtype=np.int64)
        n2b += int(b)
        nbc += int(c)
    return time.perf_counter() - t0, n2b, nbc


def cpu_baseline_one_core(n, m, pos, eps, nsample, seed=0):
    """The reference walk on one core: full tree build plus the walks of
    `nsample` uniformly sampled bodies, extrapolated to one full evaluation.
    Returns (bodies/s, build seconds, walk bodies/s, kind, what)."""
    w = RefWalker(n)
    t0 = time.perf_counter()
    w.build(m, pos)
    t1 = time.perf_counter()
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(n, size=min(nsample, n), replace=False)).astype(np.int32)
    w.walk(idx, eps)
    t2 = time.perf_counter()
    rate = len(idx) / (t2 - t1)
    return n / ((t1 - t0) + n / rate), t1 - t0, rate, w.kind, w.what


# ---------------------------------------------------------------- GPU leg

RMS_BUDGET = 1e-3            # the force-error budget of comparison (ii) and of the guard
GUARD_SAMPLE = 256
LEARNED_THRESHOLD = 0.0      # logit threshold of the learned criterion (0: the network's own decision)
BISECT_STEPS = 10           # a budget resolution of about 1% over the widest bracket (a factor 2^16)


TUNING = {"body": None, "group": {"group_max": 64, "list_depth": 64, "grouping": "tree"}}


def set_mode(ctx, mode):
    """mode: ("body", theta) | ("error", eps) | ("learned", eps, logit threshold).
    The context's tol is theta for the per-body rule and 0.5 otherwise (the
    fallback of the guard).  The per-body rule runs with the autotuner's
    choice (its interaction sets do not depend on it); the group criteria with
    tree groups of up to 64 bodies (two per lane)."""
    t = TUNING["body"] if mode[0] == "body" and TUNING["body"] else TUNING["group"]
    ctx.set_tuning(t["group_max"], t["list_depth"], t["grouping"])
    if mode[0] == "body":
        ctx.set_params(tol=mode[1])
        ctx.set_criterion("body")
    elif mode[0] == "barnes":
        ctx.set_params(tol=TOL)
        ctx.set_criterion("barnes", mode[1])
    elif mode[0] == "error":
        ctx.set_params(tol=TOL)
        ctx.set_criterion("error", mode[1])
    else:
        ctx.set_params(tol=TOL)
        ctx.set_criterion("learned", mode[1])
        ctx.learn_threshold(mode[2])


def sample_error(ctx, idx, ea):
    _, acc, _ = ctx.download(phase=False, phi=False)
    rel = np.linalg.norm(acc[idx] - ea, axis=1) / np.linalg.norm(ea, axis=1)
    return float(np.sqrt(np.mean(rel ** 2))), float(np.percentile(rel, 99))


def point(ctx, mode, idx, ea, reps=3):
    """Steady state of one criterion setting (previous accelerations from the
    same setting): best step time, RMS and p99 error, interactions."""
    set_mode(ctx, mode)
    ctx.evaluate()
    ts = []
    for _ in range(reps):
        ctx.evaluate()
        b, w, _ = ctx.timing()
        ts.append(b + w)
    d = ctx.diagnostics()
    rms, p99 = sample_error(ctx, idx, ea)
    return {"mode": list(mode), "step_ms": min(ts), "rms": rms, "p99": p99, "interactions": int(d.n2b + d.nbc)}


def calibrate(ctx, idx, ea, mode_of, lo, hi, target, geometric=True, steps=BISECT_STEPS):
    """Largest parameter in [lo, hi] whose RMS error is within the target (RMS
    grows with the parameter): bisection.  Returns (best point or None, probes)."""
    probes = [point(ctx, mode_of(hi), idx, ea)]
    if probes[-1]["rms"] <= target:
        return probes[-1], probes
    probes.append(point(ctx, mode_of(lo), idx, ea))
    if probes[-1]["rms"] > target:
        return None, probes
    best = probes[-1]
    for _ in range(steps):
        mid = (lo * hi) ** 0.5 if geometric else 0.5 * (lo + hi)
        pt = point(ctx, mode_of(mid), idx, ea)
        probes.append(pt)
        if pt["rms"] <= target:
            best, lo = pt, mid
        else:
            hi = mid
    return best, probes


def timed(ctx, mode, steps, warmup, flush, world):
    """K steps of one criterion, device-timed with CUDA events on the context
    stream, L2 flushed before each.  Returns per-step ms, build / walk ms,
    kernel launches, interactions of the last step."""
    import torch
    set_mode(ctx, mode)
    for _ in range(warmup):
        ctx.evaluate()
    step_ms, build_ms, walk_ms, launches = [], [], [], 0
    barrier(world)
    torch.cuda.synchronize()
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        ctx.timer_start()
        ctx.evaluate()          # build + walk (+ guard), replayed from a captured CUDA graph
        step_ms.append(ctx.timer_stop())
        b, w, nl = ctx.timing()
        build_ms.append(b)
        walk_ms.append(w)
        launches += nl
    torch.cuda.synchronize()
    barrier(world)
    d = ctx.diagnostics()
    ws = ctx.walk_stats()
    return {"step_ms": statistics.mean(step_ms), "build_ms": statistics.mean(build_ms),
            "walk_ms": statistics.mean(walk_ms), "launches": launches, "n2b": int(d.n2b), "nbc": int(d.nbc),
            "walk": {k: ws[k] for k in ("candidates", "entries_body", "entries_cell", "network", "network_rounds")}}


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) of the GB300s, else the fallback."""
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent)"


def build_bytes(n, nmassive, ncell, usequad=USEQUAD):
    """Algorithmic bytes of one octree build, each array moved once: keys (24 B of
    positions read, 16 B of key and index written per body), the sort (16 B per
    body read and written once), the cell linking (16 B per massive key read),
    the upward pass (every node's record read once as a child, every cell's
    record written once: 48 B monopole, 96 B with the quadrupole)."""
    rec = 96 if usequad else 48
    return n * (24 + 16) + n * 32 + nmassive * 16 + (nmassive + ncell) * rec + ncell * rec


def walk_flops(n2b, nbc):
    return FLOPS_MONO * n2b + (FLOPS_QUAD if USEQUAD else FLOPS_MONO) * nbc


def run_ours(args, world, rank, local):
    import torch
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode as hc
    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (the CUDA path has no CPU fallback)")
    torch.cuda.set_device(local)
    wl = args.workload
    n = args.n if args.n else WORKLOADS[wl]["n"]
    eps = WORKLOADS[wl]["eps"]
    m, ph = generate(hc, wl, n)
    ctx = hc.Context(n, tol=TOL, eps=eps, fcells=1.0, usequad=USEQUAD)
    ctx.upload(m, ph)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        ctx.evaluate()
    peak = ctx.fp32_peak_tflops()
    tuned = ctx.autotune()                  # per-body rule at tol = 0.5
    TUNING["body"] = tuned

    # ---- FP64 direct-sum sample (bodies do not move: one evaluation per step) ----
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(n, size=min(args.sample, n), replace=False)).astype(np.int64)
    ea, _ = ctx.direct_sample(idx)

    # ---- calibration to equal RMS (untimed): the fixed-theta rule, then the error rule ----
    fixed = point(ctx, ("body", TOL), idx, ea)
    target = fixed["rms"]
    err_pt, cal_err = calibrate(ctx, idx, ea, lambda e: ("error", e), 1e-3, 64.0, target)

    # ---- the learned criterion: labels from this system, training on the device, at the
    #      error rule's equal-RMS budget unless --train-theta names one ----
    t0 = time.perf_counter()
    set_mode(ctx, ("body", TOL))
    ctx.evaluate()                           # accelerations of the reference rule for a_min
    tg = TUNING["group"]                     # labels from the groups the learned walk uses
    ctx.set_tuning(tg["group_max"], tg["list_depth"], tg["grouping"])
    theta_train = args.train_theta if args.train_theta else (err_pt["mode"][1] if err_pt else 0.03)
    train = ctx.learn_from_self(theta=theta_train, target=1 << 20, band=tuple(args.train_band))
    torch.cuda.synchronize()
    train["seconds"] = time.perf_counter() - t0
    train["theta"] = theta_train
    train["band"] = list(args.band)
    ctx.learn_band(*args.band)

    learned_mode = lambda e: ("learned", e, LEARNED_THRESHOLD)
    lrn_pt, cal_lrn = calibrate(ctx, idx, ea, learned_mode, 1e-3, 64.0, target)
    tc1_pt, cal_tc1 = calibrate(ctx, idx, ea, lambda t: ("barnes", t), 0.3, 1.5, target, geometric=False)
    th_pt2, cal_th = calibrate(ctx, idx, ea, lambda t: ("body", t), TOL, 1.2, RMS_BUDGET, geometric=False)
    err_pt2, cal_err2 = calibrate(ctx, idx, ea, lambda e: ("error", e), 1e-3, 64.0, RMS_BUDGET)
    lrn_pt2, cal_lrn2 = calibrate(ctx, idx, ea, learned_mode, 1e-3, 64.0, RMS_BUDGET)
    head_mode = tuple(lrn_pt["mode"]) if lrn_pt else ("body", TOL)

    # ---- timed: the headline (learned, guard on) and its comparisons ----
    ctx.set_guard(GUARD_SAMPLE, RMS_BUDGET, seed=1)
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        head = timed(ctx, head_mode, args.steps, args.warmup, flush, world)
        wall = time.perf_counter() - wall0
        guard = ctx.guard_stats()
        head_err = sample_error(ctx, idx, ea)
        ws = ctx.walk_stats()
        comp = {"fixed_theta_0.5": timed(ctx, ("body", TOL), args.steps, args.warmup, flush, world)}
        comp["fixed_theta_0.5"]["rms"] = sample_error(ctx, idx, ea)[0]
        for name, pt in (("error_rule", err_pt), ("treecode1_new_rcrit", tc1_pt)):
            if pt:
                comp[name] = timed(ctx, tuple(pt["mode"]), args.steps, args.warmup, flush, world)
                comp[name]["rms"] = sample_error(ctx, idx, ea)[0]
                comp[name]["mode"] = pt["mode"]
        for name, pt in (("fixed_theta_at_1e-3", th_pt2), ("error_rule_at_1e-3", err_pt2),
                         ("learned_at_1e-3", lrn_pt2)):
            if pt:
                comp[name] = timed(ctx, tuple(pt["mode"]), args.steps, args.warmup, flush, world)
                comp[name]["rms"] = sample_error(ctx, idx, ea)[0]
                comp[name]["mode"] = pt["mode"]
    clocks = clk.summary()
    value, mean_ms = job_throughput(n, head["step_ms"], world)
    fixed_value, _ = job_throughput(n, comp["fixed_theta_0.5"]["step_ms"], world)
    for v in comp.values():
        v["bodies_per_s"] = job_throughput(n, v["step_ms"], world)[0]
        v["walk_fp32_frac"] = walk_flops(v["n2b"], v["nbc"]) / (v["walk_ms"] * 1e-3) / 1e12 / peak
    ratios = {"learned_vs_fixed_theta_equal_rms": value / fixed_value}
    if "error_rule" in comp:
        ratios["error_rule_vs_fixed_theta_equal_rms"] = comp["error_rule"]["bodies_per_s"] / fixed_value
    if "treecode1_new_rcrit" in comp:
        ratios["treecode1_group_vs_fixed_theta_equal_rms"] = (comp["treecode1_new_rcrit"]["bodies_per_s"]
                                                              / fixed_value)
    if "learned_at_1e-3" in comp and "fixed_theta_at_1e-3" in comp:
        ratios["learned_vs_fixed_theta_at_rms_1e-3"] = (comp["learned_at_1e-3"]["bodies_per_s"]
                                                        / comp["fixed_theta_at_1e-3"]["bodies_per_s"])

    # ---- end to end through the public API, host buffers (pinned): the
    # headline criterion, the host carrying positions and the previous
    # accelerations across calls; hc_evaluate_host copies the positions in,
    # the previous accelerations beside the build, and the accelerations and
    # potentials out, with one synchronisation per call ----
    set_mode(ctx, head_mode)
    hpos = torch.from_numpy(np.ascontiguousarray(ph[:, 0]).reshape(-1)).pin_memory()
    hacc = [torch.empty(3 * n, dtype=torch.float64).pin_memory() for _ in range(2)]
    hphi = torch.empty(n, dtype=torch.float64).pin_memory()
    ctx.upload(m, ph)
    ctx.evaluate()
    ctx.download_ptr(None, hacc[0].data_ptr(), hphi.data_ptr())
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ctx.timer_start()
        ctx.evaluate_host_ptr(hpos.data_ptr(), hacc[i % 2].data_ptr(), hacc[(i + 1) % 2].data_ptr(),
                              hphi.data_ptr())
        t = ctx.timer_stop()
        if i >= args.warmup:
            e2e_ms.append(t)
    e2e_value, _ = job_throughput(n, statistics.mean(e2e_ms), world)
    ctx.set_guard(0)

    # ---- roofline of the headline walk kernel ----
    flops = walk_flops(head["n2b"], head["nbc"])
    achieved = flops / (head["walk_ms"] * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "walk_traffic.json")
    if os.path.exists(tpath):
        try:
            t = json.load(open(tpath))
            if int(t.get("n", 0)) == n:
                traffic = t.get("learned" if head_mode[0] == "learned" else "body")
        except (OSError, ValueError):
            traffic = None
    # the octree build against HBM bandwidth (fixed-theta step: no guard beside it)
    ti = ctx.tree_info()
    bpk, bsrc = hbm_peak()
    bbytes = build_bytes(n, int(ti.nbody_massive), int(ti.ncell))
    b_ms = comp["fixed_theta_0.5"]["build_ms"]
    roofline_build = {"bound": "hbm", "achieved": bbytes / (b_ms * 1e-3) / 1e9, "peak": bpk, "unit": "GB/s",
                      "frac": bbytes / (b_ms * 1e-3) / 1e9 / bpk, "algorithmic_bytes": bbytes, "build_ms": b_ms,
                      "peak_source": bsrc,
                      "what": "keys + radix sort + cell linking + upward pass, each array moved once; the build "
                              "is bound by per-level latency, not bandwidth"}
    # body slots per list entry: 32 lanes, two bodies each under the group criteria
    slots = 32 if head_mode[0] == "body" else 64
    ws["mask_fill"] = (head["n2b"] + head["nbc"]) / max(1, slots * (ws["entries_body"] + ws["entries_cell"]))

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": ("synthetic: Plummer sphere drawn as mkplummer does (ran3, seed=1)" if wl == "plummer" else
                 "synthetic: Hernquist sphere (project generator, ran3 seed=7)"),
        "config": workload_config(n, head_mode, wl),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 48 * n, "d2h_bytes_per_step": 32 * n,
                "calls": "hc_evaluate_host: positions and previous accelerations in (the latter beside the "
                         "build), accelerations and potentials out"},
        "gpu_launches": head["launches"],
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": "k_walk<quad> (headline criterion)",
                     "peak_source": "measured live: FP32 FMA chain kernel (hc_fp32_peak), FMA = 2 flops",
                     "flops_per_launch": flops},
        "roofline_build": roofline_build,
        "ratios": ratios,
        "headline": {"mode": list(head_mode), "rms": head_err[0], "p99": head_err[1],
                     "target_rms": target, "guard": guard, "build_ms": head["build_ms"],
                     "walk_ms": head["walk_ms"], "interactions": head["n2b"] + head["nbc"]},
        "comparisons": comp,
        "calibration": {"fixed_theta_0.5": fixed, "error_rule": cal_err, "learned": cal_lrn, "treecode1": cal_tc1,
                        "fixed_theta_1e-3": cal_th, "error_rule_1e-3": cal_err2, "learned_1e-3": cal_lrn2},
        "training": train,
        "tuning": {"fixed_theta": tuned, "group_criteria": TUNING["group"]},
        "interactions_per_s": world * (head["n2b"] + head["nbc"]) / (mean_ms * 1e-3),
        "walk_stats": ws,
        "wall_s_timed_loop": wall,
        "force_error": {"rms": head_err[0], "p99": head_err[1], "sample": int(len(idx)),
                        "against": "FP64 direct sum (GPU)"},
        "clocks": clocks,
    }
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        pos = np.ascontiguousarray(ph[:, 0])
        v, tb, rate, kind, what = cpu_baseline_one_core(n, m, pos, eps, args.cpu_sample)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": kind,
                               "sample": f"{what}, fixed theta {TOL}, one core ({cpu_model()}): full tree build of "
                                         f"{n} bodies ({tb:.2f} s) + walks of {args.cpu_sample} uniformly sampled "
                                         f"bodies ({rate:.0f} bodies/s), extrapolated to one full evaluation"}
    ctx.close()
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        out["workloads"] = companion_workloads()
    if rank == 0:
        print(json.dumps(out), flush=True)


# the other configurations, each a short run of its own workload in a child
# process (the headline's context is closed first); their lines are
# summarised under "workloads" so that one default run records all of them
COMPANIONS = (
    ("plummer-run", ["--workload", "plummer-run", "--no-cpu-baseline"],
     ("value", "unit", "ms_per_step", "steps", "ratio_learned_vs_fixed_theta", "rms_error", "clocks")),
    ("hernquist", ["--workload", "hernquist", "--steps", "5", "--warmup", "2", "--no-cpu-baseline"],
     ("value", "unit", "ms_per_step", "steps", "ratios", "e2e", "force_error", "clocks")),
    ("ensemble", ["--workload", "ensemble", "--steps", "5", "--warmup", "2"],
     ("value", "unit", "ms_per_step", "steps", "phase_ms", "tuning", "energy_drift", "clocks")),
    ("galaxy", ["--workload", "galaxy", "--generator", "device", "--steps", "100", "--warmup", "2"],
     ("value", "unit", "ms_per_step", "steps", "evaluation_ms", "rms_error", "energy_drift",
      "angular_momentum_drift", "guard", "clocks")),
)


def companion_workloads(timeout_s=600):
    res = {}
    for name, argv, keys in COMPANIONS:
        t0 = time.perf_counter()
        try:
            p = subprocess.run([sys.executable, os.path.abspath(__file__)] + argv, capture_output=True, text=True,
                               timeout=timeout_s)
            lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
            if p.returncode != 0 or not lines:
                res[name] = {"error": f"exit {p.returncode}: {p.stderr.strip().splitlines()[-1:]}"}
                continue
            d = json.loads(lines[-1])
            res[name] = {k: d[k] for k in keys if k in d}
            res[name]["metric"] = d.get("metric")
            if name == "plummer-run":
                res[name]["runs"] = {k: {"body_steps_per_s": v.get("body_steps_per_s"),
                                         "energy_drift": v.get("energy_drift"),
                                         "angular_momentum_drift": v.get("angular_momentum_drift")}
                                     for k, v in d.get("runs", {}).items()}
        except subprocess.TimeoutExpired:
            res[name] = {"error": f"timed out after {timeout_s} s"}
        res[name]["wall_s"] = round(time.perf_counter() - t0, 1)
    return res


# ---------------------------------------------------------------- config-2 leapfrog run

RUN_DT = 1.0 / 128


def run_plummer_run(args, world, rank, local):
    """The second configuration as specified: Plummer N=1,048,576 (mkplummer
    seed=1), tol=0.5, eps=0.01, quadrupoles; one force evaluation plus
    `--steps` (default 100) leapfrog steps at dt=1/128 with the FP64 state
    (stepsystem, code.c:159-191), once with the reference's fixed-theta rule
    and once with the learned criterion (guard on) at the fixed rule's RMS
    force error.  Each step is one CUDA-graph replay (build, walk with the
    closing half-kick, diagnostics) and the kick-drift; FP64 energy and
    angular-momentum drift and guard trips are reported."""
    import torch
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode as hc
    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (the CUDA path has no CPU fallback)")
    torch.cuda.set_device(local)
    n = args.n if args.n else N_DEFAULT
    m, ph = hc.mkplummer(n, SEED)
    ctx = hc.Context(n, tol=TOL, eps=EPS, fcells=1.0, usequad=USEQUAD)
    ctx.upload(m, ph)
    ctx.evaluate()
    TUNING["body"] = ctx.autotune()
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(n, size=min(args.sample, n), replace=False)).astype(np.int64)
    ea, _ = ctx.direct_sample(idx)
    fixed = point(ctx, ("body", TOL), idx, ea)
    err_pt, _ = calibrate(ctx, idx, ea, lambda e: ("error", e), 1e-3, 64.0, fixed["rms"])
    set_mode(ctx, ("body", TOL))
    ctx.evaluate()
    tg = TUNING["group"]
    ctx.set_tuning(tg["group_max"], tg["list_depth"], tg["grouping"])
    train = ctx.learn_from_self(theta=err_pt["mode"][1] if err_pt else 0.03, target=1 << 20,
                                band=tuple(args.train_band))
    ctx.learn_band(*args.band)
    lrn_pt, _ = calibrate(ctx, idx, ea, lambda e: ("learned", e, LEARNED_THRESHOLD), 1e-3, 64.0, fixed["rms"])
    runs = {}
    with ClockSampler(local) as clk:
        for name, mode, guard in (("fixed_theta_0.5", ("body", TOL), False),
                                  ("learned", tuple(lrn_pt["mode"]) if lrn_pt else ("body", TOL), True)):
            set_mode(ctx, mode)
            ctx.set_guard(GUARD_SAMPLE if guard else 0, RMS_BUDGET, seed=1)
            ctx.upload(m, ph)                                   # the run starts from the initial conditions
            d0, _, _, _ = ctx.step(RUN_DT, 0)                   # the first force evaluation
            e0, l0 = d0.etot[0], angular_momentum(d0)
            barrier(world)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for k in range(1, args.steps + 1):
                d, _, _, _ = ctx.step(RUN_DT, k)
            torch.cuda.synchronize()
            secs = time.perf_counter() - t0
            ms = reduce_max(1e3 * secs / args.steps, world)
            runs[name] = {"mode": list(mode), "ms_per_step": ms, "body_steps_per_s": world * n / (ms * 1e-3),
                          "energy_drift": abs((d.etot[0] - e0) / e0),
                          "angular_momentum_drift": float(np.linalg.norm(angular_momentum(d) - l0)
                                                          / max(np.linalg.norm(l0), 1e-300)),
                          "interactions_last_step": int(d.n2b + d.nbc)}
            if guard:
                runs[name]["guard"] = ctx.guard_stats()
    ctx.set_guard(0)
    head = runs["learned"]
    out = {
        "metric": "Plummer N=1M leapfrog body-steps/s (config 2: one evaluation + 100 steps at dt=1/128)",
        "value": head["body_steps_per_s"], "unit": "body-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": 1, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: Plummer sphere drawn as mkplummer does (ran3, seed=1)",
        "config": {"workload": f"plummer N={n} seed={SEED} (mkplummer), tol={TOL}, eps={EPS}, quadrupole, "
                               f"dt=1/128, {args.steps} steps after the first evaluation, FP64 leapfrog state",
                   "timing": "host wall clock over the steps (each step one CUDA-graph replay, synchronised)",
                   "l2": "working set larger than L2 (no flush)"},
        "runs": runs,
        "ratio_learned_vs_fixed_theta": head["body_steps_per_s"] / runs["fixed_theta_0.5"]["body_steps_per_s"],
        "rms_error": {"fixed_theta_0.5": fixed["rms"], "learned": lrn_pt["rms"] if lrn_pt else None,
                      "sample": int(len(idx)), "against": "FP64 direct sum (GPU), initial conditions"},
        "training": train,
        "clocks": clk.summary(),
    }
    ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


# ---------------------------------------------------------------- ensemble workload

ENS_NSYS, ENS_NMIN, ENS_NMAX, ENS_SEED = 4096, 64, 16384, 1
ENS_EPS, ENS_DT, ENS_TOL, ENS_DIRECT_MAX = 0.02, 1.0 / 256, 0.6, 1024


def ensemble_systems(nsys=ENS_NSYS, seed=ENS_SEED):
    """Body counts log-uniform in [64, 16384] from a seeded generator; system i
    is mkplummer(N_i, seed + i)."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(ENS_NMIN), np.log(ENS_NMAX), nsys))).astype(np.int64)


def run_ensemble(args, world, rank, local):
    import torch
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode as hc
    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (the CUDA path has no CPU fallback)")
    torch.cuda.set_device(local)
    counts = ensemble_systems(args.nsys)
    ms, phs = [], []
    for i, n in enumerate(counts):
        m, ph = hc.mkplummer(int(n), ENS_SEED + i)
        ms.append(m)
        phs.append(ph)
    m, ph = np.concatenate(ms), np.concatenate(phs)
    ntot = int(counts.sum())
    ens = hc.Ensemble(counts, tol=ENS_TOL, eps=ENS_EPS, usequad=False, direct_max=ENS_DIRECT_MAX)
    ens.upload(m, ph)
    e0 = ens.step(ENS_DT, 0, energy=True)
    tuning = ens.autotune()                  # walk groups and direct-sum block size, timed on these bodies
    for k in range(1, args.warmup + 1):
        ens.step(ENS_DT, k)
    barrier(world)
    step_s, tree_ms, direct_ms = [], [], []
    with ClockSampler(local) as clk:
        for k in range(args.warmup + 1, args.warmup + 1 + args.steps):
            t0 = time.perf_counter()
            e1 = ens.step(ENS_DT, k, energy=(k == args.warmup + args.steps))
            step_s.append(time.perf_counter() - t0)
            inf = ens.info()
            tree_ms.append(inf["tree_ms"])
            direct_ms.append(inf["direct_ms"])
    barrier(world)
    inf = ens.info()
    mean_ms = reduce_max(1e3 * statistics.mean(step_s), world)
    value = world * ntot / (mean_ms * 1e-3)
    drift = np.abs((e1[:, 2] - e0[:, 2]) / e0[:, 2])
    out = {
        "metric": "ensemble leapfrog body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: Plummer spheres drawn as mkplummer does (ran3, seed 1 + i)",
        "config": {"workload": f"ensemble of {len(counts)} Plummer spheres, N log-uniform in "
                               f"[{ENS_NMIN},{ENS_NMAX}] ({ntot} bodies), eps={ENS_EPS}, dt=1/256; "
                               f"N<={ENS_DIRECT_MAX}: FP32 direct sum, larger: tree at tol={ENS_TOL}",
                   "l2": "working set larger than L2 (no flush)", "timing": "host wall clock per step "
                   "(each step is one CUDA-graph launch followed by a stream synchronisation)"},
        "gpu_launches": inf["launches"] * args.steps,
        "phase_ms": {"tree": statistics.mean(tree_ms), "direct": statistics.mean(direct_ms)},
        "tuning": tuning,
        "systems": {"tree": inf["nsys_tree"], "direct": inf["nsys_direct"], "bodies_tree": inf["bodies_tree"],
                    "bodies_direct": inf["bodies_direct"]},
        "interactions_per_s": (inf["interactions_tree"] + inf["interactions_direct"]) / (mean_ms * 1e-3),
        "energy_drift": {"median": float(np.median(drift)), "max": float(drift.max()),
                         "steps": args.warmup + args.steps},
        "clocks": clk.summary(),
    }
    ens.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


# ---------------------------------------------------------------- composite galaxy workload

GAL_N = (4194304, 1048576, 11534336)      # disk, bulge, halo: 2^24 bodies
GAL_SEED, GAL_EPS, GAL_DT = 11, 0.01, 1.0 / 512


def angular_momentum(d):
    a = np.array(d.amten).reshape(3, 3)      # antisymmetric: L = (A_yz, A_zx, A_xy)
    return np.array([a[1, 2], a[2, 0], a[0, 1]])


def run_galaxy(args, world, rank, local):
    """Leapfrog steps of the composite disk galaxy with the learned criterion
    (calibrated to the fixed-theta rule's RMS error, guard on), each step one
    CUDA-graph replay (build, walk with the closing half-kick, diagnostics),
    then kick-drift; FP64 energy and angular-momentum drift."""
    import torch
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode as hc
    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device (the CUDA path has no CPU fallback)")
    torch.cuda.set_device(local)
    n = sum(GAL_N)
    ctx = hc.Context(n, tol=TOL, eps=GAL_EPS, fcells=1.0, usequad=USEQUAD)
    if args.generator == "host":
        t0 = time.perf_counter()
        m, ph = hc.mkgalaxy(*GAL_N, seed=GAL_SEED)
        t_gen = time.perf_counter() - t0

    def initial_conditions():
        if args.generator == "host":
            ctx.upload(m, ph)
        else:
            ctx.generate("galaxy", GAL_SEED, list(GAL_N[:2]))

    if args.generator == "device":
        t0 = time.perf_counter()
        initial_conditions()
        t_gen = time.perf_counter() - t0
    initial_conditions()
    ctx.evaluate()
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(n, size=min(args.sample, 4096), replace=False)).astype(np.int64)
    ea, _ = ctx.direct_sample(idx)
    tg = TUNING["group"]                     # labels from the groups the learned walk uses
    ctx.set_tuning(tg["group_max"], tg["list_depth"], tg["grouping"])
    train = ctx.learn_from_self(theta=args.train_theta or 0.03, target=1 << 20, band=tuple(args.train_band))
    ctx.learn_band(*args.band)
    fixed = point(ctx, ("body", TOL), idx, ea)
    lrn_pt, cal = calibrate(ctx, idx, ea, lambda e: ("learned", e, LEARNED_THRESHOLD), 1e-3, 64.0, fixed["rms"],
                            steps=5)
    mode = tuple(lrn_pt["mode"]) if lrn_pt else ("body", TOL)
    set_mode(ctx, mode)
    ctx.set_guard(GUARD_SAMPLE, RMS_BUDGET, seed=1)
    # start the run from the initial conditions
    initial_conditions()
    d0, _, _, _ = ctx.step(GAL_DT, 0)
    e0, l0 = d0.etot[0], angular_momentum(d0)
    for k in range(1, args.warmup + 1):
        ctx.step(GAL_DT, k)
    barrier(world)
    step_ms = []
    with ClockSampler(local) as clk:
        for k in range(args.warmup + 1, args.warmup + 1 + args.steps):
            t1 = time.perf_counter()
            d, _, _, _ = ctx.step(GAL_DT, k)
            step_ms.append(1e3 * (time.perf_counter() - t1))
    barrier(world)
    guard = ctx.guard_stats()
    l1 = angular_momentum(d)
    mean_ms = reduce_max(statistics.mean(step_ms), world)
    out = {
        "metric": "composite galaxy leapfrog body-steps/s", "value": world * n / (mean_ms * 1e-3),
        "unit": "body-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: composite disk galaxy (project generator, " +
                ("ran3 seed=11)" if args.generator == "host" else "device counter-based streams, seed=11)"),
        "config": {"workload": f"disk {GAL_N[0]} + Hernquist bulge {GAL_N[1]} + NFW halo {GAL_N[2]} bodies, "
                               f"eps={GAL_EPS}, dt=1/512, quadrupole, learned criterion (guarded), one CUDA graph "
                               f"per step", "criterion_setting": list(mode),
                   "timing": "host wall clock per step (graph replay, synchronised)"},
        "energy_drift": abs((d.etot[0] - e0) / e0),
        "angular_momentum_drift": float(np.linalg.norm(l1 - l0) / np.linalg.norm(l0)),
        "steps_total": args.warmup + 1 + args.steps,
        "rms_error": {"learned": lrn_pt["rms"] if lrn_pt else None, "fixed_theta_0.5": fixed["rms"],
                      "sample": int(len(idx))},
        "evaluation_ms": {"learned": lrn_pt["step_ms"] if lrn_pt else None, "fixed_theta_0.5": fixed["step_ms"]},
        "calibration": cal, "training": train, "guard": guard,
        "generator": {"where": args.generator, "seconds": t_gen},
        "clocks": clk.summary(),
    }
    ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


# ---------------------------------------------------------------- gyrfalcON (falcON) CPU baseline

# falcON opening angles (theta_min of its mass-dependent theta(M), Plummer kernel, eps=0.01) at which
# its RMS relative force error on this file's 16,384-body sample of the headline system equals the
# fixed-theta rule's (tol 0.5: 3.62e-4) and 1e-3; found by oracle/calibrate_falcon.py (bisection
# against an FP64 direct sum): RMS 3.59e-4 and 9.85e-4 there.
FALCON_THETA = {"equal_rms_fixed_theta_0.5": 0.1587, "rms_1e-3": 0.2457}


def _fork_map(fn, items):
    """Run fn(item) in one forked worker per item; returns the results (pickled through pipes)."""
    import pickle
    kids = []
    for it in items:
        r, w = os.pipe()
        pid = os.fork()
        if pid == 0:
            os.close(r)
            try:
                data = pickle.dumps(fn(it))
                with os.fdopen(w, "wb") as f:
                    f.write(data)
            finally:
                os._exit(0)
        os.close(w)
        kids.append((pid, r))
    out = []
    for pid, r in kids:
        with os.fdopen(r, "rb") as f:
            data = f.read()
        os.waitpid(pid, 0)
        if not data:
            raise RuntimeError("bench.py: a worker failed")
        out.append(pickle.loads(data))
    return out


def falcon_leg(m, pos, eps, procs: int, nsample: int = 1024):
    """gyrfalcON's force solver (falcON, compiled from the NEMO sources) at the
    calibrated opening angles: one evaluation (tree + gravity of every body)
    per forked process, `procs` at once; RMS relative force error of one of
    them on `nsample` sampled bodies against an FP64 direct sum (oracle)."""
    import subprocess
    from oracle import oracle as O
    src = O.reference_sources()
    if src is None:
        return {"unavailable": "NEMO sources absent (falcON not staged)"}
    try:
        subprocess.run(["make", "-s", f"-j{min(procs, 16)}", "-C", os.path.join(ROOT, "oracle"), "falcon",
                        f"REFDIR={src}"], check=True, capture_output=True)
    except subprocess.CalledProcessError as e:
        return {"unavailable": "falcON build failed: " + (e.stderr or b"").decode()[-300:]}
    n = len(m)
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(n, size=nsample, replace=False)).astype(np.int64)
    chunks = np.array_split(idx, procs)
    parts = _fork_map(lambda ch: O.direct(m, pos, test_pos=pos[ch], eps=eps, skip=ch.astype(np.int32))[0], chunks)
    ea = np.concatenate(parts)
    out = {"kernel": 0, "eps": eps, "theta_mode": "theta(M), minimum theta as given (gyrfalcON's default mode)",
           "cores": procs, "cpu": cpu_model(), "precision": "FP32 (falcON's default build)"}
    for name, theta in FALCON_THETA.items():
        if theta is None:
            continue

        def one(k, theta=theta):
            acc, _, tg, tv = O.Falcon.get().forces(m, pos, eps, theta, kernel=0)
            rel = None
            if k == 0:
                r = np.linalg.norm(acc[idx] - ea, axis=1) / np.linalg.norm(ea, axis=1)
                rel = float(np.sqrt(np.mean(r ** 2)))
            return tg, tv, rel

        t0 = time.perf_counter()
        res = _fork_map(one, range(procs))
        wall = time.perf_counter() - t0
        single = statistics.median(r[0] + r[1] for r in res)
        out[name] = {"theta": theta, "rms_sampled": res[0][2], "sample": nsample,
                     "seconds_per_evaluation_one_core": single, "bodies_per_s_one_core": n / single,
                     "bodies_per_s_all_cores": procs * n / wall,
                     "all_cores": f"{procs} independent evaluations at once (nemo.bench np= style), wall {wall:.1f} s"}
    return out


# ---------------------------------------------------------------- reference arm

def run_reference(args, world, rank):
    """The reference's own CPU implementation of the path on the host cores:
    every step is one complete force evaluation of the headline workload
    (maketree + hackcofm, then hackgrav of every body; fixed theta 0.5,
    eps 0.01, quadrupoles), the walks split over all host cores."""
    if rank != 0:
        return
    from oracle import oracle as O
    n = args.n if args.n else N_DEFAULT
    m, ph = O.mkplummer(n, SEED)
    pos = np.ascontiguousarray(ph[:, 0])
    procs = host_cores()
    w = RefWalker(n)
    secs, totals = [], None
    wall0 = time.perf_counter()
    for i in range(args.warmup + args.steps):
        t, n2b, nbc = full_evaluation(w, m, pos, EPS, procs)
        if i >= args.warmup:
            secs.append(t)
        totals = (n2b, nbc)
    wall = time.perf_counter() - wall0
    mean_s = statistics.mean(secs)
    value = n / mean_s
    sample = (f"{w.what}; each step one complete evaluation of all {n} bodies: serial tree build, then "
              f"hackgrav of every body split over {procs} forked processes ({cpu_model()})")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_s * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic: Plummer (ran3, seed=1)",
           "config": dict(workload_config(n), l2="not applicable (host cores)",
                          parallelism=f"{procs} host processes (walk split by bodies)"),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": w.kind, "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "interactions": {"n2b": totals[0], "nbc": totals[1]},
           "wall_s": wall}
    if not args.no_falcon:
        out["gyrfalcON"] = falcon_leg(m, pos, EPS, procs)
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 10; plummer-run: 100)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=0, help="bodies (default: the workload's)")
    ap.add_argument("--sample", type=int, default=16384, help="bodies for the FP64 force-error sample")
    ap.add_argument("--cpu-sample", type=int, default=32768,
                    help="bodies walked by the one-core CPU baseline (about 5-10 s)")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="GPU headline only: no CPU baseline and no companion workload runs")
    ap.add_argument("--no-falcon", action="store_true", help="reference arm: skip the gyrfalcON (falcON) leg")
    ap.add_argument("--workload", default="plummer",
                    choices=["plummer", "plummer-run", "hernquist", "ensemble", "galaxy"],
                    help="plummer: the headline (N=1M); plummer-run: the same system, one evaluation + "
                         "100 leapfrog steps; hernquist: N=4M, eps=0.005; "
                         "ensemble: 4096 independent systems; galaxy: 2^24-body disk galaxy, leapfrog")
    ap.add_argument("--nsys", type=int, default=ENS_NSYS)
    ap.add_argument("--train-theta", type=float, default=0.0,
                    help="learned criterion: error budget of the label walk (default: the error rule's equal-RMS budget)")
    ap.add_argument("--train-band", type=float, nargs=2, default=[1.0, 16.0],
                    help="learned criterion: band lo hi sampled for training, -lo <= log2(proxy/budget) <= hi")
    ap.add_argument("--band", type=float, nargs=2, default=[0.5, 16.0],
                    help="learned criterion: band lo hi the network decides, -lo <= log2(proxy/budget) <= hi")
    ap.add_argument("--generator", default="host", choices=["host", "device"],
                    help="galaxy workload: draw the bodies with mkgalaxy on the host or hc_generate on the device")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 100 if args.workload == "plummer-run" else 10
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "ensemble":
        run_ensemble(args, world, rank, local)
    elif args.workload == "galaxy":
        run_galaxy(args, world, rank, local)
    elif args.workload == "plummer-run":
        run_plummer_run(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
