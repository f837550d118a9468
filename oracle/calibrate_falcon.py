"""Opening angle at which falcON (gyrfalcON's force solver) matches a force error.

TEST INFRASTRUCTURE ONLY (the benchmark's CPU baseline).  For the headline
system (mkplummer N=1,048,576 seed=1, Plummer softening eps=0.01, kernel=0)
this finds, by bisection, the largest falcON opening angle theta_min
(falcON's default mass-dependent theta(M), as gyrfalcON uses it) whose RMS
relative force error on the benchmark's sample (16,384 bodies drawn with
numpy default_rng(12345), as bench.py draws them) stays within a target,
against an FP64 direct sum computed here by the oracle (worker processes).

    python oracle/calibrate_falcon.py 3.62e-4 1e-3

prints one JSON line: {"target": theta, ...} for each target RMS.  The
results are recorded in bench.py (FALCON_THETA).
"""
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

N, SEED, EPS, NSAMPLE, SAMPLE_SEED = 1 << 20, 1, 0.01, 16384, 12345


def _direct(args):
    lo, hi = args
    from oracle import oracle as O
    m, ph = O.mkplummer(N, SEED)
    pos = ph[:, 0].copy()
    idx = sample()[lo:hi]
    a, _ = O.direct(m, pos, test_pos=pos[idx], eps=EPS, skip=idx.astype(np.int32))
    return lo, a


def sample():
    rng = np.random.default_rng(SAMPLE_SEED)
    return np.sort(rng.choice(N, size=NSAMPLE, replace=False)).astype(np.int64)


def main(targets):
    from oracle import oracle as O
    O.build(ref=None)
    subprocess_make = ["make", "-s", "-j8", "-C", HERE, "falcon", f"REFDIR={O.reference_sources()}"]
    import subprocess
    subprocess.run(subprocess_make, check=True)
    m, ph = O.mkplummer(N, SEED)
    pos = ph[:, 0].copy()
    idx = sample()
    nproc = os.cpu_count() or 1
    edges = np.linspace(0, NSAMPLE, nproc + 1).astype(int)
    ea = np.zeros((NSAMPLE, 3))
    with mp.get_context("spawn").Pool(nproc) as pool:
        for lo, a in pool.imap_unordered(_direct, list(zip(edges[:-1], edges[1:]))):
            ea[lo:lo + len(a)] = a
    F = O.Falcon.get()
    cache = {}

    def rms(theta):
        if theta not in cache:
            acc, _, tg, tv = F.forces(m, pos, EPS, theta, kernel=0)
            rel = np.linalg.norm(acc[idx] - ea, axis=1) / np.linalg.norm(ea, axis=1)
            cache[theta] = (float(np.sqrt(np.mean(rel ** 2))), tg + tv)
        return cache[theta]

    for target in targets:
        lo, hi = 0.05, 0.6
        while rms(lo)[0] > target:
            lo *= 0.7
        for _ in range(8):
            mid = (lo * hi) ** 0.5
            if rms(mid)[0] <= target:
                lo = mid
            else:
                hi = mid
        r, s = rms(lo)
        print(json.dumps({"target_rms": target, "theta": lo, "rms": r, "seconds": s}), flush=True)


if __name__ == "__main__":
    main([float(x) for x in sys.argv[1:]] or [3.62e-4, 1e-3])
