"""Golden fixture of the large force evaluation: Plummer N=1,048,576.

The input is mkplummer's model with seed=1 (src/nbody/init/mkplummer.c:257-422,
drawn by the oracle's restatement, which reproduces mkplummer's published
fingerprints), evaluated with tol=0.5, eps=0.01 and quadrupoles -- the
reference hackforce_qp / hackcode1_qp force evaluation.

Everything stored comes from the reference's own load.c / grav.c (compiled
unchanged into oracle/_ref by oracle/Makefile):

* the root box after maketree (load.c:32-62);
* SHA-256 digests of the cell set in canonical order (level, integer corner,
  body count, FP64 mass, FP64 centre of mass, FP64 quadrupole) and of each
  body's parent level -- 505,787 cells are too many to store;
* every body's interaction counts from hackgrav (grav.c:22-32), as totals and
  as a digest of the per-body int32 arrays;
* acceleration, potential and counts of 16,384 bodies drawn uniformly
  without replacement (numpy default_rng(20241204)), each skipping itself.

The walk of all 1,048,576 bodies runs in worker processes (each loads the
reference library, builds the same tree and walks a contiguous share).  The
oracle's tree is checked bit for bit against the reference's here.

    python tests/golden/make_golden_plummer1m.py     (about a minute on 8 cores)
"""
import hashlib
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "plummer1m_s1_qp.npz")
N, SEED, TOL, EPS = 1 << 20, 1, 0.5, 0.01
NSAMPLE, SAMPLE_SEED = 16384, 20241204


def canon(d):
    k = np.lexsort((d["corner"][:, 2], d["corner"][:, 1], d["corner"][:, 0], d["level"]))
    return {f: np.ascontiguousarray(d[f][k]) for f in ("level", "corner", "count", "mass", "cm", "quad")}


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def inputs():
    from oracle import oracle as O
    m, ph = O.mkplummer(N, SEED)
    return m, ph[:, 0].copy()


def _share(args):
    lo, hi = args
    from oracle import oracle as O
    m, pos = inputs()
    R = O.Reference.get(True, N)
    R.build(m, pos)
    _, _, b, c = R.forces_idx(TOL, EPS, np.arange(lo, hi, dtype=np.int32))
    return lo, b, c


def main():
    from oracle import oracle as O
    O.build(ref=True)
    m, pos = inputs()
    R = O.Reference.get(True, N)
    rmin, rsize = R.build(m, pos)
    d = R.dump()
    c = canon(d)
    # the oracle's maketree/hackcofm is the reference's, bit for bit
    T = O.Tree(N, 1.0)
    assert T.build(m, pos, True) == 0
    oc = canon(T.dump())
    for f in c:
        assert np.array_equal(c[f], oc[f]), f
    rng = np.random.default_rng(SAMPLE_SEED)
    idx = np.sort(rng.choice(N, NSAMPLE, replace=False)).astype(np.int32)
    acc, phi, sb, sc = R.forces_idx(TOL, EPS, idx)

    nproc = max(1, min(16, os.cpu_count() or 1))
    edges = np.linspace(0, N, nproc + 1).astype(int)
    n2b = np.zeros(N, np.int64)
    nbc = np.zeros(N, np.int64)
    with mp.get_context("spawn").Pool(nproc) as pool:
        for lo, b, cc in pool.imap_unordered(_share, list(zip(edges[:-1], edges[1:]))):
            n2b[lo:lo + len(b)] = b
            nbc[lo:lo + len(cc)] = cc
    assert np.array_equal(n2b[idx], sb) and np.array_equal(nbc[idx], sc)
    out = dict(
        n=N, seed=SEED, tol=TOL, eps=EPS,
        input_digest=digest(m, pos),
        rmin=rmin, rsize=rsize, ncell=len(c["level"]),
        tree_digest=digest(c["level"], c["corner"], c["count"], c["mass"], c["cm"]),
        quad_digest=digest(c["quad"]),
        parent_digest=digest(d["body_parent_level"].astype(np.int32)),
        n2b_total=int(n2b.sum()), nbc_total=int(nbc.sum()),
        counts_digest=digest(n2b.astype(np.int32), nbc.astype(np.int32)),
        sample_idx=idx, sample_acc=acc, sample_phi=phi,
        sample_n2b=sb.astype(np.int32), sample_nbc=sc.astype(np.int32),
    )
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, "ncell", out["ncell"], "n2b", out["n2b_total"], "nbc", out["nbc_total"])


if __name__ == "__main__":
    main()
