"""Generate golden fixtures from the reference's own tree and walk.

Runs the reference's load.c / grav.c (compiled unchanged into oracle/_ref by
oracle/Makefile) on seeded inputs and stores, per case, the root box after
maketree, the cell set (level, integer corner, body count, mass, centre of
mass, quadrupole) and per-body acceleration, potential and interaction
counts.  Run from the repository root:

    python tests/golden/make_golden.py

Needs the NEMO sources (for oracle/_ref); the fixtures it writes are what the
tests use where those sources are absent.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name: (generator, n, seed, tol, eps, test points)
CASES = {
    "plummer4096_s123": ("plummer", 4096, 123, 0.7, 0.05, 0),
    "testdata128_s123": ("testdata", 128, 123, 1.0, 0.05, 0),
    "plummer2048_s7_test": ("plummer", 2048, 7, 0.5, 0.01, 257),
}


def canon(d):
    k = np.lexsort((d["corner"][:, 2], d["corner"][:, 1], d["corner"][:, 0], d["level"]))
    return {f: d[f][k] for f in ("level", "corner", "count", "mass", "cm", "quad")}


def main():
    O.build(ref=True)
    for name, (gen, n, seed, tol, eps, ntest) in CASES.items():
        m, ph = O.mkplummer(n, seed) if gen == "plummer" else O.make_testdata(n, seed)
        pos = ph[:, 0].copy()
        out = {"mass": m, "pos": pos, "tol": tol, "eps": eps}
        tp = None
        if ntest:
            rng = np.random.default_rng(seed)
            tp = rng.uniform(-1.5, 1.5, size=(ntest, 3))
            out["test_pos"] = tp
        for quad in (False, True):
            R = O.Reference.get(quad, 1 << 16)
            rmin, rsize = R.build(m, pos)
            c = canon(R.dump())
            tag = "qp" if quad else "mp"
            out[f"{tag}_rmin"] = rmin
            out[f"{tag}_rsize"] = rsize
            for f, v in c.items():
                out[f"{tag}_cell_{f}"] = v
            out[f"{tag}_body_parent_level"] = R.dump()["body_parent_level"]
            acc, phi, n2b, nbc = R.forces(tol, eps, test_pos=tp)
            out[f"{tag}_acc"] = acc
            out[f"{tag}_phi"] = phi
            out[f"{tag}_n2b"] = n2b.astype(np.int32)
            out[f"{tag}_nbc"] = nbc.astype(np.int32)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
        print("wrote", name, "ncell", len(out["qp_cell_level"]))


if __name__ == "__main__":
    main()
