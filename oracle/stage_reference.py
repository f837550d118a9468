"""Stage the NEMO sources that the oracle's `ref` and `falcon` builds compile.

TEST INFRASTRUCTURE ONLY.  `oracle/Makefile ref` compiles the reference's own
hackcode1 load.c / grav.c and ran3.c (with oracle/ref_driver.c) into
oracle/_ref; `oracle/Makefile falcon` compiles falcON's force solver (the
engine of gyrfalcON, usr/dehnen/falcON) with its C interface into
oracle/_ref/libfalcon.so.  This script copies exactly those sources and the
headers they include, unchanged, from a NEMO source tree into
baseline/_ref/nemo (which is git-ignored and travels with the repository copy
to hosts where the NEMO tree itself is absent), so that the same recipes build
the reference there:

    python oracle/stage_reference.py            # NEMO tree from $NEMO_REFDIR

The NEMO tree is taken from $NEMO_REFDIR, else from /root/reference (the
read-only checkout on the machine that builds the fixtures).
"""
from __future__ import annotations

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STAGED = os.path.join(ROOT, "baseline", "_ref", "nemo")

HC1 = "src/nbody/evolve/hackcode/hackcode1"
FILES = [
    f"{HC1}/load.c", f"{HC1}/grav.c", f"{HC1}/code.h", f"{HC1}/defs.h", f"{HC1}/proto.h",
    "src/kernel/numrec/ran3.c",
    "src/nbody/evolve/hackcode/treecode1/treeload.c", "src/nbody/evolve/hackcode/treecode1/treedefs.h",
    "src/nbody/evolve/hackcode/treecode1/treecode.h",
    "src/orbit/potential/data/plummer.c", "src/orbit/potential/data/hernquist.c",
    "src/orbit/potential/data/miyamoto.c", "src/orbit/potential/data/log.c", "inc/potential_float.h",
    f"{HC1}/code_io.c", "src/kernel/io/filesecret.c", "src/kernel/io/filesecret.h", "src/kernel/io/extstring.c",
    "src/kernel/io/convert.c", "src/kernel/io/ieeehalfprecision.c", "src/kernel/io/stropen.c",
    "src/kernel/cores/strlib.c", "src/kernel/cores/bswap.c", "inc/extstring.h", "inc/filestruct.h",
    "inc/history.h", "inc/strlib.h", "inc/snapshot/snapshot.h", "inc/snapshot/get_snap.c",
    "inc/snapshot/get_snap-old.c", "inc/snapshot/put_snap.c", "inc/snapshot/put_snap-old.c",
    "inc/stdinc.h", "inc/vectmath.h", "inc/mathfns.h", "inc/getparam.h", "inc/options.h",
]
# falcON's library without NEMO I/O (its makepub's non-NEMO object list, less
# PotExp, which needs Sun RPC headers) and the WDutils sources it links
FALCON = "usr/dehnen/falcON"
UTILS = "usr/dehnen/utils"
FALCON_LIB = ["basic", "body", "tree", "gravity", "kernel", "partner", "nbody", "forcesC", "sample",
              "neighbours"]
UTILS_LIB = ["WDMath", "exception", "io", "numerics", "random"]
FILES += [f"{FALCON}/src/public/lib/{f}.cc" for f in FALCON_LIB]
FILES += [f"{UTILS}/src/{f}.cc" for f in UTILS_LIB]
DIRS = [f"{FALCON}/inc", f"{UTILS}/inc"]       # headers, copied whole
# falcON's build links falcON/inc/utils to utils/inc; the staged copy holds a copy there
COPIES = {f"{FALCON}/inc/utils": f"{UTILS}/inc"}


def source_dir() -> str | None:
    """The NEMO source tree to stage from, or None where there is none."""
    d = os.environ.get("NEMO_REFDIR") or "/root/reference"
    return d if os.path.isfile(os.path.join(d, HC1, "load.c")) else None


def staged() -> str | None:
    """The staged copy, when complete."""
    ok = all(os.path.isfile(os.path.join(STAGED, f)) for f in FILES)
    ok = ok and all(os.path.isdir(os.path.join(STAGED, d)) for d in DIRS + list(COPIES))
    return STAGED if ok else None


def stage(src: str | None = None) -> str | None:
    """Copy FILES from the NEMO tree into baseline/_ref/nemo; returns the
    staged directory, or None when no NEMO tree is present."""
    src = src or source_dir()
    if src is None:
        return staged()
    for f in FILES:
        dst = os.path.join(STAGED, f)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(src, f), dst)
    for d in DIRS:
        shutil.copytree(os.path.join(src, d), os.path.join(STAGED, d), symlinks=False, dirs_exist_ok=True,
                        copy_function=shutil.copyfile)
    for dst, d in COPIES.items():
        shutil.copytree(os.path.join(src, d), os.path.join(STAGED, dst), symlinks=False, dirs_exist_ok=True,
                        copy_function=shutil.copyfile)
    return STAGED


if __name__ == "__main__":
    out = stage()
    if out is None:
        sys.exit("no NEMO source tree found (set NEMO_REFDIR)")
    print(out)
