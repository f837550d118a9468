"""Build recipe for the GB300 hackcode1 library and programs.

Compiles the CUDA sources in nemo_gb300/csrc for sm_103a only into
nemo_gb300/libhackcode_gpu.so (the C ABI of include/hackcode_gpu.h), and the
drop-in programs hackcode1 / hackforce (C++ host code) linked against it.
In-tree build, translation units compiled in parallel, no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhackcode_gpu.so")

CU_SOURCES = ["hc_sort.cu", "hc_tree.cu", "hc_walk.cu", "hc_step.cu", "hc_api.cu", "hc_noalloc.cu", "hc_learn.cu", "hc_guard.cu", "hc_ensemble.cu", "hc_gen.cu"]
HOST_LIB_SOURCES = ["nemo_io.cpp", "galaxy.cpp"]
PROGRAMS = {"hackcode1": "hackcode1_main.cpp", "hackforce": "hackforce_main.cpp"}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd, log=None):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("build step failed: " + " ".join(cmd))
    if log:
        with open(log, "w") as f:
            f.write(r.stdout)
    return r.stdout


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    import platform
    stamp = os.path.join(BUILD, "machine")
    here = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != here:
        # objects from another machine (x86 build host vs Arm GPU host): rebuild all
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
        if os.path.exists(LIB):
            os.remove(LIB)
        with open(stamp, "w") as f:
            f.write(here)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "hackcode_gpu.h"))
    objs = []
    jobs = []
    for src in CU_SOURCES + HOST_LIB_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if _newer(obj, [path] + headers):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc()] + NVCC_FLAGS + ["-c", path, "-o", obj]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-c", path, "-o", obj]
        jobs.append((cmd, os.path.join(BUILD, src + ".log")))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda j: _run(*j), jobs))
    if jobs or not os.path.exists(LIB):
        _run([nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"])
    for prog, src in PROGRAMS.items():
        path = os.path.join(CSRC, src)
        out = os.path.join(PKG, "bin", prog)
        if not os.path.exists(path):
            continue
        os.makedirs(os.path.dirname(out), exist_ok=True)
        deps = [path, LIB, os.path.join(CSRC, "nemo_io.h")]
        if _newer(out, deps):
            continue
        _run(["g++"] + CXX_FLAGS + [path, "-o", out, "-I" + CSRC, "-I" + os.path.join(ROOT, "include"),
              "-L" + PKG, "-lhackcode_gpu", "-Wl,-rpath,$ORIGIN/..", "-lm"])
    if verbose:
        for src in CU_SOURCES:
            log = os.path.join(BUILD, src + ".log")
            if os.path.exists(log):
                print(open(log).read())
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
