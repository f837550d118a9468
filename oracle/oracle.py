"""ctypes bindings for the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline / reference arm, never by the product package.

Two libraries are wrapped:

* ``_build/libhcoracle.so`` -- the plain-C FP64 restatement of hackcode1's
  tree build, moments, walk, leapfrog and diagnostics (hackcode_oracle.c).
* ``_ref/libhcref_{mp,qp}.so`` -- the reference's own load.c / grav.c /
  ran3.c compiled unchanged (only where the NEMO sources are present; see
  oracle/Makefile).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFDIR_DEFAULT = "/root/reference"

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build(ref: bool | None = None) -> None:
    """Compile the oracle (and the reference libs when the sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    refdir = os.environ.get("NEMO_REFDIR", REFDIR_DEFAULT)
    if ref is None:
        ref = os.path.isdir(os.path.join(refdir, "src/nbody/evolve/hackcode/hackcode1"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFDIR={refdir}"], check=True)


class Params(C.Structure):
    _fields_ = [("freq", C.c_double), ("eps", C.c_double), ("tol", C.c_double),
                ("fcells", C.c_double), ("tstop", C.c_double), ("freqout", C.c_double),
                ("minor_freqout", C.c_double), ("usequad", C.c_int), ("opt_mass", C.c_int),
                ("opt_phi", C.c_int), ("opt_acc", C.c_int), ("write_out", C.c_int)]


class LogRow(C.Structure):
    _fields_ = [("tnow", C.c_double), ("etot", C.c_double * 3), ("cmphase", C.c_double * 6),
                ("nttot", C.c_int64), ("n2b", C.c_int64), ("nbc", C.c_int64),
                ("nbavg", C.c_int), ("ncavg", C.c_int)]


class Bsf(C.Structure):
    _fields_ = [("n", C.c_int64), ("sum1", C.c_double), ("sum2", C.c_double),
                ("vmin", C.c_double), ("vmax", C.c_double)]

    def text(self) -> str:
        """The bsf line 'mean sigma min max count' (bsf.c:45-88, fmt=%g)."""
        n = self.n
        if n == 0:
            return "0 0 0 0 0"
        mean = self.sum1 / n
        var = self.sum2 / n - mean * mean
        sig = 0.0 if (self.vmin == self.vmax or var <= 0) else var ** 0.5
        return "%g %g %g %g %d" % (mean, sig, self.vmin, self.vmax, n)


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "libhcoracle.so")
        if not os.path.exists(path):
            build(ref=False)
        L = C.CDLL(path)
        L.hco_xrandom_init.argtypes = [C.c_int]
        L.hco_xrandom.argtypes = [C.c_double, C.c_double]
        L.hco_xrandom.restype = C.c_double
        L.hco_make_testdata.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.hco_mkplummer.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.hco_tree_new.argtypes = [C.c_int, C.c_double]
        L.hco_tree_new.restype = C.c_void_p
        L.hco_tree_free.argtypes = [C.c_void_p]
        L.hco_tree_set_box.argtypes = [C.c_void_p, _dp, C.c_double]
        L.hco_tree_get_box.argtypes = [C.c_void_p, _dp, C.POINTER(C.c_double)]
        L.hco_tree_ncell.argtypes = [C.c_void_p]
        L.hco_maketree.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int]
        L.hco_tree_dump.argtypes = [C.c_void_p, _ip, _ip, _ip, _dp, _dp, _dp, _ip]
        L.hco_forces.argtypes = [C.c_void_p, C.c_int, _dp, C.c_void_p, C.c_double, C.c_double,
                                 C.c_int, _dp, _dp, _lp, _lp]
        L.hco_direct.argtypes = [C.c_int, _dp, _dp, C.c_int, _dp, C.c_void_p, C.c_double, _dp, _dp]
        L.hco_hackcode1.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.POINTER(Params),
                                    C.POINTER(LogRow), C.c_int, C.POINTER(Bsf), _dp,
                                    C.POINTER(C.c_double)]
        L.hco_hackcode1.restype = C.c_int
        L.hco_diagnostics.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp]
        assert L.hco_sizeof_logrow() == C.sizeof(LogRow)
        assert L.hco_sizeof_params() == C.sizeof(Params)
        assert L.hco_sizeof_bsf() == C.sizeof(Bsf)
        _lib = L
    return _lib


# ---------------------------------------------------------------- generators

def mkplummer(n: int, seed: int):
    """mkplummer defaults (src/nbody/init/mkplummer.c:257-422): mass[n], phase[n,2,3]."""
    m = np.zeros(n)
    ph = np.zeros((n, 2, 3))
    lib().hco_mkplummer(n, seed, m, ph)
    return m, ph


def make_testdata(n: int, seed: int = 123, cencon: bool = False):
    """hackcode1's nbody= initial conditions (hackcode1/code.c:129-153)."""
    m = np.zeros(n)
    ph = np.zeros((n, 2, 3))
    lib().hco_make_testdata(n, seed, int(cencon), m, ph)
    return m, ph


def ran3_sequence(seed: int, count: int) -> np.ndarray:
    L = lib()
    L.hco_xrandom_init(seed)
    return np.array([L.hco_xrandom(0.0, 1.0) for _ in range(count)])


# ---------------------------------------------------------------- tree / walk

class Tree:
    """maketree + hackcofm on the CPU (load.c:32-248)."""

    def __init__(self, nbody: int, fcells: float = 1.0):
        self._L = lib()
        self._h = self._L.hco_tree_new(nbody, fcells)
        self.n = nbody

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.hco_tree_free(self._h)
            self._h = None

    def set_box(self, rmin, rsize):
        self._L.hco_tree_set_box(self._h, np.ascontiguousarray(rmin, dtype=np.float64), float(rsize))

    def box(self):
        r = np.zeros(3)
        s = C.c_double()
        self._L.hco_tree_get_box(self._h, r, C.byref(s))
        return r, s.value

    def build(self, mass, pos, usequad=False) -> int:
        self._mass = np.ascontiguousarray(mass, dtype=np.float64)
        self._pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        return self._L.hco_maketree(self._h, len(self._mass), self._mass, self._pos, int(usequad))

    @property
    def ncell(self) -> int:
        return self._L.hco_tree_ncell(self._h)

    def dump(self):
        nc = self.ncell
        n = len(self._mass)
        d = dict(level=np.zeros(nc, np.int32), corner=np.zeros((nc, 3), np.int32),
                 count=np.zeros(nc, np.int32), mass=np.zeros(nc), cm=np.zeros((nc, 3)),
                 quad=np.zeros((nc, 6)), body_parent_level=np.zeros(n, np.int32))
        self._L.hco_tree_dump(self._h, d["level"], d["corner"], d["count"], d["mass"], d["cm"],
                              d["quad"], d["body_parent_level"])
        return d

    def forces(self, tol, eps, usequad=False, test_pos=None, skip_self=True):
        """hackgrav at every body (self skipped) or at test_pos (nothing skipped)."""
        if test_pos is None:
            tp = self._pos
            skip = np.arange(len(tp), dtype=np.int32) if skip_self else None
        else:
            tp = np.ascontiguousarray(test_pos, dtype=np.float64).reshape(-1, 3)
            skip = None
        nt = len(tp)
        acc = np.zeros((nt, 3))
        phi = np.zeros(nt)
        n2b = np.zeros(nt, np.int64)
        nbc = np.zeros(nt, np.int64)
        sp = skip.ctypes.data_as(C.c_void_p) if skip is not None else None
        self._L.hco_forces(self._h, nt, tp, sp, float(tol), float(eps), int(usequad), acc, phi, n2b, nbc)
        return acc, phi, n2b, nbc


def direct(mass, pos, test_pos=None, eps=0.05, skip=None):
    """Exact FP64 direct sum (self skipped when test_pos is None)."""
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    if test_pos is None:
        tp = pos
        skip = np.arange(len(pos), dtype=np.int32)
    else:
        tp = np.ascontiguousarray(test_pos, dtype=np.float64).reshape(-1, 3)
    nt = len(tp)
    acc = np.zeros((nt, 3))
    phi = np.zeros(nt)
    sp = None
    if skip is not None:
        skip = np.ascontiguousarray(skip, dtype=np.int32)
        sp = skip.ctypes.data_as(C.c_void_p)
    lib().hco_direct(len(mass), mass, pos, nt, tp, sp, float(eps), acc, phi)
    return acc, phi


def hackcode1(mass, phase, tnow=0.0, freq=32.0, eps=0.05, tol=1.0, fcells=1.0, tstop=2.0,
              freqout=4.0, minor_freqout=32.0, options="mass,phase", usequad=False,
              write_out=True, maxrows=100000):
    """Run the hackcode1 integration loop (code.c:57-64,159-191) on the CPU.

    Returns (phase, acc, phi, rows, bsf, (rmin, rsize))."""
    opts = [w.strip() for w in options.split(",")]
    prm = Params(freq, eps, tol, fcells, tstop, freqout, minor_freqout, int(usequad),
                 int("mass" in opts), int("phi" in opts), int("acc" in opts), int(write_out))
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    ph = np.array(phase, dtype=np.float64).reshape(-1, 2, 3).copy()
    n = len(mass)
    acc = np.zeros((n, 3))
    phi = np.zeros(n)
    rows = (LogRow * maxrows)()
    bsf = Bsf()
    rmin = np.zeros(3)
    rsize = C.c_double()
    nr = lib().hco_hackcode1(n, mass, ph, acc, phi, float(tnow), C.byref(prm), rows, maxrows,
                             C.byref(bsf), rmin, C.byref(rsize))
    if nr < 0:
        raise RuntimeError(f"oracle hackcode1 failed: status {nr}")
    return ph, acc, phi, list(rows[:min(nr, maxrows)]), bsf, (rmin, rsize.value)


def diagnostics(mass, phase, acc, phi) -> np.ndarray:
    out = np.zeros(37)
    lib().hco_diagnostics(len(mass), np.ascontiguousarray(mass, dtype=np.float64),
                          np.ascontiguousarray(phase, dtype=np.float64),
                          np.ascontiguousarray(acc, dtype=np.float64),
                          np.ascontiguousarray(phi, dtype=np.float64), out)
    return out


# ---------------------------------------------------------------- reference libs

class Reference:
    """The reference's own maketree/hackgrav (oracle/_ref), one process-wide
    instance per variant because the reference keeps global state."""

    _inst: dict = {}

    def __init__(self, quad: bool, max_nbody: int, fcells: float = 1.0):
        name = "libhcref_qp.so" if quad else "libhcref_mp.so"
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        L.ref_init.argtypes = [C.c_int, C.c_double]
        L.ref_maketree.argtypes = [C.c_int, _dp, _dp, _dp, C.POINTER(C.c_double)]
        L.ref_tree_dump.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _ip]
        L.ref_forces.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_double, _dp, _dp, _lp, _lp]
        L.ref_ran3_sequence.argtypes = [C.c_int, C.c_int, _dp]
        L.ref_error_message.restype = C.c_char_p
        L.ref_init(max_nbody, fcells)
        self._L = L
        self.max_nbody = max_nbody
        self.quad = quad

    @classmethod
    def get(cls, quad: bool, max_nbody: int = 1 << 18):
        key = bool(quad)
        inst = cls._inst.get(key)
        if inst is None:
            inst = cls._inst[key] = cls(quad, max_nbody)
        if inst.max_nbody < max_nbody:
            raise RuntimeError("reference cell pool was sized for fewer bodies")
        return inst

    @staticmethod
    def available() -> bool:
        return os.path.exists(os.path.join(HERE, "_ref", "libhcref_qp.so"))

    def build(self, mass, pos, rmin=(-2.0, -2.0, -2.0), rsize=4.0):
        self._mass = np.ascontiguousarray(mass, dtype=np.float64)
        self._pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        r = np.array(rmin, dtype=np.float64)
        s = C.c_double(rsize)
        rc = self._L.ref_maketree(len(self._mass), self._mass, self._pos, r, C.byref(s))
        if rc:
            raise RuntimeError(f"reference maketree failed ({rc}): {self._L.ref_error_message()}")
        return r, s.value

    def dump(self):
        n = len(self._mass)
        nc = self._L.ref_tree_ncell()
        d = dict(level=np.zeros(nc, np.int32), corner=np.zeros((nc, 3), np.int32),
                 count=np.zeros(nc, np.int32), mass=np.zeros(nc), cm=np.zeros((nc, 3)),
                 quad=np.zeros((nc, 6)), body_parent_level=np.zeros(n, np.int32))
        self._L.ref_tree_dump(n, d["level"], d["corner"], d["count"], d["mass"], d["cm"], d["quad"],
                              d["body_parent_level"])
        return d

    def forces(self, tol, eps, test_pos=None):
        n = len(self._mass)
        if test_pos is None:
            nt, tp = n, None
        else:
            tpa = np.ascontiguousarray(test_pos, dtype=np.float64).reshape(-1, 3)
            nt, tp = len(tpa), tpa.ctypes.data_as(C.c_void_p)
        acc = np.zeros((nt, 3))
        phi = np.zeros(nt)
        n2b = np.zeros(nt, np.int64)
        nbc = np.zeros(nt, np.int64)
        self._L.ref_forces(n, nt, tp, float(tol), float(eps), acc, phi, n2b, nbc)
        return acc, phi, n2b, nbc

    def ran3_sequence(self, seed: int, count: int) -> np.ndarray:
        out = np.zeros(count)
        self._L.ref_ran3_sequence(seed, count, out)
        return out
