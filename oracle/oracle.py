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
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def reference_sources() -> str | None:
    """Directory holding the NEMO sources of the `ref` build: the staged copy
    in baseline/_ref/nemo (staged first from the NEMO tree where there is
    one), else None."""
    from oracle import stage_reference as S
    return S.stage() if S.source_dir() else S.staged()


def build(ref: bool | None = None) -> None:
    """Compile the oracle, and the reference libs (oracle/_ref) when the
    reference sources are present (ref=None) or required (ref=True)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref is False:
        return
    refdir = reference_sources()
    if refdir is None:
        if ref:
            raise FileNotFoundError("no reference sources: set NEMO_REFDIR or stage baseline/_ref/nemo")
        print("oracle: reference sources absent, oracle/_ref not built")
        return
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
        L.hco_set_snapshot_sink.argtypes = [C.c_void_p, C.c_int]
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

    def forces(self, tol, eps, usequad=False, test_pos=None, skip_self=True, idx=None):
        """hackgrav at every body (self skipped), at the bodies idx (each
        skipping itself) or at test_pos (nothing skipped)."""
        if idx is not None:
            idx = np.ascontiguousarray(idx, dtype=np.int32)
            tp = np.ascontiguousarray(self._pos[idx])
            skip = idx
        elif test_pos is None:
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
              write_out=True, maxrows=100000, snapshots=None):
    """Run the hackcode1 integration loop (code.c:57-64,159-191) on the CPU.

    Returns (phase, acc, phi, rows, bsf, (rmin, rsize)).  When `snapshots` is
    a list, each major output (tnow, phase[n,2,3], phi[n], acc[n,3]) is
    appended to it."""
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
    sink = None
    if snapshots is not None:
        nmax = int((tstop - tnow) * freqout + 3) if freqout > 0 else 0
        sink = np.zeros((max(nmax, 1), 1 + 10 * n))
        lib().hco_set_snapshot_sink(sink.ctypes.data_as(C.c_void_p), len(sink))
    try:
        nr = lib().hco_hackcode1(n, mass, ph, acc, phi, float(tnow), C.byref(prm), rows, maxrows,
                                 C.byref(bsf), rmin, C.byref(rsize))
        if sink is not None:
            for o in sink[:lib().hco_snapshot_count()]:
                snapshots.append((float(o[0]), o[1:1 + 6 * n].reshape(n, 2, 3).copy(),
                                  o[1 + 6 * n:1 + 7 * n].copy(), o[1 + 7 * n:].reshape(n, 3).copy()))
    finally:
        if sink is not None:
            lib().hco_set_snapshot_sink(None, 0)
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

    def __init__(self, quad: bool, max_nbody: int, fcells: float = 1.0, nemo_flags: bool = False):
        name = "libhcref_qp.so" if quad else "libhcref_mp.so"
        if nemo_flags:                   # the build with NEMO's own compiler flags
            if not quad:
                raise ValueError("the NEMO-flags build is the quadrupole variant")
            name = "libhcref_qp_nemo.so"
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        L.ref_init.argtypes = [C.c_int, C.c_double]
        L.ref_maketree.argtypes = [C.c_int, _dp, _dp, _dp, C.POINTER(C.c_double)]
        L.ref_tree_dump.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _ip]
        L.ref_forces.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_double, _dp, _dp, _lp, _lp]
        L.ref_forces_idx.argtypes = [C.c_int, _ip, C.c_double, C.c_double, _dp, _dp, _lp, _lp]
        L.ref_ran3_sequence.argtypes = [C.c_int, C.c_int, _dp]
        L.ref_error_message.restype = C.c_char_p
        L.ref_init(max_nbody, fcells)
        self._L = L
        self.max_nbody = max_nbody
        self.quad = quad

    @classmethod
    def get(cls, quad: bool, max_nbody: int = 1 << 18, nemo_flags: bool = False):
        key = (bool(quad), bool(nemo_flags))
        inst = cls._inst.get(key)
        if inst is None:
            inst = cls._inst[key] = cls(quad, max_nbody, nemo_flags=nemo_flags)
        if inst.max_nbody < max_nbody:
            raise RuntimeError("reference cell pool was sized for fewer bodies")
        return inst

    @staticmethod
    def available(nemo_flags: bool = False) -> bool:
        name = "libhcref_qp_nemo.so" if nemo_flags else "libhcref_qp.so"
        return os.path.exists(os.path.join(HERE, "_ref", name))

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

    def forces_idx(self, tol, eps, idx):
        """hackgrav at the loaded bodies idx only, each skipping itself."""
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        nt = len(idx)
        acc = np.zeros((nt, 3))
        phi = np.zeros(nt)
        n2b = np.zeros(nt, np.int64)
        nbc = np.zeros(nt, np.int64)
        self._L.ref_forces_idx(nt, idx, float(tol), float(eps), acc, phi, n2b, nbc)
        return acc, phi, n2b, nbc

    def ran3_sequence(self, seed: int, count: int) -> np.ndarray:
        out = np.zeros(count)
        self._L.ref_ran3_sequence(seed, count, out)
        return out


# ---------------------------------------------------------------- falcON (gyrfalcON's solver)

class Falcon:
    """falcON's force solver, the engine of gyrfalcON (usr/dehnen/falcON,
    Dehnen 2000, 2002), through its C interface (inc/forces_C.h): compiled
    from the NEMO sources by `oracle/Makefile falcon` into _ref/libfalcon.so
    (single precision, as falcON builds by default).  One process-wide
    instance: the C interface keeps one tree."""

    _inst = None

    def __init__(self):
        path = os.path.join(HERE, "_ref", "libfalcon.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        L.falcON_initialize.argtypes = [_ip, fp, fp, C.c_void_p, fp, fp, C.c_void_p, C.c_int, C.c_int,
                                        C.c_float, C.c_float, C.c_int, C.c_float]
        L.falcON_grow.argtypes = [C.c_int]
        L.falcON_default_Ncrit.restype = C.c_int
        L.falcON_default_theta.restype = C.c_float
        self._L = L
        self._keep = None

    @classmethod
    def get(cls):
        if cls._inst is None:
            cls._inst = cls()
        return cls._inst

    @staticmethod
    def available() -> bool:
        return os.path.exists(os.path.join(HERE, "_ref", "libfalcon.so"))

    def forces(self, mass, pos, eps, theta, kernel=0, G=1.0, ncrit=None):
        """One force evaluation of every body: falcON_grow (tree) then
        falcON_approx_grav (gravity).  theta > 0: falcON's mass-dependent
        opening angle with minimum theta (gyrfalcON's default mode); theta < 0:
        fixed -theta.  Returns (acc[n,3], pot[n], grow s, approx_grav s)."""
        n = len(mass)
        flags = np.ones(n, np.int32)                 # bit 1: active (wants forces)
        m = np.ascontiguousarray(mass, dtype=np.float32)
        x = np.ascontiguousarray(pos, dtype=np.float32).reshape(n, 3)
        acc = np.zeros((n, 3), np.float32)
        pot = np.zeros(n, np.float32)
        self._keep = (flags, m, x, acc, pot)         # the library holds these pointers
        L = self._L
        L.falcON_initialize(flags, m, x, None, acc, pot, None, n, 0, float(eps), float(theta), int(kernel),
                            float(G))
        t0 = time.perf_counter()
        L.falcON_grow(int(ncrit) if ncrit else L.falcON_default_Ncrit())
        t1 = time.perf_counter()
        L.falcON_approx_grav()
        t2 = time.perf_counter()
        return acc.astype(np.float64), pot.astype(np.float64), t1 - t0, t2 - t1


# ---------------------------------------------------------------- treecode1's setrcrit (reference)

def tc1_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libtc1ref.so"))


def tc1_setrcrit(criterion: str, theta: float, rsize: float, center, size, cm) -> np.ndarray:
    """Rcrit2 of cells (geometric centre, side, centre of mass) as treecode1's
    own setrcrit assigns it (treecode1/treeload.c:232-252, compiled from the
    NEMO sources into _ref/libtc1ref.so); criterion bh86 / sw94 / barnes."""
    L = C.CDLL(os.path.join(HERE, "_ref", "libtc1ref.so"))
    L.ref_setrcrit.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp]
    center = np.ascontiguousarray(center, dtype=np.float64).reshape(-1, 3)
    size = np.ascontiguousarray(size, dtype=np.float64).reshape(-1)
    cm = np.ascontiguousarray(cm, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(len(size))
    L.ref_setrcrit({"bh86": 1, "sw94": 2, "barnes": 3}[criterion], float(theta), float(rsize), len(size),
                   center, size, cm, out)
    return out


# ---------------------------------------------------------------- NEMO potential plug-ins (reference)

def potential_available(name: str) -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", f"libpot_{name}.so"))


def ref_potential(name: str, pars, pos):
    """acc[n,3], pot[n] of NEMO's potential plug-in `name` (plummer, hernquist,
    miyamoto, log: src/orbit/potential/data/<name>.c compiled from the NEMO
    sources into _ref/libpot_<name>.so) with potpars `pars` (pattern speed
    first), at time 0."""
    # A plug-in keeps parameters that potpars= does not give from its previous
    # initialisation (file-scope statics); NEMO loads it afresh in each
    # program, so each call here loads a fresh copy.
    import shutil
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, f"libpot_{name}.so")
        shutil.copyfile(os.path.join(HERE, "_ref", f"libpot_{name}.so"), path)
        L = C.CDLL(path, mode=C.RTLD_LOCAL)
        L.ref_pot_eval.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp, _dp]
        par = np.ascontiguousarray(pars if len(pars) else [0.0], dtype=np.float64)
        x = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        acc = np.zeros_like(x)
        pot = np.zeros(len(x))
        L.ref_pot_eval(len(pars), par, len(x), x, acc, pot)
        del L
    return acc, pot


# ---------------------------------------------------------------- hackcode1 state files (reference)

_STATE_KEYS = ("freq", "tol", "eps", "fcells", "tstop", "freqout", "minor_freqout", "tnow", "tout", "minor_tout",
               "rsize")


def state_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libstateref.so"))


def _state_lib():
    L = C.CDLL(os.path.join(HERE, "_ref", "libstateref.so"))
    L.ref_state_identity.argtypes = [C.c_char_p, C.c_char_p]
    L.ref_state_write.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, _dp, C.c_int, _dp, C.c_int, _dp, _dp, _dp, _dp]
    L.ref_state_read.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, _dp, C.POINTER(C.c_int), _dp,
                                 C.POINTER(C.c_int), _dp, _dp, _dp, _dp]
    L.ref_state_error.restype = C.c_char_p
    return L


def ref_state_write(path, state: dict, program="hackcode1", version="1.5b"):
    """Write a state file with hackcode1's own savestate (code_io.c:222-248,
    NEMO's filestruct writer).  state: the _STATE_KEYS, headline, options,
    nstep, rmin, mass, phase, acc, phi."""
    L = _state_lib()
    L.ref_state_identity(program.encode(), version.encode())
    dbl = np.array([state[k] for k in _STATE_KEYS] + [0.0])
    n = len(state["mass"])
    rc = L.ref_state_write(str(path).encode(), state["headline"].encode(), state["options"].encode(), dbl,
                           int(state["nstep"]), np.ascontiguousarray(state["rmin"], dtype=np.float64), n,
                           np.ascontiguousarray(state["mass"], dtype=np.float64),
                           np.ascontiguousarray(state["phase"], dtype=np.float64),
                           np.ascontiguousarray(state["acc"], dtype=np.float64),
                           np.ascontiguousarray(state["phi"], dtype=np.float64))
    if rc:
        raise RuntimeError("reference savestate failed: " + L.ref_state_error().decode())


def ref_state_read(path, nmax: int = 1 << 20) -> dict:
    """Read a state file with hackcode1's own restorestate (code_io.c:254-284)."""
    L = _state_lib()
    hl = C.create_string_buffer(1024)
    op = C.create_string_buffer(1024)
    dbl = np.zeros(12)
    nstep = C.c_int()
    rmin = np.zeros(3)
    n = C.c_int(nmax)
    mass, phase, acc, phi = np.zeros(nmax), np.zeros((nmax, 2, 3)), np.zeros((nmax, 3)), np.zeros(nmax)
    rc = L.ref_state_read(str(path).encode(), hl, op, 1024, dbl, C.byref(nstep), rmin, C.byref(n), mass, phase,
                          acc, phi)
    if rc:
        raise RuntimeError(f"reference restorestate failed ({rc}): " + L.ref_state_error().decode())
    k = n.value
    out = {key: float(v) for key, v in zip(_STATE_KEYS, dbl)}
    out.update(headline=hl.value.decode(), options=op.value.decode(), nstep=nstep.value, rmin=rmin,
               mass=mass[:k], phase=phase[:k], acc=acc[:k], phi=phi[:k])
    return out
