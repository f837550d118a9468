"""Python mirror of the hackcode1 / hackforce interface over the GB300 library.

The reference's interface for this path is two programs (hackcode1:
src/nbody/evolve/hackcode/hackcode1/code.c:21-51; hackforce: hackforce.c:38-50).
This module offers the same operations as calls, with the same keyword names,
defaults and error behaviour, on top of the C ABI in include/hackcode_gpu.h
(``libhackcode_gpu.so``).  There is no CPU fallback: if the CUDA library is
missing or no GPU is present the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(PKG, "libhackcode_gpu.so")

HC_OK = 0
ERRORS = {-1: "bad argument", -2: "CUDA error", -3: "cell pool exhausted", -4: "coincident bodies",
          -5: "walk stack exhausted", -6: "call out of order", -7: "device allocation failed"}

# exported symbols of include/hackcode_gpu.h
EXPORTS = ["hc_create", "hc_destroy", "hc_last_error", "hc_set_params", "hc_upload", "hc_set_box", "hc_get_box",
           "hc_build_tree", "hc_tree_summary", "hc_dump_tree", "hc_tree_rcrit", "hc_forces", "hc_forces_at",
           "hc_download",
           "hc_body_counts", "hc_step", "hc_diagnostics", "hc_direct_sample", "hc_last_timing",
           "hc_timer_start", "hc_timer_stop", "hc_fp32_peak", "hc_mkplummer", "hc_mkhernquist", "hc_mkgalaxy", "hc_make_testdata",
           "hc_walk_statistics", "hc_set_forces", "hc_snapcopy", "hc_nemo_eval", "hc_evaluate", "hc_evaluate_host",
           "hc_set_graphs", "hc_diagnostics_noalloc", "hc_set_criterion", "hc_set_grouping",
           "hc_learn_nparams", "hc_learn_init", "hc_learn_set_params", "hc_learn_get_params", "hc_learn_infer",
           "hc_learn_gradient", "hc_learn_collect", "hc_learn_samples", "hc_learn_load_samples", "hc_learn_train",
           "hc_learn_set_threshold", "hc_learn_relabel", "hc_learn_set_band", "hc_set_guard", "hc_guard_stats",
           "hc_ens_create", "hc_ens_destroy", "hc_ens_last_error", "hc_ens_upload", "hc_ens_step",
           "hc_ens_download", "hc_ens_info", "hc_ens_set_tuning", "hc_ens_get_tuning", "hc_ens_autotune", "hc_set_tuning", "hc_get_tuning", "hc_autotune", "hc_set_extpot",
           "hc_generate"]


class HCError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("tol", C.c_double), ("eps", C.c_double), ("fcells", C.c_double), ("usequad", C.c_int),
                ("count_per_body", C.c_int)]


class Diag(C.Structure):
    _fields_ = [("etot", C.c_double * 3), ("keten", C.c_double * 9), ("peten", C.c_double * 9),
                ("amten", C.c_double * 9), ("cmphase", C.c_double * 6), ("mtot", C.c_double),
                ("n2b", C.c_int64), ("nbc", C.c_int64), ("nfcalc", C.c_int64)]


class WalkStats(C.Structure):
    _fields_ = [("candidates", C.c_int64), ("mixed", C.c_int64), ("entries_body", C.c_int64),
                ("entries_cell", C.c_int64), ("borderline", C.c_int64), ("max_stack", C.c_int64),
                ("network", C.c_int64), ("network_rounds", C.c_int64), ("mask_hist", C.c_int64 * 33)]

    def as_dict(self):
        d = {k: int(getattr(self, k)) for k, _ in self._fields_ if k != "mask_hist"}
        d["mask_hist"] = [int(x) for x in self.mask_hist]
        return d


class Tuning(C.Structure):
    _fields_ = [("group_max", C.c_int), ("list_depth", C.c_int), ("grouping", C.c_int), ("ms", C.c_double)]

    def as_dict(self):
        return {"group_max": self.group_max, "list_depth": self.list_depth,
                "grouping": ["consecutive", "tree"][self.grouping], "ms": self.ms}


class EnsTuning(C.Structure):
    _fields_ = [("group_max", C.c_int), ("list_depth", C.c_int), ("direct_threads", C.c_int),
                ("tree_ms", C.c_double), ("direct_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class EnsParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("eps", C.c_double), ("usequad", C.c_int), ("direct_max", C.c_int),
                ("fcells", C.c_double)]


class EnsStats(C.Structure):
    _fields_ = [("nsys_tree", C.c_int), ("nsys_direct", C.c_int), ("bodies_tree", C.c_int64),
                ("bodies_direct", C.c_int64), ("interactions_tree", C.c_int64),
                ("interactions_direct", C.c_int64), ("tree_ms", C.c_double), ("direct_ms", C.c_double),
                ("launches", C.c_int64)]


class TreeInfo(C.Structure):
    _fields_ = [("nbody_massive", C.c_int64), ("ncell", C.c_int64), ("max_level", C.c_int32),
                ("rmin", C.c_double * 3), ("rsize", C.c_double)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_vp = C.c_void_p

_lib = None


def library(build_if_missing: bool = False) -> C.CDLL:
    """Load libhackcode_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        if not build_if_missing:
            raise ImportError(f"{LIBPATH} is missing: run nemo_gb300/build.py (the CUDA path has no fallback)")
        from . import build as _b
        _b.build()
    L = C.CDLL(LIBPATH)
    L.hc_create.argtypes = [C.POINTER(_vp), C.c_int64, C.POINTER(Params)]
    L.hc_destroy.argtypes = [_vp]
    L.hc_destroy.restype = None
    L.hc_last_error.argtypes = [_vp]
    L.hc_last_error.restype = C.c_char_p
    L.hc_set_params.argtypes = [_vp, C.POINTER(Params)]
    L.hc_upload.argtypes = [_vp, _dp, _dp]
    L.hc_set_box.argtypes = [_vp, _dp, C.c_double]
    L.hc_set_forces.argtypes = [_vp, _vp, _vp]
    L.hc_get_box.argtypes = [_vp, _dp, C.POINTER(C.c_double)]
    L.hc_build_tree.argtypes = [_vp]
    L.hc_tree_summary.argtypes = [_vp, C.POINTER(TreeInfo)]
    L.hc_dump_tree.argtypes = [_vp, _ip, _ip, _ip, _dp, _dp, _dp, _ip]
    L.hc_tree_rcrit.argtypes = [_vp, C.c_int, C.c_double, _dp]
    L.hc_forces.argtypes = [_vp]
    L.hc_evaluate.argtypes = [_vp]
    L.hc_evaluate_host.argtypes = [_vp, _vp, _vp, _vp, _vp]
    L.hc_set_criterion.argtypes = [_vp, C.c_int, C.c_double]
    L.hc_set_grouping.argtypes = [_vp, C.c_int]
    L.hc_set_guard.argtypes = [_vp, C.c_int64, C.c_double, C.c_uint64]
    L.hc_set_tuning.argtypes = [_vp, C.POINTER(Tuning)]
    L.hc_set_extpot.argtypes = [_vp, C.c_char_p, _vp, C.c_int]
    L.hc_generate.argtypes = [_vp, C.c_char_p, C.c_uint64, _vp, C.c_int]
    L.hc_get_tuning.argtypes = [_vp, C.POINTER(Tuning)]
    L.hc_autotune.argtypes = [_vp, C.POINTER(Tuning)]
    L.hc_ens_create.argtypes = [C.POINTER(_vp), C.c_int, _lp, C.POINTER(EnsParams)]
    L.hc_ens_destroy.argtypes = [_vp]
    L.hc_ens_destroy.restype = None
    L.hc_ens_last_error.argtypes = [_vp]
    L.hc_ens_last_error.restype = C.c_char_p
    L.hc_ens_upload.argtypes = [_vp, _dp, _dp]
    L.hc_ens_step.argtypes = [_vp, C.c_double, C.c_int64, _vp]
    L.hc_ens_download.argtypes = [_vp, _vp, _vp, _vp]
    L.hc_ens_info.argtypes = [_vp, C.POINTER(EnsStats)]
    L.hc_ens_set_tuning.argtypes = [_vp, C.POINTER(EnsTuning)]
    L.hc_ens_get_tuning.argtypes = [_vp, C.POINTER(EnsTuning)]
    L.hc_ens_autotune.argtypes = [_vp, C.POINTER(EnsTuning)]
    L.hc_guard_stats.argtypes = [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]
    _fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    L.hc_learn_nparams.argtypes = []
    L.hc_learn_init.argtypes = [_vp, C.c_uint64]
    L.hc_learn_set_params.argtypes = [_vp, _fp, C.c_int]
    L.hc_learn_get_params.argtypes = [_vp, _fp, C.c_int]
    L.hc_learn_infer.argtypes = [_vp, _fp, C.c_int64, _fp]
    L.hc_learn_gradient.argtypes = [_vp, _fp, _fp, _vp, C.c_int64, _fp, C.POINTER(C.c_float)]
    L.hc_learn_collect.argtypes = [_vp, C.c_double, C.c_int64, C.POINTER(C.c_int64)]
    L.hc_learn_samples.argtypes = [_vp, _vp, _vp, _vp, C.c_int64, C.POINTER(C.c_int64)]
    L.hc_learn_load_samples.argtypes = [_vp, _fp, _fp, _vp, C.c_int64]
    L.hc_learn_train.argtypes = [_vp, C.c_int, C.c_int, C.c_double, C.c_uint64, C.POINTER(C.c_double)]
    L.hc_learn_set_threshold.argtypes = [_vp, C.c_double]
    L.hc_learn_relabel.argtypes = [_vp, C.c_double]
    L.hc_learn_set_band.argtypes = [_vp, C.c_double, C.c_double]
    L.hc_diagnostics_noalloc.argtypes = [C.c_int64] + [_vp] * 13
    L.hc_set_graphs.argtypes = [_vp, C.c_int]
    L.hc_forces_at.argtypes = [_vp, _dp, C.c_int64, _dp, _dp]
    L.hc_download.argtypes = [_vp, _vp, _vp, _vp]
    L.hc_body_counts.argtypes = [_vp, _ip, _ip]
    L.hc_step.argtypes = [_vp, C.c_double, C.c_int64, C.POINTER(Diag), _vp, _vp, _vp]
    L.hc_diagnostics.argtypes = [_vp, C.POINTER(Diag)]
    L.hc_direct_sample.argtypes = [_vp, _lp, C.c_int64, _dp, _dp]
    L.hc_last_timing.argtypes = [_vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    L.hc_walk_statistics.argtypes = [_vp, C.POINTER(WalkStats)]
    L.hc_timer_start.argtypes = [_vp]
    L.hc_timer_stop.argtypes = [_vp, C.POINTER(C.c_double)]
    L.hc_fp32_peak.argtypes = [_vp, C.POINTER(C.c_double)]
    L.hc_mkplummer.argtypes = [C.c_int, C.c_int, _dp, _dp]
    L.hc_mkplummer.restype = None
    L.hc_mkhernquist.argtypes = [C.c_int, C.c_int, C.c_double, _dp, _dp]
    L.hc_mkhernquist.restype = None
    L.hc_mkgalaxy.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_int, _dp, _dp]
    L.hc_mkgalaxy.restype = None
    L.hc_make_testdata.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp]
    L.hc_make_testdata.restype = None
    L.hc_snapcopy.argtypes = [C.c_char_p, C.c_char_p]
    L.hc_nemo_eval.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    L.hc_nemo_eval.restype = C.c_double
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    """One system of nbody bodies on the GPU, all memory owned.  Its work runs
    on its own CUDA streams: the evaluation's at the device's highest stream
    priority, a side stream (the guard's direct sum beside the build) at the
    lowest."""

    def __init__(self, nbody: int, tol: float = 1.0, eps: float = 0.05, fcells: float = 1.0,
                 usequad: bool = False, count_per_body: bool = False):
        self._L = library()
        self.n = int(nbody)
        self.params = Params(float(tol), float(eps), float(fcells), int(bool(usequad)), int(bool(count_per_body)))
        h = _vp()
        rc = self._L.hc_create(C.byref(h), self.n, C.byref(self.params))
        self._h = h
        if rc != HC_OK:
            msg = self._L.hc_last_error(h).decode() if h.value else "hc_create failed"
            self.close()
            raise HCError(rc, msg)

    def _check(self, rc: int):
        if rc != HC_OK:
            raise HCError(rc, self._L.hc_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.hc_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- state ----
    def set_params(self, **kw):
        p = Params.from_buffer_copy(self.params)         # kept only if the library accepts it
        for k, v in kw.items():
            setattr(p, k, type(getattr(p, k))(v))
        self._check(self._L.hc_set_params(self._h, C.byref(p)))
        self.params = p

    def upload(self, mass, phase):
        m = np.ascontiguousarray(mass, dtype=np.float64)
        ph = np.ascontiguousarray(phase, dtype=np.float64).reshape(-1, 2, 3)
        if len(m) != self.n or len(ph) != self.n:
            raise ValueError("mass/phase length must equal nbody")
        if not (np.isfinite(m).all() and np.isfinite(ph).all()):
            raise ValueError("non-finite mass or phase-space coordinates")
        self._check(self._L.hc_upload(self._h, m, ph))

    def upload_ptr(self, mass_ptr: int, phase_ptr: int):
        """Upload from raw host pointers (e.g. pinned buffers): Mass[n], PhaseSpace[n][2][3]."""
        raw = self._L["hc_upload"]          # a second handle with pointer-typed arguments
        raw.argtypes = [_vp, _vp, _vp]
        self._check(raw(self._h, mass_ptr, phase_ptr))

    def generate(self, model="plummer", seed=1, pars=()):
        """Draw initial conditions on the device (hc_generate): 'plummer' (pars: mfrac),
        'hernquist' (pars: rtrunc) or 'galaxy' (pars: n_disk, n_bulge; the rest is halo)."""
        p = np.ascontiguousarray(pars, dtype=np.float64)
        self._check(self._L.hc_generate(self._h, model.encode(), int(seed), _ptr(p) if len(p) else None, len(p)))

    def set_forces(self, acc=None, phi=None):
        """Accelerations [n][3] / potentials [n] of a previous evaluation (restart state)."""
        a = None if acc is None else np.ascontiguousarray(acc, dtype=np.float64).reshape(self.n, 3)
        p = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64).reshape(self.n)
        self._check(self._L.hc_set_forces(self._h, _ptr(a), _ptr(p)))

    def set_forces_ptr(self, acc_ptr=None, phi_ptr=None):
        self._check(self._L.hc_set_forces(self._h, acc_ptr, phi_ptr))

    def download_ptr(self, phase_ptr=None, acc_ptr=None, phi_ptr=None):
        """Download to raw host pointers (any may be None)."""
        self._check(self._L.hc_download(self._h, phase_ptr, acc_ptr, phi_ptr))

    def walk_stats(self) -> dict:
        w = WalkStats()
        self._check(self._L.hc_walk_statistics(self._h, C.byref(w)))
        return w.as_dict()

    def timer_start(self):
        self._check(self._L.hc_timer_start(self._h))

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._check(self._L.hc_timer_stop(self._h, C.byref(ms)))
        return ms.value

    def fp32_peak_tflops(self) -> float:
        t = C.c_double()
        self._check(self._L.hc_fp32_peak(self._h, C.byref(t)))
        return t.value

    def set_box(self, rmin, rsize):
        self._check(self._L.hc_set_box(self._h, np.ascontiguousarray(rmin, dtype=np.float64).reshape(3), float(rsize)))

    def box(self):
        r = np.zeros(3)
        s = C.c_double()
        self._check(self._L.hc_get_box(self._h, r, C.byref(s)))
        return r, s.value

    # ---- tree / forces ----
    def build_tree(self):
        self._check(self._L.hc_build_tree(self._h))

    def tree_info(self) -> TreeInfo:
        t = TreeInfo()
        self._check(self._L.hc_tree_summary(self._h, C.byref(t)))
        return t

    def dump_tree(self):
        t = self.tree_info()
        nc = int(t.ncell)
        d = dict(level=np.zeros(nc, np.int32), corner=np.zeros((nc, 3), np.int32), count=np.zeros(nc, np.int32),
                 mass=np.zeros(nc), cm=np.zeros((nc, 3)), quad=np.zeros((nc, 6)),
                 body_parent_level=np.zeros(self.n, np.int32))
        self._check(self._L.hc_dump_tree(self._h, d["level"], d["corner"], d["count"], d["mass"], d["cm"],
                                         d["quad"], d["body_parent_level"]))
        return d

    def tree_rcrit(self, criterion: str, theta: float):
        """Critical radius^2 per cell of treecode1's bh86 / sw94 / barnes ("new") criterion, in
        dump_tree's cell order."""
        code = {"bh86": 4, "sw94": 5, "barnes": 6}[criterion]
        out = np.zeros(int(self.tree_info().ncell))
        self._check(self._L.hc_tree_rcrit(self._h, code, float(theta), out))
        return out

    def forces(self):
        self._check(self._L.hc_forces(self._h))

    def set_criterion(self, criterion: str = "body", theta: float = 0.0):
        """'body' (the reference's per-body rule), or one decision per group of up to 64 bodies: 'group' (opening
        angle theta), 'error' (truncation-error budget theta |a|), 'learned' (the network in the error
        rule's band)."""
        code = {"body": 0, "group": 1, "error": 2, "learned": 3, "bh86": 4, "sw94": 5, "barnes": 6}[criterion]
        self._check(self._L.hc_set_criterion(self._h, code, float(theta)))

    def set_grouping(self, kind: str = "consecutive"):
        """Walk groups of the per-body rule: 'consecutive' (32 bodies in key order) or 'tree' (cells of
        <= 32 bodies); the other criteria always walk tree groups of up to 64."""
        self._check(self._L.hc_set_grouping(self._h, {"consecutive": 0, "tree": 1}[kind]))

    def set_extpot(self, name=None, pars=()):
        """External potential (hackcode3's potname= / potpars=): 'plummer', 'hernquist',
        'miyamoto' or 'log' with NEMO's parameter order (pattern speed first, must be 0)."""
        p = np.ascontiguousarray(pars, dtype=np.float64)
        self._check(self._L.hc_set_extpot(self._h, (name or "").encode(), _ptr(p) if len(p) else None, len(p)))

    def set_tuning(self, group_max=32, list_depth=64, grouping="consecutive"):
        t = Tuning(int(group_max), int(list_depth), {"consecutive": 0, "tree": 1}[grouping], 0.0)
        self._check(self._L.hc_set_tuning(self._h, C.byref(t)))

    def tuning(self) -> dict:
        t = Tuning()
        self._check(self._L.hc_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def autotune(self) -> dict:
        """Time one evaluation per candidate tuning and keep the fastest."""
        t = Tuning()
        self._check(self._L.hc_autotune(self._h, C.byref(t)))
        return t.as_dict()

    def set_guard(self, nsample: int, rms_max: float = 1e-3, seed: int = 1):
        """Per-evaluation guard of the approximate criteria (0 samples: off)."""
        self._check(self._L.hc_set_guard(self._h, int(nsample), float(rms_max), int(seed)))

    def guard_stats(self) -> dict:
        ch, tr, rms = C.c_int64(), C.c_int64(), C.c_double()
        self._check(self._L.hc_guard_stats(self._h, C.byref(ch), C.byref(tr), C.byref(rms)))
        return {"checks": ch.value, "trips": tr.value, "last_rms": rms.value}

    # ---- learned opening criterion ----
    def learn_init(self, seed: int = 1):
        self._check(self._L.hc_learn_init(self._h, int(seed)))

    def learn_params(self, params=None):
        n = self._L.hc_learn_nparams()
        if params is None:
            out = np.zeros(n, np.float32)
            self._check(self._L.hc_learn_get_params(self._h, out, n))
            return out
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self._L.hc_learn_set_params(self._h, p, len(p)))

    def learn_infer(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 12)
        out = np.zeros(len(x), np.float32)
        self._check(self._L.hc_learn_infer(self._h, x, len(x), out))
        return out

    def learn_gradient(self, x, y, w=None):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 12)
        y = np.ascontiguousarray(y, dtype=np.float32)
        wp = None
        if w is not None:
            w = np.ascontiguousarray(w, dtype=np.float32)
            wp = w.ctypes.data_as(C.c_void_p)
        g = np.zeros(self._L.hc_learn_nparams(), np.float32)
        loss = C.c_float()
        self._check(self._L.hc_learn_gradient(self._h, x, y, wp, len(x), g, C.byref(loss)))
        return loss.value, g

    def learn_collect(self, theta: float, target: int) -> int:
        n = C.c_int64()
        self._check(self._L.hc_learn_collect(self._h, float(theta), int(target), C.byref(n)))
        return n.value

    def learn_samples(self):
        n = C.c_int64()
        self._check(self._L.hc_learn_samples(self._h, None, None, None, 0, C.byref(n)))
        k = n.value
        x = np.zeros((k, 12), np.float32)
        y = np.zeros(k, np.float32)
        r = np.zeros(k, np.float32)
        self._check(self._L.hc_learn_samples(self._h, _ptr(x), _ptr(y), _ptr(r), k, C.byref(n)))
        return x, y, r

    def learn_load_samples(self, x, y, w=None):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 12)
        y = np.ascontiguousarray(y, dtype=np.float32)
        wp = None
        if w is not None:
            w = np.ascontiguousarray(w, dtype=np.float32)
            wp = w.ctypes.data_as(C.c_void_p)
        self._check(self._L.hc_learn_load_samples(self._h, x, y, wp, len(x)))

    def learn_train(self, epochs=20, batch=4096, lr=1e-3, seed=1) -> float:
        loss = C.c_double()
        self._check(self._L.hc_learn_train(self._h, int(epochs), int(batch), float(lr), int(seed), C.byref(loss)))
        return loss.value

    def learn_relabel(self, rel_threshold: float):
        self._check(self._L.hc_learn_relabel(self._h, float(rel_threshold)))

    def learn_band(self, lo: float, hi: float):
        self._check(self._L.hc_learn_set_band(self._h, float(lo), float(hi)))

    def learn_from_self(self, theta: float = 0.03, target: int = 1 << 20, epochs: int = 8, batch: int = 4096,
                        lr: float = 2e-3, seed: int = 7, band=(1.0, 4.0)) -> dict:
        """Train the opening network on labels this system generates: with the tree
        built and accelerations of a previous evaluation on the device, sample
        about `target` band candidates of the error rule at budget `theta`,
        label each against a refined walk of its subtree (accept when its
        relative error is at most the median of the sample), and train on the
        device.  Leaves the band at its previous value."""
        self.learn_band(*band)
        ns = self.learn_collect(theta, target)
        x, y, rel = self.learn_samples()
        thr = float(np.median(rel)) if len(rel) else 0.0
        self.learn_relabel(thr)
        self.learn_init(seed)
        loss = self.learn_train(epochs=epochs, batch=batch, lr=lr, seed=seed)
        z = self.learn_infer(x)
        acc = float(np.mean((z > 0) == (rel <= thr))) if len(rel) else 0.0
        return {"samples": int(ns), "label_threshold": thr, "loss": float(loss), "train_accuracy": acc}

    def learn_threshold(self, t: float):
        self._check(self._L.hc_learn_set_threshold(self._h, float(t)))

    def evaluate(self):
        """build_tree + forces as one CUDA-graph replay."""
        self._check(self._L.hc_evaluate(self._h))

    def evaluate_host_ptr(self, pos_ptr: int, prev_acc_ptr=None, acc_ptr=None, phi_ptr=None):
        """hc_evaluate_host on raw host pointers (page-locked buffers): positions [n][3] in, optionally the
        previous accelerations [n][3] in, accelerations [n][3] / potentials [n] out."""
        self._check(self._L.hc_evaluate_host(self._h, pos_ptr, prev_acc_ptr, acc_ptr, phi_ptr))

    def evaluate_host(self, pos, prev_acc=None, acc=True, phi=True):
        """hc_evaluate_host on numpy arrays: returns (acc[n,3] or None, phi[n] or None)."""
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(self.n, 3)
        pa = None if prev_acc is None else np.ascontiguousarray(prev_acc, dtype=np.float64).reshape(self.n, 3)
        a = np.zeros((self.n, 3)) if acc else None
        f = np.zeros(self.n) if phi else None
        self._check(self._L.hc_evaluate_host(self._h, _ptr(p), _ptr(pa), _ptr(a), _ptr(f)))
        return a, f

    def set_graphs(self, on: bool):
        self._check(self._L.hc_set_graphs(self._h, int(bool(on))))

    def forces_at(self, test_pos):
        tp = np.ascontiguousarray(test_pos, dtype=np.float64).reshape(-1, 3)
        acc = np.zeros((len(tp), 3))
        phi = np.zeros(len(tp))
        self._check(self._L.hc_forces_at(self._h, tp, len(tp), acc, phi))
        return acc, phi

    def download(self, phase=True, acc=True, phi=True):
        ph = np.zeros((self.n, 2, 3)) if phase else None
        a = np.zeros((self.n, 3)) if acc else None
        p = np.zeros(self.n) if phi else None
        self._check(self._L.hc_download(self._h, _ptr(ph), _ptr(a), _ptr(p)))
        return ph, a, p

    def body_counts(self):
        b = np.zeros(self.n, np.int32)
        c = np.zeros(self.n, np.int32)
        self._check(self._L.hc_body_counts(self._h, b, c))
        return b, c

    def diagnostics(self) -> Diag:
        d = Diag()
        self._check(self._L.hc_diagnostics(self._h, C.byref(d)))
        return d

    def step(self, dt: float, nstep: int, snapshot: bool = False):
        d = Diag()
        ph = a = p = None
        if snapshot:
            ph, a, p = np.zeros((self.n, 2, 3)), np.zeros((self.n, 3)), np.zeros(self.n)
        self._check(self._L.hc_step(self._h, float(dt), int(nstep), C.byref(d), _ptr(ph), _ptr(a), _ptr(p)))
        return d, ph, a, p

    def direct_sample(self, index):
        idx = np.ascontiguousarray(index, dtype=np.int64)
        acc = np.zeros((len(idx), 3))
        phi = np.zeros(len(idx))
        self._check(self._L.hc_direct_sample(self._h, idx, len(idx), acc, phi))
        return acc, phi

    def timing(self):
        b, w, n = C.c_double(), C.c_double(), C.c_int64()
        self._check(self._L.hc_last_timing(self._h, C.byref(b), C.byref(w), C.byref(n)))
        return b.value, w.value, n.value


class Ensemble:
    """Independent systems of uneven size stepped together (hc_ens_*): systems of
    more than direct_max bodies share one forest octree walked with the per-body
    rule at tol; the others use an FP32 direct sum."""

    def __init__(self, counts, tol=0.6, eps=0.02, usequad=False, direct_max=1024, fcells=1.0):
        self._L = library()
        self.counts = np.ascontiguousarray(counts, dtype=np.int64)
        self.nsys = len(self.counts)
        self.n = int(self.counts.sum())
        p = EnsParams(float(tol), float(eps), int(bool(usequad)), int(direct_max), float(fcells))
        self._h = _vp()
        r = self._L.hc_ens_create(C.byref(self._h), self.nsys, self.counts, C.byref(p))
        if r != 0:
            msg = self._L.hc_ens_last_error(self._h).decode() if self._h.value else ""
            self.close()
            raise HCError(r, msg or "hc_ens_create")

    def _check(self, r):
        if r != 0:
            raise HCError(r, self._L.hc_ens_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.hc_ens_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, mass, phase):
        m = np.ascontiguousarray(mass, dtype=np.float64)
        ph = np.ascontiguousarray(phase, dtype=np.float64).reshape(-1, 2, 3)
        if len(m) != self.n or len(ph) != self.n:
            raise ValueError("mass/phase length must equal the total body count")
        self._check(self._L.hc_ens_upload(self._h, m, ph))

    def step(self, dt: float, nstep: int, energy: bool = False):
        e = np.zeros((self.nsys, 3)) if energy else None
        self._check(self._L.hc_ens_step(self._h, float(dt), int(nstep), _ptr(e)))
        return e

    def download(self, phase=True, acc=True, phi=True):
        ph = np.zeros((self.n, 2, 3)) if phase else None
        a = np.zeros((self.n, 3)) if acc else None
        p = np.zeros(self.n) if phi else None
        self._check(self._L.hc_ens_download(self._h, _ptr(ph), _ptr(a), _ptr(p)))
        return ph, a, p

    def set_tuning(self, group_max=64, list_depth=64, direct_threads=256):
        t = EnsTuning(int(group_max), int(list_depth), int(direct_threads), 0.0, 0.0)
        self._check(self._L.hc_ens_set_tuning(self._h, C.byref(t)))

    def tuning(self) -> dict:
        t = EnsTuning()
        self._check(self._L.hc_ens_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def autotune(self) -> dict:
        """Fastest walk groups for the tree systems and block size for the direct sums, timed on the
        current bodies (nothing moves)."""
        t = EnsTuning()
        self._check(self._L.hc_ens_autotune(self._h, C.byref(t)))
        return t.as_dict()

    def info(self) -> dict:
        s = EnsStats()
        self._check(self._L.hc_ens_info(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}


# ---------------------------------------------------------------- tool-level calls

def mkplummer(n: int, seed: int = 0):
    """Plummer model as mkplummer draws it with default keywords: (mass[n], phase[n,2,3])."""
    m = np.zeros(n)
    ph = np.zeros((n, 2, 3))
    library().hc_mkplummer(int(n), int(seed), m, ph)
    return m, ph


def mkhernquist(n: int, seed: int = 7, rtrunc: float = 100.0):
    """Isotropic Hernquist sphere (G = M = a = 1, truncated at rtrunc, velocities from
    the Eddington-inverted distribution function): (mass[n], phase[n,2,3])."""
    m = np.zeros(n)
    ph = np.zeros((n, 2, 3))
    library().hc_mkhernquist(int(n), int(seed), float(rtrunc), m, ph)
    return m, ph


def mkgalaxy(n_disk: int = 4194304, n_bulge: int = 1048576, n_halo: int = 11534336, seed: int = 11):
    """Composite disk galaxy (exponential disk, Hernquist bulge, NFW halo): (mass[n], phase[n,2,3]),
    bodies in the order disk, bulge, halo."""
    n = int(n_disk) + int(n_bulge) + int(n_halo)
    m = np.zeros(n)
    ph = np.zeros((n, 2, 3))
    library().hc_mkgalaxy(int(n_disk), int(n_bulge), int(n_halo), int(seed), m, ph)
    return m, ph


def make_testdata(n: int, seed: int = 123, cencon: bool = False):
    """hackcode1's nbody= initial conditions: (mass[n], phase[n,2,3])."""
    m = np.zeros(n)
    ph = np.zeros((n, 2, 3))
    library().hc_make_testdata(int(n), int(seed), int(bool(cencon)), m, ph)
    return m, ph


def hackforce(mass, pos, test=None, tol=1.0, eps=0.05, rsize=4.0, rmin=None, fcells=0.75, usequad=False):
    """One force evaluation with hackforce semantics (hackforce.c:177-215).

    The tree holds the massive bodies of (mass, pos); forces are returned at
    every body (its own body skipped) or, with test=, at the test positions
    (nothing skipped).  Returns (acc, phi, n2btot, nbctot) with 64-bit counts.
    """
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    n = len(mass)
    if n < 1:
        raise ValueError("read_snapshot: Nobj < 1 is absurd")
    if rmin is None:
        rmin = np.full(3, -rsize / 2.0)
    phase = np.zeros((n, 2, 3))
    phase[:, 0] = pos
    with Context(n, tol=tol, eps=eps, fcells=fcells, usequad=usequad) as ctx:
        ctx.upload(mass, phase)
        ctx.set_box(rmin, rsize)
        ctx.build_tree()
        if test is None:
            ctx.forces()
            _, acc, phi = ctx.download(phase=False)
            d = ctx.diagnostics()
            return acc, phi, int(d.n2b), int(d.nbc)
        acc, phi = ctx.forces_at(test)
        d = ctx.diagnostics()
        return acc, phi, int(d.n2b), int(d.nbc)


@dataclass
class LogRow:
    """One block of hackcode1's log (code_io.c:119-129)."""
    tnow: float
    etot: tuple
    nttot: int
    nbavg: int
    ncavg: int
    cmphase: tuple
    n2b: int = 0
    nbc: int = 0


@dataclass
class RunResult:
    phase: np.ndarray
    acc: np.ndarray
    phi: np.ndarray
    rows: list = field(default_factory=list)
    snapshots: list = field(default_factory=list)   # (tnow, bits, mass, phase, phi, acc, diag)
    box: tuple = None


TIME_BIT, PHASE_BIT, MASS_BIT, PHI_BIT, ACC_BIT = 1, 2, 4, 8, 16


def hackcode1(mass, phase, tnow=0.0, freq=32.0, eps=0.05, tol=1.0, fcells=1.0, tstop=2.0, freqout=4.0,
              minor_freqout=32.0, options="mass,phase", usequad=False, keep_snapshots=True, on_output=None):
    """Integrate with hackcode1 semantics (code.c:57-64,159-191; code_io.c:111-154).

    Each step builds the tree, evaluates forces with the closing half-kick,
    records the log row and any due snapshot, then kicks and drifts.  The
    snapshot list holds what hackcode1 would write to out= (or on_output is
    called with each one)."""
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    phase = np.ascontiguousarray(phase, dtype=np.float64).reshape(-1, 2, 3)
    n = len(mass)
    opts = [w.strip() for w in options.split(",")]
    res = RunResult(phase=None, acc=None, phi=None)
    tout = minor_tout = tnow
    nstep = 0
    firstmass = True
    with Context(n, tol=tol, eps=eps, fcells=fcells, usequad=usequad) as ctx:
        ctx.upload(mass, phase)
        while tnow < tstop + 0.1 / freq:
            dt = 1.0 / freq
            bits = 0
            if minor_freqout > 0.0 and (minor_tout - 0.01 / freq) <= tnow:
                minor_tout += 1.0 / minor_freqout
                bits |= TIME_BIT
            if freqout > 0.0 and (tout - 0.01 / freq) <= tnow:
                tout += 1.0 / freqout
                bits |= TIME_BIT | PHASE_BIT
                if "mass" in opts or firstmass:
                    bits |= MASS_BIT
                    firstmass = False
                if "phi" in opts:
                    bits |= PHI_BIT
                if "acc" in opts:
                    bits |= ACC_BIT
            need = bool(bits & (PHASE_BIT | PHI_BIT | ACC_BIT))
            d, ph, a, p = ctx.step(dt, nstep, snapshot=need)
            nf = max(int(d.nfcalc), 1)
            res.rows.append(LogRow(tnow, tuple(d.etot), int(d.n2b + d.nbc), int(d.n2b / nf), int(d.nbc / nf),
                                   tuple(d.cmphase), int(d.n2b), int(d.nbc)))
            if bits:
                snap = (tnow, bits, mass, ph, p, a, d)
                if on_output:
                    on_output(snap)
                if keep_snapshots:
                    res.snapshots.append(snap)
            nstep += 1
            tnow = tnow + dt
        res.phase, res.acc, res.phi = ctx.download()
        res.box = ctx.box()
    return res
