"""CPU-only checks of the library boundary and host services (no GPU calls).

* the C-ABI library builds and exports every function include/hackcode_gpu.h
  declares;
* the host generators (mkplummer, hackcode1 nbody= data) are bit-identical to
  the oracle and reproduce NEMO's published mkplummer fingerprint;
* filestruct snapshots round-trip through the C++ reader/writer, including
  byte-swapped input;
* the drop-in programs honour NEMO's keyword rules (unknown / missing /
  duplicated keywords, help=) without touching the GPU;
* getdparam-style expressions evaluate as the reference's keywords do.
"""
import io
import json
import os
import re
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib():
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode
    return hackcode


def declared_functions():
    src = open(os.path.join(ROOT, "include", "hackcode_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hc_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIBPATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(hc_[a-z0-9_]+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    L = lib.library()
    for n in names:
        assert getattr(L, n) is not None
    assert sorted(lib.EXPORTS) == sorted(names)


def test_create_rejects_sizes_and_parameters_out_of_range(lib):
    """hc_create's and hc_ens_create's argument checks run before any device
    call: more than 2^28 bodies, bodies + cells reaching 2^30 (the sort's
    30-bit look-back counts), non-finite tol / eps / fcells, empty systems."""
    import ctypes as C
    L = lib.library()
    bad = [(1 << 28) + 1, 1.0, 0.05, 1.0], [1 << 28, 1.0, 0.05, 3.0], [1000, float("nan"), 0.05, 1.0], \
        [1000, 1.0, float("inf"), 1.0], [1000, 1.0, 0.05, float("nan")], [0, 1.0, 0.05, 1.0]
    for n, tol, eps, fcells in bad:
        h = C.c_void_p()
        prm = lib.Params(tol, eps, fcells, 1, 0)
        assert L.hc_create(C.byref(h), n, C.byref(prm)) == -1, (n, tol, eps, fcells)   # HC_ERR_ARG
        assert not h.value
    for counts, tol in (([1 << 28, 1], 0.6), ([1 << 62, 1 << 62], 0.6), ([100, 0], 0.6), ([100], float("inf"))):
        with pytest.raises(lib.HCError) as e:
            lib.Ensemble(counts, tol=tol)
        assert e.value.code == -1


def test_host_generators_match_oracle_and_pin(lib, oracle_lib):
    O = oracle_lib
    for n, seed in ((10240, 123), (777, 5)):
        m1, p1 = lib.mkplummer(n, seed)
        m2, p2 = O.mkplummer(n, seed)
        assert np.array_equal(m1, m2) and np.array_equal(p1, p2)
    for cencon in (False, True):
        m1, p1 = lib.make_testdata(128, 123, cencon)
        m2, p2 = O.make_testdata(128, 123, cencon)
        assert np.array_equal(p1, p2) and np.array_equal(m1, m2)
    pins = json.load(open(os.path.join(HERE, "golden", "reference_pins.json")))
    m, ph = lib.mkplummer(10240, 123)
    from nemo_gb300 import filestruct as fs
    buf = io.BytesIO()
    fs.write_snapshot(fs.Writer(buf), m, ph, 0.0)
    path = os.path.join(HERE, "_p0.snap")
    open(path, "wb").write(buf.getvalue())
    try:
        assert fs.bsf(path) == pins["nemobench_p0_bsf"]["value"]
    finally:
        os.remove(path)


def _swap_file(src, dst):
    """Rewrite a little-endian filestruct file in big-endian byte order."""
    from nemo_gb300 import filestruct as fs
    items = fs.read_items(src)
    out = io.BytesIO()

    def hdr(typ, tag, dims):
        out.write(struct.pack(">h", fs.PLUR if dims else fs.SING))
        out.write(typ.encode() + b"\0")
        if tag is not None:
            out.write(tag.encode() + b"\0")
        if dims:
            out.write(struct.pack(">%di" % (len(dims) + 1), *dims, 0))

    def emit(it):
        hdr(it.type, it.tag, it.dims)
        if it.type == "(":
            for s in it.items:
                emit(s)
            hdr(")", None, None)
        else:
            dt, size = fs.TYPES[it.type]
            a = np.frombuffer(it.data, dtype=np.dtype("<" + dt) if size > 1 else dt)
            out.write(a.astype(np.dtype(">" + dt)).tobytes() if size > 1 else a.tobytes())

    for it in items:
        emit(it)
    open(dst, "wb").write(out.getvalue())


def test_filestruct_roundtrip_through_cpp(lib, tmp_path):
    from nemo_gb300 import filestruct as fs
    rng = np.random.default_rng(3)
    a = tmp_path / "a.snap"
    with open(a, "wb") as f:
        w = fs.Writer(f)
        w.string("Headline", "round trip")
        w.string("History", "test_host_cpu")
        for t in (0.0, 0.5):
            n = 37
            fs.write_snapshot(w, rng.random(n), rng.normal(size=(n, 2, 3)), t, phi=-rng.random(n),
                              acc=rng.normal(size=(n, 3)))
    b = tmp_path / "b.snap"
    assert lib.library().hc_snapcopy(str(a).encode(), str(b).encode()) == 2
    assert open(a, "rb").read() == open(b, "rb").read()
    # byte-swapped input is read (gethdr's swapped-magic path) and written natively
    s = tmp_path / "s.snap"
    _swap_file(str(a), str(s))
    c = tmp_path / "c.snap"
    assert lib.library().hc_snapcopy(str(s).encode(), str(c).encode()) == 2
    assert open(a, "rb").read() == open(c, "rb").read()
    snaps = fs.snapshots(str(c))
    assert [x.time for x in snaps] == [0.0, 0.5] and snaps[0].phase.shape == (37, 2, 3)


def test_malformed_snapshots_are_rejected(lib, tmp_path):
    """Inputs get_snap refuses come back as an error, not a crash: arrays of
    the wrong length, a negative dimension, a file cut short."""
    from nemo_gb300 import filestruct as fs
    n = 5

    def frame(path, mass_n=n, phase_dims=(n, 2, 3), pos_n=None):
        with open(path, "wb") as f:
            w = fs.Writer(f)
            w.set("SnapShot")
            w.set("Parameters")
            w.data("Nobj", "i", np.array(n, dtype=np.int32))
            w.tes()
            w.set("Particles")
            w.data("Mass", "d", np.ones(mass_n), [mass_n])
            if pos_n is None:
                w.data("PhaseSpace", "d", np.zeros(6 * n), list(phase_dims))
            else:
                w.data("Position", "d", np.zeros(3 * pos_n), [pos_n, 3])
                w.data("Velocity", "d", np.zeros(3 * n), [n, 3])
            w.tes()
            w.tes()

    out = str(tmp_path / "out.snap").encode()
    good = tmp_path / "good.snap"
    frame(good)
    assert lib.library().hc_snapcopy(str(good).encode(), out) == 1
    cases = {"mass": dict(mass_n=4), "negative": dict(phase_dims=(-n, 2, 3)), "position": dict(pos_n=4)}
    for name, kw in cases.items():
        p = tmp_path / f"{name}.snap"
        frame(p, **kw)
        assert lib.library().hc_snapcopy(str(p).encode(), out) == -1, name
    cut = tmp_path / "cut.snap"
    cut.write_bytes(good.read_bytes()[:-40])
    assert lib.library().hc_snapcopy(str(cut).encode(), out) == -1


def test_short_state_items_are_rejected(lib, tmp_path):
    """restorestate with an item shorter than its type needs (a 4-byte tnow)
    stops with hackcode1's fatal-error line before any device work."""
    from nemo_gb300 import filestruct as fs
    st = tmp_path / "state"
    with open(st, "wb") as f:
        w = fs.Writer(f)
        w.string("program", "hackcode1")
        w.data("tnow", "f", np.array(1.0, dtype=np.float32))
    r = _run("hackcode1", f"restart={st}", "out=.")
    assert r.returncode != 0 and "### Fatal error [hackcode1]" in r.stderr and "too short" in r.stderr


def _run(prog, *args):
    exe = os.path.join(ROOT, "nemo_gb300", "bin", prog)
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=60)


def test_program_keywords(lib):
    r = _run("hackcode1", "help=")
    assert r.returncode == 0 and "freq" in r.stdout and "minor_freqout" in r.stdout
    r = _run("hackcode1", "bogus=1")
    assert r.returncode != 0 and 'Parameter "bogus" unknown' in r.stderr and "### Fatal error [hackcode1]" in r.stderr
    r = _run("hackcode1", "tol=1", "tol=2")
    assert r.returncode != 0 and "duplicated" in r.stderr
    r = _run("hackforce")
    assert r.returncode != 0 and 'Parameter "in" missing' in r.stderr
    r = _run("hackforce", "in=/nonexistent", "out=.", "debug=1")     # system keyword accepted
    assert r.returncode != 0 and "cannot open" in r.stderr


@pytest.mark.parametrize("expr,val", [("1/32", 1 / 32), ("2*(3+4)", 14.0), ("-0.5", -0.5), ("2^10", 1024.0),
                                      ("sqrt(4)+pi", 2 + np.pi), ("1e-3", 1e-3)])
def test_keyword_expressions(lib, expr, val):
    import ctypes as C
    ok = C.c_int()
    v = lib.library().hc_nemo_eval(expr.encode(), C.byref(ok))
    assert ok.value == 1 and v == pytest.approx(val, rel=1e-15)


def test_keyword_expression_errors(lib):
    import ctypes as C
    ok = C.c_int()
    lib.library().hc_nemo_eval(b"1/", C.byref(ok))
    assert ok.value == 0


def test_mkhernquist_moments():
    """The Hernquist generator (no reference counterpart, parity unpinned):
    radii follow the truncated mass profile, kinetic energy and isotropy
    match the model's distribution function."""
    from nemo_gb300 import hackcode as hc
    n = 100000
    m, ph = hc.mkhernquist(n, 7, 100.0)
    m2, ph2 = hc.mkhernquist(n, 7, 100.0)
    np.testing.assert_array_equal(ph, ph2)                      # deterministic for a seed
    mt = 100.0 ** 2 / 101.0 ** 2
    np.testing.assert_allclose(m.sum(), mt, rtol=1e-12)
    assert np.abs(ph[:, 0].mean(0)).max() < 1e-12 and np.abs(ph[:, 1].mean(0)).max() < 1e-12
    r = np.sort(np.linalg.norm(ph[:, 0], axis=1))
    cdf = (r / (1 + r)) ** 2 / mt
    ks = np.max(np.abs(np.arange(1, n + 1) / n - cdf))
    assert ks < 1.63 / np.sqrt(n), ks                            # 1% level
    v = ph[:, 1]
    ke = 0.5 * np.sum(m * (v ** 2).sum(1))
    assert abs(ke - 1.0 / 12.0) < 0.02 / 12.0, ke               # 2K = |W| = 1/6 for the model
    x = ph[:, 0]
    rr = np.linalg.norm(x, axis=1)
    vr2 = np.mean((np.sum(x * v, 1) / rr) ** 2)
    vt2 = np.mean((v ** 2).sum(1)) - vr2
    assert abs(vt2 / (2 * vr2) - 1.0) < 0.02, vt2 / (2 * vr2)   # isotropic


def test_mkgalaxy_moments():
    """The composite galaxy generator (no reference counterpart, parity
    unpinned): component masses, the disk's exponential scale length and
    sech^2 thickness, rotation, the halo's NFW mass profile and the bulge and
    halo velocity dispersions against the isotropic Jeans equation in the
    same spherical potential."""
    from nemo_gb300 import hackcode as hc
    nd, nb, nh = 100000, 40000, 200000
    m, ph = hc.mkgalaxy(nd, nb, nh, 11)
    x, v = ph[:, 0], ph[:, 1]
    d, b, h = slice(0, nd), slice(nd, nd + nb), slice(nd + nb, None)
    np.testing.assert_allclose([m[d].sum(), m[b].sum(), m[h].sum()], [0.1, 0.033, 1.0], rtol=1e-12)
    # centre: the disk's mid-plane (the total centre of mass is at the origin)
    c = np.median(x[d], axis=0)
    R = np.hypot(x[d, 0] - c[0], x[d, 1] - c[1])
    assert abs(R.mean() - 2.0) < 0.02                                   # <R> = 2 R_d
    assert abs(np.mean(np.abs(x[d, 2] - c[2])) - 0.1 * np.log(2)) < 0.002   # sech^2: <|z|> = z0 ln 2
    lz = (x[d, 0] - c[0]) * v[d, 1] - (x[d, 1] - c[1]) * v[d, 0]
    assert np.mean(lz > 0) > 0.95                                       # rotating about +z
    rh = np.linalg.norm(x[h] - c, axis=1)
    nfw = lambda y: np.log1p(y) - y / (1 + y)
    assert abs(np.mean(rh < 3.0) - nfw(1.0) / nfw(10.0)) < 0.005
    assert rh.max() < 30.5
    # isotropic Jeans: rho sigma^2(r) = int_r^rvir rho G M_tot / r'^2 dr'
    rr = np.logspace(-4, np.log10(30.0), 4000)
    mb = 0.033 * (rr / (rr + 0.2)) ** 2 / (30.0 / 30.2) ** 2
    mh = nfw(rr / 3.0) / nfw(10.0)
    md = 0.1 * (1 - (1 + rr) * np.exp(-rr)) / (1 - 16 * np.exp(-15))
    mt = mb + mh + md
    for sl, rho, r0 in ((b, lambda r: 0.2 / (r * (r + 0.2) ** 3), 0.3), (h, lambda r: 1 / (r / 3 * (1 + r / 3) ** 2), 3.0)):
        w = rho(rr) * mt / rr ** 2
        k = np.searchsorted(rr, r0)
        s2 = np.trapezoid(w[k:], rr[k:]) / rho(rr[k])
        r = np.linalg.norm(x[sl] - c, axis=1)
        sel = (r > 0.9 * r0) & (r < 1.1 * r0)
        meas = np.mean(np.sum(v[sl][sel] ** 2, axis=1)) / 3
        assert abs(meas / s2 - 1) < 0.08, (r0, meas, s2)
