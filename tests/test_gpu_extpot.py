"""GPU tests of the external potential (hackcode3's potname= / potpars=):
the added field against NEMO's own plug-ins (src/orbit/potential/data/
{plummer,hernquist,miyamoto,log}.c, compiled from the NEMO sources into
oracle/_ref) where those are staged, else against the plug-ins' formulas
restated below (the two agree: tests/test_oracle_golden.py); the energy
convention of the diagnostics, energy conservation of test bodies orbiting
in the field through graph-replayed leapfrog steps, argument errors, and the
drop-in program's keywords."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hc():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode
    return hackcode


def field(kind, pars, x):
    """NEMO's potential plug-ins with pattern speed 0 (plummer.c, hernquist.c,
    miyamoto.c, log.c), in numpy: (acc[n,3], phi[n])."""
    p = list(pars[1:])
    x0, y0, z0 = x[:, 0], x[:, 1], x[:, 2]
    if kind == "plummer":
        M, a = (p + [1.0, 1.0][len(p):])[:2]
        t = 1 / (a * a + (x ** 2).sum(1))
        return -M * (t ** 1.5)[:, None] * x, -M * np.sqrt(t)
    if kind == "hernquist":
        M, a = (p + [1.0, 1.0][len(p):])[:2]
        r = np.linalg.norm(x, axis=1)
        return (-M / (r * (r + a) ** 2))[:, None] * x, -M / (r + a)
    if kind == "miyamoto":
        # NEMO's default build of miyamoto.c: symmetry axis y (its "XZY setup")
        M, a, b = (p + [1.0, 0.0, 1.0][len(p):])[:3]
        q = np.sqrt(y0 ** 2 + b * b)
        s = np.sqrt(x0 ** 2 + z0 ** 2 + (a + q) ** 2)
        f = -M / s ** 3
        return np.stack([f * x0, f * y0 * ((a + q) / q if a > 0 else 1.0), f * z0], 1), -M / s
    mc, rc, q = (p + [1.0, 1.0, 1.0][len(p):])[:3]
    r = p[3] if len(p) > 3 else q
    mor = mc / rc if rc > 0 else mc
    rad = rc * rc + x0 ** 2 + y0 ** 2 / q ** 2 + z0 ** 2 / r ** 2
    f = -2 * mor / rad
    return np.stack([f * x0, f * y0 / q ** 2, f * z0 / r ** 2], 1), mor * np.log(rad)


CASES = [("plummer", [0.0, 2.0, 1.5]), ("hernquist", [0.0, 3.0, 0.5]), ("miyamoto", [0.0, 1.0, 0.6, 0.1]),
         ("log", [0.0, 1.0, 0.8, 0.9, 0.7]), ("plummer", [0.0])]


@pytest.mark.parametrize("kind,pars", CASES)
def test_field_added_after_the_walk(hc, oracle_lib, kind, pars):
    n = 4096
    m, ph = hc.mkplummer(n, 21)
    ctx = hc.Context(n, tol=0.6, eps=0.02, usequad=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    _, a0, p0 = ctx.download(phase=False)
    ctx.set_extpot(kind, pars)
    ctx.evaluate()
    _, a1, p1 = ctx.download(phase=False)
    if oracle_lib.potential_available(kind):
        ae, pe = oracle_lib.ref_potential(kind, pars, ph[:, 0])       # the reference's plug-in
    else:
        ae, pe = field(kind, pars, ph[:, 0])
    np.testing.assert_allclose(a1 - a0, ae, rtol=1e-10, atol=1e-12 * np.abs(ae).max())
    np.testing.assert_allclose(p1 - p0, pe, rtol=1e-10, atol=1e-12)
    # energy: hackcode3 counts the external potential once more in U
    d, _, _, _ = ctx.step(1 / 64, 0)
    ke = 0.5 * np.sum(m * (ph[:, 1] ** 2).sum(1))
    u = 0.5 * np.sum(m * (p1 + pe))
    np.testing.assert_allclose([d.etot[1], d.etot[2]], [ke, u], rtol=1e-9)
    ctx.set_extpot(None)
    ctx.upload(m, ph)
    ctx.evaluate()
    _, a2, _ = ctx.download(phase=False, phi=False)
    np.testing.assert_allclose(a2, a0, rtol=1e-12, atol=1e-15)


def test_test_bodies_conserve_energy_in_the_field(hc):
    n = 64
    rng = np.random.default_rng(3)
    m = np.full(n, 1e-12)
    ph = np.zeros((n, 2, 3))
    ph[:, 0] = rng.normal(0, 1.0, (n, 3))
    r = np.linalg.norm(ph[:, 0], axis=1)
    vc = np.sqrt(r ** 2 / (r ** 2 + 1.0) ** 1.5)            # circular speed in a unit Plummer field
    t = np.cross(ph[:, 0], rng.normal(0, 1, (n, 3)))
    ph[:, 1] = 0.9 * vc[:, None] * t / np.linalg.norm(t, axis=1)[:, None]
    ctx = hc.Context(n, tol=0.5, eps=0.01)
    ctx.upload(m, ph)
    ctx.set_extpot("plummer", [0.0, 1.0, 1.0])
    e = []
    for k in range(400):
        d, _, _, _ = ctx.step(1 / 256, k)
        e.append(d.etot[0])
    e = np.array(e)
    assert np.max(np.abs(e / e[0] - 1)) < 1e-5, np.max(np.abs(e / e[0] - 1))


def test_errors(hc):
    ctx = hc.Context(128, tol=0.5, eps=0.01)
    for name, pars in (("kepler", [0.0]), ("plummer", [0.5, 1.0, 1.0]), ("plummer", [0.0, 1, 1, 1])):
        with pytest.raises(hc.HCError):
            ctx.set_extpot(name, pars)


def test_drop_in_keywords(hc, tmp_path):
    prog = os.path.join(ROOT, "nemo_gb300", "bin", "hackcode1")
    args = [prog, "nbody=256", "tstop=0.25", "freq=32", "freqout=32", "minor_freqout=32", "eps=0.05", "tol=0.7"]
    plain = subprocess.run(args, capture_output=True, text=True, timeout=300)
    ext = subprocess.run(args + ["potname=plummer", "potpars=0,1.0,1.0"], capture_output=True, text=True,
                         timeout=300)
    assert plain.returncode == 0 and ext.returncode == 0, ext.stderr
    assert plain.stdout != ext.stdout                     # the field changes the run
    bad = subprocess.run(args + ["potname=plummer", "potpars=0.1,1,1"], capture_output=True, text=True, timeout=300)
    assert bad.returncode != 0 and "Fatal error" in bad.stderr
