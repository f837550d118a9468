"""GPU tests of the device generators (hc_generate): the drawn bodies follow
the same distributions as the host generators' (two-sample KS tests of radii
and speeds against mkplummer / mkhernquist samples, of each galaxy
component's radii, heights, speeds and angular momenta against mkgalaxy's,
the analytic cumulative mass profile), the systems are in virial equilibrium, the centre of mass is at rest
at the origin, a seed gives the same bodies every time, and bad arguments
raise."""
import numpy as np
import pytest

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


def ks2(a, b):
    """Two-sample Kolmogorov-Smirnov statistic and its 0.1% critical value."""
    a, b = np.sort(a), np.sort(b)
    x = np.concatenate([a, b])
    d = np.abs(np.searchsorted(a, x, "right") / len(a) - np.searchsorted(b, x, "right") / len(b)).max()
    return d, 1.95 * np.sqrt((len(a) + len(b)) / (len(a) * len(b)))


def _draw(hc, n, model, seed, pars=()):
    ctx = hc.Context(n, tol=0.6, eps=0.01, usequad=True)
    ctx.generate(model, seed, pars)
    ph, _, _ = ctx.download(acc=False, phi=False)
    return ctx, ph


@pytest.mark.parametrize("model", ["plummer", "hernquist"])
def test_same_distributions_as_the_host_generators(hc, model):
    n = 200000
    ctx, ph = _draw(hc, n, model, 5)
    m_h, ph_h = hc.mkplummer(n, 6) if model == "plummer" else hc.mkhernquist(n, 6)
    r, v = np.linalg.norm(ph[:, 0], axis=1), np.linalg.norm(ph[:, 1], axis=1)
    rh, vh = np.linalg.norm(ph_h[:, 0], axis=1), np.linalg.norm(ph_h[:, 1], axis=1)
    for a, b in ((r, rh), (v, vh)):
        d, crit = ks2(a, b)
        assert d < crit, (d, crit)
    # the same total mass and the centre of mass at rest at the origin
    d = ctx.diagnostics()
    np.testing.assert_allclose(d.mtot, m_h.sum(), rtol=1e-10)
    np.testing.assert_allclose(np.asarray(d.cmphase[:]), 0, atol=1e-12)
    ctx.close()


def test_galaxy_components_match_the_host_generator(hc):
    nd, nb, nh = 100000, 40000, 200000
    ctx = hc.Context(nd + nb + nh, tol=0.6, eps=0.01, usequad=True)
    ctx.generate("galaxy", 8, [nd, nb])
    ph, _, _ = ctx.download(acc=False, phi=False)
    m_h, ph_h = hc.mkgalaxy(nd, nb, nh, 9)
    d = ctx.diagnostics()
    np.testing.assert_allclose(d.mtot, m_h.sum(), rtol=1e-10)
    np.testing.assert_allclose(np.asarray(d.cmphase[:]), 0, atol=1e-12)
    # each sample relative to its disk's centre: the total centre of mass the
    # generators remove moves with the halo's sampling noise (~0.02 per axis)
    ph = ph - np.median(ph[:nd], axis=0)
    ph_h = ph_h - np.median(ph_h[:nd], axis=0)
    sl = (slice(0, nd), slice(nd, nd + nb), slice(nd + nb, None))
    for k, s in enumerate(sl):
        a, b = ph[s], ph_h[s]
        if k == 0:
            qa = (np.hypot(a[:, 0, 0], a[:, 0, 1]), a[:, 0, 2], a[:, 1, 0] * a[:, 0, 1] - a[:, 1, 1] * a[:, 0, 0])
            qb = (np.hypot(b[:, 0, 0], b[:, 0, 1]), b[:, 0, 2], b[:, 1, 0] * b[:, 0, 1] - b[:, 1, 1] * b[:, 0, 0])
        else:
            qa = (np.linalg.norm(a[:, 0], axis=1), np.linalg.norm(a[:, 1], axis=1))
            qb = (np.linalg.norm(b[:, 0], axis=1), np.linalg.norm(b[:, 1], axis=1))
        for x, y in zip(qa, qb):
            dks, crit = ks2(x, y)
            assert dks < crit, (k, dks, crit)
    ctx.close()


def test_plummer_profile_and_virial_equilibrium(hc):
    n = 262144
    ctx, ph = _draw(hc, n, "plummer", 11)
    a = 3 * np.pi / 16                                 # Plummer scale length in virial units
    r = np.sort(np.linalg.norm(ph[:, 0], axis=1))
    cdf = r ** 3 / (r * r + a * a) ** 1.5 / 0.999
    assert np.abs(cdf - np.arange(1, n + 1) / n).max() < 1.95 / np.sqrt(n) + 2e-3
    ctx.evaluate()
    d = ctx.diagnostics()
    ke, pe = d.etot[1], d.etot[2]
    assert abs(2 * ke / -pe - 1) < 0.02 and abs(pe + 0.5) < 0.01, (ke, pe)
    ctx.close()


def test_seed_determinism(hc):
    n = 50000
    c1, p1 = _draw(hc, n, "hernquist", 3, [50.0])
    c2, p2 = _draw(hc, n, "hernquist", 3, [50.0])
    c3, p3 = _draw(hc, n, "hernquist", 4, [50.0])
    assert np.array_equal(p1, p2) and not np.array_equal(p1, p3)
    assert np.linalg.norm(p1[:, 0], axis=1).max() < 50.0 * 1.001
    for c in (c1, c2, c3):
        c.close()


def test_generated_bodies_run(hc):
    n = 65536
    ctx, _ = _draw(hc, n, "plummer", 21)
    e = []
    for k in range(16):
        d, _, _, _ = ctx.step(1 / 64, k)
        e.append(d.etot[0])
    assert abs(e[-1] / e[0] - 1) < 1e-3


def test_errors(hc):
    ctx = hc.Context(1024, tol=0.6, eps=0.01)
    for model, pars in (("king", []), ("plummer", [0.0]), ("plummer", [1.5]), ("hernquist", [-1.0]),
                        ("galaxy", [1000, 100]), ("galaxy", [10.5, 10]), ("galaxy", [10, 10, 10])):
        with pytest.raises(hc.HCError):
            ctx.generate(model, 1, pars)
    ctx.generate("plummer", 1)                         # the context is still usable
    ctx.evaluate()
    ctx.close()
