"""GPU tests of the ensemble engine (hc_ens_*): independent Plummer systems of
uneven size stepped together.

Tree systems are checked against the single-system path (the same build and
walk, bit-exact with the reference tree for one system); direct-sum systems
against an FP64 direct sum on the host; energies against sums of the
downloaded state; a few leapfrog steps against per-system runs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUNTS = [64, 3000, 300, 1025, 1024, 5000, 100, 2048, 777, 4096]
TOL, EPS, DT = 0.6, 0.02, 1.0 / 256


@pytest.fixture(scope="module")
def hc():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode
    return hackcode


@pytest.fixture(scope="module")
def systems(hc):
    out = []
    for i, n in enumerate(COUNTS):
        m, ph = hc.mkplummer(n, 100 + i)
        out.append((m, ph))
    return out


def _concat(systems):
    return np.concatenate([m for m, _ in systems]), np.concatenate([ph for _, ph in systems])


def _direct(m, pos, eps):
    d = pos[None, :, :] - pos[:, None, :]
    r2 = (d ** 2).sum(-1) + eps * eps
    np.fill_diagonal(r2, np.inf)
    rinv = 1.0 / np.sqrt(r2)
    acc = (m[None, :, None] * d * (rinv ** 3)[:, :, None]).sum(1)
    phi = -(m[None, :] * rinv).sum(1)
    return acc, phi


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


def test_errors(hc):
    with pytest.raises(hc.HCError):
        hc.Ensemble([10, 0, 5])
    with pytest.raises(hc.HCError):
        hc.Ensemble([10, 20], direct_max=100000)


def test_first_forces_and_energies(hc, systems):
    m, ph = _concat(systems)
    ens = hc.Ensemble(COUNTS, tol=TOL, eps=EPS, usequad=False, direct_max=1024)
    ens.upload(m, ph)
    energy = ens.step(DT, 0, energy=True)
    _, acc, phi = ens.download(phase=False)
    info = ens.info()
    assert info["nsys_tree"] == sum(c > 1024 for c in COUNTS)
    assert info["nsys_direct"] == sum(c <= 1024 for c in COUNTS)
    assert info["interactions_tree"] > 0 and info["launches"] > 0
    off = np.concatenate([[0], np.cumsum(COUNTS)])
    for s, (ms, phs) in enumerate(systems):
        a, p = acc[off[s]:off[s + 1]], phi[off[s]:off[s + 1]]
        if COUNTS[s] > 1024:
            ctx = hc.Context(COUNTS[s], tol=TOL, eps=EPS, usequad=False)
            ctx.set_grouping("tree")
            ctx.upload(ms, phs)
            ctx.evaluate()
            _, ar, pr = ctx.download(phase=False)
            ctx.close()
            rel = _rel(a, ar)
            assert np.quantile(rel, 0.999) < 1e-5, (s, np.quantile(rel, 0.999))
            assert rel.max() < 1e-3, (s, rel.max())
            assert np.max(np.abs(p - pr) / np.abs(pr)) < 1e-3
        else:
            ar, pr = _direct(ms, phs[:, 0], EPS)
            rel = _rel(a, ar)
            assert rel.max() < 1e-5, (s, rel.max())
            assert np.max(np.abs(p - pr) / np.abs(pr)) < 1e-5
        ke = 0.5 * np.sum(ms * (phs[:, 1] ** 2).sum(1))
        pe = 0.5 * np.sum(ms * p)
        np.testing.assert_allclose(energy[s], [ke, pe, ke + pe], rtol=1e-10)
    ens.close()


def test_steps_follow_single_system_runs(hc, systems):
    m, ph = _concat(systems)
    ens = hc.Ensemble(COUNTS, tol=TOL, eps=EPS, usequad=False, direct_max=1024)
    ens.upload(m, ph)
    nsteps = 4
    for k in range(nsteps):
        ens.step(DT, k)
    pe_, _, _ = ens.download(acc=False, phi=False)
    off = np.concatenate([[0], np.cumsum(COUNTS)])
    for s, (ms, phs) in enumerate(systems):
        got = pe_[off[s]:off[s + 1]]
        if COUNTS[s] > 1024:
            ctx = hc.Context(COUNTS[s], tol=TOL, eps=EPS, usequad=False)
            ctx.set_grouping("tree")
            ctx.upload(ms, phs)
            for k in range(nsteps):
                ctx.step(DT, k)
            ref, _, _ = ctx.download(acc=False, phi=False)
            ctx.close()
        else:
            # FP64 leapfrog with the direct sum, as stepsystem does it
            x, v = phs[:, 0].copy(), phs[:, 1].copy()
            a_old = None
            for k in range(nsteps):
                a, _ = _direct(ms, x, EPS)
                if k > 0:
                    v += (a - a_old) * (0.5 * DT)
                v1 = v + a * (0.5 * DT)
                x = x + v1 * DT
                v = v1 + a * (0.5 * DT)
                a_old = a
            ref = np.stack([x, v], axis=1)
        dx = np.abs(got - ref).max()
        # FP32 forces (relative error ~1e-6) over 4 steps of 1/256
        assert dx < 1e-6, (s, COUNTS[s], dx)
    ens.close()


def test_autotune_keeps_the_state_and_the_physics(hc, systems):
    """hc_ens_autotune times walk-group and direct-sum block candidates on the
    current bodies without moving them; stepping afterwards gives the same
    trajectory as an untuned ensemble to the tree walk's FP32 level, and any
    tuning keeps the direct-sum systems' forces bit for bit."""
    m, ph = _concat(systems)
    runs = []
    for tune in (False, True):
        ens = hc.Ensemble(COUNTS, tol=TOL, eps=EPS, direct_max=1024)
        ens.upload(m, ph)
        ens.step(DT, 0)
        if tune:
            before = ens.download()
            best = ens.autotune()
            assert best["group_max"] in (32, 48, 64) and best["list_depth"] in (32, 48, 64)
            assert best["direct_threads"] in (128, 256, 512)
            assert best["tree_ms"] > 0 and best["direct_ms"] > 0
            assert ens.tuning()["direct_threads"] == best["direct_threads"]
            after = ens.download()
            for x, y in zip(before, after):                 # nothing moved, forces as they were
                assert np.array_equal(x, y)
        for k in range(1, 4):
            ens.step(DT, k)
        runs.append(ens.download())
        ens.close()
    (p0, a0, f0), (p1, a1, f1) = runs
    np.testing.assert_allclose(p1, p0, rtol=0, atol=1e-6)
    rel = np.linalg.norm(a1 - a0, axis=1) / np.linalg.norm(a0, axis=1)
    assert np.percentile(rel, 99.9) < 1e-4
    ens = hc.Ensemble(COUNTS, tol=TOL, eps=EPS, direct_max=1024)
    with pytest.raises(hc.HCError):
        ens.set_tuning(64, 64, 200)
    ens.close()
