"""GPU edge cases of the additions: ensembles that are all-direct, all-tree or
a single system, the rejection of massless ensemble bodies, caller-order
independence of ensemble results, the approximate criteria and the guard
without quadrupoles, test points under a group criterion, the guard's direct
sum against the FP64 one, the guard with CUDA graphs off, and more test points
than tree nodes between graph replays."""
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


def _systems(hc, counts, seed0=200):
    ms, phs = [], []
    for i, n in enumerate(counts):
        m, ph = hc.mkplummer(int(n), seed0 + i)
        ms.append(m)
        phs.append(ph)
    return ms, phs


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


@pytest.mark.parametrize("direct_max", [0, 4096])
def test_ensemble_all_tree_or_all_direct(hc, direct_max):
    counts = [1500, 2100, 3000]
    ms, phs = _systems(hc, counts)
    ens = hc.Ensemble(counts, tol=0.6, eps=0.02, usequad=True, direct_max=direct_max)
    ens.upload(np.concatenate(ms), np.concatenate(phs))
    ens.step(1 / 256, 0)
    _, acc, _ = ens.download(phase=False, phi=False)
    info = ens.info()
    assert (info["nsys_tree"], info["nsys_direct"]) == ((3, 0) if direct_max == 0 else (0, 3))
    off = np.concatenate([[0], np.cumsum(counts)])
    for s, n in enumerate(counts):
        ctx = hc.Context(n, tol=0.6, eps=0.02, usequad=True)
        ctx.upload(ms[s], phs[s])
        ctx.evaluate()
        ref, _ = ctx.direct_sample(np.arange(n, dtype=np.int64))
        if direct_max == 0:
            ctx.set_grouping("tree")
            ctx.evaluate()
            _, ref, _ = ctx.download(phase=False, phi=False)
            assert np.quantile(_rel(acc[off[s]:off[s + 1]], ref), 0.999) < 1e-5
        else:
            assert _rel(acc[off[s]:off[s + 1]], ref).max() < 1e-5
        ctx.close()
    ens.close()


def test_ensemble_single_system_and_order(hc):
    counts = [5000, 700, 2500]
    ms, phs = _systems(hc, counts, 300)
    e1 = hc.Ensemble(counts, tol=0.6, eps=0.02, direct_max=1024)
    e1.upload(np.concatenate(ms), np.concatenate(phs))
    e1.step(1 / 256, 0)
    _, a1, p1 = e1.download(phase=False)
    # the same systems in another order give the same per-system results
    perm = [2, 0, 1]
    c2 = [counts[i] for i in perm]
    e2 = hc.Ensemble(c2, tol=0.6, eps=0.02, direct_max=1024)
    e2.upload(np.concatenate([ms[i] for i in perm]), np.concatenate([phs[i] for i in perm]))
    e2.step(1 / 256, 0)
    _, a2, p2 = e2.download(phase=False)
    o1 = np.concatenate([[0], np.cumsum(counts)])
    o2 = np.concatenate([[0], np.cumsum(c2)])
    for j, i in enumerate(perm):
        np.testing.assert_allclose(a2[o2[j]:o2[j + 1]], a1[o1[i]:o1[i + 1]], rtol=1e-5, atol=1e-9)
        np.testing.assert_allclose(p2[o2[j]:o2[j + 1]], p1[o1[i]:o1[i + 1]], rtol=1e-5)
    # one system alone
    e3 = hc.Ensemble([counts[0]], tol=0.6, eps=0.02, direct_max=1024)
    e3.upload(ms[0], phs[0])
    e3.step(1 / 256, 0)
    _, a3, _ = e3.download(phase=False, phi=False)
    assert np.quantile(_rel(a3, a1[:counts[0]]), 0.999) < 1e-5
    for e in (e1, e2, e3):
        e.close()


def test_ensemble_rejects_massless_bodies(hc):
    counts = [3000, 2000]
    ms, phs = _systems(hc, counts, 400)
    ms[0][::10] = 0.0
    ens = hc.Ensemble(counts, tol=0.6, eps=0.02, direct_max=1024)
    with pytest.raises(hc.HCError):
        ens.upload(np.concatenate(ms), np.concatenate(phs))
    ens.close()


@pytest.mark.parametrize("criterion,value", [("error", 0.03), ("barnes", 0.6), ("bh86", 0.6), ("sw94", 0.6)])
def test_criteria_without_quadrupoles(hc, criterion, value):
    n = 65536
    m, ph = hc.mkplummer(n, 9)
    ctx = hc.Context(n, tol=0.5, eps=0.01, usequad=False)
    ctx.upload(m, ph)
    ctx.evaluate()
    idx = np.arange(0, n, 32, dtype=np.int64)
    ea, _ = ctx.direct_sample(idx)
    ctx.set_criterion(criterion, value)
    ctx.set_guard(256, 1e-2, seed=2)
    ctx.evaluate()
    ctx.evaluate()
    _, acc, _ = ctx.download(phase=False, phi=False)
    rel = _rel(acc[idx], ea)
    st = ctx.guard_stats()
    assert np.sqrt(np.mean(rel ** 2)) < 1e-2 and st["trips"] == 0, (np.sqrt(np.mean(rel ** 2)), st)
    assert st["last_rms"] < 1e-2


def test_learned_without_quadrupoles(hc):
    n = 131072
    m, ph = hc.mkplummer(n, 10)
    ctx = hc.Context(n, tol=0.5, eps=0.01, usequad=False)
    ctx.upload(m, ph)
    ctx.evaluate()
    idx = np.arange(0, n, 64, dtype=np.int64)
    ea, _ = ctx.direct_sample(idx)
    info = ctx.learn_from_self(theta=0.03, target=1 << 17)
    assert info["samples"] > 5000 and info["train_accuracy"] > 0.7
    ctx.learn_band(0.5, 3.0)
    ctx.set_criterion("learned", 0.03)
    ctx.evaluate()
    ctx.evaluate()
    _, acc, _ = ctx.download(phase=False, phi=False)
    rms = np.sqrt(np.mean(_rel(acc[idx], ea) ** 2))
    assert rms < 3e-3, rms
    assert ctx.walk_stats()["network"] > 0


def test_test_points_under_group_criteria(hc):
    """hackforce's test= path (hc_forces_at: groups of 64 consecutive test
    points, no self term) under the error rule agrees with the per-body rule
    to the criteria's accuracy, and with an FP64 direct sum."""
    n = 65536
    m, ph = hc.mkplummer(n, 12)
    rng = np.random.default_rng(5)
    tp = rng.normal(0.0, 0.7, (5000, 3))
    ctx = hc.Context(n, tol=0.4, eps=0.01, usequad=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    ab, pb = ctx.forces_at(tp)
    ctx.set_criterion("error", 0.01)
    ctx.evaluate()
    ae, pe = ctx.forces_at(tp)
    rel = _rel(ae, ab)
    assert np.sqrt(np.mean(rel ** 2)) < 2e-3 and np.quantile(rel, 0.999) < 2e-2, (np.sqrt(np.mean(rel ** 2)),)
    assert np.max(np.abs(pe / pb - 1)) < 1e-3
    # direct sum for a few points
    x = ph[:, 0]
    for j in range(0, 5000, 997):
        d = x - tp[j]
        r2 = (d ** 2).sum(1) + 0.01 ** 2
        a = (m[:, None] * d / r2[:, None] ** 1.5).sum(0)
        assert np.linalg.norm(ae[j] - a) / np.linalg.norm(a) < 1e-2


def _guard_sample(n, nsample, seed):
    """hc_set_guard's seeded sample: Floyd's algorithm over splitmix64, ascending."""
    M = (1 << 64) - 1
    st = (seed * 0x9E3779B97F4A7C15 + 0x632BE59BD9B4E019) & M
    seen, pick = set(), []
    for j in range(n - nsample, n):
        st = (st + 0x9E3779B97F4A7C15) & M
        z = st
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z ^= z >> 31
        t = z % (j + 1)
        if t in seen:
            t = j
        seen.add(t)
        pick.append(t)
    return np.array(sorted(pick), dtype=np.int64)


@pytest.mark.parametrize("eps", [0.01, 0.0])
def test_guard_direct_sum_matches_the_fp64_sum(hc, eps):
    """The guard's RMS error over its sample, from its FP32 direct sum (FP32
    positions with softening, hi + lo positions without), equals the RMS
    against the FP64 direct sum of the same bodies to 1e-3 of itself."""
    n = 65536
    m, ph = hc.mkplummer(n, 21)
    ctx = hc.Context(n, tol=0.5, eps=eps, usequad=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    ctx.set_criterion("error", 0.05)
    ctx.set_guard(256, 1.0, seed=5)
    ctx.evaluate()
    _, acc, _ = ctx.download(phase=False, phi=False)
    idx = _guard_sample(n, 256, 5)
    ea, _ = ctx.direct_sample(idx)
    rms = float(np.sqrt(np.mean(_rel(acc[idx], ea) ** 2)))
    st = ctx.guard_stats()
    ctx.close()
    assert st["checks"] == 1 and st["trips"] == 0
    assert abs(st["last_rms"] - rms) <= 1e-3 * rms + 1e-7, (st["last_rms"], rms)


def test_guard_without_graphs(hc):
    """The guard's direct sum on its side stream, with CUDA graphs off (plain
    launches on two streams): the same statistics and forces as with graphs."""
    n = 131072
    m, ph = hc.mkplummer(n, 13)
    out = {}
    for graphs in (True, False):
        ctx = hc.Context(n, tol=0.5, eps=0.01, usequad=True)
        ctx.set_graphs(graphs)
        ctx.upload(m, ph)
        ctx.evaluate()
        ctx.set_criterion("error", 0.03)
        ctx.set_guard(256, 1e-2, seed=4)
        for _ in range(3):
            ctx.evaluate()
        _, a, _ = ctx.download(phase=False, phi=False)
        out[graphs] = (a, ctx.guard_stats())
        ctx.close()
    np.testing.assert_array_equal(out[True][0], out[False][0])
    assert out[True][1]["checks"] == out[False][1]["checks"] == 3
    assert out[True][1]["last_rms"] == out[False][1]["last_rms"]


def test_many_test_points_keep_the_captured_graphs(hc):
    """More test points than the context has tree nodes: their sort's scratch
    grows on its own, so the evaluation graph captured before them (which
    holds the tree sort's scratch) replays afterwards to the same forces, and
    a second, smaller call reuses the grown buffers."""
    n = 1000
    m, ph = hc.mkplummer(n, 21)
    rng = np.random.default_rng(8)
    test = rng.uniform(-1.0, 1.0, (40000, 3))          # about 20 times the node capacity
    with hc.Context(n, tol=0.6, eps=0.05, usequad=True) as ctx:
        ctx.upload(m, ph)
        ctx.evaluate()
        _, a0, p0 = ctx.download(phase=False)
        acc, phi = ctx.forces_at(test)
        acc2, phi2 = ctx.forces_at(test[:5000])
        ctx.upload(m, ph)
        ctx.evaluate()
        _, a1, p1 = ctx.download(phase=False)
    np.testing.assert_array_equal(a0, a1)
    np.testing.assert_array_equal(p0, p1)
    assert np.isfinite(acc).all() and np.isfinite(phi).all()
    # the same interaction sets; group centres differ with the test set, so
    # the FP32 sums agree to rounding, not bit for bit
    assert _rel(acc2, acc[:5000]).max() < 1e-5
    assert (np.abs(phi2 - phi[:5000]) / np.abs(phi[:5000])).max() < 1e-5


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("crit", [("body", 0.0), ("error", 0.05), ("learned", 0.05)])
def test_evaluate_host_matches_the_device_path(hc, graphs, crit):
    """hc_evaluate_host (positions and previous accelerations from the host,
    the latter copied beside the build; results back in one round trip) gives
    the same bits as hc_upload + hc_set_forces + hc_evaluate + hc_download."""
    n = 20000
    m, ph = hc.mkplummer(n, 3)
    ph2 = ph.copy()
    ph2[:, 0] += 0.01 * ph[:, 1]                       # the next positions
    out = []
    for host in (False, True):
        with hc.Context(n, tol=0.5, eps=0.01, usequad=True) as ctx:
            ctx.set_graphs(graphs)
            ctx.upload(m, ph)
            if crit[0] == "learned":
                ctx.learn_init(3)                          # an untrained network still decides the band
            ctx.set_criterion(*crit)
            ctx.evaluate()                                 # same box history in both paths
            _, a_prev, _ = ctx.download(phase=False, phi=False)
            if host:
                a, p = ctx.evaluate_host(ph2[:, 0], prev_acc=a_prev)
                a2, p2 = ctx.evaluate_host(ph2[:, 0])       # keeps the accelerations it computed
            else:
                ctx.upload(m, ph2)
                ctx.set_forces(a_prev)
                ctx.evaluate()
                _, a, p = ctx.download(phase=False)
                ctx.evaluate()
                _, a2, p2 = ctx.download(phase=False)
            out.append((a, p, a2, p2))
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)
