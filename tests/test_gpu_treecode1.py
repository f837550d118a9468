"""GPU tests of treecode1's critical-radius criteria (bh86, sw94 and its
default "new" radius, treecode1/treeload.c:232-252) in the group walk.

The per-cell radii the walk uses are pinned to treecode1's own setrcrit
(compiled from the NEMO sources into oracle/_ref/libtc1ref.so) on every cell
of a GPU tree; the walk is checked by the criteria's defining properties:
accuracy improves as theta shrinks; at one theta the bh86 radius is the
smallest of the three (size/theta <= both others), so it accepts the most;
theta = 0 opens every cell (exact direct sum).  Also: the upward pass counts
each cell's bodies, which the learned criterion's features read."""
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


def _err(ctx, idx, ea):
    ctx.evaluate()
    d = ctx.diagnostics()
    _, acc, _ = ctx.download(phase=False, phi=False)
    rel = np.linalg.norm(acc[idx] - ea, axis=1) / np.linalg.norm(ea, axis=1)
    return int(d.n2b + d.nbc), float(np.sqrt(np.mean(rel ** 2)))


def test_critical_radius_criteria(hc):
    n = 65536
    m, ph = hc.mkplummer(n, 5)
    ctx = hc.Context(n, tol=0.5, eps=0.01, usequad=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    idx = np.arange(0, n, 16, dtype=np.int64)
    ea, _ = ctx.direct_sample(idx)
    res = {}
    for kind in ("bh86", "sw94", "barnes"):
        for th in (1.0, 0.7, 0.5):
            ctx.set_criterion(kind, th)
            res[kind, th] = _err(ctx, idx, ea)
        errs = [res[kind, th][1] for th in (1.0, 0.7, 0.5)]
        inter = [res[kind, th][0] for th in (1.0, 0.7, 0.5)]
        assert errs[0] > errs[1] > errs[2], (kind, errs)
        assert inter[0] < inter[1] < inter[2], (kind, inter)
        assert errs[2] < 2e-3, (kind, errs)
    for th in (1.0, 0.7, 0.5):
        assert res["bh86", th][0] <= res["sw94", th][0]
        assert res["bh86", th][0] <= res["barnes", th][0]
    # theta = 0: every cell opened, every pair a body-body interaction
    small = 2048
    m2, ph2 = hc.mkplummer(small, 6)
    c2 = hc.Context(small, tol=0.5, eps=0.01, usequad=True)
    c2.upload(m2, ph2)
    c2.set_criterion("barnes", 0.0)
    c2.evaluate()
    d = c2.diagnostics()
    assert (d.n2b, d.nbc) == (small * (small - 1), 0)
    _, acc, phi = c2.download(phase=False)
    ea2, ep2 = c2.direct_sample(np.arange(small, dtype=np.int64))
    assert np.max(np.linalg.norm(acc - ea2, axis=1) / np.linalg.norm(ea2, axis=1)) < 1e-5
    assert np.max(np.abs(phi - ep2) / np.abs(ep2)) < 1e-5


def test_cell_body_counts_reach_the_features(hc):
    n = 65536
    m, ph = hc.mkplummer(n, 7)
    ctx = hc.Context(n, tol=0.5, eps=0.01, usequad=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    ctx.learn_band(1.0, 4.0)
    ns = ctx.learn_collect(0.03, 20000)
    assert ns > 1000
    x, _, _ = ctx.learn_samples()
    # feature 7 = log2(bodies in the cell) / 8: band cells hold from 2 to many bodies
    f7 = x[:, 7]
    assert f7.min() >= 0.124 and f7.max() > 0.5 and len(np.unique(f7)) > 5, (f7.min(), f7.max())


def test_small_theta_keeps_the_stack_bounded(hc):
    """At small theta the group walk opens almost every cell; near the stack's
    capacity it takes one node at a time instead of failing."""
    n = 262144
    m, ph = hc.mkplummer(n, 8)
    ctx = hc.Context(n, tol=0.5, eps=0.01, usequad=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    idx = np.arange(0, n, 64, dtype=np.int64)
    ea, _ = ctx.direct_sample(idx)
    ctx.set_criterion("barnes", 0.3)
    i3, e3 = _err(ctx, idx, ea)
    ctx.set_criterion("barnes", 0.15)
    i2, e2 = _err(ctx, idx, ea)
    assert ctx.walk_stats()["max_stack"] <= 256
    assert e2 < e3 and i2 > i3, (e2, e3, i2, i3)


@pytest.mark.parametrize("criterion", ["bh86", "sw94", "barnes"])
def test_radii_match_treecode1_setrcrit(hc, oracle_lib, criterion):
    """Every cell's critical radius^2 equals treecode1's setrcrit for the same
    cell (geometric centre and side from the cell's integer corner and level,
    FP64 centre of mass from the upward pass) to FP32 rounding."""
    O = oracle_lib
    if not O.tc1_available():
        pytest.skip("reference sources not staged (oracle/_ref/libtc1ref.so absent)")
    n = 30000
    m, ph = hc.mkplummer(n, 8)
    with hc.Context(n, tol=0.5, eps=0.01, usequad=True) as ctx:
        ctx.upload(m, ph)
        ctx.build_tree()
        rmin, rsize = ctx.box()
        d = ctx.dump_tree()
        for theta in (0.4, 0.75, 0.0):
            got = ctx.tree_rcrit(criterion, theta)
            size = rsize / 2.0 ** d["level"]
            center = rmin + (d["corner"] + 0.5 * 2.0 ** (30 - d["level"][:, None])) * (rsize / 2.0 ** 30)
            ref = O.tc1_setrcrit(criterion, theta, rsize, center, size, d["cm"])
            assert len(got) == len(ref) == len(d["level"])
            rel = np.abs(got - ref) / ref
            assert rel.max() <= 1.2e-7, (criterion, theta, rel.max())
