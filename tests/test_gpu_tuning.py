"""GPU tests of the walk tuning and the autotuner: with the per-body rule the
interaction sets (hence the reference's counts) do not depend on the tuning,
the autotuner returns one of its candidates and leaves it set, and the group
criteria's 64-body groups (two bodies per lane) give the same forces as
32-body groups to the accuracy of their criterion."""
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


def test_tuning_keeps_the_reference_interactions(hc):
    n = 65536
    m, ph = hc.mkplummer(n, 3)
    ctx = hc.Context(n, tol=0.6, eps=0.02, usequad=True, count_per_body=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    d0 = ctx.diagnostics()
    b0, c0 = ctx.body_counts()
    _, a0, _ = ctx.download(phase=False)
    with pytest.raises(hc.HCError):
        ctx.set_tuning(group_max=65)
    with pytest.raises(hc.HCError):
        ctx.set_tuning(list_depth=16)
    # group_max above 32 walks 32-body groups under the per-body rule
    for gm, ld, gk in ((16, 32, "tree"), (24, 48, "tree"), (32, 64, "tree"), (64, 64, "tree"), (32, 40, "consecutive")):
        ctx.set_tuning(gm, ld, gk)
        assert ctx.tuning()["group_max"] == gm and ctx.tuning()["list_depth"] == ld
        ctx.evaluate()
        d = ctx.diagnostics()
        assert (d.n2b, d.nbc) == (d0.n2b, d0.nbc)
        b, c = ctx.body_counts()
        np.testing.assert_array_equal(b, b0)
        np.testing.assert_array_equal(c, c0)
        _, a, _ = ctx.download(phase=False)
        rel = np.linalg.norm(a - a0, axis=1) / np.linalg.norm(a0, axis=1)
        assert rel.max() < 1e-5
    best = ctx.autotune()
    assert best["group_max"] in (16, 24, 32) and best["list_depth"] in (32, 48, 64) and best["ms"] > 0
    assert {k: best[k] for k in ("group_max", "list_depth", "grouping")} == \
        {k: ctx.tuning()[k] for k in ("group_max", "list_depth", "grouping")}
    ctx.evaluate()
    d = ctx.diagnostics()
    assert (d.n2b, d.nbc) == (d0.n2b, d0.nbc)


def test_group_criteria_two_bodies_per_lane(hc):
    """Tree groups of up to 64 bodies under the error rule: the forces stay
    within the rule's accuracy of the FP64 direct sum, per-body counts add up
    to the interaction totals, and the autotuner picks one of 32/48/64."""
    n = 65536
    m, ph = hc.mkplummer(n, 4)
    ctx = hc.Context(n, tol=0.5, eps=0.01, usequad=True, count_per_body=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    idx = np.arange(0, n, 16, dtype=np.int64)
    ea, _ = ctx.direct_sample(idx)
    ctx.set_criterion("error", 0.02)
    rms = {}
    for gm in (32, 64):
        ctx.set_tuning(gm, 64, "tree")
        ctx.evaluate()
        ctx.evaluate()
        _, a, _ = ctx.download(phase=False, phi=False)
        rel = np.linalg.norm(a[idx] - ea, axis=1) / np.linalg.norm(ea, axis=1)
        rms[gm] = float(np.sqrt(np.mean(rel ** 2)))
        d = ctx.diagnostics()
        b, c = ctx.body_counts()
        assert (b.sum(), c.sum()) == (d.n2b, d.nbc)
        assert b.min() >= 0 and c.min() > 0
    assert rms[64] < 1e-3 and rms[32] < 1e-3 and 0.5 < rms[64] / rms[32] < 2.0, rms
    best = ctx.autotune()
    assert best["group_max"] in (32, 48, 64) and best["grouping"] == "tree"
