"""GPU tests of the walk tuning and the autotuner: with the per-body rule the
interaction sets (hence the reference's counts) do not depend on the tuning,
and the autotuner returns one of its candidates and leaves it set."""
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
        ctx.set_tuning(group_max=40)
    with pytest.raises(hc.HCError):
        ctx.set_tuning(list_depth=16)
    for gm, ld, gk in ((16, 32, "tree"), (24, 48, "tree"), (32, 64, "tree"), (32, 40, "consecutive")):
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
