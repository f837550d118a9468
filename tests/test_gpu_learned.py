"""GPU tests of the learned opening criterion and of the guard.

  * the walk's network (mma.sync BF16, FP32 accumulate) against the FP64
    oracle of oracle/mlp_oracle.py: logits and training gradients;
  * the training kernels learn a known rule;
  * the method end to end -- labels from its own tree against refined
    partial forces, training on the device, the learned walk -- needs fewer
    interactions than the same walk without the network (the error rule) at
    the same RMS force error against the FP64 direct sum;
  * the guard: a passing check leaves the forces untouched, a failing one
    replaces them by the per-body rule's.
"""
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


@pytest.fixture(scope="module")
def mo():
    from oracle import mlp_oracle
    return mlp_oracle


def _params(mo, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, scale / np.sqrt(12), (64, 12))
    b1 = rng.normal(0, 0.1, 64)
    W2 = rng.normal(0, scale / np.sqrt(64), (64, 64))
    b2 = rng.normal(0, 0.1, 64)
    W3 = rng.normal(0, scale / np.sqrt(64), 64)
    b3 = rng.normal(0, 0.1, 1)
    p = np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3, b3]).astype(np.float32)
    assert len(p) == mo.NP
    return p


def _features(n, seed):
    rng = np.random.default_rng(seed)
    return np.clip(rng.normal(0, 1.5, (n, 12)), -8, 8).astype(np.float32)


def test_inference_matches_oracle(hc, mo):
    ctx = hc.Context(1024, tol=0.5, eps=0.01, usequad=True)
    for seed, n in ((1, 37), (2, 1000), (3, 4099)):          # ragged: partial warps and m-tiles
        p = _params(mo, seed, scale=2.0)
        ctx.learn_params(p)
        x = _features(n, seed + 10)
        z = ctx.learn_infer(x)
        zr, _ = mo.forward(p.astype(np.float64), x)
        err = np.abs(z - zr)
        # activations are rounded to BF16 (2^-9 relative) on both sides; the
        # GPU's tanh-form SiLU can move a value to the neighbouring BF16 step
        assert np.mean(err) < 4e-3 * (1 + np.mean(np.abs(zr))), (seed, np.mean(err))
        assert np.max(err) < 0.03 * (1 + np.max(np.abs(zr))), (seed, np.max(err))
        assert np.mean(np.sign(z) == np.sign(zr)) > 0.99


def test_gradient_matches_oracle(hc, mo):
    ctx = hc.Context(1024, tol=0.5, eps=0.01, usequad=True)
    rng = np.random.default_rng(5)
    for seed, n in ((4, 64), (5, 3000)):
        p = _params(mo, seed)
        ctx.learn_params(p)
        x = _features(n, seed + 20)
        y = (rng.random(n) < 0.4).astype(np.float32)
        w = rng.uniform(0.5, 2.0, n).astype(np.float32)
        loss, g = ctx.learn_gradient(x, y, w)
        lr, gr = mo.loss_and_grad(p.astype(np.float64), x, y, w)
        assert abs(loss - lr) <= 2e-3 * abs(lr), (loss, lr)
        rel = np.linalg.norm(g - gr) / np.linalg.norm(gr)
        assert rel < 2e-2, rel
        # every parameter block agrees (W1, b1, W2, b2, W3, b3)
        o = 0
        for size in (64 * 12, 64, 64 * 64, 64, 64, 1):
            gb, rb = g[o:o + size], gr[o:o + size]
            assert np.linalg.norm(gb - rb) <= 3e-2 * np.linalg.norm(rb) + 1e-7, (o, size)
            o += size


def test_training_learns_a_rule(hc, mo):
    ctx = hc.Context(1024, tol=0.5, eps=0.01, usequad=True)
    x = _features(60000, 31)
    rule = lambda x: (x[:, 0] + 0.5 * x[:, 3] - 0.25 * x[:, 7] < 0.2).astype(np.float32)
    ctx.learn_load_samples(x[:50000], rule(x[:50000]))
    ctx.learn_init(3)
    loss = ctx.learn_train(epochs=10, batch=2048, lr=3e-3)
    z = ctx.learn_infer(x[50000:])
    acc = np.mean((z > 0) == (rule(x[50000:]) > 0.5))
    assert loss < 0.15 and acc > 0.96, (loss, acc)


N_PLUMMER = 262144


@pytest.fixture(scope="module")
def plummer(hc):
    m, ph = hc.mkplummer(N_PLUMMER, 1)
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(N_PLUMMER, size=4096, replace=False)).astype(np.int64)
    return m, ph, idx


def _run(ctx, idx, ea):
    """One evaluation: (interactions, RMS relative force error on the sample)."""
    ctx.evaluate()
    d = ctx.diagnostics()
    _, acc, _ = ctx.download(phase=False, phi=False)
    rel = np.linalg.norm(acc[idx] - ea, axis=1) / np.linalg.norm(ea, axis=1)
    return int(d.n2b + d.nbc), float(np.sqrt(np.mean(rel ** 2)))


def _fresh_acc(ctx):
    ctx.set_criterion("body")
    ctx.evaluate()


def test_learned_beats_the_rule_without_network(hc, plummer):
    m, ph, idx = plummer
    ctx = hc.Context(N_PLUMMER, tol=0.5, eps=0.01, usequad=True)
    ctx.upload(m, ph)
    ctx.evaluate()
    ea, _ = ctx.direct_sample(idx)
    # the method without the network: the error rule over a range of budgets
    curve = []
    for eps in (0.01, 0.02, 0.03, 0.05, 0.08):
        _fresh_acc(ctx)
        ctx.set_criterion("error", eps)
        curve.append(_run(ctx, idx, ea))
    curve.sort(key=lambda t: t[1])
    # the method with it: labels from this system, training on the device
    _fresh_acc(ctx)
    ctx.learn_band(1.0, 4.0)
    ns = ctx.learn_collect(0.03, 1 << 18)
    assert ns > 10000
    xs, ys, rs = ctx.learn_samples()
    ctx.learn_relabel(float(np.median(rs)))
    ctx.learn_init(7)
    loss = ctx.learn_train(epochs=8, batch=4096, lr=2e-3)
    assert loss < 0.45
    ctx.learn_band(0.5, 3.0)
    _fresh_acc(ctx)
    ctx.set_criterion("learned", 0.03)
    ctx.learn_threshold(-1.0)
    inter, rms = _run(ctx, idx, ea)
    ws = ctx.walk_stats()
    assert ws["network"] > 0 and ws["network_rounds"] > 0
    assert ws["network"] <= 32 * ws["network_rounds"]
    # interactions the error rule needs at the learned walk's RMS (log-log interpolation)
    r = np.log([c[1] for c in curve])
    k = np.log([c[0] for c in curve])
    assert r[0] <= np.log(rms) <= r[-1], (rms, curve)
    need = float(np.exp(np.interp(np.log(rms), r, k)))
    print(f"learned: {inter} interactions at RMS {rms:.3e}; error rule needs {need:.0f}; curve {curve}")
    assert inter < 0.95 * need, (inter, need, rms, curve)


def test_guard(hc, plummer):
    m, ph, idx = plummer
    ctx = hc.Context(N_PLUMMER, tol=0.5, eps=0.01, usequad=True)
    ctx.upload(m, ph)
    with pytest.raises(hc.HCError):
        ctx.set_guard(N_PLUMMER + 1, 1e-3)
    with pytest.raises(hc.HCError):
        ctx.set_guard(256, 0.0)
    # per-body rule: reference forces and counts.  The fallback walks 32
    # consecutive bodies per group (the approximate criteria's tree groups hold
    # up to 64); the per-body rule's interaction sets do not depend on the
    # grouping, the rounding of its FP32 sums does.
    ctx.set_grouping("consecutive")
    ctx.evaluate()
    db = ctx.diagnostics()
    _, acc_body, phi_body = ctx.download(phase=False)
    ea, _ = ctx.direct_sample(idx)

    # error rule without guard, then with a guard it passes: identical forces
    ctx.set_criterion("error", 0.05)
    ctx.evaluate()
    _, acc_e, phi_e = ctx.download(phase=False)
    rel = np.linalg.norm(acc_e[idx] - ea, axis=1) / np.linalg.norm(ea, axis=1)
    rms = float(np.sqrt(np.mean(rel ** 2)))
    ctx.set_criterion("body")
    ctx.evaluate()
    ctx.set_criterion("error", 0.05)
    ctx.set_guard(512, 1.0, seed=3)
    ctx.evaluate()
    _, acc_g, phi_g = ctx.download(phase=False)
    np.testing.assert_array_equal(acc_g, acc_e)
    np.testing.assert_array_equal(phi_g, phi_e)
    st = ctx.guard_stats()
    assert st["checks"] == 1 and st["trips"] == 0
    assert rms / 3 < st["last_rms"] < 3 * rms, (st, rms)

    # a budget it cannot meet: the per-body rule's forces and counts
    ctx.set_criterion("body")
    ctx.evaluate()
    ctx.set_criterion("error", 0.05)
    ctx.set_guard(512, 1e-9, seed=3)
    ctx.evaluate()
    _, acc_t, phi_t = ctx.download(phase=False)
    np.testing.assert_array_equal(acc_t, acc_body)
    np.testing.assert_array_equal(phi_t, phi_body)
    d = ctx.diagnostics()
    assert (d.n2b, d.nbc) == (db.n2b, db.nbc)
    st = ctx.guard_stats()
    assert st["checks"] == 2 and st["trips"] == 1

    # leapfrog steps with a failing guard follow the per-body rule's run
    ref = hc.Context(N_PLUMMER, tol=0.5, eps=0.01, usequad=True)
    ref.set_grouping("consecutive")
    for c in (ctx, ref):
        c.upload(m, ph)
    ctx.set_criterion("body")
    ctx.step(1 / 128, 0)                   # first step: no closing kick
    ref.step(1 / 128, 0)
    ctx.set_criterion("error", 0.05)
    for k in range(1, 3):
        ctx.step(1 / 128, k)
        ref.step(1 / 128, k)
    pa, aa, _ = ctx.download()
    pb, ab, _ = ref.download()
    # the two kicks (a_err - a_old) h + (a_body - a_err) h round differently
    # from (a_body - a_old) h, so positions may differ in the last bit
    dv = np.linalg.norm(pa[:, 1] - pb[:, 1], axis=1) / np.linalg.norm(pb[:, 1], axis=1)
    da = np.linalg.norm(aa - ab, axis=1) / np.linalg.norm(ab, axis=1)
    assert np.quantile(dv, 0.9999) < 1e-12 and np.quantile(da, 0.9999) < 1e-10, (dv.max(), da.max())
    assert dv.max() < 1e-6 and da.max() < 1e-3
    st = ctx.guard_stats()
    assert st["checks"] == 4 and st["trips"] == 3, st
    ctx.set_guard(0)
