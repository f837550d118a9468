"""hc_diagnostics_noalloc: the diagnostics sums without device allocation.

Some callers cannot allocate device memory when they need these sums (a
runtime that only lends them pre-registered buffers from its own pool, or a
real-time loop that must not pay cudaMalloc's implicit synchronisation).  The
entry point takes device pointers to the body arrays and to the result and
keeps its per-block partials in a static device array.  This test calls it
through the C ABI once, then twice in a row, and checks both results against
the regular entry point (hc_diagnostics), to the 1e-12 relative tolerance used
for FP64 reductions here, and checks that the device's free memory is the same
before and after those two calls.  It lives in a file of its own that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def _finish(raw):
    """36 raw sums -> (etot[3], keten, peten, amten, cmphase, mtot) as hc_diag holds them."""
    ke, pe = raw[0], raw[1]
    keten, peten, am = raw[2:11], raw[11:20], raw[20:29].reshape(3, 3)
    mtot = raw[35]
    return {"etot": np.array([ke + pe, ke, pe]), "keten": keten, "peten": peten,
            "amten": (am - am.T).ravel(), "cmphase": np.concatenate([raw[29:32], raw[32:35]]) / mtot, "mtot": mtot}


def test_noalloc_diagnostics_match_regular_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nemo_gb300 import build as B
    B.build()
    from nemo_gb300 import hackcode as hc

    n = 50000
    m, ph = hc.mkplummer(n, 17)
    with hc.Context(n, tol=0.7, eps=0.05, usequad=True) as ctx:
        ctx.upload(m, ph)
        ctx.evaluate()
        d = ctx.diagnostics()
        phase, acc, phi = ctx.download()
    ref = {"etot": np.array(d.etot[:]), "keten": np.array(d.keten[:]), "peten": np.array(d.peten[:]),
           "amten": np.array(d.amten[:]), "cmphase": np.array(d.cmphase[:]), "mtot": d.mtot}

    dev = "cuda"
    cols = [m, phase[:, 0, 0], phase[:, 0, 1], phase[:, 0, 2], phase[:, 1, 0], phase[:, 1, 1], phase[:, 1, 2],
            acc[:, 0], acc[:, 1], acc[:, 2], phi]
    tens = [torch.tensor(np.ascontiguousarray(c), dtype=torch.float64, device=dev) for c in cols]
    out = torch.zeros(36, dtype=torch.float64, device=dev)
    L = hc.library()
    results = []
    # the first call on the device looks the static array up, and the CUDA
    # driver may load the entry point's kernels then (lazy loading takes
    # device memory for their code); the calls measured below follow it
    assert L.hc_diagnostics_noalloc(n, *[t.data_ptr() for t in tens], out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()           # cudaMemGetInfo
    for _ in range(2):                                   # two calls in a row share the static array
        out.fill_(np.nan)
        rc = L.hc_diagnostics_noalloc(n, *[t.data_ptr() for t in tens], out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        results.append(out.cpu().numpy().copy())
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)     # nothing was allocated
    for raw in results:
        got = _finish(raw)
        for k, v in ref.items():
            # virial units: every sum is O(1) or smaller, so 1e-12 is also the absolute floor
            # (the centre-of-mass sums of this zero-momentum system are ~1e-17)
            np.testing.assert_allclose(got[k], v, rtol=RTOL, atol=RTOL)
    assert np.array_equal(results[0], results[1])

    # sizes beyond the static array are rejected before any GPU work
    assert L.hc_diagnostics_noalloc(8388609, *[t.data_ptr() for t in tens], out.data_ptr(), None) == -1
