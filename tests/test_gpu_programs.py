"""The drop-in programs on the GPU, checked the way NEMO checks hackcode1.

* ``hackcode1 out=bench.dat`` (all defaults) must reproduce the Testfile bsf
  fingerprint (src/nbody/evolve/hackcode/hackcode1/Testfile:27) and the
  man-page log lines;
* ``hackforce`` must agree with the oracle per body (counts exact, forces to
  1e-5) with and without test=;
* a run saved with save= and continued with restart= must end in the same
  state as an uninterrupted run, and its state file is the one hackcode1's
  own savestate writes (read and re-written by the reference's code);
* the extensions dtime= / nstep= / usequad= drive the same integration as
  freq= / tstop= with the quadrupole build.
"""
import json
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
PINS = json.load(open(os.path.join(HERE, "golden", "reference_pins.json")))
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def progs():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nemo_gb300 import build as B
    B.build()
    return os.path.join(ROOT, "nemo_gb300", "bin")


def run(progs, prog, *args, cwd=None):
    r = subprocess.run([os.path.join(progs, prog), *args], capture_output=True, text=True, timeout=600, cwd=cwd)
    assert r.returncode == 0, r.stderr
    return r.stdout


def log_rows(text):
    rows = []
    lines = text.splitlines()
    for i, l in enumerate(lines):
        if l.split()[:2] == ["tnow", "T+U"]:
            f = lines[i + 1].split()
            rows.append((float(f[0]), f[1], f[2], int(f[3]), int(f[4]), int(f[5])))
    return rows


def test_hackcode1_testfile(progs, tmp_path):
    from nemo_gb300 import filestruct as fs
    out = run(progs, "hackcode1", "out=bench.dat", cwd=tmp_path)
    assert fs.bsf(str(tmp_path / "bench.dat")) == PINS["hackcode1_testfile_bsf"]["value"]
    rows = log_rows(out)
    assert len(rows) == 65
    for row, key in ((rows[0], "manpage_first"), (rows[-1], "manpage_last")):
        p = PINS[key]
        assert row[1:] == ("%.4f" % p["T+U"], "%.4f" % p["T/U"], p["nttot"], p["nbavg"], p["ncavg"])
    assert "particle data written" in out


def test_hackcode1_nemobench_h0(progs, tmp_path):
    from nemo_gb300 import filestruct as fs
    run(progs, "hackcode1", "nbody=10240", "out=h0", "seed=123", cwd=tmp_path)
    got = fs.bsf(str(tmp_path / "h0")).split()
    want = PINS["nemobench_h0_bsf"]["value"].split()
    assert got[4] == want[4]                            # same values written
    # 64 leapfrog steps of a 10240-body system amplify the FP32 walk's 1e-7
    # force differences; the fingerprint must still agree to 1e-4
    for g, w in zip(got[:4], want[:4]):
        assert float(g) == pytest.approx(float(w), rel=1e-4)


def _snap(tmp_path, name, m, ph, t=0.0):
    from nemo_gb300 import filestruct as fs
    p = tmp_path / name
    with open(p, "wb") as f:
        w = fs.Writer(f)
        w.string("History", "test")
        fs.write_snapshot(w, m, ph, t)
    return str(p)


@pytest.mark.parametrize("quad", [False, True])
def test_hackforce_vs_oracle(progs, tmp_path, oracle_lib, quad):
    from nemo_gb300 import filestruct as fs
    O = oracle_lib
    m, ph = O.mkplummer(3000, 11)
    src = _snap(tmp_path, "in.snap", m, ph, 0.25)
    q = "usequad=t" if quad else "usequad=f"
    run(progs, "hackforce", f"in={src}", "out=f.snap", "tol=0.6", "eps=0.02", q, cwd=tmp_path)
    s = fs.snapshots(str(tmp_path / "f.snap"))[0]
    T = O.Tree(3000, 0.75)
    assert T.build(m, ph[:, 0].copy(), quad) == 0
    ra, rp, rb, rc = T.forces(0.6, 0.02, quad)
    assert s.time == 0.25
    assert int(s.diagnostics["n2btot"]) == rb.sum() and int(s.diagnostics["nbctot"]) == rc.sum()
    ea = np.linalg.norm(s.acc - ra, axis=1) / np.linalg.norm(ra, axis=1)
    assert (ea <= 1e-5).mean() >= 0.999 and np.allclose(s.phi, rp, rtol=1e-5)
    # test= positions: separate points, nothing skipped
    rng = np.random.default_rng(2)
    tph = np.zeros((100, 2, 3))
    tph[:, 0] = rng.uniform(-1, 1, size=(100, 3))
    tst = _snap(tmp_path, "t.snap", np.zeros(100), tph)
    run(progs, "hackforce", f"in={src}", f"test={tst}", "out=g.snap", "tol=0.6", "eps=0.02", q, cwd=tmp_path)
    g = fs.snapshots(str(tmp_path / "g.snap"))[0]
    ta, tp, tb, tc = T.forces(0.6, 0.02, quad, test_pos=tph[:, 0])
    assert int(g.diagnostics["n2btot"]) == tb.sum() and int(g.diagnostics["nbctot"]) == tc.sum()
    assert np.allclose(g.acc, ta, rtol=1e-5, atol=1e-9) and np.allclose(g.phi, tp, rtol=1e-5)


def test_save_and_restart_continue_the_run(progs, tmp_path):
    from nemo_gb300 import filestruct as fs
    common = ["nbody=512", "seed=7", "freqout=4", "minor_freqout=4", "options=mass,phase,phi,acc"]
    run(progs, "hackcode1", "out=full.snap", "tstop=1.0", *common, cwd=tmp_path)
    run(progs, "hackcode1", "out=a.snap", "tstop=0.5", "save=state", *common, cwd=tmp_path)
    run(progs, "hackcode1", "out=b.snap", "restart=state", "tstop=1.0", "freqout=4", "minor_freqout=4",
        "options=mass,phase,phi,acc", cwd=tmp_path)
    full = fs.snapshots(str(tmp_path / "full.snap"))
    b = fs.snapshots(str(tmp_path / "b.snap"))
    assert b[-1].time == full[-1].time == 1.0
    assert np.array_equal(b[-1].phase, full[-1].phase)
    assert np.array_equal(b[-1].acc, full[-1].acc)


def test_state_file_is_the_references(progs, tmp_path, oracle_lib):
    """The drop-in's save= file against hackcode1's own savestate/restorestate
    (code_io.c:222-284 on NEMO's filestruct library, built from the NEMO
    sources into oracle/_ref): the reference's reader reads every item of it,
    the reference's writer given those values writes the same bytes, and the
    drop-in restarts from a state file the reference wrote."""
    from nemo_gb300 import filestruct as fs
    O = oracle_lib
    if not O.state_available():
        pytest.skip("reference sources not staged (oracle/_ref/libstateref.so absent)")
    common = ["nbody=512", "seed=7", "freqout=4", "minor_freqout=4", "options=mass,phase,phi,acc"]
    run(progs, "hackcode1", "out=full.snap", "tstop=1.0", *common, cwd=tmp_path)
    run(progs, "hackcode1", "out=a.snap", "tstop=0.5", "save=state", *common, cwd=tmp_path)
    st = O.ref_state_read(tmp_path / "state")
    a = fs.snapshots(str(tmp_path / "a.snap"))
    # saved at the last output, after its force evaluation (code_io.c:152-153)
    assert st["tnow"] == a[-1].time == 0.5 and len(st["mass"]) == 512
    assert st["freq"] == 32.0 and st["options"] == "mass,phase,phi,acc"
    assert np.array_equal(st["mass"], a[-1].mass) and np.array_equal(st["phase"], a[-1].phase)
    assert np.array_equal(st["acc"], a[-1].acc) and np.array_equal(st["phi"], a[-1].phi)
    O.ref_state_write(tmp_path / "state_ref", st, program="hackcode1", version="1.5b-gb300")
    assert (tmp_path / "state_ref").read_bytes() == (tmp_path / "state").read_bytes()
    # a state file written by the reference (its own VERSION) restarts the drop-in
    O.ref_state_write(tmp_path / "state_nemo", st, program="hackcode1", version="1.5b")
    run(progs, "hackcode1", "out=b.snap", "restart=state_nemo", "tstop=1.0", "freqout=4", "minor_freqout=4",
        "options=mass,phase,phi,acc", cwd=tmp_path)
    full = fs.snapshots(str(tmp_path / "full.snap"))
    b = fs.snapshots(str(tmp_path / "b.snap"))
    assert b[-1].time == full[-1].time == 1.0
    assert np.array_equal(b[-1].phase, full[-1].phase)


def test_extension_keywords(progs, tmp_path, oracle_lib):
    O = oracle_lib
    m, ph = O.mkplummer(4096, 123)
    src = _snap(tmp_path, "p4k", m, ph)
    out = run(progs, "hackcode1", f"in={src}", "tol=0.7", "eps=0.05", "dtime=1/32", "nstep=8", "usequad=true",
              "out=.", cwd=tmp_path)
    rows = log_rows(out)
    _, _, _, orows, _, _ = O.hackcode1(m, ph, freq=32.0, eps=0.05, tol=0.7, tstop=0.25, usequad=True,
                                       write_out=False)
    assert len(rows) == len(orows) == 9
    for r, o in zip(rows, orows):
        assert (r[3], r[4], r[5]) == (o.nttot, o.nbavg, o.ncavg)
        assert r[1] == "%.4f" % o.etot[0]
