"""The CPU oracle pinned against the reference.

Three kinds of pin:
  * the known-answer values NEMO publishes for this path (bsf fingerprints,
    bench12's interaction count, the man-page log table),
  * fixtures made by the reference's own load.c / grav.c (tests/golden/*.npz,
    written by tests/golden/make_golden.py), and
  * where the NEMO sources are present, the reference libraries themselves.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
PINS = json.load(open(os.path.join(HERE, "golden", "reference_pins.json")))


def bsf_text(values):
    s1 = s2 = 0.0
    for v in values:
        s1 += v
        s2 += v * v
    n = len(values)
    mean = s1 / n
    var = s2 / n - mean * mean
    sig = 0.0 if var <= 0 else var ** 0.5
    return "%g %g %g %g %d" % (mean, sig, min(values), max(values), n)


def test_ran3_matches_reference_sequence(oracle_lib):
    O = oracle_lib
    if not O.Reference.available():
        pytest.skip("reference sources not present")
    R = O.Reference.get(True)
    assert np.array_equal(O.ran3_sequence(123, 2000), R.ran3_sequence(123, 2000))
    assert np.array_equal(O.ran3_sequence(7, 500), R.ran3_sequence(7, 500))


@pytest.mark.parametrize("n,key", [(10, "mkplummer_testfile_bsf"), (10240, "nemobench_p0_bsf")])
def test_mkplummer_bsf(oracle_lib, n, key):
    m, ph = oracle_lib.mkplummer(n, 123)
    vals = [0.0] + list(m) + list(ph.ravel())     # Time, Mass, PhaseSpace
    assert bsf_text(vals) == PINS[key]["value"]


def test_hackcode1_testfile_bsf_and_manpage(oracle_lib):
    O = oracle_lib
    m, ph = O.make_testdata(128, 123)
    _, _, _, rows, bsf, _ = O.hackcode1(m, ph)
    assert bsf.text() == PINS["hackcode1_testfile_bsf"]["value"]
    for row, key in ((rows[0], "manpage_first"), (rows[-1], "manpage_last")):
        pin = PINS[key]
        assert "%.3f" % row.tnow == "%.3f" % pin["tnow"]
        assert "%.4f" % row.etot[0] == "%.4f" % pin["T+U"]
        assert "%.4f" % (row.etot[1] / row.etot[2]) == "%.4f" % pin["T/U"]
        assert (row.nttot, row.nbavg, row.ncavg) == (pin["nttot"], pin["nbavg"], pin["ncavg"])
        for k in range(3):
            assert "%.4f" % row.cmphase[k] == "%.4f" % pin["cmpos"][k]
            assert "%.4f" % row.cmphase[3 + k] == "%.4f" % pin["cmvel"][k]


def test_nemobench_h0_bsf(oracle_lib):
    m, ph = oracle_lib.make_testdata(10240, 123)
    _, _, _, _, bsf, _ = oracle_lib.hackcode1(m, ph)
    assert bsf.text() == PINS["nemobench_h0_bsf"]["value"]


@pytest.mark.slow
def test_bench12_interaction_count(oracle_lib):
    m, ph = oracle_lib.mkplummer(200000, 123)
    _, _, _, rows, _, _ = oracle_lib.hackcode1(m, ph, eps=0.05, tstop=0.125, freq=128, write_out=False)
    r = rows[-1]
    pin = PINS["bench12_line"]
    assert r.nttot == pin["nttot"]
    assert (r.nbavg, r.ncavg) == (pin["nbavg"], pin["ncavg"])
    assert "%.4f" % r.etot[0] == "%.4f" % pin["T+U"]
    assert "%.4f" % (r.etot[1] / r.etot[2]) == "%.4f" % pin["T/U"]


def _canon(d):
    k = np.lexsort((d["corner"][:, 2], d["corner"][:, 1], d["corner"][:, 0], d["level"]))
    return {f: d[f][k] for f in ("level", "corner", "count", "mass", "cm", "quad")}


@pytest.mark.parametrize("case", ["plummer4096_s123", "testdata128_s123", "plummer2048_s7_test"])
@pytest.mark.parametrize("quad", [False, True])
def test_oracle_bit_exact_vs_reference_fixture(oracle_lib, case, quad):
    O = oracle_lib
    g = np.load(os.path.join(HERE, "golden", case + ".npz"))
    tag = "qp" if quad else "mp"
    m, pos = g["mass"], g["pos"]
    T = O.Tree(len(m), 1.0)
    assert T.build(m, pos, quad) == 0
    rmin, rsize = T.box()
    assert np.array_equal(rmin, g[f"{tag}_rmin"]) and rsize == float(g[f"{tag}_rsize"])
    c = _canon(T.dump())
    for f in ("level", "corner", "count", "mass", "cm", "quad"):
        assert np.array_equal(c[f], g[f"{tag}_cell_{f}"]), f
    assert np.array_equal(T.dump()["body_parent_level"], g[f"{tag}_body_parent_level"])
    tp = g["test_pos"] if "test_pos" in g.files else None
    acc, phi, n2b, nbc = T.forces(float(g["tol"]), float(g["eps"]), quad, test_pos=tp)
    assert np.array_equal(acc, g[f"{tag}_acc"])
    assert np.array_equal(phi, g[f"{tag}_phi"])
    assert np.array_equal(n2b, g[f"{tag}_n2b"]) and np.array_equal(nbc, g[f"{tag}_nbc"])


def test_oracle_vs_live_reference_expansion_chain(oracle_lib):
    """Second massive body far away: expandbox grafts a chain of one-body
    cells (load.c:74-93); the oracle must reproduce that cell set."""
    O = oracle_lib
    if not O.Reference.available():
        pytest.skip("reference sources not present")
    far = np.array([[0.1, 0.2, 0.3], [40.0, -70.0, 15.0], [45.0, -65.0, 18.0], [38.0, -71.0, 12.0]])
    m4 = np.full(4, 0.25)
    m, ph = O.mkplummer(300, 5)
    pos = ph[:, 0].copy()
    pos[1] = [40.0, -70.0, 15.0]
    for masses, posn, lone in ((m4, far, True), (m, pos, False)):
        for quad in (False, True):
            R = O.Reference.get(quad)
            R.build(masses, posn)
            T = O.Tree(len(masses), 4.0)
            assert T.build(masses, posn, quad) == 0
            a, b = _canon(T.dump()), _canon(R.dump())
            for f in a:
                assert np.array_equal(a[f], b[f]), f
            assert (b["count"] == 1).any() == lone
            r1 = T.forces(0.6, 0.02, quad)
            r2 = R.forces(0.6, 0.02)
            for x, y in zip(r1, r2):
                assert np.array_equal(x, y)


def test_oracle_direct_sum_is_tol0_walk(oracle_lib):
    O = oracle_lib
    m, ph = O.mkplummer(512, 3)
    pos = ph[:, 0].copy()
    T = O.Tree(512)
    T.build(m, pos)
    acc_t, phi_t, _, _ = T.forces(0.0, 0.05)
    acc_d, phi_d = O.direct(m, pos, eps=0.05)
    assert np.allclose(acc_t, acc_d, rtol=1e-12, atol=1e-14)
    assert np.allclose(phi_t, phi_d, rtol=1e-12)


def test_oracle_errors(oracle_lib):
    O = oracle_lib
    m, ph = O.mkplummer(256, 9)
    pos = ph[:, 0].copy()
    T = O.Tree(256, 0.1)                 # fcells too small -> makecell error
    assert T.build(m, pos) == 1
    pos2 = pos.copy()
    pos2[3] = pos2[7]                    # coincident -> assert(l != 0)
    T2 = O.Tree(256, 1.0)
    assert T2.build(m, pos2) == 2


def test_oracle_at_1m_against_reference_fixture(oracle_lib):
    """Plummer N=1,048,576 (mkplummer seed=1), tol=0.5, eps=0.01, quadrupoles:
    the oracle's tree (digest of the canonical cell set and quadrupoles) and
    the forces and counts of the fixture's 16,384 sampled bodies are the
    reference's bit for bit (tests/golden/make_golden_plummer1m.py)."""
    import hashlib
    O = oracle_lib
    g = np.load(os.path.join(HERE, "golden", "plummer1m_s1_qp.npz"))

    def digest(*arrays):
        h = hashlib.sha256()
        for a in arrays:
            h.update(np.ascontiguousarray(a).tobytes())
        return h.hexdigest()

    n = int(g["n"])
    m, ph = O.mkplummer(n, int(g["seed"]))
    pos = ph[:, 0].copy()
    assert digest(m, pos) == str(g["input_digest"])
    T = O.Tree(n, 1.0)
    assert T.build(m, pos, True) == 0
    r, s = T.box()
    assert np.array_equal(r, g["rmin"]) and s == float(g["rsize"])
    d = T.dump()
    c = _canon(d)
    assert digest(c["level"], c["corner"], c["count"], c["mass"], c["cm"]) == str(g["tree_digest"])
    assert digest(c["quad"]) == str(g["quad_digest"])
    assert digest(d["body_parent_level"].astype(np.int32)) == str(g["parent_digest"])
    idx = g["sample_idx"][::8]                      # 2,048 of the sampled bodies: a few seconds
    acc, phi, n2b, nbc = T.forces(float(g["tol"]), float(g["eps"]), True, idx=idx)
    assert np.array_equal(acc, g["sample_acc"][::8]) and np.array_equal(phi, g["sample_phi"][::8])
    assert np.array_equal(n2b, g["sample_n2b"][::8]) and np.array_equal(nbc, g["sample_nbc"][::8])


def test_treecode1_setrcrit_reference_driver(oracle_lib):
    """treecode1's own setrcrit (treeload.c:232-252), built from the NEMO
    sources, on random cells: the three criteria's formulas as published in
    Barnes (1994) / Salmon & Warren (1994) -- (s/theta)^2, bmax^2/theta^2
    with bmax the largest corner distance from the centre of mass, and
    (s/theta + |cm - centre|)^2."""
    O = oracle_lib
    if not O.tc1_available():
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(5)
    n = 200
    center = rng.normal(size=(n, 3))
    size = 2.0 ** rng.integers(-8, 2, n)
    cm = center + (rng.uniform(-0.5, 0.5, (n, 3)) * size[:, None])
    th = 0.7
    np.testing.assert_allclose(O.tc1_setrcrit("bh86", th, 4.0, center, size, cm), (size / th) ** 2, rtol=1e-15)
    d = cm - center + size[:, None] / 2
    bmax2 = (np.maximum(d, size[:, None] - d) ** 2).sum(1)
    np.testing.assert_allclose(O.tc1_setrcrit("sw94", th, 4.0, center, size, cm), bmax2 / th ** 2, rtol=1e-14)
    off = np.linalg.norm(cm - center, axis=1)
    np.testing.assert_allclose(O.tc1_setrcrit("barnes", th, 4.0, center, size, cm), (size / th + off) ** 2,
                               rtol=1e-14)
    assert np.all(O.tc1_setrcrit("barnes", 0.0, 4.0, center, size, cm) == 64.0)   # theta 0: (2 rsize)^2


@pytest.mark.parametrize("kind,pars", [("plummer", [0.0, 2.0, 1.5]), ("hernquist", [0.0, 3.0, 0.5]),
                                       ("miyamoto", [0.0, 1.0, 0.6, 0.1]), ("log", [0.0, 1.0, 0.8, 0.9, 0.7]),
                                       ("plummer", [0.0]), ("miyamoto", [0.0, 1.0, 0.0, 0.3])])
def test_potential_plugins_match_restated_field(oracle_lib, kind, pars):
    """NEMO's own potential plug-ins (built from the NEMO sources) against the
    restatement the GPU tests fall back to where those sources are absent."""
    O = oracle_lib
    if not O.potential_available(kind):
        pytest.skip("reference sources not present")
    from tests.test_gpu_extpot import field
    x = np.random.default_rng(3).normal(size=(500, 3)) * 2.0
    ra, rp = O.ref_potential(kind, pars, x)
    fa, fp = field(kind, pars, x)
    np.testing.assert_allclose(fa, ra, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(fp, rp, rtol=1e-12, atol=1e-15)


def test_reference_state_file_round_trip(oracle_lib, tmp_path):
    """hackcode1's own savestate and restorestate (code_io.c:222-284 on NEMO's
    filestruct library, built from the NEMO sources) round-trip every item."""
    O = oracle_lib
    if not O.state_available():
        pytest.skip("reference sources not present")
    m, ph = O.mkplummer(300, 4)
    rng = np.random.default_rng(1)
    st = dict(freq=32.0, tol=0.7, eps=0.05, fcells=1.0, tstop=2.0, freqout=4.0, minor_freqout=32.0, tnow=0.5,
              tout=0.75, minor_tout=0.53125, rsize=8.0, headline="state test", options="mass,phi", nstep=16,
              rmin=np.array([-4.0, -4.0, -4.0]), mass=m, phase=ph, acc=rng.normal(size=(300, 3)),
              phi=-rng.uniform(size=300))
    f = tmp_path / "state"
    O.ref_state_write(f, st)
    back = O.ref_state_read(f)
    for k, v in st.items():
        if isinstance(v, np.ndarray):
            assert np.array_equal(back[k], v), k
        else:
            assert back[k] == v, k
