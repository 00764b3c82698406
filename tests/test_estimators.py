"""Estimators (3pcf_gb300/estimators.py) against the element-by-element
restatement of the reference scripts (oracle/estimators_ref.py)."""
import numpy as np

import estimators
import estimators_ref
import oracle
import synth


def _hists(seed):
    d = synth.blobs(140, n_blobs=3, sigma=4.0, box=40.0, seed=seed)
    r = synth.uniform(150, box=30.0, seed=seed + 1)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    h = {k: oracle.triangle(c, w, spec)[0] for k, c, w in (("DDD", [d, d, d], 0), ("DDR", [d, d, r], 1),
                                                          ("DRR", [d, r, r], 1), ("RRR", [r, r, r], 0))}
    n = {"DDD": (140, 140, 140), "DDR": (140, 140, 150), "DRR": (140, 150, 150), "RRR": (150, 150, 150)}
    return h, n, spec, d, r


def test_zeta_matches_reference_restatement():
    h, n, spec, _, _ = _hists(5)
    z = estimators.zeta(h["DDD"], h["DDR"], h["DRR"], h["RRR"], n["DDD"], n["DDR"], n["DRR"], n["RRR"])
    want = estimators_ref.zeta(h["DDD"], h["DDR"], h["DRR"], h["RRR"], n["DDD"], n["DDR"], n["DRR"], n["RRR"])
    assert np.array_equal(z, np.array(want))
    assert np.count_nonzero(z) > 0


def test_zeta_of_identical_catalogs_is_zero():
    """D = R: every term cancels exactly where RRR is populated."""
    d = synth.uniform(120, box=25.0, seed=9)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    ddd, _ = oracle.triangle([d, d, d], 0, spec)
    ddr, _ = oracle.triangle([d, d, d], 1, spec)
    n = (120, 120, 120)
    z = estimators.zeta(ddd, ddr, ddr, ddd, n, n, n, n)
    nd = estimators.norms_3pcf(n, n, n, n)
    with np.errstate(divide="ignore", invalid="ignore"):  # empty bins: 0/0, set to 0 as the script does
        expect = (ddd / nd[0] - 3 * ddr / nd[1] + 3 * ddr / nd[2] - ddd / nd[3]) / (ddd / nd[3])
    expect[~np.isfinite(expect)] = 0
    assert np.allclose(z, expect, rtol=0, atol=1e-12)


def test_xi_matches_reference_restatement():
    d = synth.blobs(800, n_blobs=6, sigma=5.0, box=80.0, seed=3)
    r = synth.uniform(700, box=80.0, seed=4)
    dd, _ = oracle.pair([d, d], 0, 0.0, 70.0, 700)
    dr, _ = oracle.pair([d, r], 1, 0.0, 70.0, 700)
    rr, _ = oracle.pair([r, r], 0, 0.0, 70.0, 700)
    x = estimators.xi(dd, dr, rr, (800, 800), (800, 700), (700, 700))
    want = estimators_ref.xi(dd, dr, rr, (800, 800), (800, 700), (700, 700))
    assert np.array_equal(x, np.array(want))
    tab = estimators.xi_table(x, 0.0, 70.0, 700)
    text = estimators.format_xi_table(tab)
    assert text.splitlines()[0] == "%f %f" % (0.1, x[0])
    assert len(text.splitlines()) == 700


def test_reduced_zeta_shape_and_finite_denominator():
    h, n, spec, d, r = _hists(11)
    z = estimators.zeta(h["DDD"], h["DDR"], h["DRR"], h["RRR"], n["DDD"], n["DDR"], n["DRR"], n["RRR"])
    tab = np.stack([np.linspace(0.5, 70, 140), np.linspace(2.0, 0.01, 140)], axis=1)
    q = estimators.reduced_zeta(z, spec, 3, [0, 1, 2], tab)
    assert q.shape == (3, 16)
    assert np.all(np.isfinite(q))
    want = estimators_ref.reduced_zeta(z, spec, 3, [0, 1, 2], list(tab[:, 0]), list(tab[:, 1]))
    assert np.allclose(q, np.array(want), rtol=1e-13, atol=0)


def test_zeta_error_summary():
    z_ref = np.array([0.5, -0.25, 2.0, 0.0])
    z = z_ref + np.array([1e-3, 0.0, -2e-3, 5.0])
    rrr = np.array([3, 1, 7, 0])  # the last bin is unpopulated and ignored
    e = estimators.zeta_error(z, z_ref, rrr)
    assert e["bins"] == 3
    assert abs(e["max_abs"] - 2e-3) < 1e-15
    assert abs(e["rms"] - np.sqrt((1e-6 + 4e-6) / 3)) < 1e-15
    assert abs(e["max_rel"] - 2e-3) < 1e-12


# ---- pins: the reference's own scripts run on committed histogram files ----
# (tests/golden/make_estimator_pins.py executes examples/plot_MICE_2pcf.py and
# examples/plot_MICE_3pcf.py under Python 3, matplotlib replaced by a recorder)

import os  # noqa: E402

import refformat as rf  # noqa: E402

PINS = np.load(os.path.join(rf.GOLDEN, "estimator_pins.npz"))
LRG = "Debbie_LRG_CPU_10degx10deg_LRG_binning_SLAC_1k.dat"


def _triangle_files(paths):
    hs, ns = [], []
    for p in paths:
        ngal, nb, counts = rf.parse_triangle(rf.read_bytes(p))
        hs.append(counts)
        ns.append(tuple(ngal))
    return hs, ns, nb


def _pair_file(path):
    vals = rf.read_bytes(path).split()
    ngal = (int(vals[0]), int(vals[1]))
    lo, hi = float(vals[3]), float(vals[4])
    return np.array([int(v) for v in vals[6:]], dtype=np.uint64), ngal, int(vals[2]), lo, hi


def _same(a, b):
    """Identical float64 values (NaN never occurs: the scripts set it to 0)."""
    a, b = np.asarray(a, dtype=np.float64).ravel(), np.asarray(b, dtype=np.float64).ravel()
    return a.shape == b.shape and np.array_equal(a, b)


def test_zeta_pinned_to_the_reference_script():
    for var in ("tp_s8_q8_t16", "tp_default"):
        hs, ns, nb = _triangle_files([os.path.join(rf.GOLDEN, "ref", "%s_%s.dat.gz" % (var, h))
                                      for h in ("DDD", "DDR", "DRR", "RRR")])
        z = estimators.zeta(*hs, *ns)
        assert _same(z, PINS["zeta_" + var]), var
    hs, ns, nb = _triangle_files([os.path.join(rf.GOLDEN, "sandbox", "%s_%s.gz" % (h, LRG))
                                  for h in ("DDD", "DDR", "DRR", "RRR")])
    z = estimators.zeta(*hs, *ns)
    assert _same(z, PINS["zeta_lrg"])
    assert np.count_nonzero(z) > 1000


def test_xi_and_table_pinned_to_the_reference_script():
    for var in ("2pcf_default", "2pcf_s40_1_21"):
        files = [_pair_file(os.path.join(rf.GOLDEN, "ref", "%s_%s.dat.gz" % (var, h))) for h in ("DD", "DR", "RR")]
        (dd, ndd, nbins, lo, hi), (dr, ndr, _, _, _), (rr, nrr, _, _, _) = files
        x = estimators.xi(dd, dr, rr, ndd, ndr, nrr)
        assert _same(x, PINS["xi_" + var]), var
        # the script's table: x + width with the width as the file prints it
        text = estimators.format_xi_table(estimators.xi_table(x, lo, hi, nbins))
        assert text == str(PINS["table_" + var]), var


def test_reduced_zeta_pinned_to_the_reference_script():
    """LRG golden files (25 theta bins) with the xi table of 2pcf_default."""
    hs, ns, nb = _triangle_files([os.path.join(rf.GOLDEN, "sandbox", "%s_%s.gz" % (h, LRG))
                                  for h in ("DDD", "DDR", "DRR", "RRR")])
    z = estimators.zeta(*hs, *ns)
    table = np.array([[float(v) for v in line.split()] for line in str(PINS["table_2pcf_default"]).splitlines()])
    spec = ((50, 2.0, 12.0), (16, 0.9, 4.1), (25, 0.0, 1.0))
    q = estimators.reduced_zeta(z, spec, int(PINS["sbin"]), [int(v) for v in PINS["qbins"]], table)
    want = PINS["reduced_lrg"]
    assert q.shape == want.shape
    assert np.allclose(q, want, rtol=1e-12, atol=0, equal_nan=True)


def test_jackknife_covariance_matches_restatement():
    rng = np.random.default_rng(3)
    x = rng.normal(size=(16, 12)) * rng.uniform(0.1, 3.0, size=12)
    mean, cov = estimators.jackknife_covariance(x)
    wmean, wcov = estimators_ref.jackknife_covariance(x.tolist())
    assert np.allclose(mean, wmean, rtol=1e-14, atol=1e-15)
    assert np.allclose(cov, np.array(wcov), rtol=1e-12, atol=1e-14)
    # (N-1)/N sum of squares = (N-1) times the biased sample covariance
    assert np.allclose(cov, 15 * np.cov(x, rowvar=False, bias=True), rtol=1e-12, atol=1e-14)
    assert np.allclose(cov, cov.T)
    assert np.linalg.eigvalsh(cov).min() > -1e-12


def test_zeta_jackknife_of_identical_subsamples_has_no_spread():
    h, n, spec, d, r = _hists(21)
    full = (h["DDD"], h["DDR"], h["DRR"], h["RRR"])
    out = estimators.zeta_jackknife(full, [full] * 4, (140, 150), [(140, 150)] * 4)
    assert np.array_equal(out["mean"], out["zeta"])
    assert np.all(out["sigma"] == 0)


def test_zeta_jackknife_from_region_subsamples():
    """Subsamples of the oracle's counts with one of 4 regions removed: the
    error bars are the restated formula applied to their zetas."""
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    d = synth.blobs(160, n_blobs=3, sigma=4.0, box=30.0, seed=31)
    r = synth.uniform(150, box=30.0, seed=32)
    reg_d, reg_r = (d[:, 0] // 7.5).astype(int).clip(0, 3), (r[:, 0] // 7.5).astype(int).clip(0, 3)

    def four(dd, rr):
        return tuple(oracle.triangle(c, w, spec)[0] for c, w in (([dd, dd, dd], 0), ([dd, dd, rr], 1),
                                                                 ([dd, rr, rr], 1), ([rr, rr, rr], 0)))
    full = four(d, r)
    subs = [four(d[reg_d != k], r[reg_r != k]) for k in range(4)]
    ns = [(int((reg_d != k).sum()), int((reg_r != k).sum())) for k in range(4)]
    bins = np.nonzero(full[3])[0][:20]
    out = estimators.zeta_jackknife(full, subs, (len(d), len(r)), ns, bins=bins)
    zs = [estimators_ref.zeta(*h, *estimators.norms_counts(*n)) for h, n in zip(subs, ns)]
    wmean, wcov = estimators_ref.jackknife_covariance([[z[b] for b in bins] for z in zs])
    assert np.allclose(out["mean"], wmean, rtol=1e-12, atol=1e-14)
    assert np.allclose(out["cov"], np.array(wcov), rtol=1e-10, atol=1e-14)
    assert out["sigma"].max() > 0
