"""GPU parity at the benchmark workloads' own scale: the engine, through the
C ABI, against the oracle (tolerance 0, every bin) on

* the three-side workload in full: DDD and RRR of 1000 clustered + 1000
  uniform points in a 100^3 cube, 16 bins on [0,40) with the reference's
  overflow aliasing (sides >= 40 give index n+1, src/3pcf_C_version.cc:27-30,139);
  1e9 ordered triples per histogram;
* a 2,000 + 2,000-point sub-sample of the triangle-parametrization workload
  (the first 2,000 points of each of its catalogs: clustered blobs in a 100^3
  cube, uniform randoms in a 200^3 cube), all four histograms DDD/DDR/DRR/RRR
  with s 8 bins on [2,10), q 8 on [1,3), theta 16 on [0,pi)
  (src/3pcf_C_version_triangle_parametrization.cc:477-533); 1.1e10 triangles;
* a 2,000-point sub-sample of the lattice workload at its density (30 % of the
  points on the integer lattice, box scaled so that the number density is that
  of 500k points in 500^3), three-side 32 bins on [0,32), triples with a side
  >= 32 left out; 8e9 ordered triples.

Each is counted with the guarded FP32 path and the plain FP64 kernel."""
import platform

import numpy as np
import pytest

import oracle
import synth
import tpcf

pytestmark = pytest.mark.gpu

NATIVE_NAN = tpcf.NAN_ZERO if platform.machine() == "aarch64" else tpcf.NAN_INT_MIN
PRECISIONS = (tpcf.GUARDED_FP32, tpcf.PLAIN_FP64)


@pytest.fixture(scope="module")
def eng():
    e = tpcf.Engine(0)
    yield e
    e.close()


def test_three_side_workload_in_full(eng):
    d = synth.blobs(1000, n_blobs=20, sigma=5.0, box=100.0, seed=1)
    r = synth.uniform(1000, box=100.0, seed=0)
    axis = (16, 0.0, 40.0)
    hd, hr = eng.catalog(d), eng.catalog(r)
    for h, cat in ((hd, d), (hr, r)):
        want, n = oracle.three_side([cat] * 3, axis[1], axis[2], axis[0])
        assert n == 1000 ** 3
        # sides >= 40 occur: their code n+1 aliases into other bins or gives
        # an index past the reference's array (not counted)
        assert 0 < want.sum() < n
        for prec in PRECISIONS:
            s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [axis], precision=prec)
            got = eng.count(s, eng.job([h, h, h]))
            assert np.array_equal(got, want), prec
            assert eng.stats()["loop_units"] == n
    eng.release(hd)
    eng.release(hr)


def test_triangle_workload_subsample(eng):
    d = synth.blobs(10000, n_blobs=20, sigma=5.0, box=100.0, seed=1)[:2000]
    r = synth.uniform(10000, box=200.0, seed=0)[:2000]
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    hd, hr = eng.catalog(d), eng.catalog(r)
    combos = [("DDD", [hd, hd, hd], [d, d, d], 0), ("DDR", [hd, hd, hr], [d, d, r], 1),
              ("DRR", [hd, hr, hr], [d, r, r], 1), ("RRR", [hr, hr, hr], [r, r, r], 0)]
    want = {}
    for name, _, cats, which in combos:
        want[name] = oracle.triangle(cats, which, spec, nan_zero=NATIVE_NAN == tpcf.NAN_ZERO)
    for prec in PRECISIONS:
        specs = [tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_ONE if w else tpcf.LOOP_SAME, spec, precision=prec,
                                nan_policy=NATIVE_NAN) for _, _, _, w in combos]
        got = eng.count_batch(specs, [eng.job(hs) for _, hs, _, _ in combos])
        for (name, _, _, _), g in zip(combos, got):
            w, _ = want[name]
            assert w.sum() > 0, name
            assert np.array_equal(g, w), (name, prec, int((g != w).sum()))
        assert eng.stats()["loop_units"] == sum(n for _, n in want.values())
    eng.release(hd)
    eng.release(hr)


def test_lattice_workload_subsample(eng):
    n = 2000
    pts = synth.lattice_mix(n, box=500.0 * (n / 500000.0) ** (1.0 / 3.0), frac=0.3, seed=3)
    axis = (32, 0.0, 32.0)
    want, units = oracle.three_side([pts] * 3, axis[1], axis[2], axis[0], clean=True)
    assert units == n ** 3
    assert want.sum() > 10 ** 6
    h = eng.catalog(pts)
    for prec in PRECISIONS:
        s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [axis], precision=prec, overflow=tpcf.OVERFLOW_CLEAN)
        got = eng.count(s, eng.job([h, h, h]))
        assert np.array_equal(got, want), prec
    eng.release(h)
