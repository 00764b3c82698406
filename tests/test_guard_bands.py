"""GPU: the guarded FP32 triangle path where its guard bands decide.

Triangles are built so that a ratio q (each of the three permutations) or an
angle theta (each of the three angles) lies on a bin edge, including the
range ends, and with nearly collinear points (|cos| -> 1, where the band
widens without bound).  Each base triangle A, B, C becomes one small catalog:
A, B and C moved by -6..6 units in the last place in x and in y (169 copies
of C), so that the reference's rounded q or theta falls on both sides of the
edge within a few ulps.  The copies of C also form near-degenerate triangles
(A or B with two copies of C: q a few ulps above 1, theta near 0).

The guarded FP32 kernel (with its exact recheck) must give exactly the
histograms of the plain FP64 kernel and of the oracle, with a nonzero number
of rechecked triangles.  A second test lowers the recheck queue's capacity
(TPCF_RECHECK_CAP) so that the queue overflows: the engine grows it, counts
again, and the histograms are still exact."""
import math
import platform

import numpy as np
import pytest

import oracle
import tpcf

pytestmark = pytest.mark.gpu

NATIVE_NAN = tpcf.NAN_ZERO if platform.machine() == "aarch64" else tpcf.NAN_INT_MIN
PI_REF = 3.14159  # the reference's PI: theta = acos(c) / 3.14159
SPECS = {
    "bench": ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0)),
    "sandbox": ((50, 2.0, 12.0), (16, 0.9, 4.1), (25, 0.0, 1.0)),
}


def _edges(axis):
    n, lo, hi = axis
    lo32, hi32 = np.float32(lo), np.float32(hi)
    w = np.float32((hi32 - lo32) / np.float32(n))
    return [float(np.float32(lo32 + np.float32(k) * w)) for k in range(n + 1)]


def _third_point(b, c, phi):
    """A at 0, B at (b, 0), C at distance c from A, angle phi at A."""
    return (c * math.cos(phi), c * math.sin(phi))


def _base_triangles(spec, rng):
    """(b, c, phi): sides AB = b, AC = c and the angle phi at A."""
    (ns, slo, shi), (nq, qlo, qhi), (nt, tlo, thi) = spec
    out = []
    s_mid = lambda: rng.uniform(max(slo, 0.5) + 0.3, shi - 0.3)  # noqa: E731
    for e in _edges(spec[1]):
        if e <= 1.0:
            continue
        # q = m/s (permutation 0): b = s, c = s*e, the third side longest
        s = s_mid()
        out.append((s, s * e, rng.uniform(0.62, 0.9) * math.pi))
        # q = l/s (permutation 2): b = s, c = l = s*e, the third side between
        lo_c, hi_c = 1.0 / (2.0 * e), min(e / 2.0, 0.999)
        if lo_c < hi_c:
            out.append((s, s * e, math.acos(rng.uniform(lo_c, hi_c))))
        # q = l/m (permutation 1): b = m, c = l = m*e, the third side shortest
        if e < 2.0:
            m = s_mid()
            out.append((m, m * e, math.acos(rng.uniform(e / 2.0, 1.0) * 0.999 + 0.0005)))
    for t in _edges(spec[2]):
        phi = t * PI_REF
        if not (0.0 < phi < math.pi):
            continue
        for _ in range(3):
            # sides around the angle: the opposite side is longest, shortest or
            # between for different ratios (theta0, theta1, theta2)
            b = s_mid()
            c = b * rng.uniform(1.02, 2.8)
            out.append((b, c, phi))
    # nearly collinear: |cos| -> 1 at the angle and at the other vertices
    for phi in (1e-3, 1e-4, 1e-5, math.pi - 1e-3, math.pi - 1e-4, PI_REF, PI_REF - 1e-6):
        b = s_mid()
        out.append((b, b * rng.uniform(1.05, 2.5), phi))
    return out


def _catalogs(spec, seed):
    rng = np.random.default_rng(seed)
    cats = []
    for b, c, phi in _base_triangles(spec, rng):
        origin = rng.uniform(5.0, 40.0, size=3)
        a = np.array(origin, dtype=np.float32)
        bp = np.array(origin + [b, 0.0, 0.0], dtype=np.float32)
        cx, cy = _third_point(b, c, phi)
        cp = np.array(origin + [cx, cy, 0.0], dtype=np.float32)
        pts = [a, bp]
        for dx in range(-6, 7):
            for dy in range(-6, 7):
                q = cp.copy()
                for _ in range(abs(dx)):
                    q[0] = np.nextafter(q[0], np.float32(np.inf if dx > 0 else -np.inf))
                for _ in range(abs(dy)):
                    q[1] = np.nextafter(q[1], np.float32(np.inf if dy > 0 else -np.inf))
                pts.append(q)
        cats.append(np.stack(pts).astype(np.float32))
    return cats


def _count_all(eng, cats, spec, precision):
    hs = [eng.catalog(c) for c in cats]
    specs = [tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_SAME, spec, precision=precision, nan_policy=NATIVE_NAN)] * len(hs)
    got = eng.count_batch(specs, [eng.job([h, h, h]) for h in hs])
    st = eng.stats()
    for h in hs:
        eng.release(h)
    return got, st


@pytest.mark.parametrize("name", sorted(SPECS))
def test_guard_bands_at_every_edge(name):
    spec = SPECS[name]
    cats = _catalogs(spec, seed=11 if name == "bench" else 12)
    with tpcf.Engine(0) as eng:
        fast, st = _count_all(eng, cats, spec, tpcf.GUARDED_FP32)
        exact, _ = _count_all(eng, cats, spec, tpcf.PLAIN_FP64)
    assert st["recheck_units"] > 0
    total = 0
    for c, f, x in zip(cats, fast, exact):
        want, _ = oracle.triangle([c, c, c], 0, spec, nan_zero=NATIVE_NAN == tpcf.NAN_ZERO)
        assert np.array_equal(x, want)
        assert np.array_equal(f, want)
        total += int(want.sum())
    assert total > 0


def test_recheck_queue_overflow_regrows(monkeypatch):
    spec = SPECS["bench"]
    cats = _catalogs(spec, seed=13)
    with tpcf.Engine(0) as eng:
        exact, _ = _count_all(eng, cats, spec, tpcf.PLAIN_FP64)
    monkeypatch.setenv("TPCF_RECHECK_CAP", "16")
    monkeypatch.setenv("TPCF_GRAPHS", "0")
    with tpcf.Engine(0) as eng:
        fast, st = _count_all(eng, cats, spec, tpcf.GUARDED_FP32)
    assert st["recheck_units"] > 16
    assert st["recheck_regrows"] >= 1
    for f, x in zip(fast, exact):
        assert np.array_equal(f, x)
