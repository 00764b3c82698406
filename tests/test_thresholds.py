"""The squared-length threshold method of the three-side (clean mode) and pair
kernels, restated on the CPU: a bin is a non-decreasing step function of the
squared length as the reference sums it; with the exact float threshold of
every step (bisection over the ordered float bit patterns), a first guess
that is off by at most one step and two compares give the reference's bin for
every input.  The engine's own thresholds are exercised on the GPU by the
parity tests (lattice catalogs put separations exactly on bin edges)."""
import numpy as np

f32 = np.float32


def three_side_code(d2, lo, hi, bw, n):
    """distance_to_bin of the three-side program on sqrtf(d2); n + 1 for d >= hi."""
    d = np.sqrt(f32(d2))
    if d < lo:
        return 0
    if d >= hi:
        return n + 1
    return int(f32(f32(d - lo) / bw))


def pair_code(d2, lo, hi, bw, n):
    """The pair program's bin + 1 on sqrtf(d2); 0 below lo, n + 2 at or above hi."""
    d = np.sqrt(f32(d2))
    if d < lo:
        return 0
    if d >= hi:
        return n + 2
    return int(f32(f32(d - lo) / bw)) + 1


def smallest_d2(code, v):
    lo, hi = 0, 0x7F800000
    while lo < hi:
        mid = (lo + hi) // 2
        if code(np.array(mid, dtype=np.uint32).view(np.float32)) >= v:
            hi = mid
        else:
            lo = mid + 1
    return np.array(lo, dtype=np.uint32).view(np.float32)


def thresholds(code, top):
    u = [f32(-np.inf)] + [smallest_d2(code, v) for v in range(1, top + 1)] + [f32(np.nan)]
    return np.array(u, dtype=np.float32)


def lookup(d2, u, lo, inv_bw, offset, top, rel_err):
    """The kernels' correction of a guess from a square root with relative
    error rel_err (offset: 0 for three-side codes, 1 for pair codes).  The
    guess rounds to nearest: the code skips a value where d reaches hi (from
    the last bin to "at or above hi" when no rounding gives bin nbins), and a
    truncated guess just below that edge would be two steps short."""
    da = f32(np.sqrt(np.float64(d2)) * (1.0 + rel_err))
    g = int(np.rint(f32(f32(da - lo) * inv_bw))) + offset if np.isfinite(da) else top
    g = min(max(g, 0), top)
    return g - 1 + int(d2 >= u[g]) + int(d2 >= u[g + 1])


def _samples(u, rng):
    """Squared lengths at and around every threshold, and random ones."""
    out = []
    for t in u[1:-1]:
        bits = np.array(t, dtype=np.float32).view(np.uint32)
        for k in (-2, -1, 0, 1, 2):
            out.append(np.array(max(int(bits) + k, 0), dtype=np.uint32).view(np.float32))
    out += list(rng.uniform(0, float(u[-2]) * 1.5, 2000).astype(np.float32))
    out += [f32(0.0)]
    return out


def test_three_side_thresholds():
    rng = np.random.default_rng(1)
    for n, lo, hi in ((32, 0.0, 32.0), (16, 0.0, 40.0), (7, 1.5, 12.0), (24, 2.0, 20.0)):
        lo, hi = f32(lo), f32(hi)
        bw = f32(f32(hi - lo) / f32(n))
        code = lambda x: three_side_code(x, lo, hi, bw, n)
        u = thresholds(code, n + 1)
        assert np.all(np.diff(u[1:-1]) >= 0)
        inv = f32(1.0) / bw
        for d2 in _samples(u, rng):
            want = code(d2)
            for err in (-2.0 ** -20, 0.0, 2.0 ** -20):
                assert lookup(d2, u, lo, inv, 0, n + 1, err) == want, (n, lo, hi, float(d2), err)


def test_pair_thresholds():
    rng = np.random.default_rng(2)
    for n, lo, hi in ((700, 0.0, 70.0), (40, 1.0, 21.0), (10, 0.0, 10.0)):
        lo, hi = f32(lo), f32(hi)
        bw = f32(f32(hi - lo) / f32(n))
        code = lambda x: pair_code(x, lo, hi, bw, n)
        u = thresholds(code, n + 2)
        inv = f32(1.0) / bw
        for d2 in _samples(u, rng)[::3]:
            want = code(d2)
            for err in (-2.0 ** -20, 2.0 ** -20):
                assert lookup(d2, u, lo, inv, 1, n + 2, err) == want, (n, float(d2), err)


def test_truncated_guess_misses_the_step_at_hi():
    """Why the guess rounds: with 32 bins on [0, 32), d2 = 1024 (d = hi) has
    code 33 after code 31 (code 32 never occurs); a guess from a square root a
    little below 32, truncated, lands on 31 and two compares reach only 32."""
    lo, hi, n = f32(0.0), f32(32.0), 32
    bw = f32(f32(hi - lo) / f32(n))
    code = lambda x: three_side_code(x, lo, hi, bw, n)
    u = thresholds(code, n + 1)
    assert u[32] == u[33] == f32(1024.0)
    assert code(f32(1024.0)) == 33
    da = f32(32.0 * (1 - 2.0 ** -20))
    g = min(max(int(np.trunc(f32(da - lo) * f32(1.0) / bw)), 0), n + 1)
    assert g - 1 + int(f32(1024.0) >= u[g]) + int(f32(1024.0) >= u[g + 1]) == 32
    assert lookup(f32(1024.0), u, lo, f32(1.0) / bw, 0, n + 1, -2.0 ** -20) == 33



def test_fast_arc_cosine_fit_error():
    """The guarded triangle kernel's arc cosine acos(x) ~ sqrt(1 - x) P(x) on
    [0, 1] (coefficients in engine.cpp): a minimax fit whose error
    equioscillates at 7 points and stays within the 6.4e-7 rad its guard band
    budgets for it."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "3pcf_gb300", "csrc",
                            "engine.cpp")).read()
    body = re.search(r"static const double coef\[6\] = \{([^}]*)\}", src).group(1)
    coef = np.array([float(v) for v in body.split(",")])
    x = np.linspace(0.0, 1.0, 2000001)
    err = np.sqrt(1.0 - x) * np.polyval(coef[::-1], x) - np.arccos(x)
    assert np.abs(err).max() <= 6.4e-7
    sign = np.sign(err[np.abs(err) > 1e-9])
    assert int((np.diff(sign) != 0).sum()) == 6  # 7 alternating extrema: the minimax form
