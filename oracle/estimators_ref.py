"""TEST INFRASTRUCTURE ONLY: element-by-element restatement of the reference's
estimator scripts, used to check 3pcf_gb300/estimators.py.

  zeta: examples/plot_MICE_3pcf.py:98-151
  xi:   examples/plot_MICE_2pcf.py:44-75, table file :128-132
"""
import math


def zeta(ddd, ddr, drr, rrr, n_ddd, n_ddr, n_drr, n_rrr):
    # :98-107 (normalisations use each file's own header counts)
    ddd_norm = float(n_ddd[0] * (n_ddd[1] - 1) * (n_ddd[2] - 2)) / 6.
    ddr_norm = float(n_ddr[0] * (n_ddr[1] - 1) * n_ddr[2]) / 2.
    drr_norm = float(n_drr[0] * n_drr[1] * (n_drr[2] - 1)) / 2.
    rrr_norm = float(n_rrr[0] * (n_rrr[1] - 1) * (n_rrr[2] - 2)) / 6.
    out = []
    for a, b, c, d in zip(ddd, ddr, drr, rrr):
        a, b, c, d = (float(int(v) % 2 ** 32) for v in (a, b, c, d))  # the files hold unsigned int
        a /= ddd_norm
        b /= ddr_norm
        c /= drr_norm
        d /= rrr_norm
        num = a - 3 * b + 3 * c - d
        if d == 0.0:
            t = float("nan") if num == 0.0 else math.copysign(float("inf"), num)
        else:
            t = num / d
        if t != t or t == float("inf"):  # :150-151
            t = 0.0
        out.append(t)
    return out


def xi(dd, dr, rr, n_dd, n_dr, n_rr):
    dd_norm = float((n_dd[0] * n_dd[0]) - n_dd[0]) / 2.
    dr_norm = float(n_dr[0] * n_dr[1])
    rr_norm = float((n_rr[0] * n_rr[0]) - n_rr[0]) / 2.
    out = []
    for a, b, c in zip(dd, dr, rr):
        a, b, c = (float(int(v) % 2 ** 32) for v in (a, b, c))
        a /= dd_norm
        b /= dr_norm
        c /= rr_norm
        num = a - 2 * b + c
        if c == 0.0:
            t = float("nan") if num == 0.0 else math.copysign(float("inf"), num)
        else:
            t = num / c
        if t != t or t == float("inf"):
            t = 0.0
        out.append(t)
    return out


def reduced_zeta(z, spec, sbin, qbins, xi_x, xi_y):
    """Element-by-element restatement of examples/plot_MICE_3pcf.py:175-232:
    sxx2cf (:7-28, nearest tabulated separation, first on ties), bin2val
    (:30-36), sqtheta2s1s2s3 (:39-45), Q = zeta / (x12 x23 + x23 x31 + x31 x12)."""
    import math
    (S, slo, shi), (Q, qlo, qhi), (T, tlo, thi) = spec
    tw = (thi - tlo) / T

    def bin2val(b, lo, hi, n):
        w = (hi - lo) / float(n)
        return lo + (w * b) + (w / 2.0)

    def nearest(s):
        diffs = [abs(s - x) for x in xi_x]
        m = min(diffs)
        return xi_y[diffs.index(m)]

    sval = bin2val(sbin, slo, shi, S)
    out = []
    for qb in qbins:
        qval = bin2val(qb, qlo, qhi, Q)
        row = []
        for t in range(T):
            x = tlo + t * tw
            theta = math.pi * (x + tw / 2.0)
            s12, s23 = sval, sval * qval
            s31 = sval * math.sqrt(1 + qval * qval - 2 * qval * math.cos(theta))
            c12, c23, c31 = nearest(s12), nearest(s23), nearest(s31)
            den = c12 * c23 + c23 * c31 + c31 * c12
            zz = z[(sbin * Q + qb) * T + t]
            row.append(zz / den if den != 0 else (math.copysign(math.inf, zz) if zz != 0 else math.nan))
        out.append(row)
    return out


def jackknife_covariance(samples):
    """Element-by-element restatement of the jackknife covariance of
    3pcf_gb300/estimators.py (no reference counterpart):
    mean_b = (1/N) sum_r x_r[b]; C[a][b] = (N-1)/N sum_r (x_r[a]-mean_a)(x_r[b]-mean_b)."""
    n = len(samples)
    nb = len(samples[0])
    mean = [sum(float(samples[r][b]) for r in range(n)) / n for b in range(nb)]
    cov = [[0.0] * nb for _ in range(nb)]
    for a in range(nb):
        for b in range(nb):
            acc = 0.0
            for r in range(n):
                acc += (float(samples[r][a]) - mean[a]) * (float(samples[r][b]) - mean[b])
            cov[a][b] = (n - 1) / n * acc
    return mean, cov
