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
