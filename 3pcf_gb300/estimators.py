"""Correlation-function estimators from the engine's histograms (host, FP64).

Mirrors the reference's post-processing scripts:
  * three-point (Szapudi-Szalay) zeta, examples/plot_MICE_3pcf.py:98-151:
      norms  DDD, RRR: N0 (N1-1) (N2-2) / 6      (each file's own header counts)
             DDR:      N0 (N1-1) N2 / 2
             DRR:      N0 N1 (N2-1) / 2
      zeta = (DDD/n - 3 DDR/n + 3 DRR/n - RRR/n) / (RRR/n); NaN -> 0, +inf -> 0
  * reduced zeta Q = zeta / (xi12 xi23 + xi23 xi31 + xi31 xi12), :175-223, with
    the triangle of bin centres s12 = s, s23 = s q, s31 = s sqrt(1 + q^2 - 2 q cos theta),
    theta = pi (x + w/2), and xi looked up at the nearest tabulated separation;
  * two-point xi, examples/plot_MICE_2pcf.py:44-75:
      norms  DD: (N0^2 - N0)/2,  DR: N0 N1,  RR: (N0^2 - N0)/2
      xi = (DD/n - 2 DR/n + RR/n) / (RR/n); NaN -> 0, +inf -> 0
    and the table file master_2pcf_reference.dat ("%f %f" of x + w and xi), :128-132.
  * jackknife covariance of zeta (no counterpart in the reference, whose
    estimator ends at zeta): for N subsamples, subsample r being the catalogs
    with the points of region r removed and zeta_r its zeta (norms from the
    subsample's own catalog sizes),
      mean_b  = (1/N) sum_r zeta_r[b]
      C[a, b] = (N - 1)/N sum_r (zeta_r[a] - mean_a) (zeta_r[b] - mean_b)
    and sigma_b = sqrt(C[b, b]), the error bar of zeta[b] of the full sample.

Histograms are the engine's uint64 counts; the reference reads the written files,
whose triangle and pair counts are unsigned int, so counts are wrapped mod 2^32
first (as the files hold them).
"""
import numpy as np

U32 = np.uint64(0xFFFFFFFF)


def _as_file_counts(h):
    return (np.asarray(h, dtype=np.uint64) & U32).astype(np.float64)


def norms_3pcf(n_ddd, n_ddr, n_drr, n_rrr):
    """Normalisations of the four histograms from their files' header counts
    (N0, N1, N2) each."""
    a, b, c = (float(v) for v in n_ddd)
    ddd = a * (b - 1) * (c - 2) / 6.0
    a, b, c = (float(v) for v in n_ddr)
    ddr = a * (b - 1) * c / 2.0
    a, b, c = (float(v) for v in n_drr)
    drr = a * b * (c - 1) / 2.0
    a, b, c = (float(v) for v in n_rrr)
    rrr = a * (b - 1) * (c - 2) / 6.0
    return ddd, ddr, drr, rrr


def zeta(ddd, ddr, drr, rrr, n_ddd, n_ddr, n_drr, n_rrr):
    """Szapudi-Szalay three-point function per (s, q, theta) bin."""
    nd = norms_3pcf(n_ddd, n_ddr, n_drr, n_rrr)
    h = [_as_file_counts(x) / n for x, n in zip((ddd, ddr, drr, rrr), nd)]
    with np.errstate(divide="ignore", invalid="ignore"):
        z = (h[0] - 3 * h[1] + 3 * h[2] - h[3]) / h[3]
    z[z != z] = 0
    z[z == np.inf] = 0
    return z


def xi(dd, dr, rr, n_dd, n_dr, n_rr):
    """Two-point function per separation bin; n_* are each file's (N0, N1)."""
    ndd = (float(n_dd[0]) * float(n_dd[0]) - float(n_dd[0])) / 2.0
    ndr = float(n_dr[0]) * float(n_dr[1])
    nrr = (float(n_rr[0]) * float(n_rr[0]) - float(n_rr[0])) / 2.0
    a, b, c = _as_file_counts(dd) / ndd, _as_file_counts(dr) / ndr, _as_file_counts(rr) / nrr
    with np.errstate(divide="ignore", invalid="ignore"):
        x = (a - 2 * b + c) / c
    x[x != x] = 0
    x[x == np.inf] = 0
    return x


def xi_table(xi_values, lo, hi, nbins):
    """(separation, xi) rows as master_2pcf_reference.dat holds them: the bin's
    lower edge plus one width."""
    w = (hi - lo) / nbins
    x = np.arange(lo, hi, w)[:nbins]
    return np.stack([x + w, np.asarray(xi_values, dtype=np.float64)], axis=1)


def format_xi_table(table):
    return "".join("%f %f\n" % (a, b) for a, b in table)


def _bin_centre(b, lo, hi, n):
    w = (hi - lo) / float(n)
    return lo + w * b + w / 2.0


def _nearest(s, xs, ys):
    return ys[int(np.argmin(np.abs(s - xs)))]


def reduced_zeta(z, spec, sbin, qbins, xi_tab):
    """Q(theta) for one s bin and the given q bins (rows), from zeta
    (S x Q x T) and a (separation, xi) table."""
    (S, slo, shi), (Q, qlo, qhi), (T, tlo, thi) = spec
    z = np.asarray(z, dtype=np.float64).reshape(S, Q, T)
    tw = (thi - tlo) / T
    x = np.arange(tlo, thi, tw)[:T]
    theta = np.pi * (x + tw / 2.0)
    s = _bin_centre(sbin, slo, shi, S)
    xs, ys = xi_tab[:, 0], xi_tab[:, 1]
    out = []
    for qb in qbins:
        q = _bin_centre(qb, qlo, qhi, Q)
        s12 = np.full(T, s)
        s23 = np.full(T, s * q)
        s31 = s * np.sqrt(1 + q * q - 2 * q * np.cos(theta))
        c12 = np.array([_nearest(v, xs, ys) for v in s12])
        c23 = np.array([_nearest(v, xs, ys) for v in s23])
        c31 = np.array([_nearest(v, xs, ys) for v in s31])
        den = c12 * c23 + c23 * c31 + c31 * c12
        with np.errstate(divide="ignore", invalid="ignore"):
            out.append(z[sbin, qb] / den)
    return np.array(out)


def zeta_error(z, z_ref, rrr):
    """Error of zeta against a reference zeta (e.g. from FP64-geometry counts)
    over the bins where RRR is populated: max and RMS absolute difference and
    the largest difference relative to max(|z_ref|, 1e-12)."""
    z = np.asarray(z, dtype=np.float64).ravel()
    z_ref = np.asarray(z_ref, dtype=np.float64).ravel()
    m = np.asarray(rrr).ravel() > 0
    if not m.any():
        return {"bins": 0, "max_abs": 0.0, "rms": 0.0, "max_rel": 0.0}
    d = np.abs(z[m] - z_ref[m])
    rel = d / np.maximum(np.abs(z_ref[m]), 1e-12)
    return {"bins": int(m.sum()), "max_abs": float(d.max()), "rms": float(np.sqrt(np.mean(d * d))),
            "max_rel": float(rel.max())}


def norms_counts(nd, nr):
    """Header counts (N0, N1, N2) of the DDD, DDR, DRR, RRR files for nd data
    and nr random points."""
    return (nd, nd, nd), (nd, nd, nr), (nd, nr, nr), (nr, nr, nr)


def jackknife_covariance(samples):
    """(mean, covariance) of N jackknife samples (N x B): the mean over the
    samples and (N - 1)/N times the sum of the outer products of the
    deviations from it."""
    x = np.asarray(samples, dtype=np.float64)
    n = x.shape[0]
    mean = x.mean(axis=0)
    dev = x - mean
    cov = (n - 1) / n * (dev.T @ dev)
    return mean, cov


def zeta_jackknife(full, subsamples, n_full, n_sub, bins=None):
    """zeta of the full sample with its jackknife error.

    full: (DDD, DDR, DRR, RRR) histograms of the full catalogs; subsamples:
    one such tuple per region r, counted on the catalogs without region r;
    n_full: (nd, nr) catalog sizes; n_sub: one (nd, nr) per region.  bins:
    the flat bin indices the covariance is kept for (default all; a
    covariance of B bins holds B^2 doubles).  Returns a dict with zeta (all
    bins), the jackknife mean, covariance and sigma over the chosen bins."""
    z = zeta(*full, *norms_counts(*n_full))
    zs = np.stack([zeta(*h, *norms_counts(*n)) for h, n in zip(subsamples, n_sub)])
    sel = np.arange(z.size) if bins is None else np.asarray(bins)
    mean, cov = jackknife_covariance(zs[:, sel])
    return {"zeta": z, "bins": sel, "mean": mean, "cov": cov, "sigma": np.sqrt(np.diag(cov))}
