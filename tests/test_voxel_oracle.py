"""GPU: the batched form (every job of a light-cone count in ONE
tpcf_count_batch_into launch) against the oracle, not against the engine's
own counts.

1,500 clustered + 1,500 uniform points in a 20 x 20 degree light cone
(comoving depth 100-300), cut into 2 x 2 x 4 voxels of at least 40 (the
longest counted side of the s8 q8 t16 binning) and 2 x 2 angular jackknife
regions.  One launch holds: the four full histograms, every canonical
neighbour-voxel job of each (summed on the device per kind), the four D-D-R
subsamples as jobs of their own, and the region decomposition of the DDD,
DRR and RRR loops (jobs grouped on the device by the regions they touch).
Checked, bin for bin, against oracle.triangle:
  * full histograms and voxel sums: the oracle on the full catalogs;
  * each of the 4 x 4 jackknife subsamples (decomposed or direct): the oracle
    on the catalogs with that region's points removed."""
import platform

import numpy as np
import pytest

import oracle
import synth
import tpcf
import voxels

pytestmark = pytest.mark.gpu

TP = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
LOOP = {"same": tpcf.LOOP_SAME, "one": tpcf.LOOP_ONE, "all": tpcf.LOOP_ALL}
NATIVE_NAN = tpcf.NAN_ZERO if platform.machine() == "aarch64" else tpcf.NAN_INT_MIN
KINDS = (("DDD", tpcf.LOOP_SAME, 0), ("DDR", tpcf.LOOP_ONE, 1), ("DRR", tpcf.LOOP_ONE, 1),
         ("RRR", tpcf.LOOP_SAME, 0))


def _region(x):
    a = np.deg2rad(10.0)
    tx = np.clip(((x[:, 0] / x[:, 2] + a) / (2 * a) * 2).astype(int), 0, 1)
    ty = np.clip(((x[:, 1] / x[:, 2] + a) / (2 * a) * 2).astype(int), 0, 1)
    return tx * 2 + ty


def _oracle4(d, r):
    cats = {"D": d, "R": r}
    return [oracle.triangle([cats[x] for x in k], w, TP, nan_zero=NATIVE_NAN == tpcf.NAN_ZERO)[0]
            for k, _, w in KINDS]


def test_light_cone_batch_against_oracle():
    d = synth.lightcone(1500, clustered=True, n_blobs=40, sigma=5.0, seed=31, r_min=100.0, r_max=300.0)
    r = synth.lightcone(1500, seed=32, r_min=100.0, r_max=300.0)
    lo = np.minimum(d.min(0), r.min(0)).astype(np.float64) - 1e-3
    hi = np.maximum(d.max(0), r.max(0)).astype(np.float64) + 1e-3
    grid = (2, 2, 4)
    assert ((hi - lo) / np.array(grid) >= 40.0).all()
    od, sd, ed = voxels.voxel_order(d, lo, hi, grid)
    orr, sr, er = voxels.voxel_order(r, lo, hi, grid)
    d, r = d[od], r[orr]
    rd, rr = _region(d), _region(r)
    # region-ordered copies for the decomposition
    gd, gr = np.argsort(rd, kind="stable"), np.argsort(rr, kind="stable")
    dg, rgc, rdg, rrg = d[gd], r[gr], rd[gd], rr[gr]
    cd = np.searchsorted(rdg, np.arange(4), "left"), np.searchsorted(rdg, np.arange(4), "right")
    cr = np.searchsorted(rrg, np.arange(4), "left"), np.searchsorted(rrg, np.arange(4), "right")
    blo, bhi = voxels.cell_boxes([dg, rgc], [cd[0], cr[0]], [cd[1], cr[1]], 4)
    neighbours, near = voxels.box_near(blo, bhi, 10.0 * (1.0 + 3.0))  # longest counted side < s_hi (1 + q_hi)

    spec = {lp: tpcf.make_spec(tpcf.TRIANGLE, lp, TP, nan_policy=NATIVE_NAN) for lp in LOOP.values()}
    with tpcf.Engine(0) as eng:
        hd, hr, hdg, hrg = eng.catalog(d), eng.catalog(r), eng.catalog(dg), eng.catalog(rgc)
        cat, gcat = {"D": hd, "R": hr}, {"D": hdg, "R": hrg}
        sub = [{"D": eng.catalog(d[rd != k]), "R": eng.catalog(r[rr != k])} for k in range(4)]
        specs, jobs, outs = [], [], []
        for o, (k, lp, _) in enumerate(KINDS):  # 0-3 full histograms
            specs.append(spec[lp])
            jobs.append(eng.job([cat[x] for x in k]))
            outs.append(o)
        nvox = 0
        for o, (k, lp, _) in enumerate(KINDS):  # 4-7 voxel sums
            for roles, ranges, loop, glob in voxels.spatial_jobs(k, (sd, ed), (sr, er), grid):
                specs.append(spec[LOOP[loop]])
                jobs.append(eng.job([cat[x] for x in roles], ranges, global_index=glob))
                outs.append(4 + o)
                nvox += 1
        for reg in range(4):  # 8-11 D-D-R subsamples as jobs of their own
            specs.append(spec[tpcf.LOOP_ONE])
            jobs.append(eng.job([sub[reg][x] for x in "DDR"]))
            outs.append(8 + reg)
        n_out, group_base = 12, {}
        for k, _, _ in KINDS:
            if k == "DDR":
                continue
            cj, gid, groups = voxels.jackknife_groups(k, cd, cr, neighbours, near)
            for j, g in zip(cj, gid):
                specs.append(spec[LOOP[j[2]]])
                jobs.append(eng.job([gcat[x] for x in j[0]], j[1], global_index=j[3]))
                outs.append(n_out + g)
            group_base[k] = (n_out, groups)
            n_out += len(groups)
        got = eng.count_batch_into(specs, jobs, outs, n_out)
        st = eng.stats()
    assert nvox > 20
    assert st["kernel_launches"] == 2  # one counting launch + the guard-band recheck

    want_full = _oracle4(d, r)
    for o, (k, _, _) in enumerate(KINDS):
        assert want_full[o].sum() > 0, k
        assert np.array_equal(got[o], want_full[o]), ("full", k)
        assert np.array_equal(got[4 + o], want_full[o]), ("voxel sum", k)
    for reg in range(4):
        want = _oracle4(d[rd != reg], r[rr != reg])
        assert np.array_equal(got[8 + reg], want[1]), ("DDR subsample", reg)
        for o, (k, _, _) in enumerate(KINDS):
            if k == "DDR":
                continue
            base, groups = group_base[k]
            full, jk = voxels.jackknife_from_groups(got[base:base + len(groups)], groups, 4)
            assert np.array_equal(full, want_full[o]), ("decomposition total", k)
            assert jk[reg].sum() > 0
            assert np.array_equal(jk[reg], want[o]), ("decomposed subsample", k, reg)
