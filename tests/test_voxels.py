"""Spatial voxel decomposition: the sum of the canonical neighbour-voxel jobs
(tpcf_count_batch_into, catalog-wide loop indices for DDR) equals the one-job
count of every histogram, exactly; plus the summed-output batch semantics."""
import numpy as np
import pytest

import synth
import tpcf
import voxels

TP = [(8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0)]  # longest counted side < 40
LOOP = {"same": tpcf.LOOP_SAME, "one": tpcf.LOOP_ONE, "all": tpcf.LOOP_ALL}


def test_spatial_jobs_cover_each_canonical_triple_once():
    """CPU check of the enumeration: on a 3x3x3 grid with every voxel
    occupied, DDD jobs cover each unordered neighbour triple of voxels once."""
    grid = (3, 3, 3)
    n = 27
    occ_range = (np.arange(n) * 10, np.arange(n) * 10 + 10)
    jobs = voxels.spatial_jobs("DDD", occ_range, occ_range, grid)
    seen = set()
    for roles, ranges, loop, glob in jobs:
        vs = tuple(sorted(r[0] // 10 for r in ranges))
        assert vs not in seen
        seen.add(vs)
    want = set()
    for a in range(n):
        for b in range(a, n):
            for c in range(b, n):
                if voxels._adjacent(a, b, grid) and voxels._adjacent(a, c, grid) and voxels._adjacent(b, c, grid):
                    want.add((a, b, c))
    assert seen == want


def test_cell_jobs_cover_every_cell_multiset_once():
    """With every pair of cells near, the DDD cell jobs cover each multiset of
    cells once, and the DDR/DRR jobs each ordered role pattern once."""
    n = 5
    rng_ = (np.arange(n) * 10, np.arange(n) * 10 + 10)
    allnb = lambda v, occ: [int(c) for c in np.nonzero(occ)[0]]
    near = lambda a, b: True
    seen = [tuple(sorted(j[4])) for j in voxels.cell_jobs("DDD", rng_, rng_, allnb, near)]
    assert len(seen) == len(set(seen))
    assert set(seen) == {(a, b, c) for a in range(n) for b in range(a, n) for c in range(b, n)}
    drr = [(j[4][0],) + tuple(sorted(j[4][1:])) for j in voxels.cell_jobs("DRR", rng_, rng_, allnb, near)]
    assert len(drr) == len(set(drr)) == n * n * (n + 1) // 2
    ddr = [j[4] for j in voxels.cell_jobs("DDR", rng_, rng_, allnb, near)]
    # ordered data-cell pairs (u, v) with u == v once, u != v both ways, each with every random cell
    assert len(ddr) == len(set(ddr)) == n * n * n
    for j in voxels.cell_jobs("DDD", rng_, rng_, allnb, near):
        for (lo, hi), c in zip(j[1], j[4]):
            assert lo == c * 10 and hi == c * 10 + 10


def test_cell_jobs_with_a_sparse_neighbour_relation():
    """A random symmetric neighbour relation: the DDD jobs cover exactly the
    cell multisets whose cells are pairwise near, once each; DRR jobs every
    (data cell, unordered random pair) within reach, DDR jobs every ordered
    (data cell pair, random cell) within reach, each once."""
    rng = np.random.default_rng(7)
    n = 9
    m = rng.random((n, n)) < 0.45
    near_m = m | m.T | np.eye(n, dtype=bool)
    rng_ = (np.arange(n) * 10, np.arange(n) * 10 + 10)
    neighbours = lambda v, occ: [int(c) for c in np.nonzero(occ)[0] if near_m[v, c]]
    near = lambda a, b: bool(near_m[a, b])
    ok = lambda cells: all(near_m[x, y] for x in cells for y in cells)
    ddd = [tuple(sorted(j[4])) for j in voxels.cell_jobs("DDD", rng_, rng_, neighbours, near)]
    assert len(ddd) == len(set(ddd))
    assert set(ddd) == {(a, b, c) for a in range(n) for b in range(a, n) for c in range(b, n) if ok((a, b, c))}
    drr = [(j[4][0],) + tuple(sorted(j[4][1:])) for j in voxels.cell_jobs("DRR", rng_, rng_, neighbours, near)]
    assert len(drr) == len(set(drr))
    assert set(drr) == {(u, v, w) for u in range(n) for v in range(n) for w in range(v, n) if ok((u, v, w))}
    ddr = [j[4] for j in voxels.cell_jobs("DDR", rng_, rng_, neighbours, near)]
    assert len(ddr) == len(set(ddr))
    assert set(ddr) == {(u, v, w) for u in range(n) for v in range(n) for w in range(n) if ok((u, v, w))}


def test_box_near_is_conservative():
    """Two cells whose points come within the reach of each other are always
    near (the box gap never exceeds a point distance)."""
    rng = np.random.default_rng(8)
    pts = rng.uniform(0, 100, size=(3000, 3)).astype(np.float32)
    cell = (pts[:, 0] // 25).astype(int) * 4 + (pts[:, 1] // 25).astype(int)
    order = np.argsort(cell, kind="stable")
    pts, cell = pts[order], cell[order]
    st = np.searchsorted(cell, np.arange(16), "left")
    en = np.searchsorted(cell, np.arange(16), "right")
    lo, hi = voxels.cell_boxes([pts], [st], [en], 16)
    reach = 12.0
    neighbours, near = voxels.box_near(lo, hi, reach)
    sample = rng.choice(len(pts), 400, replace=False)
    for i in sample:
        dd = np.sqrt(((pts - pts[i]) ** 2).sum(1))
        for c in np.unique(cell[dd < reach]):
            assert near(int(cell[i]), int(c)) and near(int(c), int(cell[i]))
    occ = en > st
    for v in range(16):
        assert v in neighbours(v, occ)


def _ref_dist32(a, b):
    """The reference's float side length: sqrt((dx*dx + dy*dy) + dz*dz) in float32."""
    d = (a - b).astype(np.float32)
    s = np.float32(d[0] * d[0]) + np.float32(d[1] * d[1])
    s = np.float32(s) + np.float32(d[2] * d[2])
    return np.float32(np.sqrt(np.float32(s)))


def test_box_near_keeps_pairs_that_round_below_the_edge():
    """Pairs of points in two cells whose exact distance is at or just above
    the edge hi, but whose float32 length (as the kernels compute it) is below
    hi, must still make the two cells near."""
    rng = np.random.default_rng(9)
    hi = np.float32(12.0)
    found = 0
    for _ in range(4000):
        a = rng.uniform(0, 30, size=3).astype(np.float32)
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        b = (a.astype(np.float64) + u * float(hi) * (1 + rng.uniform(0, 2e-7))).astype(np.float32)
        exact = np.linalg.norm(a.astype(np.float64) - b.astype(np.float64))
        if exact < hi or _ref_dist32(a, b) >= hi:
            continue
        found += 1
        lo_ = np.stack([a, b]).astype(np.float64)
        neighbours, near = voxels.box_near(lo_, lo_, float(hi))
        assert near(0, 1) and near(1, 0)
    assert found > 0


def test_jackknife_from_groups_arithmetic():
    """JK_r = full - (groups touching r), on made-up group histograms."""
    groups = [frozenset({0}), frozenset({0, 1}), frozenset({1, 2}), frozenset({2})]
    hs = [np.full(4, v, dtype=np.uint64) for v in (1, 10, 100, 1000)]
    full, jk = voxels.jackknife_from_groups(hs, groups, 3)
    assert (full == 1111).all()
    assert (jk[0] == 1100).all() and (jk[1] == 1001).all() and (jk[2] == 11).all()


def _setup(seed):
    d = synth.blobs(2500, n_blobs=12, sigma=5.0, box=130.0, seed=seed)
    r = synth.uniform(2000, box=130.0, seed=seed + 1)
    lo = np.minimum(d.min(0), r.min(0)).astype(np.float64) - 1e-3
    hi = np.maximum(d.max(0), r.max(0)).astype(np.float64) + 1e-3
    assert ((hi - lo) / 3 >= 40.0).all()
    od, sd, ed = voxels.voxel_order(d, lo, hi, (3, 3, 3))
    orr, sr, er = voxels.voxel_order(r, lo, hi, (3, 3, 3))
    return d[od], r[orr], (sd, ed), (sr, er)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5])
def test_voxel_sum_equals_full_count(seed):
    d, r, dr, rr = _setup(seed)
    with tpcf.Engine(0) as eng:
        hd, hr = eng.catalog(d), eng.catalog(r)
        cat = {"D": hd, "R": hr}
        full = {"DDD": ([hd, hd, hd], tpcf.LOOP_SAME), "DDR": ([hd, hd, hr], tpcf.LOOP_ONE),
                "DRR": ([hd, hr, hr], tpcf.LOOP_ONE), "RRR": ([hr, hr, hr], tpcf.LOOP_SAME)}
        specs, jobs, outs = [], [], []
        for o, k in enumerate(full):
            hs, loop = full[k]
            specs.append(tpcf.make_spec(tpcf.TRIANGLE, loop, TP))
            jobs.append(eng.job(hs))
            outs.append(o)
        for o, k in enumerate(full):
            for roles, ranges, loop, glob in voxels.spatial_jobs(k, dr, rr, (3, 3, 3)):
                specs.append(tpcf.make_spec(tpcf.TRIANGLE, LOOP[loop], TP))
                jobs.append(eng.job([cat[x] for x in roles], ranges, global_index=glob))
                outs.append(4 + o)
        got = eng.count_batch_into(specs, jobs, outs, 8)
        assert eng.stats()["kernel_launches"] == 2  # one counting launch + recheck
        for o, k in enumerate(full):
            assert got[o].sum() > 0, k
            assert np.array_equal(got[o], got[4 + o]), (k, int(np.abs(got[o].astype(np.int64) - got[4 + o].astype(np.int64)).sum()))
        # the same full counts through the plain batch
        plain = eng.count_batch(specs[:4], jobs[:4])
        for a, b in zip(plain, got[:4]):
            assert np.array_equal(a, b)


@pytest.mark.gpu
def test_count_batch_into_sums_and_checks():
    d = synth.blobs(800, n_blobs=3, sigma=5.0, box=50.0, seed=9)
    with tpcf.Engine(0) as eng:
        h = eng.catalog(d)
        sp = tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [(100, 0.0, 50.0)])
        chunks = [voxels.vox2gal(4, i, len(d)) for i in range(4)]
        jobs = [eng.job([h, h], [chunks[i], chunks[j]]) for i in range(4) for j in range(4)]
        single = eng.count_batch([sp] * len(jobs), jobs)
        summed = eng.count_batch_into([sp] * len(jobs), jobs, [0] * len(jobs), 1)[0]
        assert np.array_equal(summed, sum(single))
        two = eng.count_batch_into([sp] * len(jobs), jobs, [i % 2 for i in range(len(jobs))], 2)
        assert np.array_equal(two[0], sum(single[0::2])) and np.array_equal(two[1], sum(single[1::2]))
        with pytest.raises(tpcf.EngineError):
            eng.count_batch_into([sp], jobs[:1], [3], 2)


@pytest.mark.gpu
def test_radecz_conversion_matches_script():
    """Device conversion of ra/dec/redshift against the numpy restatement of
    the reference's script: equal floats except at a float rounding boundary
    of the double result (then one float ulp)."""
    import convert_ref
    rng = np.random.Generator(np.random.PCG64(77))
    n = 200000
    ra = 20.0 * rng.random(n)
    dec = np.rad2deg(np.arccos(np.cos(np.deg2rad(70)) * rng.random(n))) - 70
    zr = ((0.55 ** 3 - 0.15 ** 3) * rng.random(n) + 0.15 ** 3) ** (1.0 / 3)
    want = convert_ref.radecz_to_xyz(ra, dec, zr).astype(np.float32)
    with tpcf.Engine(0) as eng:
        got = eng.convert_radecz(ra, dec, zr)
        other = eng.convert_radecz(ra[:10], dec[:10], zr[:10], poly=(0.0, 1000.0, 0.0))
    ulp = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
    assert ulp.max() <= 1
    assert (ulp == 0).mean() > 0.9999
    assert np.allclose(other, convert_ref.radecz_to_xyz(ra[:10], dec[:10], zr[:10], (0.0, 1000.0, 0.0)), rtol=1e-6)


@pytest.mark.gpu
def test_count_batch_into_mixed_kinds():
    """Jobs of different kinds and binnings in one call (one launch each):
    every output gets the sum of its own jobs."""
    d = synth.blobs(900, n_blobs=3, sigma=5.0, box=50.0, seed=19)
    r = synth.uniform(800, box=50.0, seed=20)
    with tpcf.Engine(0) as eng:
        hd, hr = eng.catalog(d), eng.catalog(r)
        tp = tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_SAME, TP)
        tp1 = tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_ONE, TP)
        jbj = tpcf.make_spec(tpcf.TRIANGLE_JBJ, tpcf.LOOP_SAME, [(10, 1.0, 11.0), (8, 0.2, 1.0), (10, 0.0, 1.0)])
        pr = tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [(100, 0.0, 50.0)])
        specs = [tp, tp1, jbj, pr, pr, tp]
        jobs = [eng.job([hd, hd, hd]), eng.job([hd, hd, hr]), eng.job([hd, hd, hd]), eng.job([hd, hd]),
                eng.job([hr, hr]), eng.job([hr, hr, hr])]
        outs = [0, 0, 1, 2, 2, 3]
        got = eng.count_batch_into(specs, jobs, outs, 4)
        single = [eng.count(s, j) for s, j in zip(specs, jobs)]
        assert np.array_equal(got[0], single[0] + single[1])
        assert np.array_equal(got[1], single[2])
        assert np.array_equal(got[2], single[3] + single[4])
        assert np.array_equal(got[3], single[5])
        assert all(g.sum() > 0 for g in got)


@pytest.mark.gpu
def test_jackknife_by_cells_equals_subsample_counts():
    """Jackknife subsamples (one region of points removed from both catalogs)
    from one cell decomposition equal the direct counts of the subsamples,
    for the histograms whose loop compares indices of one catalog only (DDD,
    DRR, RRR; the D-D-R loop compares a data index with a random index, so
    removing points shifts that comparison and its subsamples are counted
    directly)."""
    d = synth.lightcone(3000, clustered=True, seed=21)
    r = synth.lightcone(3000, seed=22)
    # 2 x 2 angular regions of the flat-sky slab, as region ids 0..3; the
    # catalogs in region order
    reg = lambda x: (np.clip(((x[:, 0] / x[:, 2] + np.deg2rad(10)) / np.deg2rad(20) * 2).astype(int), 0, 1) * 2
                     + np.clip(((x[:, 1] / x[:, 2] + np.deg2rad(10)) / np.deg2rad(20) * 2).astype(int), 0, 1))
    d, r = d[np.argsort(reg(d), kind="stable")], r[np.argsort(reg(r), kind="stable")]
    rd, rr = reg(d), reg(r)
    sd = np.searchsorted(rd, np.arange(4), "left"), np.searchsorted(rd, np.arange(4), "right")
    sr = np.searchsorted(rr, np.arange(4), "left"), np.searchsorted(rr, np.arange(4), "right")
    lo, hi = voxels.cell_boxes([d, r], [sd[0], sr[0]], [sd[1], sr[1]], 4)
    neighbours, near = voxels.box_near(lo, hi, 40.0 * 1.001)
    kinds = {"DDD": tpcf.LOOP_SAME, "DRR": tpcf.LOOP_ONE, "RRR": tpcf.LOOP_SAME}
    with tpcf.Engine(0) as eng:
        hd, hr = eng.catalog(d), eng.catalog(r)
        cat = {"D": hd, "R": hr}
        specs, jobs, outs, per_kind = [], [], [], {}
        for k in kinds:
            cj, gid, groups = voxels.jackknife_groups(k, sd, sr, neighbours, near)
            base = max(outs) + 1 if outs else 0
            for j, g in zip(cj, gid):
                specs.append(tpcf.make_spec(tpcf.TRIANGLE, LOOP[j[2]], TP))
                jobs.append(eng.job([cat[x] for x in j[0]], j[1], global_index=j[3]))
                outs.append(base + g)
            per_kind[k] = (base, groups)
        got = eng.count_batch_into(specs, jobs, outs, max(outs) + 1)
        for k, loop in kinds.items():
            base, groups = per_kind[k]
            full, jk = voxels.jackknife_from_groups(got[base:base + len(groups)], groups, 4)
            sp = tpcf.make_spec(tpcf.TRIANGLE, loop, TP)
            assert np.array_equal(full, eng.count(sp, eng.job([cat[x] for x in k]))), k
            for rg in range(4):
                sub = {"D": eng.catalog(d[rd != rg]), "R": eng.catalog(r[rr != rg])}
                assert jk[rg].sum() > 0
                assert np.array_equal(jk[rg], eng.count(sp, eng.job([sub[x] for x in k]))), (k, rg)
                for h in sub.values():
                    eng.release(h)
