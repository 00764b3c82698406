"""The reference's voxel decomposition (`-X division -x iiijjjkkk`) as jobs.

src/3pcf_C_version_triangle_parametrization.cc:52-80 (vox2gal) cuts each
catalog's index range into `division` chunks, the last one taking the
remainder; :306-313 decode `-x iiijjjkkk` into one chunk index per input
file.  examples/build_voxel_submission_scripts.py submits every (i, j, k) in
range(division)^3 as its own job and examples/sum_voxels.py adds the files.
The loops of a chunk job compare LOCAL indices, so the sum over chunk jobs is
what the reference's voxel workflow produces (not the one-file count).
"""
import numpy as np


def vox2gal(division, index, ngals):
    """[lo, hi) of chunk `index` of `ngals` points cut into `division` chunks."""
    per = ngals // division
    if per == 0:
        raise ValueError("Voxel chunks are bigger than the number of galaxies!")
    lo = per * index
    hi = per * (index + 1)
    if index == division - 1:
        hi += ngals % division
    return lo, hi


def decode(vtemp, ncat=3):
    """-x iiijjjkkk -> chunk index per input file."""
    idx = [vtemp // 1000000, (vtemp // 1000) % 1000, vtemp % 1000]
    return idx[:ncat]


def chunk_ranges(division, sizes):
    """Every chunk-index triple (pair for two catalogs) with its per-catalog
    [lo, hi) ranges, in the order the submission script visits them."""
    out = []
    if len(sizes) == 2:
        for i in range(division):
            for j in range(division):
                out.append(((i, j), [vox2gal(division, i, sizes[0]), vox2gal(division, j, sizes[1])]))
        return out
    for i in range(division):
        for j in range(division):
            for k in range(division):
                out.append(((i, j, k), [vox2gal(division, i, sizes[0]), vox2gal(division, j, sizes[1]),
                                        vox2gal(division, k, sizes[2])]))
    return out


# ---------------------------------------------------------------------------
# Spatial voxels whose job sum equals the one-job count.
#
# The catalogs are ordered by voxel (a grid over their common bounding box);
# a voxel is then a contiguous index range.  With voxel edges at least the
# longest side a counted triangle can have, every counted triangle lies in
# voxels that are pairwise neighbours (index difference <= 1 on each axis), so
# canonical neighbour-voxel triples cover every counted triangle exactly once:
#   DDD, RRR (unordered distinct triples of one catalog):
#       V=V=V -> (V, V, V) same-array loop; V=V<W -> (W, V, V) one-array loop;
#       U<V=V -> (U, V, V) one-array loop;  U<V<W -> (U, V, W) every triple
#   DRR (every data point with every unordered random pair):
#       (U, V, V) one-array loop; (U, V, W), V<W, every triple
#   DDR (ordered data pairs (i, j), randoms k, k >= j in catalog order):
#       (U, U, W) one-array loop; (U, V, W) and (V, U, W), U<V, one-array loop,
#       all with catalog-wide loop indices.


def voxel_order(points, lo, hi, grid):
    """Stable order of the points by voxel id (x-major), the voxel id of each
    sorted point, and the [start, end) of every voxel id."""
    pts = np.asarray(points, dtype=np.float64)
    g = np.asarray(grid)
    cell = np.floor((pts - lo) / (hi - lo) * g).astype(np.int64)
    cell = np.clip(cell, 0, g - 1)
    vid = (cell[:, 0] * g[1] + cell[:, 1]) * g[2] + cell[:, 2]
    order = np.argsort(vid, kind="stable")
    svid = vid[order]
    nvox = int(g.prod())
    start = np.searchsorted(svid, np.arange(nvox), side="left")
    end = np.searchsorted(svid, np.arange(nvox), side="right")
    return order, start, end


def _coords(v, grid):
    return v // (grid[1] * grid[2]), (v // grid[2]) % grid[1], v % grid[2]


def _adjacent(a, b, grid):
    ca, cb = _coords(a, grid), _coords(b, grid)
    return all(abs(x - y) <= 1 for x, y in zip(ca, cb))


def _neighbours(v, grid, occupied):
    x, y, z = _coords(v, grid)
    out = []
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                a, b, c = x + dx, y + dy, z + dz
                if 0 <= a < grid[0] and 0 <= b < grid[1] and 0 <= c < grid[2]:
                    w = (a * grid[1] + b) * grid[2] + c
                    if occupied[w]:
                        out.append(w)
    return sorted(out)


def spatial_jobs(kind, d_range, r_range, grid):
    """Voxel jobs of one histogram kind ("DDD", "DDR", "DRR", "RRR").
    d_range / r_range: (start, end) arrays per voxel id of the voxel-ordered
    data and random catalogs.  Returns a list of (roles, ranges, loop,
    global_index) with roles 'D'/'R' per position and loop one of
    "same", "one", "all"."""
    grid = tuple(int(x) for x in grid)
    return [j[:4] for j in cell_jobs(kind, d_range, r_range, lambda v, occ: _neighbours(v, grid, occ),
                                     lambda a, b: _adjacent(a, b, grid))]


def cell_jobs(kind, d_range, r_range, neighbours, near):
    """Jobs of one histogram kind over the cells of cell-ordered catalogs.
    neighbours(v, occupied) lists the occupied cells (v included) whose
    points may lie within the longest counted side of a point of cell v, and
    near(a, b) says the same of two cells; every counted triangle then falls
    in exactly one job.  Returns (roles, ranges, loop, global_index, cells)
    with the cell of each role."""
    ds, de = d_range
    rs, rend = r_range
    occ_d = de > ds
    occ_r = rend > rs
    rng = lambda role, v: (int(ds[v]), int(de[v])) if role == "D" else (int(rs[v]), int(rend[v]))
    jobs = []
    if kind in ("DDD", "RRR"):
        X = kind[0]
        occ = occ_d if X == "D" else occ_r
        for a in np.nonzero(occ)[0]:
            a = int(a)
            nb = neighbours(a, occ)
            jobs.append(((X, X, X), [rng(X, a)] * 3, "same", False, (a, a, a)))
            for b in nb:
                if b <= a:
                    continue
                jobs.append(((X, X, X), [rng(X, b), rng(X, a), rng(X, a)], "one", False, (b, a, a)))  # a=a<b
                jobs.append(((X, X, X), [rng(X, a), rng(X, b), rng(X, b)], "one", False, (a, b, b)))  # a<b=b
                for c in nb:
                    if c > b and near(b, c):
                        jobs.append(((X, X, X), [rng(X, a), rng(X, b), rng(X, c)], "all", False, (a, b, c)))
    elif kind == "DRR":
        for u in np.nonzero(occ_d)[0]:
            u = int(u)
            nb = neighbours(u, occ_r)
            for v in nb:
                jobs.append((("D", "R", "R"), [rng("D", u), rng("R", v), rng("R", v)], "one", False, (u, v, v)))
                for w in nb:
                    if w > v and near(v, w):
                        jobs.append((("D", "R", "R"), [rng("D", u), rng("R", v), rng("R", w)], "all", False,
                                     (u, v, w)))
    elif kind == "DDR":
        for u in np.nonzero(occ_d)[0]:
            u = int(u)
            nbd = neighbours(u, occ_d)
            nbr = neighbours(u, occ_r)
            for w in nbr:
                jobs.append((("D", "D", "R"), [rng("D", u), rng("D", u), rng("R", w)], "one", True, (u, u, w)))
            for v in nbd:
                if v <= u:
                    continue
                for w in nbr:
                    if near(v, w):
                        jobs.append((("D", "D", "R"), [rng("D", u), rng("D", v), rng("R", w)], "one", True,
                                     (u, v, w)))
                        jobs.append((("D", "D", "R"), [rng("D", v), rng("D", u), rng("R", w)], "one", True,
                                     (v, u, w)))
    else:
        raise ValueError(kind)
    return jobs


# ---------------------------------------------------------------------------
# Jackknife subsamples from one decomposition.
#
# With the catalogs ordered by jackknife region (cells), every counted
# triangle falls in exactly one cell job, so the subsample without region r
# (points of r removed from both catalogs) is the sum of the jobs that involve
# no point of r: JK_r = F - sum of the jobs whose cells include r, F the sum
# of all jobs.  Jobs are grouped by their set of distinct cells; the engine
# sums each group on the device and the subsamples are sums of groups.

def cell_boxes(points_by_cat, starts_by_cat, ends_by_cat, ncell):
    """Bounding box (lo, hi; float64) of each cell over every catalog."""
    lo = np.full((ncell, 3), np.inf)
    hi = np.full((ncell, 3), -np.inf)
    for pts, st, en in zip(points_by_cat, starts_by_cat, ends_by_cat):
        pts = np.asarray(pts, dtype=np.float64)
        for c in range(ncell):
            if en[c] > st[c]:
                seg = pts[st[c]:en[c]]
                lo[c] = np.minimum(lo[c], seg.min(0))
                hi[c] = np.maximum(hi[c], seg.max(0))
    return lo, hi


def box_near(lo, hi, reach):
    """near(a, b): the boxes of cells a and b are closer than reach, with
    reach the largest side that can be counted (the upper bin edge).  The
    kernels decide with the reference's float32 side length, which can round
    below the edge for points whose exact distance is at or slightly above
    it, so the test uses reach * (1 + 1e-5) + 1e-6: a float32 length is within
    a few units in the last place (~2.4e-7 relative) of the exact one.  The
    box gap never exceeds the exact distance of two of their points."""
    limit = float(reach) * (1.0 + 1e-5) + 1e-6

    def near(a, b):
        gap = np.maximum(0.0, np.maximum(lo[a] - hi[b], lo[b] - hi[a]))
        return bool(np.sqrt((gap ** 2).sum()) < limit)

    def neighbours(v, occ):
        return [int(c) for c in np.nonzero(occ)[0] if near(v, int(c))]
    return neighbours, near


def jackknife_groups(kind, d_range, r_range, neighbours, near):
    """Cell jobs of one kind and their groups: returns (jobs, group of each
    job, cell set of each group)."""
    jobs = cell_jobs(kind, d_range, r_range, neighbours, near)
    groups, key_of = [], {}
    gid = []
    for j in jobs:
        key = frozenset(j[4])
        if key not in key_of:
            key_of[key] = len(groups)
            groups.append(key)
        gid.append(key_of[key])
    return jobs, gid, groups


def jackknife_from_groups(group_hists, groups, nregions):
    """(full histogram, [JK_r for r in range(nregions)]) from the summed
    histogram of each group (uint64 arrays)."""
    full = np.zeros_like(group_hists[0])
    touch = [np.zeros_like(group_hists[0]) for _ in range(nregions)]
    for h, g in zip(group_hists, groups):
        full += h
        for r in g:
            touch[r] += h
    return full, [full - t for t in touch]
