"""The reference's voxel decomposition (`-X division -x iiijjjkkk`) as jobs.

src/3pcf_C_version_triangle_parametrization.cc:52-80 (vox2gal) cuts each
catalog's index range into `division` chunks, the last one taking the
remainder; :306-313 decode `-x iiijjjkkk` into one chunk index per input
file.  examples/build_voxel_submission_scripts.py submits every (i, j, k) in
range(division)^3 as its own job and examples/sum_voxels.py adds the files.
The loops of a chunk job compare LOCAL indices, so the sum over chunk jobs is
what the reference's voxel workflow produces (not the one-file count).
"""


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
