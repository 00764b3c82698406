"""GPU parity: the CUDA engine, called through the C ABI, against the
reference's own outputs (golden files and compiled-reference fixtures) and the
oracle restatement.  Integer histograms must be identical (tolerance 0)."""
import json
import os
import platform
import subprocess

import numpy as np
import pytest

import oracle
import refformat as rf
import synth
import tpcf

pytestmark = pytest.mark.gpu

SANDBOX = os.path.join(rf.GOLDEN, "sandbox")
SANDBOX_SPEC = ((50, 2.0, 12.0), (16, 0.9, 4.1), (25, 0.0, 1.0))
WIDE_SPEC = ((60, 0.0, 120.0), (16, 0.9, 4.1), (25, 0.0, 1.0))
NATIVE_NAN = tpcf.NAN_ZERO if platform.machine() == "aarch64" else tpcf.NAN_INT_MIN


@pytest.fixture(scope="module")
def eng():
    e = tpcf.Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="module")
def eng_x86():
    """Engine using x86-64 glibc's acosf: the reference's golden files and the
    compiled-reference fixtures were produced on x86-64, whose glibc acosf
    differs from aarch64 glibc's on some inputs."""
    e = tpcf.Engine(0)
    e.set_acos_exceptions(*rf.x86_acos_exceptions())
    yield e
    e.close()


def _tp_spec(spec, loop, precision=tpcf.GUARDED_FP32, nan=tpcf.NAN_INT_MIN, prune=True):
    return tpcf.make_spec(tpcf.TRIANGLE, loop, spec, precision=precision, nan_policy=nan, prune=prune)


def _loop_of(which):
    return tpcf.LOOP_ONE if which else tpcf.LOOP_SAME


CASES = rf.ref_cases()["cases"]


def _case_inputs(eng, name):
    case = CASES[name]
    program, spec = rf.ref_binning(case["variant"])
    flags = case["flags"]
    if "-m" in flags or "-s" in flags:
        cats = [oracle.read_header(os.path.join(rf.GOLDEN, "ref", c + ".dat"), rf.flags_scale(flags))
                for c in case["catalogs"]]
    else:
        cats = [rf.load_catalog(c) for c in case["catalogs"]]
    ngal = [len(c) for c in cats]
    # one engine catalog per distinct argv string, as the reference CLI sees them
    handles = {}
    for cname, c in zip(case["catalogs"], cats):
        if cname not in handles:
            handles[cname] = eng.catalog(c)
    hs = [handles[c] for c in case["catalogs"]]
    ranges = None
    if "-X" in flags:
        div = int(flags[flags.index("-X") + 1])
        idx = rf.voxel_indices(int(flags[flags.index("-x") + 1]), len(cats))
        ranges = [rf.vox2gal(div, idx[a], len(c)) for a, c in enumerate(cats)]
    return case, program, spec, cats, ngal, hs, ranges


@pytest.mark.parametrize("precision", [tpcf.GUARDED_FP32, tpcf.PLAIN_FP64])
@pytest.mark.parametrize("name", sorted(CASES))
def test_engine_matches_compiled_reference(eng_x86, name, precision):
    eng = eng_x86
    case, program, spec, cats, ngal, hs, ranges = _case_inputs(eng, name)
    which = rf.which_mode(case["catalogs"])
    want = rf.read_bytes(os.path.join(rf.GOLDEN, "ref", name + ".dat.gz"))
    job = eng.job(hs, ranges)
    if program == "3side":
        n, lo, hi = spec
        s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [spec], precision=precision)
        got = rf.format_three_side(eng.count(s, job), n)
    elif program == "tp":
        got = rf.format_triangle(eng.count(_tp_spec(spec, _loop_of(which), precision), job), ngal, spec)
    elif program == "jbj":
        s = tpcf.make_spec(tpcf.TRIANGLE_JBJ, _loop_of(which), spec, precision=precision)
        got = rf.format_triangle(eng.count(s, job), ngal, spec)
    else:
        n, lo, hi = spec
        s = tpcf.make_spec(tpcf.PAIR, _loop_of(which), [spec], precision=precision)
        got = rf.format_pair(eng.count(s, job), ngal, n, lo, hi)
    for h in set(hs):
        eng.release(h)
    assert got == want


def _sandbox_cat(tmp_path, name):
    return tpcf.read_catalog(rf.gunzip_to(os.path.join(SANDBOX, name + ".gz"), str(tmp_path / name)), 1)


@pytest.mark.parametrize("vox", ["000000000", "000000001", "000001000", "000001001",
                                 "001000000", "001000001", "001001000", "001001001"])
def test_sandbox_voxel2(eng_x86, tmp_path, vox):
    eng = eng_x86
    cat = _sandbox_cat(tmp_path, "MICE_5degx5deg_1k_randomized.dat")
    h = eng.catalog(cat)
    idx = rf.voxel_indices(int(vox), 3)
    ranges = [rf.vox2gal(2, idx[a], len(cat)) for a in range(3)]
    got = eng.count(_tp_spec(SANDBOX_SPEC, tpcf.LOOP_SAME), eng.job([h, h, h], ranges))
    eng.release(h)
    want = rf.read_bytes(os.path.join(SANDBOX, "DDD_voxel2_%s_evenbinning_CPU_5degx5deg_LRG_binning_1k.dat.gz" % vox))
    assert rf.format_triangle(got, [len(cat)] * 3, SANDBOX_SPEC) == want


def test_sandbox_voxel4(eng_x86, tmp_path):
    """All 64 DDD_voxel4_* chunk files (an earlier revision: k starts at j+1),
    as the current loop with the third chunk shifted by one point."""
    eng = eng_x86
    cat = _sandbox_cat(tmp_path, "MICE_5degx5deg_1k_randomized.dat")
    h = eng.catalog(cat)
    for i in range(4):
        for j in range(4):
            for k in range(4):
                r = [rf.vox2gal(4, v, len(cat)) for v in (i, j, k)]
                r[2] = (r[2][0] + 1, r[2][1])
                got = eng.count(_tp_spec(SANDBOX_SPEC, tpcf.LOOP_SAME), eng.job([h, h, h], r))
                name = "DDD_voxel4_%03d%03d%03d_evenbinning_CPU_5degx5deg_LRG_binning_1k.dat.gz" % (i, j, k)
                assert rf.format_triangle(got, [len(cat)] * 3, SANDBOX_SPEC) == rf.read_bytes(os.path.join(SANDBOX, name))
    eng.release(h)


PROVENANCE = json.load(open(os.path.join(SANDBOX, "provenance.json")))["sets"]


def _earlier_revision_ddr(eng, hd, hr, nd, nr, spec):
    """DDR of an earlier revision of the triangle program: k >= j+1 (the
    commented-out bound at :502) and no zero-side test, so pairs i == j add
    permutation 1 of (D_i, D_i, R_k): s = |D_i R_k|, q = 1, theta = 0.
    Emulated as the current loop with R's range shifted by one, plus the pair
    histogram of (D_i, R_k), k >= i+1, in bins (s, q=0, theta=0)."""
    h = eng.count(_tp_spec(spec, tpcf.LOOP_ONE), eng.job([hd, hd, hr], [(0, nd), (0, nd), (1, nr)]))
    pairs = eng.count(tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [spec[0]]), eng.job([hd, hr], [(0, nd), (1, nr)]))
    S, Q, T = spec[0][0], spec[1][0], spec[2][0]
    q0 = int(np.floor((np.float32(1.0) - np.float32(spec[1][1])) / np.float32((np.float32(spec[1][2]) - np.float32(spec[1][1])) / Q)))
    for sb in range(S):
        h[Q * T * sb + T * q0 + 0] += pairs[sb]
    return h


@pytest.mark.parametrize("setname,histo", [(s, h) for s in sorted(PROVENANCE) for h in sorted(PROVENANCE[s]["histos"])])
def test_sandbox_full_sets(eng_x86, tmp_path, setname, histo):
    """The reference's full-scale golden histograms (up to 1.6e12 triangles),
    reproduced the way each was made: a full run, a sum of -X V index-chunk
    runs (Q9: chunk-local loop indices), or an earlier loop-bound revision;
    counted with x86-64 glibc's acosf, as the golden files were."""
    eng = eng_x86
    info = PROVENANCE[setname]
    h = info["histos"][histo]
    spec = tuple(tuple(a) for a in info["spec"])
    d, r = _sandbox_cat(tmp_path, info["data"]), _sandbox_cat(tmp_path, info["randoms"])
    hd, hr = eng.catalog(d), eng.catalog(r)
    roles = {"DDD": ([hd, hd, hd], [d, d, d], tpcf.LOOP_SAME), "DDR": ([hd, hd, hr], [d, d, r], tpcf.LOOP_ONE),
             "DRR": ([hd, hr, hr], [d, r, r], tpcf.LOOP_ONE), "RRR": ([hr, hr, hr], [r, r, r], tpcf.LOOP_SAME)}[histo]
    hs, cats, loop = roles
    ns = [len(c) for c in cats]
    if h["how"] == "full":
        got = eng.count(_tp_spec(spec, loop), eng.job(hs))
    elif h["how"] == "voxel":
        V = h["division"]
        specs, jobs = [], []
        for a in range(V):
            for b in range(V):
                for c in range(V):
                    specs.append(_tp_spec(spec, loop))
                    jobs.append(eng.job(hs, [rf.vox2gal(V, x, ns[q]) for q, x in enumerate((a, b, c))]))
        got = sum(eng.count_batch(specs, jobs))
    else:
        got = _earlier_revision_ddr(eng, hd, hr, len(d), len(r), spec)
    eng.release(hd)
    eng.release(hr)
    if "compare" in h:
        # the golden file came from another build (compare_note): the
        # reference compiled here, summed over the same chunk runs, is the pin
        want = np.array(rf.read_bytes(os.path.join(rf.GOLDEN, h["compare"])).split(), dtype=np.uint64)
    else:
        _, _, want = rf.parse_triangle(rf.read_bytes(os.path.join(SANDBOX, h["file"] + ".gz")))
    got = (got & np.uint64(0xFFFFFFFF)).astype(np.int64)
    assert np.array_equal(got, want.astype(np.int64)), int((got != want.astype(np.int64)).sum())


@pytest.mark.parametrize("chunks", ["002000008", "000005009"])
def test_lrg_rrr_chunk_jobs(eng_x86, tmp_path, chunks):
    """Two -X 10 chunk jobs of the LRG randoms run by the reference binary
    compiled here (tests/golden/make_lrg_rrr.py): 002000008 holds the
    triangle whose ratio rounds to exactly Q_HI, 000005009 the triangle of
    bin (33, 12, 17) closest to its q edge.  Byte-identical output files in
    both precisions."""
    eng = eng_x86
    cat = _sandbox_cat(tmp_path, "flat_MICE_LRGs_10degx10deg.dat")
    h = eng.catalog(cat)
    idx = rf.voxel_indices(int(chunks), 3)
    ranges = [rf.vox2gal(10, idx[a], len(cat)) for a in range(3)]
    want = rf.read_bytes(os.path.join(rf.GOLDEN, "ref", "lrg_rrr_x10_%s.dat.gz" % chunks))
    for prec in (tpcf.GUARDED_FP32, tpcf.PLAIN_FP64):
        got = eng.count(_tp_spec(SANDBOX_SPEC, tpcf.LOOP_SAME, prec), eng.job([h, h, h], ranges))
        assert rf.format_triangle(got, [len(cat)] * 3, SANDBOX_SPEC) == want, prec
    eng.release(h)


def _random_case(seed, n_d=220, n_r=200):
    d = synth.blobs(n_d, n_blobs=3, sigma=4.0, box=40.0, seed=seed)
    r = synth.uniform(n_r, box=28.0, seed=seed + 1)
    return d, r


@pytest.mark.parametrize("seed", [101, 202])
@pytest.mark.parametrize("spec", [((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0)),
                                  ((50, 2.0, 12.0), (16, 0.9, 4.1), (32, 0.0, 1.0)),
                                  ((6, 0.0, 15.0), (5, 1.0, 2.5), (7, 0.1, 0.9))])
def test_triangle_vs_oracle_native_nan(eng, seed, spec):
    """All four loop nests plus the generic three-array nest, with the NaN
    convention of the machine the oracle runs on."""
    d, r = _random_case(seed)
    x = synth.blobs(150, n_blobs=2, sigma=3.0, box=25.0, seed=seed + 2)
    hd, hr, hx = eng.catalog(d), eng.catalog(r), eng.catalog(x)
    combos = [([hd, hd, hd], [d, d, d], 0), ([hd, hd, hr], [d, d, r], 1), ([hd, hr, hr], [d, r, r], 1),
              ([hr, hr, hr], [r, r, r], 0), ([hd, hr, hx], [d, r, x], 0), ([hd, hr, hd], [d, r, d], 0),
              ([hr, hd, hx], [r, d, x], 1)]
    specs = [_tp_spec(spec, _loop_of(w), nan=NATIVE_NAN) for _, _, w in combos]
    hists = eng.count_batch(specs, [eng.job(h) for h, _, _ in combos])
    for (h, cats, w), got in zip(combos, hists):
        want, _ = oracle.triangle(cats, w, spec, nan_zero=NATIVE_NAN == tpcf.NAN_ZERO)
        assert np.array_equal(got, want), (w, int((got != want).sum()))
    for h in (hd, hr, hx):
        eng.release(h)


@pytest.mark.parametrize("seed", [303])
def test_geometry_fp64_vs_oracle(eng, seed):
    """TPCF_GEOMETRY_FP64 (the FP64 truth, not the reference's counts) against
    the oracle's double-precision loop: identical operations except acos
    (CUDA's double acos vs the host's), so at most a couple of triangles may
    sit on the other side of an edge."""
    d, r = _random_case(seed)
    hd, hr = eng.catalog(d), eng.catalog(r)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    combos = [([hd, hd, hd], [d, d, d], 0), ([hd, hd, hr], [d, d, r], 1), ([hd, hr, hr], [d, r, r], 1),
              ([hr, hr, hr], [r, r, r], 0)]
    specs = [_tp_spec(spec, _loop_of(w), precision=tpcf.GEOMETRY_FP64, nan=NATIVE_NAN) for _, _, w in combos]
    hists = eng.count_batch(specs, [eng.job(h) for h, _, _ in combos])
    for (h, cats, w), got in zip(combos, hists):
        want, _ = oracle.triangle_geom64(cats, w, spec, nan_zero=NATIVE_NAN == tpcf.NAN_ZERO)
        diff = np.abs(got.astype(np.int64) - want.astype(np.int64)).sum()
        assert diff <= 6, (w, int(diff))
        assert got.sum() > 0
    # the float-arithmetic counts differ from the FP64 truth only near edges
    exact = eng.count_batch([_tp_spec(spec, _loop_of(w), nan=NATIVE_NAN) for _, _, w in combos],
                            [eng.job(h) for h, _, _ in combos])
    for a, b in zip(exact, hists):
        assert np.abs(a.astype(np.int64) - b.astype(np.int64)).sum() <= 1e-3 * a.sum()
    with pytest.raises(tpcf.EngineError):
        eng.count(tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [(10, 0.0, 10.0)], precision=tpcf.GEOMETRY_FP64),
                  eng.job([hd, hd]))
    eng.release(hd)
    eng.release(hr)


def test_lattice_nan_policies(eng):
    """Degenerate lattice triangles produce rounded cosines beyond +-1; both
    int(NaN) conventions must match the oracle."""
    cat = rf.load_catalog("c_lattice")
    h = eng.catalog(cat)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    for nan in (tpcf.NAN_INT_MIN, tpcf.NAN_ZERO):
        for prec in (tpcf.GUARDED_FP32, tpcf.PLAIN_FP64):
            got = eng.count(_tp_spec(spec, tpcf.LOOP_SAME, prec, nan), eng.job([h, h, h]))
            want, _ = oracle.triangle([cat] * 3, 0, spec, nan_zero=nan == tpcf.NAN_ZERO)
            assert np.array_equal(got, want), (nan, prec)
    eng.release(h)


def test_prune_is_exact(eng):
    d, r = _random_case(7, 600, 500)
    hd, hr = eng.catalog(d), eng.catalog(r)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    for hs, loop in (([hd, hd, hd], tpcf.LOOP_SAME), ([hd, hd, hr], tpcf.LOOP_ONE), ([hd, hr, hr], tpcf.LOOP_ONE)):
        a = eng.count(_tp_spec(spec, loop, prune=True), eng.job(hs))
        st_a = eng.stats()
        b = eng.count(_tp_spec(spec, loop, prune=False), eng.job(hs))
        st_b = eng.stats()
        assert np.array_equal(a, b)
        assert st_a["loop_units"] == st_b["loop_units"]
        assert st_a["evaluated_units"] <= st_b["evaluated_units"]
    eng.release(hd)
    eng.release(hr)


@pytest.mark.parametrize("overflow", [tpcf.OVERFLOW_COMPAT, tpcf.OVERFLOW_CLEAN])
@pytest.mark.parametrize("axis", [(16, 0.0, 40.0), (32, 0.0, 32.0), (8, 5.0, 25.0)])
def test_three_side_vs_oracle(eng, overflow, axis):
    d = synth.blobs(140, n_blobs=4, sigma=5.0, box=60.0, seed=31)
    r = synth.lattice_mix(120, box=40.0, frac=0.5, seed=32)
    hd, hr = eng.catalog(d), eng.catalog(r)
    for hs, cats in (([hd, hd, hd], [d, d, d]), ([hd, hr, hr], [d, r, r]), ([hr, hd, hr], [r, d, r])):
        for prec in (tpcf.GUARDED_FP32, tpcf.PLAIN_FP64):
            s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [axis], precision=prec, overflow=overflow)
            got = eng.count(s, eng.job(hs))
            want, n = oracle.three_side(cats, axis[1], axis[2], axis[0], clean=overflow == tpcf.OVERFLOW_CLEAN)
            assert np.array_equal(got, want)
            assert eng.stats()["loop_units"] == n
    eng.release(hd)
    eng.release(hr)


@pytest.mark.parametrize("axis", [(32, 0.0, 32.0), (24, 2.0, 20.0), (12, 0.0, 36.0)])
def test_three_side_clean_spread_catalog(eng, axis):
    """Clean three-side mode on a catalog much wider than the largest side
    (most tile triples and most points of a tile are out of reach, 30 % of the
    points on the integer lattice): every launch shape the autotuner tries
    (32-warp CTAs around one large histogram, the global histogram, 8-warp
    CTAs) and the FP64 kernel give the oracle's counts."""
    pts = synth.lattice_mix(1500, box=150.0, frac=0.3, seed=41)
    h = eng.catalog(pts)
    job = eng.job([h, h, h])
    want, n = oracle.three_side([pts, pts, pts], axis[1], axis[2], axis[0], clean=True)
    assert want.sum() > 0
    for prec in (tpcf.GUARDED_FP32, tpcf.PLAIN_FP64):
        s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [axis], precision=prec, overflow=tpcf.OVERFLOW_CLEAN)
        for _ in range(4):  # the repeated batch is autotuned over the candidate shapes
            got = eng.count(s, job)
            assert np.array_equal(got, want)
            assert eng.stats()["loop_units"] == n
    eng.release(h)


@pytest.mark.parametrize("overflow", [tpcf.OVERFLOW_COMPAT, tpcf.OVERFLOW_CLEAN])
@pytest.mark.parametrize("axis", [(16, 0.0, 40.0), (50, 0.0, 30.0)])
def test_three_side_every_launch_shape(eng, overflow, axis):
    """One catalog in all roles (multiset counting) and two catalogs (ordered
    tasks) in one batch, counted repeatedly so that the autotuner runs every
    launch shape (histogram copies per CTA, the grouped kernel, the global
    histogram; 50 bins do not fit shared memory at all): the oracle's counts
    every time."""
    d = synth.blobs(300, n_blobs=4, sigma=5.0, box=60.0, seed=47)
    r = synth.lattice_mix(260, box=60.0, frac=0.4, seed=48)
    hd, hr = eng.catalog(d), eng.catalog(r)
    s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [axis], overflow=overflow)
    clean = overflow == tpcf.OVERFLOW_CLEAN
    combos = [([hd, hd, hd], [d, d, d]), ([hr, hr, hr], [r, r, r]), ([hd, hr, hr], [d, r, r])]
    want = [oracle.three_side(c, axis[1], axis[2], axis[0], clean=clean)[0] for _, c in combos]
    jobs = [eng.job(h) for h, _ in combos]
    for _ in range(4):
        got = eng.count_batch([s] * 3, jobs)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)
    eng.release(hd)
    eng.release(hr)


@pytest.mark.parametrize("axis", [(32, 0.0, 32.0), (10, 0.0, 10.0), (12, 2.0, 14.0)])
def test_three_side_clean_sides_on_hist_max(eng, axis):
    """Integer lattice points: many sides exactly at hist_max (d = hi drops the
    triple; the code jumps over nbins there) and on every bin edge."""
    pts = synth.lattice_mix(500, box=36.0, frac=1.0, seed=50)
    h = eng.catalog(pts)
    s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [axis], overflow=tpcf.OVERFLOW_CLEAN)
    want, _ = oracle.three_side([pts, pts, pts], axis[1], axis[2], axis[0], clean=True)
    assert np.array_equal(eng.count(s, eng.job([h, h, h])), want)
    eng.release(h)


def test_three_side_clean_batch_of_jobs(eng):
    """Several clean three-side jobs with a 32^3-bin histogram in one launch
    (one CTA per SM of task pipelines that meet to flush at every change of
    job), symmetric and ordered tasks mixed, two jobs summed into one output:
    each output equals the oracle's."""
    d = synth.blobs(700, n_blobs=5, sigma=6.0, box=90.0, seed=45)
    r = synth.lattice_mix(600, box=90.0, frac=0.3, seed=46)
    hd, hr = eng.catalog(d), eng.catalog(r)
    axis = (32, 0.0, 32.0)
    s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [axis], overflow=tpcf.OVERFLOW_CLEAN)
    combos = [([hd, hd, hd], [d, d, d]), ([hd, hr, hr], [d, r, r]), ([hr, hr, hr], [r, r, r]),
              ([hr, hd, hr], [r, d, r])]
    want = [oracle.three_side(c, axis[1], axis[2], axis[0], clean=True)[0] for _, c in combos]
    jobs = [eng.job(h) for h, _ in combos]
    for _ in range(3):  # the repeated batch is autotuned, then replayed
        got = eng.count_batch([s] * 4, jobs)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)
    got = eng.count_batch_into([s] * 4, jobs, [0, 1, 0, 1], 2)
    assert np.array_equal(got[0], want[0] + want[2])
    assert np.array_equal(got[1], want[1] + want[3])
    eng.release(hd)
    eng.release(hr)


@pytest.mark.parametrize("sym", ["1", "0"])
def test_three_side_clean_duplicates(eng, monkeypatch, sym):
    """Clean three-side mode on a catalog where every point appears three
    times (zero-length sides between distinct indices) beside the repeated
    indices of the ordered loop (i == j, j == k, i == j == k): the symmetric
    tasks (each multiset of three points counted for its distinct orderings)
    and the ordered ones (TPCF_SYM3=0) give the oracle's counts."""
    monkeypatch.setenv("TPCF_SYM3", sym)
    base = synth.lattice_mix(70, box=30.0, frac=0.5, seed=43)
    pts = np.concatenate([base, base, base])[np.random.default_rng(44).permutation(210)]
    h = eng.catalog(pts)
    for axis in ((16, 0.0, 24.0), (10, 1.0, 11.0)):
        s = tpcf.make_spec(tpcf.THREE_SIDE, tpcf.LOOP_ALL, [axis], overflow=tpcf.OVERFLOW_CLEAN)
        want, n = oracle.three_side([pts, pts, pts], axis[1], axis[2], axis[0], clean=True)
        got = eng.count(s, eng.job([h, h, h]))
        assert np.array_equal(got, want), axis
        # a sub-range of the catalog (tiles of a range view) and two roles alike
        r = [(13, 190)] * 3
        want_r, _ = oracle.three_side([pts[13:190]] * 3, axis[1], axis[2], axis[0], clean=True)
        assert np.array_equal(eng.count(s, eng.job([h, h, h], r)), want_r), axis
    eng.release(h)


@pytest.mark.parametrize("axis", [(700, 0.0, 70.0), (40, 1.0, 21.0)])
def test_pairs_vs_oracle(eng, axis):
    d = synth.blobs(3000, n_blobs=10, sigma=5.0, box=100.0, seed=41)
    r = synth.uniform(2500, box=100.0, seed=42)
    hd, hr = eng.catalog(d), eng.catalog(r)
    for hs, cats, w in (([hd, hd], [d, d], 0), ([hd, hr], [d, r], 1), ([hr, hr], [r, r], 0)):
        s = tpcf.make_spec(tpcf.PAIR, _loop_of(w), [axis])
        got = eng.count(s, eng.job(hs))
        want, n = oracle.pair(cats, w, axis[1], axis[2], axis[0])
        assert np.array_equal(got, want)
        assert eng.stats()["loop_units"] == n
    # index chunks of one catalog: the reference's j >= i on chunk-local indices
    got = eng.count(tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [axis]), eng.job([hd, hd], [(1500, 3000), (0, 1500)]))
    want, _ = oracle.pair([d[1500:3000], d[0:1500]], 0, axis[1], axis[2], axis[0])
    assert np.array_equal(got, want)
    eng.release(hd)
    eng.release(hr)


@pytest.mark.parametrize("axis", [(10, 0.0, 10.0), (7, 1.5, 12.0), (2000, 0.0, 40.0)])
def test_pairs_bin_edges(eng, axis):
    """Lattice points (separations exactly on bin edges, zero separations
    between duplicates): the squared-length thresholds of the guarded kernel
    (up to 700 bins; 2000 bins take the reference formula) and the FP64
    kernel give the oracle's counts."""
    pts = synth.lattice_mix(2500, box=40.0, frac=0.8, seed=49)
    pts = np.concatenate([pts, pts[:300]])
    h = eng.catalog(pts)
    for prec in (tpcf.GUARDED_FP32, tpcf.PLAIN_FP64):
        got = eng.count(tpcf.make_spec(tpcf.PAIR, tpcf.LOOP_SAME, [axis], precision=prec), eng.job([h, h]))
        want, _ = oracle.pair([pts, pts], 0, axis[1], axis[2], axis[0])
        assert got.sum() > 0
        assert np.array_equal(got, want), prec
    eng.release(h)


def test_empty_and_tiny_catalogs(eng):
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    one = np.array([[1.0, 2.0, 3.0]], dtype=np.float32)
    two = np.array([[1.0, 2.0, 3.0], [4.0, 2.0, 3.0]], dtype=np.float32)
    h0 = eng.catalog(np.zeros((0, 3), dtype=np.float32))
    h1, h2 = eng.catalog(one), eng.catalog(two)
    for hs in ([h0, h0, h0], [h1, h1, h1], [h2, h2, h2], [h2, h2, h0], [h2, h0, h0]):
        got = eng.count(_tp_spec(spec, tpcf.LOOP_SAME), eng.job(hs))
        assert got.sum() == 0
    for h in (h0, h1, h2):
        eng.release(h)


def test_duplicate_points_zero_sides(eng):
    """Coincident points give zero sides: the reference drops all three
    permutations even when the low s edge is 0."""
    base = synth.blobs(80, n_blobs=1, sigma=3.0, box=10.0, seed=51)
    cat = np.concatenate([base, base[:30], base[:10]])
    h = eng.catalog(cat)
    for spec in (((6, 0.0, 15.0), (5, 1.0, 2.5), (7, 0.1, 0.9)), ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))):
        for loop, w in ((tpcf.LOOP_SAME, 0), (tpcf.LOOP_ONE, 1)):
            got = eng.count(_tp_spec(spec, loop), eng.job([h, h, h]))
            want, _ = oracle.triangle([cat] * 3, w, spec)
            assert np.array_equal(got, want)
    eng.release(h)


@pytest.mark.parametrize("name", ["tp_s8_q8_t16_DDR", "tp_s8_q8_t16_vox3_DDD", "tp_default_DRR",
                                  "3side_n16_0_40_DDR", "2pcf_default_DD", "2pcf_default_vox2",
                                  "jbj_default_DDD", "jbj_s10_q8_t10_vox2_DDR"])
def test_cli_byte_exact(tmp_path, name):
    case = CASES[name]
    var = case["variant"]
    prog = {"3side": "tpcf_3side", "tp": "tpcf_tp", "2pcf": "tpcf_2pcf", "jbj": "tpcf_jbj"}[rf.ref_binning(var)[0]]
    program, spec = rf.ref_binning(var)
    extra = []
    if program in ("tp", "jbj"):
        extra = ["--s-axis", "%d,%r,%r" % spec[0], "--q-axis", "%d,%r,%r" % spec[1],
                 "--theta-axis", "%d,%r,%r" % spec[2], "--nan-policy", "int_min"]
    elif program == "3side":
        extra = ["--nbins", str(spec[0]), "--hist-min", repr(spec[1]), "--hist-max", repr(spec[2])]
    else:
        extra = ["--pair-axis", "%d,%r,%r" % spec]
    cats = [os.path.join(rf.GOLDEN, "ref", c + ".dat") for c in case["catalogs"]]
    out = tmp_path / "out.dat"
    r = subprocess.run([os.path.join(tpcf.BIN_DIR, prog)] + cats + case["flags"] + extra + ["-o", str(out), "--quiet"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert out.read_bytes() == rf.read_bytes(os.path.join(rf.GOLDEN, "ref", name + ".dat.gz"))


def test_acos_exception_table(eng):
    mism, n = eng.acos_selfcheck()
    assert mism == 0
    assert 1_000_000 < n < 20_000_000


@pytest.mark.parametrize("spec", [((50, 2.0, 12.0), (16, 0.9, 4.1), (32, 0.0, 1.0)),
                                  ((10, 1.0, 11.0), (8, 0.2, 1.0), (10, 0.0, 1.0))])
def test_jbj_vs_oracle_both_overflow_modes(eng, spec):
    """JBJ parametrization: compat (the reference's two extra bin-0 counts per
    visited triangle) and clean, every loop nest, pruned and unpruned."""
    d, r = _random_case(404)
    hd, hr = eng.catalog(d), eng.catalog(r)
    combos = [([hd, hd, hd], [d, d, d], 0), ([hd, hd, hr], [d, d, r], 1), ([hd, hr, hr], [d, r, r], 1),
              ([hr, hr, hr], [r, r, r], 0)]
    for overflow in (tpcf.OVERFLOW_COMPAT, tpcf.OVERFLOW_CLEAN):
        for prune in (True, False):
            specs = [tpcf.make_spec(tpcf.TRIANGLE_JBJ, _loop_of(w), spec, overflow=overflow, prune=prune)
                     for _, _, w in combos]
            hists = eng.count_batch(specs, [eng.job(h) for h, _, _ in combos])
            for (h, cats, w), got in zip(combos, hists):
                want, n = oracle.triangle_jbj(cats, w, spec, compat=overflow == tpcf.OVERFLOW_COMPAT)
                assert np.array_equal(got, want), (overflow, prune, w)
    eng.release(hd)
    eng.release(hr)


@pytest.mark.parametrize("tile_points", [17, 32, 48])
def test_counts_do_not_depend_on_tile_size(monkeypatch, tile_points):
    """Smaller spatial tiles (many partial tiles) give the same histograms as
    the default 64-point tiles.  (The number of candidates binned may differ:
    tile triples that provably hold no counted triangle are pruned, and with
    them class-level candidates that the exact binning would reject.)"""
    d = synth.blobs(3000, n_blobs=6, sigma=5.0, box=80.0, seed=77)
    r = synth.uniform(2500, box=120.0, seed=78)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    loops = [tpcf.LOOP_SAME, tpcf.LOOP_ONE, tpcf.LOOP_ONE, tpcf.LOOP_SAME]

    def run():
        with tpcf.Engine(0) as e:
            hd, hr = e.catalog(d), e.catalog(r)
            jobs = [e.job([hd, hd, hd]), e.job([hd, hd, hr]), e.job([hd, hr, hr]), e.job([hr, hr, hr])]
            out = []
            return [e.count(_tp_spec(spec, lp, nan=NATIVE_NAN), jb) for lp, jb in zip(loops, jobs)]

    monkeypatch.delenv("TPCF_TILE_POINTS", raising=False)
    want = run()
    monkeypatch.setenv("TPCF_TILE_POINTS", str(tile_points))
    got = run()
    for hw, hg in zip(want, got):
        assert np.array_equal(hw, hg)
        assert hw.sum() > 0


_GROUP_WANT = {}


@pytest.mark.parametrize("group_tasks", ["1", "3", "64"])
def test_counts_do_not_depend_on_task_groups(monkeypatch, group_tasks):
    """The fast triangle kernel takes groups of tasks that share tiles B and C
    (one j-k table per group, rows skipped from the union box of the group's
    A tiles): any group size gives the oracle's histograms, TP and JBJ."""
    monkeypatch.setenv("TPCF_GROUP_TASKS", group_tasks)
    d = synth.blobs(900, n_blobs=3, sigma=5.0, box=50.0, seed=81)
    r = synth.uniform(800, box=60.0, seed=82)
    tp = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    jbj = ((8, 2.0, 10.0), (8, 0.2, 1.0), (10, 0.0, 1.0))
    combos = [([d, d, d], 0), ([d, d, r], 1), ([d, r, r], 1), ([r, r, r], 0)]
    if not _GROUP_WANT:
        for (cats, w) in combos:
            _GROUP_WANT[("tp", w, len(cats[1]), len(cats[2]))] = \
                oracle.triangle(cats, w, tp, nan_zero=NATIVE_NAN == tpcf.NAN_ZERO)[0]
            _GROUP_WANT[("jbj", w, len(cats[1]), len(cats[2]))] = oracle.triangle_jbj(cats, w, jbj)[0]
    with tpcf.Engine(0) as e:
        hd, hr = e.catalog(d), e.catalog(r)
        hmap = {id(d): hd, id(r): hr}
        jobs = [e.job([hmap[id(c)] for c in cats]) for cats, _ in combos]
        for name, kind, spec in (("tp", tpcf.TRIANGLE, tp), ("jbj", tpcf.TRIANGLE_JBJ, jbj)):
            specs = [tpcf.make_spec(kind, _loop_of(w), spec, nan_policy=NATIVE_NAN) for _, w in combos]
            got = e.count_batch(specs, jobs)
            for (cats, w), g in zip(combos, got):
                want = _GROUP_WANT[(name, w, len(cats[1]), len(cats[2]))]
                assert want.sum() > 0
                assert np.array_equal(g, want), (name, w)


@pytest.mark.parametrize("kind", ["tp", "jbj"])
def test_many_s_bins_counted_exactly(kind):
    """The fast kernel's side words hold s-bins below 255; a guarded-FP32 count
    with more s bins runs in the plain FP64 kernel and gives the oracle's
    histogram all the same."""
    d = synth.blobs(500, n_blobs=3, sigma=4.0, box=40.0, seed=91)
    r = synth.uniform(400, box=40.0, seed=92)
    if kind == "tp":
        spec = ((300, 2.0, 10.0), (4, 1.0, 3.0), (4, 0.0, 1.0))
        want = oracle.triangle([d, d, r], 1, spec, nan_zero=NATIVE_NAN == tpcf.NAN_ZERO)[0]
        s = tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_ONE, spec, nan_policy=NATIVE_NAN)
    else:
        spec = ((300, 2.0, 10.0), (4, 0.2, 1.0), (4, 0.0, 1.0))
        want = oracle.triangle_jbj([d, d, r], 1, spec)[0]
        s = tpcf.make_spec(tpcf.TRIANGLE_JBJ, tpcf.LOOP_ONE, spec, nan_policy=NATIVE_NAN)
    with tpcf.Engine(0) as e:
        hd, hr = e.catalog(d), e.catalog(r)
        got = e.count(s, e.job([hd, hd, hr]))
    assert want.sum() > 0
    assert np.array_equal(got, want)


def test_catalogs_built_in_the_background():
    """A catalog's spatial view is built on a library thread: releasing it before
    any use, counting right after creation, counting many new catalogs in one
    batch and asking for the resident bytes all see the finished view."""
    d = synth.blobs(700, n_blobs=3, sigma=4.0, box=40.0, seed=95)
    r = synth.uniform(600, box=40.0, seed=96)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    want = oracle.triangle([d, d, r], 1, spec, nan_zero=NATIVE_NAN == tpcf.NAN_ZERO)[0]
    with tpcf.Engine(0) as e:
        for _ in range(5):
            e.release(e.catalog(d))  # released while (or after) its view is built
        hs = [(e.catalog(d), e.catalog(r)) for _ in range(4)]
        assert e.resident_bytes() >= 4 * (700 + 600) * 16
        s = tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_ONE, spec, nan_policy=NATIVE_NAN)
        got = e.count_batch([s] * 4, [e.job([hd, hd, hr]) for hd, hr in hs])
        for g in got:
            assert np.array_equal(g, want)
        for hd, hr in hs:
            e.release(hd)
            e.release(hr)
        assert e.resident_bytes() == 0


def test_pipelined_batches_with_empty_jobs():
    """A new batch of a few fast-kernel jobs launches its first job while the
    rest are planned; an empty first or later job (a zero-length catalog
    range) leaves its histogram zero and the others exact."""
    d = synth.blobs(600, n_blobs=3, sigma=4.0, box=40.0, seed=97)
    r = synth.uniform(500, box=40.0, seed=98)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    nz = NATIVE_NAN == tpcf.NAN_ZERO
    want_ddr = oracle.triangle([d, d, r], 1, spec, nan_zero=nz)[0]
    want_rrr = oracle.triangle([r, r, r], 0, spec, nan_zero=nz)[0]
    s_one = tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_ONE, spec, nan_policy=NATIVE_NAN)
    s_same = tpcf.make_spec(tpcf.TRIANGLE, tpcf.LOOP_SAME, spec, nan_policy=NATIVE_NAN)
    with tpcf.Engine(0) as e:
        hd, hr = e.catalog(d), e.catalog(r)
        empty = e.job([hd, hd, hd], [(0, 0)] * 3)
        for specs, jobs, wants in (
                ([s_same, s_one, s_same], [empty, e.job([hd, hd, hr]), e.job([hr, hr, hr])],
                 [None, want_ddr, want_rrr]),
                ([s_one, s_same, s_same], [e.job([hd, hd, hr]), empty, e.job([hr, hr, hr])],
                 [want_ddr, None, want_rrr])):
            got = e.count_batch(specs, jobs)
            again = e.count_batch(specs, jobs)  # the merged plan of the repeat
            for g, a, w in zip(got, again, wants):
                assert np.array_equal(g, a)
                if w is None:
                    assert g.sum() == 0
                else:
                    assert w.sum() > 0 and np.array_equal(g, w)
