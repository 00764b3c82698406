"""Pins the oracle restatement (oracle/tpcf_oracle.c) to the reference itself:
the reference's shipped golden histograms and outputs of the reference
programs compiled from source (tests/golden/ref, made by make_fixtures.py on
an x86-64 host, where int(NaN) is INT_MIN)."""
import os

import numpy as np
import pytest

import oracle
import refformat as rf
import synth

SANDBOX = os.path.join(rf.GOLDEN, "sandbox")
SANDBOX_SPEC = ((50, 2.0, 12.0), (16, 0.9, 4.1), (25, 0.0, 1.0))


def sandbox_catalog(tmp_path, name):
    return oracle.read_7col(rf.gunzip_to(os.path.join(SANDBOX, name + ".gz"), str(tmp_path / name)))


@pytest.mark.parametrize("vox", ["000000000", "000000001", "000001000", "000001001",
                                 "001000000", "001000001", "001001000", "001001001"])
def test_sandbox_voxel2_byte_exact(tmp_path, vox):
    """examples/sandbox/DDD_voxel2_*: TP DDD with -X 2 -x vox on the 1k catalog."""
    cat = sandbox_catalog(tmp_path, "MICE_5degx5deg_1k_randomized.dat")
    idx = rf.voxel_indices(int(vox), 3)
    subs = []
    for a in range(3):
        lo, hi = rf.vox2gal(2, idx[a], len(cat))
        subs.append(cat[lo:hi])
    hist, _ = oracle.triangle(subs, 0, SANDBOX_SPEC)
    got = rf.format_triangle(hist, [len(cat)] * 3, SANDBOX_SPEC)
    want = rf.read_bytes(os.path.join(SANDBOX, "DDD_voxel2_%s_evenbinning_CPU_5degx5deg_LRG_binning_1k.dat.gz" % vox))
    assert got == want


VOXEL4 = ["%03d%03d%03d" % (i, j, k) for i in range(4) for j in range(4) for k in range(4)]


def test_sandbox_voxel4_byte_exact(tmp_path):
    """examples/sandbox/DDD_voxel4_* (all 64 chunk triples of -X 4): made by a
    revision whose same-file loop starts k at j+1; the current j >= i, k >= j
    loop over the third chunk shifted by one point reproduces it."""
    cat = sandbox_catalog(tmp_path, "MICE_5degx5deg_1k_randomized.dat")
    for vox in VOXEL4:
        idx = rf.voxel_indices(int(vox), 3)
        r = [rf.vox2gal(4, idx[a], len(cat)) for a in range(3)]
        subs = [cat[r[0][0]:r[0][1]], cat[r[1][0]:r[1][1]], cat[r[2][0] + 1:r[2][1]]]
        hist, _ = oracle.triangle(subs, 0, SANDBOX_SPEC)
        got = rf.format_triangle(hist, [len(cat)] * 3, SANDBOX_SPEC)
        want = rf.read_bytes(os.path.join(SANDBOX, "DDD_voxel4_%s_evenbinning_CPU_5degx5deg_LRG_binning_1k.dat.gz" % vox))
        assert got == want, vox


def test_sandbox_lrg_full_ddd(tmp_path):
    """DDD_Debbie_LRG_..._1k.dat: full TP DDD on 1316 LRGs (3.8e8 triangles).
    The golden carries one extra trailing newline from sum_voxels.py's print."""
    cat = sandbox_catalog(tmp_path, "MICE_LRGs_10degx10deg.dat")
    hist, ncalc = oracle.triangle([cat] * 3, 0, SANDBOX_SPEC)
    n = len(cat)
    assert ncalc == n * (n + 1) * (n + 2) // 6
    got = rf.format_triangle(hist, [n] * 3, SANDBOX_SPEC)
    want = rf.read_bytes(os.path.join(SANDBOX, "DDD_Debbie_LRG_CPU_10degx10deg_LRG_binning_SLAC_1k.dat.gz"))
    assert got.split() == want.split()
    assert want == got + b"\n"


CASES = rf.ref_cases()["cases"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_compiled_reference(name):
    case = CASES[name]
    program, spec = rf.ref_binning(case["variant"])
    flags = case["flags"]
    cats = [rf.load_catalog(c) for c in case["catalogs"]]
    if "-m" in flags or "-s" in flags:
        cats = [oracle.read_header(os.path.join(rf.GOLDEN, "ref", c + ".dat"), rf.flags_scale(flags))
                for c in case["catalogs"]]
    ngal = [len(c) for c in cats]
    want = rf.read_bytes(os.path.join(rf.GOLDEN, "ref", name + ".dat.gz"))
    if "-X" in flags:
        div = int(flags[flags.index("-X") + 1])
        idx = rf.voxel_indices(int(flags[flags.index("-x") + 1]), len(cats))
        cats = [c[slice(*rf.vox2gal(div, idx[a], len(c)))] for a, c in enumerate(cats)]
    which = rf.which_mode(case["catalogs"])
    if program == "3side":
        n, lo, hi = spec
        hist, _ = oracle.three_side(cats, lo, hi, n)
        got = rf.format_three_side(hist, n)
    elif program == "tp":
        hist, _ = oracle.triangle(cats, which, spec, nan_zero=False)
        got = rf.format_triangle(hist, ngal, spec)
    elif program == "jbj":
        hist, _ = oracle.triangle_jbj(cats, which, spec, compat=True)
        got = rf.format_triangle(hist, ngal, spec)
    else:
        n, lo, hi = spec
        hist, _ = oracle.pair(cats, which, lo, hi, n)
        got = rf.format_pair(hist, ngal, n, lo, hi)
    assert got == want


def test_lattice_fixture_has_nan_triangles():
    """The lattice catalog holds degenerate triangles whose rounded cosine falls
    outside [-1, 1]; the two NaN conventions must then give different counts."""
    spec = ((6, 0.0, 15.0), (5, 1.0, 2.5), (7, 0.1, 0.9))
    cat = rf.load_catalog("c_lattice")
    h_int_min, _ = oracle.triangle([cat] * 3, 0, ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0)), nan_zero=False)
    h_zero, _ = oracle.triangle([cat] * 3, 0, ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0)), nan_zero=True)
    assert h_zero.sum() > h_int_min.sum()
    assert spec  # the zero-low-edge binning is covered by the compiled-reference cases


def test_oracle_acosf_is_host_libm():
    import ctypes
    libm = ctypes.CDLL("libm.so.6")
    libm.acosf.restype = ctypes.c_float
    libm.acosf.argtypes = [ctypes.c_float]
    for c in np.linspace(-1, 1, 1001, dtype=np.float32):
        assert oracle.acosf(c) == libm.acosf(float(c))


def test_geometry_fp64_oracle_matches_python_restatement():
    """The FP64-geometry loop (oracle_triangle_geom64) against a plain-Python
    double restatement of the same formulas on a small case."""
    import math
    d = synth.blobs(36, n_blobs=2, sigma=3.0, box=12.0, seed=21)
    spec = ((8, 2.0, 10.0), (8, 1.0, 3.0), (16, 0.0, 1.0))
    got, n = oracle.triangle_geom64([d, d, d], 0, spec, nthreads=2)
    want = np.zeros(8 * 8 * 16, dtype=np.uint64)
    lo = [float(np.float32(a[1])) for a in spec]
    hi = [float(np.float32(a[2])) for a in spec]
    nb = [a[0] for a in spec]
    pts = [tuple(float(v) for v in p) for p in d]

    def bin_(v, a):
        if v < lo[a] or v >= hi[a]:
            return -1
        return int((v - lo[a]) / ((hi[a] - lo[a]) / nb[a]))

    def dist(p, q):
        dx, dy, dz = p[0] - q[0], p[1] - q[1], p[2] - q[2]
        return math.sqrt(dx * dx + dy * dy + dz * dz)

    count = 0
    for i in range(len(pts)):
        for j in range(i, len(pts)):
            for k in range(j, len(pts)):
                count += 1
                s = sorted((dist(pts[i], pts[j]), dist(pts[i], pts[k]), dist(pts[j], pts[k])))
                if s[0] == 0:
                    continue
                a, b, c = s
                t0 = math.acos((a * a + b * b - c * c) / (2 * a * b)) / 3.14159
                t1 = math.acos((b * b + c * c - a * a) / (2 * b * c)) / 3.14159
                for sv, qv, tv in ((a, b / a, t0), (b, c / b, t1), (a, c / a, 1.0 - t0 - t1)):
                    i0, i1, i2 = bin_(sv, 0), bin_(qv, 1), bin_(tv, 2)
                    if min(i0, i1, i2) >= 0:
                        want[128 * i0 + 16 * i1 + i2] += 1
    assert n == count
    assert np.array_equal(got, want)
    assert want.sum() > 0


def test_lrg_rrr_chunk_job_matches_compiled_reference(tmp_path):
    """The oracle on one -X 10 chunk job of the LRG randoms (1.56e9 triangles)
    against the output file of the reference binary compiled here for the
    same job: the job holding the triangle whose ratio m/s rounds to exactly
    Q_HI (tests/golden/make_lrg_rrr.py)."""
    cat = sandbox_catalog(tmp_path, "flat_MICE_LRGs_10degx10deg.dat")
    idx = rf.voxel_indices(2000008, 3)
    subs = [cat[slice(*rf.vox2gal(10, idx[a], len(cat)))] for a in range(3)]
    hist, _ = oracle.triangle(subs, 0, SANDBOX_SPEC)
    got = rf.format_triangle(hist, [len(cat)] * 3, SANDBOX_SPEC)
    assert got == rf.read_bytes(os.path.join(rf.GOLDEN, "ref", "lrg_rrr_x10_002000008.dat.gz"))
