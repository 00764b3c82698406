"""Reference file formats and loop helpers shared by the tests.

Formatters reproduce the reference programs' printf output byte for byte:
  three-side  src/3pcf_C_version.cc:440-460
  triangle    src/3pcf_C_version_triangle_parametrization.cc:537-569
  pairs       src/2pcf_C_version.cc:391-404
"""
import gzip
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "3pcf_gb300"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def read_bytes(path):
    if path.endswith(".gz"):
        with gzip.open(path, "rb") as f:
            return f.read()
    with open(path, "rb") as f:
        return f.read()


def gunzip_to(path_gz, dst):
    with open(dst, "wb") as f:
        f.write(read_bytes(path_gz))
    return dst


def fmt3(v):
    return "%-6.3f" % v


def format_three_side(hist, nbins):
    out = ["%d %d %d\n" % (nbins, nbins, nbins)]
    h = np.asarray(hist, dtype=np.uint64)
    n = nbins
    for i in range(n):
        out.append("%d\n" % i)
        for j in range(n):
            out.append("".join("%d " % int(h[n * n * k + n * j + i]) for k in range(n)) + "\n")
    return "".join(out).encode()


def format_triangle(hist, ngal, spec_macros):
    """spec_macros: ((S, lo, hi), (Q, lo, hi), (T, lo, hi)) with lo/hi the
    reference's double macro values; counts are wrapped to unsigned int."""
    (S, slo, shi), (Q, qlo, qhi), (T, tlo, thi) = spec_macros
    h = np.asarray(hist, dtype=np.uint64) & np.uint64(0xFFFFFFFF)
    out = ["%d\n" % ngal[0], "%d\n" % ngal[1], "%d\n" % ngal[2], "%d %d %d\n" % (S, Q, T)]
    for lo, hi, n in ((slo, shi, S), (qlo, qhi, Q), (tlo, thi, T)):
        out.append("%s %s %s\n" % (fmt3(lo), fmt3(hi), fmt3((hi - lo) / n)))
    for i in range(S):
        for j in range(Q):
            base = Q * T * i + T * j
            out.append("".join("%d " % int(h[base + k]) for k in range(T)) + "\n")
    return "".join(out).encode()


def format_pair(hist, ngal, nbins, lo, hi):
    h = np.asarray(hist, dtype=np.uint64) & np.uint64(0xFFFFFFFF)
    out = ["%d\n" % ngal[0], "%d\n" % ngal[1], "%d\n" % nbins, "%s %s %s\n" % (fmt3(lo), fmt3(hi), fmt3((hi - lo) / nbins))]
    out += ["%d\n" % int(v) for v in h]
    return "".join(out).encode()


def parse_triangle(data):
    vals = data.split()
    ngal = [int(v) for v in vals[0:3]]
    nb = [int(v) for v in vals[3:6]]
    counts = np.array([int(v) for v in vals[15:]], dtype=np.uint64)
    return ngal, nb, counts


def vox2gal(division, index, ngals):
    """Index chunk of one catalog, src/3pcf_C_version_triangle_parametrization.cc:52-80."""
    per = ngals // division
    if per == 0:
        raise ValueError("Voxel chunks are bigger than the number of galaxies!")
    lo = per * index
    hi = per * (index + 1)
    if index == division - 1:
        hi += ngals % division
    return lo, hi


def voxel_indices(vtemp, ncat):
    """-x iiijjjkkk decoding, :306-313 (and src/2pcf_C_version.cc:188-194)."""
    idx = [vtemp // 1000000, (vtemp // 1000) % 1000, vtemp % 1000]
    return idx[:ncat]


def which_mode(argv_cats):
    """Loop mode from argv string identity, as the reference decides it (:333-353),
    after the bool collapse: 0 (j>=i,k>=j) or 1 (j from 0, k>=j)."""
    if len(argv_cats) == 2:
        return 0 if argv_cats[0] == argv_cats[1] else 1
    a0, a1, a2 = argv_cats
    w = 0
    if a0 == a1 and a0 == a2:
        w = 0
    elif a0 != a1 and a1 == a2:
        w = 1
    elif a0 != a2 and a0 == a2:  # dead branch in the reference
        w = 2
    elif a0 == a1 and a0 != a2:
        w = 2
    return 1 if w else 0


def ref_binning(variant):
    """(program, spec) of a compiled reference variant with float-ready values."""
    import ref_build
    program, p = ref_build.binning(variant)
    if program == "3side":
        hi = float(np.float32(math.sqrt(1728.0))) if p["hi"] is None else float(p["hi"])
        return program, (int(p["nbins"]), float(p["lo"]), hi)
    if program in ("tp", "jbj"):
        return program, tuple((int(n), float(lo), float(hi)) for n, lo, hi in (p["S"], p["Q"], p["T"]))
    n, lo, hi = p["S"]
    return program, (int(n), float(lo), float(hi))


def ref_cases():
    with open(os.path.join(GOLDEN, "ref", "manifest.json")) as f:
        return json.load(f)


def load_catalog(name):
    """Fixture catalog by name via the oracle's fscanf-faithful readers."""
    import oracle
    path = os.path.join(GOLDEN, "ref", name + ".dat")
    if name.startswith("h_"):
        return oracle.read_header(path)
    return oracle.read_7col(path)


def flags_scale(flags):
    if "-s" in flags:
        return 206264.0
    if "-m" in flags:
        return 3437.74677
    return 1.0


def x86_acos_exceptions():
    """The x86-64 glibc 2.39 acosf exception table (keys, up flags) the
    reference's golden files were made with (tests/golden/make_acos_fixture.py)."""
    z = np.load(os.path.join(GOLDEN, "acosf_exceptions_x86_64_glibc2.39.npz"))
    n = int(z["n"])
    keys = np.cumsum(z["key_deltas"].astype(np.int64)).astype(np.uint32)
    up = np.unpackbits(z["up_bits"])[:n].astype(bool)
    return keys, up
