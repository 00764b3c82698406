#!/usr/bin/env python3
"""Fixtures for the reference's LRG RRR golden file (test infrastructure only).

RRR_Debbie_LRG_CPU_10degx10deg_LRG_binning_SLAC_1k.dat is the sum of the 1000
``-X 10`` index-chunk runs of the triangle program (sandbox binning) on
flat_MICE_LRGs_10degx10deg.dat (21,056 points).  This script records what the
reference compiled here gives for the same runs:

* ``ref/lrg_rrr_x10_chunk_sum.txt.gz``: the chunk sum, each triangle binned by
  the reference's own ``distance()`` (tests/golden/chunk_sum_driver.cc compiled
  against the configured copy oracle/_ref/src/tp_sandbox.cc; 20,000 counts,
  one per line);
* ``ref/lrg_rrr_x10_<chunks>.dat.gz``: the output files of the compiled
  reference binary (oracle/_ref/bin/tp_sandbox) for the chunk jobs that hold
  the triangles closest to the bins in which the golden file differs from
  the sum above (about 130 s each).

Needs the configured copies and binaries of oracle/ref_build.py (run it with
the reference checkout first) and g++ with OpenMP.
"""
import gzip
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"), os.path.join(ROOT, "3pcf_gb300")):
    sys.path.insert(0, p)
import numpy as np  # noqa: E402
import oracle  # noqa: E402
import ref_build  # noqa: E402
import refformat as rf  # noqa: E402

CATALOG = "flat_MICE_LRGs_10degx10deg.dat"
DIVISION = 10
# chunk jobs (iii jjj kkk) run with the reference binary itself:
#  002000008 holds triangle (1504, 4417, 18592) (catalog rows), whose
#            permutation-0 ratio m/s rounds to exactly Q_HI = 4.1f in single
#            precision (exact ratio 4.09999965): dropped by the reference
#            compiled here, counted at (s, q, theta) = (41, 15, 21) in the file;
#  000005009 holds triangle (508, 11932, 20555), the one of bin (33, 12, 17)
#            closest to the q edge 3.3 (ratio 3.3000052).
CHUNK_JOBS = ["002000008", "000005009"]


def gz_write(path, data):
    with gzip.GzipFile(path, "wb", mtime=0) as g:
        g.write(data)


def main():
    src = os.path.join(ref_build.SRC_OUT, "tp_sandbox.cc")
    exe = ref_build.binary("tp_sandbox")
    if not os.path.exists(src) or exe is None:
        print("oracle/_ref has no tp_sandbox; run oracle/ref_build.py first")
        return 1
    out = os.path.join(HERE, "ref")
    with tempfile.TemporaryDirectory() as tmp:
        cat_txt = rf.gunzip_to(os.path.join(HERE, "sandbox", CATALOG + ".gz"), os.path.join(tmp, CATALOG))
        pts = oracle.read_7col(cat_txt)
        raw = os.path.join(tmp, "points.f32")
        np.ascontiguousarray(pts, dtype=np.float32).tofile(raw)
        drv = os.path.join(tmp, "chunk_sum")
        subprocess.run(["g++", "-O1", "-ffp-contract=off", "-fopenmp", "-w", "-Dmain=ref_main", "-include", src,
                        "-o", drv, os.path.join(HERE, "chunk_sum_driver.cc"), "-lm"], check=True)
        r = subprocess.run([drv, raw, str(DIVISION)], check=True, capture_output=True)
        gz_write(os.path.join(out, "lrg_rrr_x10_chunk_sum.txt.gz"), r.stdout)
        for job in CHUNK_JOBS:
            o = os.path.join(tmp, "o.dat")
            subprocess.run([exe, cat_txt, cat_txt, cat_txt, "-X", str(DIVISION), "-x", job, "-o", o],
                           check=True, stdout=subprocess.DEVNULL, cwd=tmp)
            with open(o, "rb") as f:
                gz_write(os.path.join(out, "lrg_rrr_x10_%s.dat.gz" % job), f.read())
    print("written to", out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
