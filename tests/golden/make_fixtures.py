#!/usr/bin/env python3
"""Generates the committed parity fixtures under tests/golden/.

Run where the reference checkout exists (it reads it); the fixtures it writes
travel with the repository so that tests never need the checkout.

1. ``sandbox/``: golden histogram files shipped by the reference
   (examples/sandbox) together with the input catalogs they were made from
   (sample_data).  Large files are stored gzip-compressed.
2. ``ref/``: outputs of the reference programs themselves, compiled from source
   by oracle/ref_build.py, on small seeded synthetic catalogs (3pcf_gb300/synth.py)
   that exercise every loop mode, the index-chunk voxel flags (-X/-x), bins whose
   edges are hit exactly (lattice points), duplicate points (zero sides) and
   degenerate triangles (acos of a rounded cosine beyond +-1).
   ``ref/manifest.json`` records each case's program variant, argument vector
   and the machine it ran on (its NaN-to-int convention).
"""
import gzip
import json
import os
import platform
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "3pcf_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import numpy as np  # noqa: E402
import synth  # noqa: E402
import ref_build  # noqa: E402

# the reference checkout (required): TPCF_REFERENCE_DIR or the first argument
REFERENCE = os.environ.get("TPCF_REFERENCE_DIR") or (sys.argv[1] if len(sys.argv) > 1 else None)

SANDBOX_INPUTS = [
    "MICE_5degx5deg_1k_randomized.dat",
    "MICE_LRGs_10degx10deg.dat",
    "flat_MICE_LRGs_10degx10deg.dat",
    "MICE_5degx5deg_10k_randomized.dat",
    "flat_MICE_5degx5deg_10k.dat",
    "MICE_20degx20deg_10k_randomized.dat",
    "flat_MICE_20degx20deg_10k.dat",
]
SANDBOX_GOLDENS = (
    ["DDD_voxel2_%s_evenbinning_CPU_5degx5deg_LRG_binning_1k.dat" % v
     for v in ("000000000", "000000001", "000001000", "000001001",
               "001000000", "001000001", "001001000", "001001001")]
    + ["%s_Debbie_LRG_CPU_10degx10deg_LRG_binning_SLAC_1k.dat" % h for h in ("DDD", "DDR", "DRR", "RRR")]
    + ["%s_evenbinning_CPU_5degx5deg_LRG_binning_10k.dat" % h for h in ("DDD", "DDR", "DRR", "RRR")]
    + ["%s_evenbinning_CPU_20degx20deg_10k.dat" % h for h in ("DDD", "DDR", "DRR", "RRR")]
    + ["DDD_voxel4_%03d%03d%03d_evenbinning_CPU_5degx5deg_LRG_binning_1k.dat" % (i, j, k)
       for i in range(4) for j in range(4) for k in range(4)]
)


def gz_copy(src, dst_gz):
    with open(src, "rb") as f, gzip.GzipFile(dst_gz, "wb", mtime=0) as g:
        g.write(f.read())


def sandbox():
    out = os.path.join(HERE, "sandbox")
    os.makedirs(out, exist_ok=True)
    for name in SANDBOX_INPUTS:
        gz_copy(os.path.join(REFERENCE, "sample_data", name), os.path.join(out, name + ".gz"))
    for name in SANDBOX_GOLDENS:
        gz_copy(os.path.join(REFERENCE, "examples", "sandbox", name), os.path.join(out, name + ".gz"))


def catalogs():
    """Small seeded catalogs (float32, written so fscanf reads them exactly)."""
    cats = {
        # three-side, header-count format
        "h_blobs": ("h", synth.blobs(110, n_blobs=3, sigma=6.0, box=60.0, seed=11)),
        "h_unif": ("h", synth.uniform(100, box=60.0, seed=12)),
        "h_lattice": ("h", np.concatenate([synth.lattice_mix(60, box=16.0, frac=1.0, seed=13),
                                           synth.lattice_mix(20, box=16.0, frac=1.0, seed=13)[:10]])),
        # triangle parametrization / pairs, seven-column format
        "c_blobs": ("7", synth.blobs(170, n_blobs=3, sigma=4.0, box=60.0, seed=21)),
        "c_unif": ("7", synth.uniform(150, box=30.0, seed=22)),
        "c_third": ("7", synth.blobs(90, n_blobs=2, sigma=3.0, box=30.0, seed=23)),
        "c_lattice": ("7", np.concatenate([synth.lattice_mix(150, box=9.0, frac=1.0, seed=24),
                                           synth.lattice_mix(40, box=9.0, frac=1.0, seed=24)[:20]])),
        "c_pairs_d": ("7", synth.blobs(1500, n_blobs=10, sigma=5.0, box=100.0, seed=25)),
        "c_pairs_r": ("7", synth.uniform(1300, box=100.0, seed=26)),
    }
    return cats


def cases():
    """(case name, reference variant, positional catalogs, extra flags)."""
    c = []
    for var in ("3side_n16_0_40", "3side_n8_5_25"):
        c += [(var + "_DDD", var, ["h_blobs"] * 3, []),
              (var + "_RRR", var, ["h_unif"] * 3, []),
              (var + "_DDR", var, ["h_blobs", "h_blobs", "h_unif"], []),
              (var + "_DRR", var, ["h_blobs", "h_unif", "h_unif"], [])]
    c += [("3side_n16_0_40_lattice", "3side_n16_0_40", ["h_lattice"] * 3, []),
          ("3side_n16_0_40_arcmin", "3side_n16_0_40", ["h_unif", "h_blobs", "h_unif"], ["-m"]),
          ("3side_n32_0_32_lattice", "3side_n32_0_32", ["h_lattice", "h_lattice", "h_unif"], [])]
    for var in ("tp_s8_q8_t16", "tp_default"):
        c += [(var + "_DDD", var, ["c_blobs"] * 3, []),
              (var + "_DDR", var, ["c_blobs", "c_blobs", "c_unif"], []),
              (var + "_DRR", var, ["c_blobs", "c_unif", "c_unif"], []),
              (var + "_RRR", var, ["c_unif"] * 3, [])]
    c += [("tp_s8_q8_t16_DRD", "tp_s8_q8_t16", ["c_blobs", "c_unif", "c_blobs"], []),
          ("tp_s8_q8_t16_three", "tp_s8_q8_t16", ["c_blobs", "c_unif", "c_third"], []),
          ("tp_s8_q8_t16_RDD", "tp_s8_q8_t16", ["c_unif", "c_blobs", "c_blobs"], []),
          ("tp_s8_q8_t16_vox3_DDD", "tp_s8_q8_t16", ["c_blobs"] * 3, ["-X", "3", "-x", "000001002"]),
          ("tp_s8_q8_t16_vox3_diag", "tp_s8_q8_t16", ["c_blobs"] * 3, ["-X", "3", "-x", "002002002"]),
          ("tp_s8_q8_t16_vox2_DDR", "tp_s8_q8_t16", ["c_blobs", "c_blobs", "c_unif"], ["-X", "2", "-x", "001000001"]),
          ("tp_s8_q8_t16_lattice", "tp_s8_q8_t16", ["c_lattice"] * 3, []),
          ("tp_s6_q5_t7_zero_lattice", "tp_s6_q5_t7_zero", ["c_lattice"] * 3, []),
          ("tp_s6_q5_t7_zero_DDR", "tp_s6_q5_t7_zero", ["c_lattice", "c_lattice", "c_third"], []),
          ("tp_sandbox_lattice", "tp_sandbox", ["c_lattice"] * 3, [])]
    for var in ("jbj_s10_q8_t10", "jbj_default"):
        c += [(var + "_DDD", var, ["c_blobs"] * 3, []),
              (var + "_DDR", var, ["c_blobs", "c_blobs", "c_unif"], []),
              (var + "_DRR", var, ["c_blobs", "c_unif", "c_unif"], []),
              (var + "_RRR", var, ["c_unif"] * 3, [])]
    c += [("jbj_s10_q8_t10_lattice", "jbj_s10_q8_t10", ["c_lattice"] * 3, []),
          ("jbj_s10_q8_t10_vox2_DDR", "jbj_s10_q8_t10", ["c_blobs", "c_blobs", "c_unif"], ["-X", "2", "-x", "001000001"]),
          ("jbj_s10_q8_t10_three", "jbj_s10_q8_t10", ["c_blobs", "c_unif", "c_third"], [])]
    for var in ("2pcf_default", "2pcf_s40_1_21"):
        c += [(var + "_DD", var, ["c_pairs_d"] * 2, []),
              (var + "_DR", var, ["c_pairs_d", "c_pairs_r"], []),
              (var + "_RR", var, ["c_pairs_r"] * 2, [])]
    c += [("2pcf_default_vox2", "2pcf_default", ["c_pairs_d", "c_pairs_d"], ["-X", "2", "-x", "001000000"]),
          ("2pcf_default_lattice", "2pcf_default", ["c_lattice"] * 2, [])]
    return c


def reference_outputs():
    ref_build.write_configured(REFERENCE)
    ref_build.compile_all()
    out = os.path.join(HERE, "ref")
    os.makedirs(out, exist_ok=True)
    cats = catalogs()
    for name, (fmt, xyz) in cats.items():
        path = os.path.join(out, name + ".dat")
        if fmt == "h":
            synth.write_header_catalog(path, xyz)
        else:
            synth.write_7col_catalog(path, xyz)
    manifest = {"machine": platform.machine(), "cases": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for name, var, pos, flags in cases():
            exe = ref_build.binary(var)
            # the reference decides its loop mode from argv string identity,
            # so identical catalogs are passed as identical strings
            argv = [exe] + [os.path.join(out, p + ".dat") for p in pos] + flags + ["-o", os.path.join(tmp, "o.dat")]
            r = subprocess.run(argv, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, cwd=tmp)
            if r.returncode != 0:
                raise RuntimeError("%s failed: %s" % (name, r.stderr))
            gz_copy(os.path.join(tmp, "o.dat"), os.path.join(out, name + ".dat.gz"))
            manifest["cases"][name] = {"variant": var, "catalogs": pos, "flags": flags}
    with open(os.path.join(out, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


def main():
    if not REFERENCE or not os.path.isdir(REFERENCE):
        print("make_fixtures: give the reference checkout (TPCF_REFERENCE_DIR or the first argument);"
              " fixtures unchanged")
        return 1
    sandbox()
    reference_outputs()
    print("fixtures written to", HERE)
    return 0


if __name__ == "__main__":
    sys.exit(main())
