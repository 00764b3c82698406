#!/usr/bin/env python3
"""Recipe that builds the reference's own C programs as parity checkers.

TEST INFRASTRUCTURE ONLY: the outputs are used by the test-suite and by the
CPU-baseline leg of bench.py; the product never runs them.

The reference programs fix their binning with unconditional ``#define`` lines
(src/3pcf_C_version_triangle_parametrization.cc:31-42, src/2pcf_C_version.cc:14-16)
or local initialisers (src/3pcf_C_version.cc:169-173), so ``-D`` cannot override
them.  Step 1 (only where the reference checkout exists) writes one configured
copy per binning variant into ``oracle/_ref/src/`` -- a gitignored build
directory, never part of the repository.  Two further edits are made:

* the histogram ``malloc`` is enlarged eightfold.  Out-of-range sides give bin
  indices past the end of the reference's array (src/3pcf_C_version.cc:30,137-139
  and a rounding case in the other two programs); those writes are undefined
  behaviour that never reaches the printed histogram.  The padding makes them
  defined without changing any printed count.
* nothing else: loops, arithmetic and output formats are untouched.

Step 2 compiles every configured copy in ``oracle/_ref/src/`` into
``oracle/_ref/bin/`` with ``g++ -O1 -ffp-contract=off`` (the reference Makefile's
``-O1``, src/Makefile:105-115, plus no FMA contraction so that an aarch64 build
performs the same IEEE single operations as the x86-64 build that produced the
reference's golden files).  Step 2 needs only the configured copies, so it also
runs on a machine without the reference checkout.
"""
import concurrent.futures
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC_OUT = os.path.join(OUT, "src")
BIN_OUT = os.path.join(OUT, "bin")
# the reference checkout: TPCF_REFERENCE_DIR, or the argument of write_configured
REFERENCE = os.environ.get("TPCF_REFERENCE_DIR")

# name -> (program, parameters).  Parameters are the macro values as the
# reference writes them (double literals).
VARIANTS = {
    # three-side: nbins, hist_min, hist_max (None keeps the reference's own value)
    "3side_default": ("3side", dict(nbins=None, lo=None, hi=None)),
    "3side_n16_0_40": ("3side", dict(nbins=16, lo="0.0", hi="40.0")),
    "3side_n32_0_32": ("3side", dict(nbins=32, lo="0.0", hi="32.0")),
    "3side_n8_5_25": ("3side", dict(nbins=8, lo="5.0", hi="25.0")),
    # triangle parametrization: S, Q, THETA (nbins, lo, hi)
    "tp_default": ("tp", None),
    "tp_sandbox": ("tp", dict(S=(50, "2.0", "12.0"), Q=(16, "0.9", "4.1"), T=(25, "0.", "1."))),
    "tp_sandbox_wide": ("tp", dict(S=(60, "0.", "120."), Q=(16, "0.9", "4.1"), T=(25, "0.", "1."))),
    "tp_s8_q8_t16": ("tp", dict(S=(8, "2.0", "10.0"), Q=(8, "1.0", "3.0"), T=(16, "0.", "1."))),
    "tp_s6_q5_t7_zero": ("tp", dict(S=(6, "0.0", "15.0"), Q=(5, "1.0", "2.5"), T=(7, "0.1", "0.9"))),
    # JBJ shape parametrization (s, s/m, (l-m)/s): S, Q, THETA (nbins, lo, hi)
    "jbj_default": ("jbj", None),
    "jbj_s10_q8_t10": ("jbj", dict(S=(10, "1.0", "11.0"), Q=(8, "0.2", "1.0"), T=(10, "0.", "1."))),
    # 2pcf: S (nbins, lo, hi)
    "2pcf_default": ("2pcf", None),
    "2pcf_s40_1_21": ("2pcf", dict(S=(40, "1.0", "21.0"))),
}

SOURCES = {
    "3side": "3pcf_C_version.cc",
    "tp": "3pcf_C_version_triangle_parametrization.cc",
    "2pcf": "2pcf_C_version.cc",
    "jbj": "3pcf_C_version_triangle_parametrization_JBJ.cc",
}


def _sub1(pattern, repl, text, what):
    new, n = re.subn(pattern, repl, text, flags=re.M)
    if n == 0:
        raise RuntimeError("ref_build: pattern for %s not found" % what)
    return new


def configure(program, params, text):
    """Return the configured copy of one reference source."""
    if program == "3side":
        if params["nbins"] is not None:
            text = _sub1(r"^#define DEFAULT_NBINS \d+.*$", "#define DEFAULT_NBINS %d" % params["nbins"], text, "DEFAULT_NBINS")
        if params["lo"] is not None:
            text = _sub1(r"^(\s*)float hist_min = 0;", r"\g<1>float hist_min = %s;" % params["lo"], text, "hist_min")
        if params["hi"] is not None:
            text = _sub1(r"^(\s*)float hist_max = sqrt\(3\*24\*24\);", r"\g<1>float hist_max = %s;" % params["hi"], text, "hist_max")
        text = _sub1(r"malloc\(size_hist_bytes\)", "malloc(8*(size_t)size_hist_bytes)", text, "hist malloc")
        return text
    if program in ("tp", "jbj"):
        if params is not None:
            for ax, key in (("S", "S"), ("Q", "Q"), ("THETA", "T")):
                n, lo, hi = params[key]
                text = _sub1(r"^#define %s_NBINS \d+.*$" % ax, "#define %s_NBINS %d" % (ax, n), text, ax + "_NBINS")
                text = _sub1(r"^#define %s_LO .*$" % ax, "#define %s_LO %s" % (ax, lo), text, ax + "_LO")
                text = _sub1(r"^#define %s_HI .*$" % ax, "#define %s_HI %s" % (ax, hi), text, ax + "_HI")
        text = _sub1(r"malloc\(size_hist_bytes\)", "malloc(8*(size_t)size_hist_bytes)", text, "hist malloc")
        return text
    if program == "2pcf":
        if params is not None:
            n, lo, hi = params["S"]
            text = _sub1(r"^#define S_NBINS \d+.*$", "#define S_NBINS %d" % n, text, "S_NBINS")
            text = _sub1(r"^#define S_LO .*$", "#define S_LO %s" % lo, text, "S_LO")
            text = _sub1(r"^#define S_HI .*$", "#define S_HI %s" % hi, text, "S_HI")
        text = _sub1(r"malloc\(size_hist_bytes\)", "malloc(8*(size_t)size_hist_bytes)", text, "hist malloc")
        return text
    raise ValueError(program)


def write_configured(reference=None):
    """Step 1: write configured copies (needs the reference checkout, given
    as the argument or by TPCF_REFERENCE_DIR; without one nothing is written
    and False is returned)."""
    reference = reference or REFERENCE
    if not reference:
        return False
    src_dir = os.path.join(reference, "src")
    if not os.path.isdir(src_dir):
        return False
    os.makedirs(SRC_OUT, exist_ok=True)
    manifest = {}
    for name, (program, params) in VARIANTS.items():
        with open(os.path.join(src_dir, SOURCES[program])) as f:
            text = f.read()
        text = configure(program, params, text)
        path = os.path.join(SRC_OUT, name + ".cc")
        old = open(path).read() if os.path.exists(path) else None
        if old != text:
            with open(path, "w") as f:
                f.write(text)
        manifest[name] = {"program": program, "params": params}
    with open(os.path.join(OUT, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    return True


def _compile(name):
    src = os.path.join(SRC_OUT, name + ".cc")
    exe = os.path.join(BIN_OUT, name)
    if os.path.exists(exe) and os.path.getmtime(exe) >= os.path.getmtime(src):
        return name, 0, ""
    cmd = ["g++", "-O1", "-ffp-contract=off", "-w", "-o", exe, src, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return name, r.returncode, r.stderr


def compile_all():
    """Step 2: compile every configured copy present in oracle/_ref/src."""
    if not os.path.isdir(SRC_OUT):
        return []
    os.makedirs(BIN_OUT, exist_ok=True)
    names = sorted(f[:-3] for f in os.listdir(SRC_OUT) if f.endswith(".cc"))
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        results = list(ex.map(_compile, names))
    bad = [(n, e) for n, rc, e in results if rc != 0]
    if bad:
        raise RuntimeError("reference build failed: %s" % bad)
    return names


# the reference's own values for variants that keep them
_DEFAULTS = {
    "3side": dict(nbins=64, lo="0", hi=None),  # hist_max = (float)sqrt(3*24*24), src/3pcf_C_version.cc:172
    "tp": dict(S=(50, "2.0", "12.0"), Q=(16, "0.9", "4.1"), T=(32, "0.", "1.")),  # :31-42
    "2pcf": dict(S=(700, "0.0", "70.0")),  # src/2pcf_C_version.cc:14-16
    "jbj": dict(S=(50, "2.0", "12.0"), Q=(16, "0.9", "4.1"), T=(32, "0.", "1.")),  # _JBJ.cc:31-42
}


def binning(name):
    """Explicit binning of a variant: (program, params) with every value set.
    Three-side params are nbins/lo/hi with hi=None meaning sqrt(1728.0)."""
    program, params = VARIANTS[name]
    if program == "3side":
        p = dict(_DEFAULTS["3side"])
        for k, v in params.items():
            if v is not None:
                p[k] = v
        return program, p
    return program, (params if params is not None else _DEFAULTS[program])


def binary(name):
    """Path of a compiled reference variant, or None."""
    p = os.path.join(BIN_OUT, name)
    return p if os.path.exists(p) else None


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else REFERENCE
    if not ref and not os.path.isdir(SRC_OUT):
        print("ref_build: give the reference checkout (argument or TPCF_REFERENCE_DIR)")
        return 1
    wrote = write_configured(ref)
    names = compile_all()
    print("reference variants: configured=%s built=%d" % (wrote, len(names)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
