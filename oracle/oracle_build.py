#!/usr/bin/env python3
"""Builds the oracle (test infrastructure only): the C restatement in
tpcf_oracle.c as a shared library in oracle/_build/, and the reference's own
programs via ref_build.py (configured copies are written only where the
reference checkout exists; compilation runs wherever the copies are)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtpcf_oracle.so")


def build_oracle():
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "tpcf_oracle.c")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    # -ffp-contract=off: the reference's float expressions are evaluated as
    # separate IEEE operations (no fused multiply-add), on x86-64 and aarch64.
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-Wall",
           "-o", LIB, src, "-lm", "-lpthread"]
    subprocess.run(cmd, check=True)
    return LIB


def build_all(reference=None):
    """reference: the reference checkout, if this machine has one (else
    TPCF_REFERENCE_DIR; without either, the configured copies already in
    oracle/_ref/src are compiled)."""
    sys.path.insert(0, HERE)
    import ref_build
    build_oracle()
    ref_build.write_configured(reference)
    ref_build.compile_all()


if __name__ == "__main__":
    build_all()
    print("oracle built:", LIB)
