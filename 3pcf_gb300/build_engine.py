#!/usr/bin/env python3
"""Builds the engine in-tree: 3pcf_gb300/_build/libtpcf.so (CUDA kernels for
sm_103a + host engine + C ABI) and the command-line shims in 3pcf_gb300/bin/.

Translation units compile in parallel; no cmake.  nvcc cross-compiles for
sm_103a without a GPU, so this also runs on a build machine without one.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
BIN = os.path.join(HERE, "bin")
LIB = os.path.join(BUILD, "libtpcf.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
PROGRAMS = {"tpcf_3side": 0, "tpcf_tp": 1, "tpcf_2pcf": 2, "tpcf_jbj": 3}

HEADERS = ["engine.h", "exact_acos.h"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    errs = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errs.append("$ %s\n%s" % (" ".join(c), out))
    if errs:
        raise RuntimeError("build failed:\n" + "\n".join(errs))


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    hdr = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "tpcf.h")]
    objs = []
    cmds = []
    k_src = os.path.join(CSRC, "kernels.cu")
    k_obj = os.path.join(BUILD, "kernels.o")
    objs.append(k_obj)
    # TPCF_NVCC_FLAGS: extra defines for kernel tuning sweeps (e.g. -DTRI_MIN_BLOCKS=2)
    extra = os.environ.get("TPCF_NVCC_FLAGS", "").split()
    stamp = os.path.join(BUILD, "kernels.flags")
    if not os.path.exists(stamp) or open(stamp).read() != " ".join(extra):
        with open(stamp, "w") as f:
            f.write(" ".join(extra))
    if _newer(k_obj, [k_src, stamp] + hdr):
        cmds.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"] + extra +
                    ["-Xptxas", "-v" if verbose else "-O3", "-c", k_src, "-o", k_obj])
    for name in ("engine.cpp", "io.cpp"):
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name.replace(".cpp", ".o"))
        objs.append(obj)
        if _newer(obj, [src] + hdr):
            # -ffp-contract=off: host float/double expressions are evaluated as
            # written (the exact acos and the reference's bin widths depend on it)
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I" + os.path.join(CUDA, "include"), "-c", src, "-o", obj])
    _run_all(cmds)
    if _newer(LIB, objs):
        subprocess.run(["g++", "-shared", "-o", LIB] + objs +
                       ["-L" + os.path.join(CUDA, "lib64"), "-lcudart_static", "-ldl", "-lrt", "-lpthread"],
                       check=True)
    cmds = []
    cli = os.path.join(CSRC, "cli.cpp")
    for prog, num in PROGRAMS.items():
        exe = os.path.join(BIN, prog)
        if _newer(exe, [cli, LIB] + hdr):
            cmds.append(["g++", "-O2", "-std=c++17", "-Wall", "-DTPCF_PROGRAM=%d" % num, cli, "-o", exe,
                         "-L" + BUILD, "-ltpcf", "-Wl,-rpath,$ORIGIN/../_build"])
    sv = os.path.join(CSRC, "sum_voxels.cpp")
    exe = os.path.join(BIN, "tpcf_sum_voxels")
    if _newer(exe, [sv]):
        cmds.append(["g++", "-O2", "-std=c++17", "-Wall", sv, "-o", exe])
    _run_all(cmds)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", LIB)
