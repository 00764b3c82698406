#!/usr/bin/env python3
"""Writes tests/golden/acosf_exceptions_<arch>_glibc<ver>.npz: every float c in
[-1, 1] for which this machine's glibc acosf differs from (float)tpcf_acos_d(c)
(3pcf_gb300/csrc/exact_acos.h), stored as key deltas and the +-1 ulp direction.

The reference's golden files were made on x86-64; the GPU tests load this x86-64
table into the engine on any machine so those files can be compared exactly
(glibc's acosf on aarch64 differs from x86-64 glibc's on some inputs)."""
import ctypes
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    lib = ctypes.CDLL(os.path.join(ROOT, "3pcf_gb300", "_build", "libtpcf.so"))
    n = ctypes.c_uint64()
    lib.tpcf_debug_acos_exceptions(None, None, ctypes.c_uint64(0), ctypes.byref(n))
    keys = np.zeros(n.value, dtype=np.uint32)
    dirs = np.zeros(n.value, dtype=np.int8)
    lib.tpcf_debug_acos_exceptions(keys.ctypes.data_as(ctypes.c_void_p), dirs.ctypes.data_as(ctypes.c_void_p),
                                   ctypes.c_uint64(n.value), ctypes.byref(n))
    libc = ctypes.CDLL("libc.so.6")
    libc.gnu_get_libc_version.restype = ctypes.c_char_p
    ver = libc.gnu_get_libc_version().decode()
    deltas = np.diff(keys.astype(np.int64), prepend=0).astype(np.uint32)
    up = np.packbits(dirs > 0)
    name = "acosf_exceptions_%s_glibc%s.npz" % (platform.machine(), ver)
    np.savez_compressed(os.path.join(HERE, name), key_deltas=deltas, up_bits=up, n=np.int64(n.value))
    print(name, n.value)


if __name__ == "__main__":
    sys.exit(main())
