"""ctypes wrapper of the oracle restatement (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class _Cat(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p), ("n", ctypes.c_long)]


def lib():
    global _LIB
    if _LIB is None:
        import oracle_build as build
        path = build.build_oracle()
        L = ctypes.CDLL(path)
        L.oracle_three_side.restype = ctypes.c_ulonglong
        L.oracle_three_side.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        L.oracle_triangle.restype = ctypes.c_ulonglong
        L.oracle_triangle.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        L.oracle_triangle_jbj.restype = ctypes.c_ulonglong
        L.oracle_triangle_jbj.argtypes = L.oracle_triangle.argtypes
        L.oracle_triangle_geom64.restype = ctypes.c_ulonglong
        L.oracle_triangle_geom64.argtypes = L.oracle_triangle.argtypes
        L.oracle_triangle_one.restype = None
        L.oracle_triangle_one.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_void_p]
        L.oracle_pair.restype = ctypes.c_ulonglong
        L.oracle_pair.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                  ctypes.c_void_p, ctypes.c_int]
        L.oracle_acosf.restype = ctypes.c_float
        L.oracle_acosf.argtypes = [ctypes.c_float]
        L.oracle_read_header.restype = ctypes.c_long
        L.oracle_read_header.argtypes = [ctypes.c_char_p, ctypes.c_float] + [ctypes.c_void_p] * 3 + [ctypes.c_long]
        L.oracle_read_7col.restype = ctypes.c_long
        L.oracle_read_7col.argtypes = [ctypes.c_char_p] + [ctypes.c_void_p] * 3 + [ctypes.c_long]
        _LIB = L
    return _LIB


def _threads():
    return max(1, os.cpu_count() or 1)


def _cats(cats):
    """cats: list of (n,3) float32 arrays -> (ctypes array, keepalive)."""
    keep = []
    arr = (_Cat * len(cats))()
    for i, c in enumerate(cats):
        c = np.ascontiguousarray(np.asarray(c, dtype=np.float32).reshape(-1, 3))
        cols = [np.ascontiguousarray(c[:, a]) for a in range(3)]
        keep += cols
        arr[i].x, arr[i].y, arr[i].z = (cols[0].ctypes.data, cols[1].ctypes.data, cols[2].ctypes.data)
        arr[i].n = len(c)
    return arr, keep


def three_side(cats, lo, hi, nbins, clean=False, nthreads=None):
    """Histogram (nbins^3 uint64, reference index layout) and triples visited."""
    arr, keep = _cats(cats)
    hist = np.zeros(nbins ** 3, dtype=np.uint64)
    n = lib().oracle_three_side(arr, np.float32(lo), np.float32(hi), nbins, int(clean),
                                hist.ctypes.data, nthreads or _threads())
    return hist, n


def triangle(cats, which, spec, nan_zero=False, nthreads=None):
    """spec: ((S, s_lo, s_hi), (Q, q_lo, q_hi), (T, t_lo, t_hi)); limits are
    converted to float32 exactly as the reference converts its macros."""
    arr, keep = _cats(cats)
    lohi = np.array([spec[0][1], spec[0][2], spec[1][1], spec[1][2], spec[2][1], spec[2][2]], dtype=np.float32)
    nb = np.array([spec[0][0], spec[1][0], spec[2][0]], dtype=np.int32)
    hist = np.zeros(int(nb.prod()), dtype=np.uint64)
    n = lib().oracle_triangle(arr, int(which), lohi.ctypes.data, nb.ctypes.data, int(nan_zero),
                              hist.ctypes.data, nthreads or _threads())
    return hist, n


def triangle_jbj(cats, which, spec, compat=True, nthreads=None):
    """JBJ shape histogram (s, s/m, (l-m)/s) with the reference's loop nest;
    compat adds the reference's 2 counts per visited triangle to bin 0."""
    arr, keep = _cats(cats)
    lohi = np.array([spec[0][1], spec[0][2], spec[1][1], spec[1][2], spec[2][1], spec[2][2]], dtype=np.float32)
    nb = np.array([spec[0][0], spec[1][0], spec[2][0]], dtype=np.int32)
    hist = np.zeros(int(nb.prod()), dtype=np.uint64)
    n = lib().oracle_triangle_jbj(arr, int(which), lohi.ctypes.data, nb.ctypes.data, int(compat),
                                  hist.ctypes.data, nthreads or _threads())
    return hist, n


def triangle_geom64(cats, which, spec, nan_zero=False, nthreads=None):
    """The same loop nest with the triangle formulas in double (not the
    reference's counts: the FP64 geometry truth)."""
    arr, keep = _cats(cats)
    lohi = np.array([spec[0][1], spec[0][2], spec[1][1], spec[1][2], spec[2][1], spec[2][2]], dtype=np.float32)
    nb = np.array([spec[0][0], spec[1][0], spec[2][0]], dtype=np.int32)
    hist = np.zeros(int(nb.prod()), dtype=np.uint64)
    n = lib().oracle_triangle_geom64(arr, int(which), lohi.ctypes.data, nb.ctypes.data, int(nan_zero),
                                     hist.ctypes.data, nthreads or _threads())
    return hist, n


def triangle_one(p0, p1, p2, spec, nan_zero=False):
    lohi = np.array([spec[0][1], spec[0][2], spec[1][1], spec[1][2], spec[2][1], spec[2][2]], dtype=np.float32)
    nb = np.array([spec[0][0], spec[1][0], spec[2][0]], dtype=np.int32)
    ps = [np.ascontiguousarray(np.asarray(p, dtype=np.float32)) for p in (p0, p1, p2)]
    out = np.zeros(3, dtype=np.int32)
    lib().oracle_triangle_one(ps[0].ctypes.data, ps[1].ctypes.data, ps[2].ctypes.data, lohi.ctypes.data,
                              nb.ctypes.data, int(nan_zero), out.ctypes.data)
    return out


def pair(cats, which, lo, hi, nbins, nthreads=None):
    arr, keep = _cats(cats)
    hist = np.zeros(nbins, dtype=np.uint64)
    n = lib().oracle_pair(arr, int(which), np.float32(lo), np.float32(hi), nbins, hist.ctypes.data,
                          nthreads or _threads())
    return hist, n


def acosf(c):
    return lib().oracle_acosf(float(np.float32(c)))


def read_header(path, scale_factor=1.0):
    n = lib().oracle_read_header(path.encode(), np.float32(scale_factor), None, None, None, 0)
    if n < 0:
        raise OSError(path)
    out = np.zeros((3, max(n, 1)), dtype=np.float32)
    lib().oracle_read_header(path.encode(), np.float32(scale_factor), out[0].ctypes.data, out[1].ctypes.data,
                             out[2].ctypes.data, n)
    return np.ascontiguousarray(out[:, :n].T)


def read_7col(path):
    n = lib().oracle_read_7col(path.encode(), None, None, None, 0)
    if n < 0:
        raise OSError(path)
    out = np.zeros((3, max(n, 1)), dtype=np.float32)
    lib().oracle_read_7col(path.encode(), out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data, n)
    return np.ascontiguousarray(out[:, :n].T)
