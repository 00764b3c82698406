"""ctypes binding of include/tpcf.h (the engine's C ABI) for Python callers.

The counting itself always runs in the CUDA engine (3pcf_gb300/_build/libtpcf.so);
this module only marshals arrays.  Loading fails loudly when the library has not
been built, and every engine call raises EngineError on a non-zero status.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("TPCF_LIB") or os.path.join(HERE, "_build", "libtpcf.so")
BIN_DIR = os.path.join(HERE, "bin")

THREE_SIDE, TRIANGLE, PAIR, TRIANGLE_JBJ = 0, 1, 2, 3
LOOP_ALL, LOOP_SAME, LOOP_ONE = 0, 1, 2
GUARDED_FP32, PLAIN_FP64, GEOMETRY_FP64 = 0, 1, 2
NAN_INT_MIN, NAN_ZERO = 0, 1
OVERFLOW_COMPAT, OVERFLOW_CLEAN = 0, 1

# every function include/tpcf.h declares
ABI_SYMBOLS = [
    "tpcf_create", "tpcf_destroy", "tpcf_last_error", "tpcf_status_string", "tpcf_abi_version",
    "tpcf_catalog_create", "tpcf_catalog_release", "tpcf_resident_bytes", "tpcf_hist_len", "tpcf_count",
    "tpcf_count_batch", "tpcf_submit", "tpcf_wait", "tpcf_cancel", "tpcf_last_stats", "tpcf_loop_units",
    "tpcf_read_catalog", "tpcf_pair_count_noalloc", "tpcf_wait_timed", "tpcf_count_batch_into",
    "tpcf_convert_radecz",
]


class EngineError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("tpcf status %d: %s" % (status, msg))
        self.status = status


class Axis(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_float), ("hi", ctypes.c_float), ("nbins", ctypes.c_int32)]


class Spec(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("loop", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("nan_policy", ctypes.c_int32), ("overflow", ctypes.c_int32), ("prune", ctypes.c_int32),
                ("axis", Axis * 3)]


class Job(ctypes.Structure):
    _fields_ = [("catalog", ctypes.c_uint64 * 3), ("begin", ctypes.c_int64 * 3), ("end", ctypes.c_int64 * 3),
                ("flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


JOB_GLOBAL_INDEX = 1


class Stats(ctypes.Structure):
    _fields_ = [("kernel_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("loop_units", ctypes.c_uint64),
                ("evaluated_units", ctypes.c_uint64), ("recheck_units", ctypes.c_uint64),
                ("tasks", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("main_kernel_ms", ctypes.c_double), ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("binned_units", ctypes.c_uint64), ("graph_replays", ctypes.c_uint64),
                ("tuned_shapes", ctypes.c_uint64), ("hist_copies", ctypes.c_uint64), ("ctas_per_sm", ctypes.c_uint64),
                ("plan_ms", ctypes.c_double), ("recheck_regrows", ctypes.c_uint64)]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("CUDA engine not built: %s is missing (run __graft_entry__.build())" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.tpcf_create.argtypes = [ctypes.POINTER(P), ctypes.c_int32]
        L.tpcf_destroy.argtypes = [P]
        L.tpcf_last_error.restype = ctypes.c_char_p
        L.tpcf_last_error.argtypes = [P]
        L.tpcf_status_string.restype = ctypes.c_char_p
        L.tpcf_catalog_create.argtypes = [P, P, P, P, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64)]
        L.tpcf_catalog_release.argtypes = [P, ctypes.c_uint64]
        L.tpcf_resident_bytes.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
        L.tpcf_hist_len.argtypes = [ctypes.POINTER(Spec), ctypes.POINTER(ctypes.c_int64)]
        L.tpcf_count.argtypes = [P, ctypes.POINTER(Spec), ctypes.POINTER(Job), P, ctypes.c_int64]
        L.tpcf_count_batch.argtypes = [P, P, P, ctypes.c_int32, P]
        L.tpcf_count_batch_into.argtypes = [P, P, P, ctypes.c_int32, P, ctypes.c_int32, P]
        L.tpcf_convert_radecz.argtypes = [P, P, P, P, ctypes.c_int64, P, P, P, P]
        L.tpcf_submit.argtypes = [P, ctypes.POINTER(Spec), ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_uint64)]
        L.tpcf_wait.argtypes = [P, ctypes.c_uint64, P, ctypes.c_int64, ctypes.c_int64]
        L.tpcf_cancel.argtypes = [P, ctypes.c_uint64]
        L.tpcf_wait_timed.argtypes = [P, ctypes.c_uint64, P, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.tpcf_last_stats.argtypes = [P, ctypes.POINTER(Stats)]
        L.tpcf_loop_units.argtypes = [P, ctypes.POINTER(Spec), ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_uint64)]
        L.tpcf_read_catalog.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_float, P, P, P,
                                        ctypes.POINTER(ctypes.c_int64)]
        L.tpcf_pair_count_noalloc.restype = ctypes.c_int32
        L.tpcf_pair_count_noalloc.argtypes = [P, P, P, ctypes.c_int64, P, P, P, ctypes.c_int64, ctypes.c_int32,
                                              ctypes.c_float, ctypes.c_float, ctypes.c_int32, P, P]
        L.tpcf_debug_set_acos_exceptions.restype = ctypes.c_int32
        L.tpcf_debug_set_acos_exceptions.argtypes = [P, P, P, ctypes.c_uint64]
        L.tpcf_debug_acos_selfcheck.restype = ctypes.c_int64
        L.tpcf_debug_acos_selfcheck.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
        _LIB = L
    return _LIB


def status_string(s):
    return lib().tpcf_status_string(s).decode()


def make_spec(kind, loop, axes, precision=GUARDED_FP32, nan_policy=NAN_INT_MIN, overflow=OVERFLOW_COMPAT, prune=True):
    """axes: list of (nbins, lo, hi); lo/hi are the reference's macro values,
    converted to float exactly as the reference converts them."""
    s = Spec()
    s.kind, s.loop, s.precision, s.nan_policy, s.overflow, s.prune = kind, loop, precision, nan_policy, overflow, int(prune)
    for i, (n, lo, hi) in enumerate(axes):
        s.axis[i].nbins = int(n)
        s.axis[i].lo = float(np.float32(lo))
        s.axis[i].hi = float(np.float32(hi))
    return s


def hist_len(spec):
    n = ctypes.c_int64()
    lib().tpcf_hist_len(ctypes.byref(spec), ctypes.byref(n))
    return n.value


def read_catalog(path, fmt, scale_factor=1.0):
    """Reference catalog file -> (n,3) float32 (fscanf-identical parsing)."""
    n = ctypes.c_int64(0)
    st = lib().tpcf_read_catalog(path.encode(), fmt, np.float32(scale_factor), None, None, None, ctypes.byref(n))
    if st != 0:
        raise EngineError(st, "read_catalog %s" % path)
    cols = np.zeros((3, max(n.value, 1)), dtype=np.float32)
    st = lib().tpcf_read_catalog(path.encode(), fmt, np.float32(scale_factor), cols[0].ctypes.data,
                                 cols[1].ctypes.data, cols[2].ctypes.data, ctypes.byref(n))
    if st != 0:
        raise EngineError(st, "read_catalog %s" % path)
    return np.ascontiguousarray(cols[:, :n.value].T)


class Engine:
    """One engine context on one CUDA device."""

    def __init__(self, device=0):
        self._ctx = ctypes.c_void_p()
        st = lib().tpcf_create(ctypes.byref(self._ctx), device)
        if st != 0:
            raise EngineError(st, lib().tpcf_last_error(None).decode())

    def _check(self, st, what):
        if st != 0:
            raise EngineError(st, "%s: %s" % (what, lib().tpcf_last_error(self._ctx).decode()))

    def close(self):
        if self._ctx:
            lib().tpcf_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def catalog(self, xyz):
        xyz = np.asarray(xyz, dtype=np.float32).reshape(-1, 3)
        cols = [np.ascontiguousarray(xyz[:, a]) for a in range(3)]
        h = ctypes.c_uint64()
        self._check(lib().tpcf_catalog_create(self._ctx, cols[0].ctypes.data, cols[1].ctypes.data,
                                              cols[2].ctypes.data, len(xyz), ctypes.byref(h)), "catalog_create")
        return h.value

    def release(self, handle):
        self._check(lib().tpcf_catalog_release(self._ctx, handle), "catalog_release")

    @staticmethod
    def job(handles, ranges=None, global_index=False):
        """ranges: per catalog [begin, end) (end -1: to the end).  global_index:
        the mode predicates compare positions in the whole catalog."""
        j = Job()
        hs = list(handles) + [handles[-1]] * (3 - len(handles))
        for r in range(3):
            j.catalog[r] = hs[r]
            lo, hi = (0, -1) if ranges is None else (list(ranges) + [ranges[-1]] * 3)[r]
            j.begin[r], j.end[r] = lo, hi
        j.flags = JOB_GLOBAL_INDEX if global_index else 0
        return j

    def count(self, spec, job):
        n = hist_len(spec)
        h = np.zeros(n, dtype=np.uint64)
        self._check(lib().tpcf_count(self._ctx, ctypes.byref(spec), ctypes.byref(job), h.ctypes.data, n), "count")
        return h

    def count_batch(self, specs, jobs):
        n = len(specs)
        sa = (Spec * n)(*specs)
        ja = (Job * n)(*jobs)
        hists = [np.zeros(hist_len(s), dtype=np.uint64) for s in specs]
        ptrs = (ctypes.c_void_p * n)(*[h.ctypes.data for h in hists])
        self._check(lib().tpcf_count_batch(self._ctx, sa, ja, n, ptrs), "count_batch")
        return hists

    class Batch:
        """Specs, jobs and output map packed once for repeated counts of a large
        batch (count_batch_into rebuilds them on every call)."""

        def __init__(self, specs, jobs, out_index, n_out):
            self.n = len(specs)
            self.specs = (Spec * self.n)(*specs)
            self.jobs = (Job * self.n)(*jobs)
            self.out_index = np.ascontiguousarray(np.asarray(out_index, dtype=np.int32))
            self.n_out = n_out
            self.lens = [0] * n_out
            for s, o in zip(specs, self.out_index):
                if 0 <= int(o) < n_out:  # the engine rejects the rest
                    self.lens[int(o)] = hist_len(s)
            self.hists = [np.zeros(max(1, ln), dtype=np.uint64) for ln in self.lens]
            self.ptrs = (ctypes.c_void_p * n_out)(*[h.ctypes.data for h in self.hists])

    def prepare(self, specs, jobs, out_index, n_out):
        return Engine.Batch(specs, jobs, out_index, n_out)

    def count_prepared(self, b):
        """Counts a prepared batch; returns copies of the n_out summed histograms."""
        self._check(lib().tpcf_count_batch_into(self._ctx, b.specs, b.jobs, b.n, b.out_index.ctypes.data, b.n_out,
                                                b.ptrs), "count_batch_into")
        return [h[:ln].copy() for h, ln in zip(b.hists, b.lens)]

    def count_batch_into(self, specs, jobs, out_index, n_out):
        """Job i adds into output out_index[i]; returns the n_out summed histograms."""
        return self.count_prepared(Engine.Batch(specs, jobs, out_index, n_out))

    def convert_radecz(self, ra, dec, redshift, poly=None):
        """(n,3) float32 Cartesian coordinates of ra/dec (degrees) and redshift."""
        cols = [np.ascontiguousarray(np.asarray(v, dtype=np.float64)) for v in (ra, dec, redshift)]
        n = len(cols[0])
        out = [np.zeros(n, dtype=np.float32) for _ in range(3)]
        pc = None if poly is None else np.ascontiguousarray(np.asarray(poly, dtype=np.float64))
        self._check(lib().tpcf_convert_radecz(self._ctx, cols[0].ctypes.data, cols[1].ctypes.data,
                                              cols[2].ctypes.data, n, None if pc is None else pc.ctypes.data,
                                              out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data),
                    "convert_radecz")
        return np.stack(out, axis=1)

    def submit(self, spec, job):
        t = ctypes.c_uint64()
        self._check(lib().tpcf_submit(self._ctx, ctypes.byref(spec), ctypes.byref(job), ctypes.byref(t)), "submit")
        return t.value

    def wait(self, ticket, spec, timeout_ms=-1):
        n = hist_len(spec)
        h = np.zeros(n, dtype=np.uint64)
        self._check(lib().tpcf_wait(self._ctx, ticket, h.ctypes.data, n, timeout_ms), "wait")
        return h

    def wait_timed(self, ticket, spec, timeout_ms=-1):
        """(histogram, latency ms from submit to completion, ms of its batch)."""
        n = hist_len(spec)
        h = np.zeros(n, dtype=np.uint64)
        lat, run = ctypes.c_double(), ctypes.c_double()
        self._check(lib().tpcf_wait_timed(self._ctx, ticket, h.ctypes.data, n, timeout_ms, ctypes.byref(lat),
                                          ctypes.byref(run)), "wait")
        return h, lat.value, run.value

    def cancel(self, ticket):
        return lib().tpcf_cancel(self._ctx, ticket)

    def stats(self):
        s = Stats()
        self._check(lib().tpcf_last_stats(self._ctx, ctypes.byref(s)), "last_stats")
        return {f: getattr(s, f) for f, _ in Stats._fields_}

    def loop_units(self, spec, job):
        u = ctypes.c_uint64()
        self._check(lib().tpcf_loop_units(self._ctx, ctypes.byref(spec), ctypes.byref(job), ctypes.byref(u)),
                    "loop_units")
        return u.value

    def resident_bytes(self):
        b = ctypes.c_int64()
        self._check(lib().tpcf_resident_bytes(self._ctx, ctypes.byref(b)), "resident_bytes")
        return b.value

    def set_acos_exceptions(self, keys, up):
        """Test hook: use another machine's glibc acosf (exception keys sorted,
        up[i] True when glibc rounds one ulp above (float)tpcf_acos_d)."""
        keys = np.ascontiguousarray(keys, dtype=np.uint32)
        dirs = np.where(np.asarray(up, dtype=bool), 1, -1).astype(np.int8)
        self._check(lib().tpcf_debug_set_acos_exceptions(self._ctx, keys.ctypes.data, dirs.ctypes.data, len(keys)),
                    "set_acos_exceptions")

    def acos_selfcheck(self):
        n = ctypes.c_int64()
        r = lib().tpcf_debug_acos_selfcheck(self._ctx, ctypes.byref(n))
        return r, n.value
