/*
 * tpcf.h -- C ABI of the GB300 triplet/pair counting engine.
 *
 * The reference (mattbellis/3pcf) has no library interface: each histogram is a
 * stand-alone program whose main() reads catalogs, runs a nested loop over point
 * triples (or pairs) and writes a histogram file.  This ABI exposes exactly that
 * loop as a call, with the reference's semantics (same loop bounds, same float
 * arithmetic, same bins, bit-identical integer counts), computed on one GPU.
 * The command-line shims (tpcf_3side, tpcf_tp, tpcf_2pcf) are thin callers of
 * this ABI that keep the reference's flags and file formats.
 *
 * Conventions
 *   - plain C types and pointers only; every call returns a tpcf_status
 *     (0 = success, negative = error) and never throws;
 *   - histograms returned to the caller are uint64 counts in the reference's
 *     index layout; the reference's own unsigned-int wrap (triangle and pair
 *     programs) is applied only by the file writers;
 *   - a context is bound to one CUDA device and is not thread-safe: use one
 *     context per host thread (calls on one context are serialised internally);
 *   - catalogs are uploaded once and stay resident in device memory until
 *     released or the context is destroyed.
 */
#ifndef TPCF_H
#define TPCF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TPCF_ABI_VERSION 3

typedef int32_t tpcf_status;
enum {
    TPCF_OK = 0,
    TPCF_ERR_INVALID = -1,        /* bad argument (message in tpcf_last_error) */
    TPCF_ERR_CUDA = -2,           /* CUDA runtime error */
    TPCF_ERR_NO_DEVICE = -3,      /* no CUDA device, or extension built without one */
    TPCF_ERR_OOM = -4,            /* device memory admission failed */
    TPCF_ERR_TIMEOUT = -5,        /* tpcf_wait timed out; the job keeps running */
    TPCF_ERR_NOT_FOUND = -6,      /* unknown catalog handle or ticket */
    TPCF_ERR_CANCELLED = -7,      /* job cancelled before it ran */
    TPCF_ERR_INTERNAL = -8,       /* invariant violated (device error flag set) */
    TPCF_ERR_IO = -9              /* file could not be read or written */
};

/* Which histogram. */
enum {
    TPCF_THREE_SIDE = 0, /* src/3pcf_C_version.cc: sides d01,d02,d12 binned unsorted */
    TPCF_TRIANGLE = 1,   /* src/3pcf_C_version_triangle_parametrization.cc: (s,q,theta) */
    TPCF_PAIR = 2,       /* src/2pcf_C_version.cc: pair separation */
    TPCF_TRIANGLE_JBJ = 3 /* src/3pcf_C_version_triangle_parametrization_JBJ.cc:116-229:
                             one count per triangle at (s, q, theta) = (shortest,
                             shortest/middle, (longest-middle)/shortest); with
                             TPCF_OVERFLOW_COMPAT bin 0 also gets the reference's 2
                             counts per visited triangle (:455, :511-518), with
                             TPCF_OVERFLOW_CLEAN it does not */
};

/* Loop nest.  The reference decides it from argv string identity and keeps it
 * in a bool (src/3pcf_C_version_triangle_parametrization.cc:333-353), so only
 * two nests exist in the triangle and pair programs. */
enum {
    TPCF_LOOP_ALL = 0,  /* every ordered triple: the three-side loop,
                           src/3pcf_C_version.cc:363-432; pairs: every (i,j) */
    TPCF_LOOP_SAME = 1, /* j >= i, k >= j (which_three_input_files == 0, :484-509);
                           pairs: j >= i (src/2pcf_C_version.cc:365-370) */
    TPCF_LOOP_ONE = 2   /* j from 0, k >= j (which_three_input_files == 1) */
};

/* Arithmetic of the per-triangle kernel.  The first two give identical
 * histograms (the reference's); the third is a different, more accurate count. */
enum {
    TPCF_GUARDED_FP32 = 0, /* FP32 fast path; values within a bounded guard band of
                              a bin edge are recomputed exactly */
    TPCF_PLAIN_FP64 = 1,   /* every reference float operation done in FP64 and
                              rounded to float (exact for + - * / sqrt) */
    TPCF_GEOMETRY_FP64 = 2 /* triangle only: the same formulas evaluated in double
                              from the float coordinates (acos in double); NOT the
                              reference's counts -- the FP64 truth that the error of
                              the derived correlation function is measured against
                              (no counterpart in the reference) */
};

/* int(NaN) in distance_to_bin (src/3pcf_C_version_triangle_parametrization.cc:99)
 * is platform-defined in the reference: x86-64 cvttss2si yields INT_MIN (the
 * permutation is dropped); aarch64 fcvtzs yields 0 (counted in bin 0). */
enum {
    TPCF_NAN_INT_MIN = 0,
    TPCF_NAN_ZERO = 1
};

/* Three-side handling of sides at or above hist_max. */
enum {
    TPCF_OVERFLOW_COMPAT = 0, /* reference: bin nbins+1, index aliases; indices
                                 past nbins^3 are not counted */
    TPCF_OVERFLOW_CLEAN = 1   /* skip triples with any side >= hist_max */
};

typedef struct {
    float lo;       /* lower edge, as the float the reference converts it to */
    float hi;       /* upper edge */
    int32_t nbins;
} tpcf_axis;

typedef struct {
    int32_t kind;       /* TPCF_THREE_SIDE / TPCF_TRIANGLE / TPCF_PAIR */
    int32_t loop;       /* TPCF_LOOP_* */
    int32_t precision;  /* TPCF_GUARDED_FP32 / TPCF_PLAIN_FP64 */
    int32_t nan_policy; /* TPCF_NAN_* (triangle only; pair counts always follow
                           x86-64: a NaN separation is not counted) */
    int32_t overflow;   /* TPCF_OVERFLOW_* (three-side and JBJ) */
    int32_t prune;      /* 1: skip point tiles that provably cannot contribute
                           (exact); 0: visit every tile of the loop nest */
    tpcf_axis axis[3];  /* three-side: axis[0]; triangle: s, q, theta; pair: axis[0] */
} tpcf_spec;

/* One histogram request: 3 catalog ranges (2 for pairs).  The loop indices of
 * the reference are positions inside [begin, end) of each range, which is how
 * the reference's -X/-x index chunks (vox2gal, :52-80) behave. */
/* Job flags. */
enum {
    /* The loop indices the mode predicates compare (j >= i, k >= j) are
     * positions in the whole catalog instead of positions inside [begin, end).
     * The reference's -x chunk jobs use positions inside the chunk (default);
     * spatial sub-jobs whose sum must equal the one-job count use this flag. */
    TPCF_JOB_GLOBAL_INDEX = 1
};

typedef struct {
    uint64_t catalog[3];
    int64_t begin[3];
    int64_t end[3];     /* -1: to the end of the catalog */
    uint32_t flags;     /* TPCF_JOB_* */
    uint32_t reserved;  /* 0 */
} tpcf_job;

typedef struct {
    double kernel_ms;            /* device time of the counting kernels */
    double total_ms;             /* wall time of the last call */
    uint64_t loop_units;         /* triangles (pairs) the reference's loop visits */
    uint64_t evaluated_units;    /* triangles (pairs) the kernels evaluated */
    uint64_t recheck_units;      /* guard-band cases recomputed exactly */
    uint64_t tasks;              /* tile tasks launched */
    uint64_t kernel_launches;    /* engine kernels launched by the last call */
    double main_kernel_ms;       /* device time of the counting kernel alone (no recheck) */
    uint64_t h2d_bytes;          /* host-to-device bytes copied since the previous tpcf_last_stats */
    uint64_t d2h_bytes;          /* device-to-host bytes copied since the previous tpcf_last_stats */
    uint64_t binned_units;       /* triangles (pairs) that reached the full binning arithmetic */
    uint64_t graph_replays;      /* launches replayed from a captured CUDA graph (a repeated
                                    batch); the rest were issued one by one */
    uint64_t tuned_shapes;       /* launch shapes the autotuner timed in this call (0: none) */
    uint64_t hist_copies;        /* launch shape of the last group: histogram copies per CTA
                                    in shared memory (0: global histogram) ... */
    uint64_t ctas_per_sm;        /* ... and resident CTAs per SM */
    double plan_ms;              /* host time of views, planning and the task upload
                                    (near 0 when a repeated batch reuses its plan) */
    uint64_t recheck_regrows;    /* times the guard-band recheck queue overflowed and the
                                    count was repeated with a larger queue */
} tpcf_stats;

typedef struct tpcf_ctx tpcf_ctx;

/* ---- context -------------------------------------------------------------- */
/* New context on a CUDA device.  Fails with TPCF_ERR_NO_DEVICE without a GPU. */
tpcf_status tpcf_create(tpcf_ctx** ctx, int32_t device);
tpcf_status tpcf_destroy(tpcf_ctx* ctx);
const char* tpcf_last_error(tpcf_ctx* ctx);
const char* tpcf_status_string(tpcf_status s);
int32_t tpcf_abi_version(void);

/* ---- catalogs --------------------------------------------------------------- */
/* Upload n points (SoA float arrays) as a resident catalog.  Replaces the
 * reference's per-program read + malloc of h_x/h_y/h_z
 * (src/3pcf_C_version.cc:311-332, src/3pcf_C_version_triangle_parametrization.cc:366-439).
 * The arrays are copied before the call returns; the catalog's spatial order
 * and its device copy are built on a thread of the library meanwhile, and the
 * first count that uses the catalog waits for them (and reports their errors). */
tpcf_status tpcf_catalog_create(tpcf_ctx* ctx, const float* x, const float* y, const float* z,
                                int64_t n, uint64_t* handle);
tpcf_status tpcf_catalog_release(tpcf_ctx* ctx, uint64_t handle);
/* Device bytes held by catalogs and their cached spatial views. */
tpcf_status tpcf_resident_bytes(tpcf_ctx* ctx, int64_t* bytes);

/* ---- counting ------------------------------------------------------------- */
/* Number of histogram entries of a spec: nbins^3, S*Q*T or nbins. */
tpcf_status tpcf_hist_len(const tpcf_spec* spec, int64_t* len);

/* Synchronous count.  Replaces the hot loops and their distance()/
 * distance_to_bin() helpers:
 *   three-side  src/3pcf_C_version.cc:363-432, :54-142, :23-51
 *   triangle    src/3pcf_C_version_triangle_parametrization.cc:477-533, :116-240, :84-113
 *   pairs       src/2pcf_C_version.cc:358-387, :89-113, :57-86
 * hist (host, hist_len entries) receives the counts. */
tpcf_status tpcf_count(tpcf_ctx* ctx, const tpcf_spec* spec, const tpcf_job* job, uint64_t* hist,
                       int64_t hist_len);

/* Batched count: n jobs in one persistent launch (e.g. DDD, DDR, DRR and RRR,
 * or every voxel job of a decomposition).  hists[i] receives job i. */
tpcf_status tpcf_count_batch(tpcf_ctx* ctx, const tpcf_spec* specs, const tpcf_job* jobs, int32_t n,
                             uint64_t* const* hists);

/* Batched count with summed outputs: job i adds its counts into
 * hists[out_index[i]] (0 <= out_index[i] < n_out; every job of one output has
 * the same histogram length), all in one persistent launch per binning.  This
 * is examples/sum_voxels.py done on the device: a spatial or index-chunk
 * decomposition of one count into many jobs (up to 4,194,303 per binning)
 * returns the summed histogram.  No counterpart in the reference. */
tpcf_status tpcf_count_batch_into(tpcf_ctx* ctx, const tpcf_spec* specs, const tpcf_job* jobs, int32_t n,
                                  const int32_t* out_index, int32_t n_out, uint64_t* const* hists);

/* Asynchronous submit / wait (serving).  Serving workers (TPCF_SERVING_LANES,
 * default 2), each with its own stream, take the oldest pending job together
 * with every pending job of the same binning, while the device bytes of all
 * running batches stay within the admission budget (TPCF_ADMIT_BYTES, default
 * 8 GiB), and count them in one launch; jobs submitted meanwhile go to the next
 * free worker, so batches overlap on the device.  A heavy job (product of its
 * catalog sizes above TPCF_HEAVY_COST, default 1e12) runs alone, and only the
 * first worker takes heavy jobs, so light jobs keep flowing beside them.
 * tpcf_wait blocks up to timeout_ms (<0: forever); tpcf_cancel drops a job that
 * has not started. */
tpcf_status tpcf_submit(tpcf_ctx* ctx, const tpcf_spec* spec, const tpcf_job* job, uint64_t* ticket);
tpcf_status tpcf_wait(tpcf_ctx* ctx, uint64_t ticket, uint64_t* hist, int64_t hist_len, int64_t timeout_ms);
/* As tpcf_wait; also returns the job's milliseconds from submission to
 * completion (latency_ms) and of the device batch it ran in (run_ms). */
tpcf_status tpcf_wait_timed(tpcf_ctx* ctx, uint64_t ticket, uint64_t* hist, int64_t hist_len, int64_t timeout_ms,
                            double* latency_ms, double* run_ms);
tpcf_status tpcf_cancel(tpcf_ctx* ctx, uint64_t ticket);

tpcf_status tpcf_last_stats(tpcf_ctx* ctx, tpcf_stats* stats);

/* Number of reference loop iterations (triangles or pairs) of a job, the
 * reference's numcalc / fake_tot counter (:520, src/3pcf_C_version.cc:429). */
tpcf_status tpcf_loop_units(tpcf_ctx* ctx, const tpcf_spec* spec, const tpcf_job* job, uint64_t* units);

/* ---- catalog conversion ---------------------------------------------------- */
/* ra/dec in degrees and redshift -> Cartesian comoving coordinates (Mpc), on the
 * device, as sample_data/gen_flat_MICE_data.py:53-99 computes them: r = p0 +
 * p1 z + p2 z^2 with poly = {p0, p1, p2} (NULL: the script's MICE fit
 * {-1.07199554, 3013.13296, -638.827998}), x = r sin((90-dec) deg) sin(ra deg),
 * y = r sin((90-dec) deg) cos(ra deg), z = r cos((90-dec) deg), in double,
 * rounded to float.  Host arrays in and out.  The double sin/cos are the GPU's
 * (within 2 ulp of a correctly rounded one), so a coordinate can differ from
 * the script's by one float ulp where the double result sits at a float
 * rounding boundary. */
tpcf_status tpcf_convert_radecz(tpcf_ctx* ctx, const double* ra, const double* dec, const double* redshift,
                                int64_t n, const double* poly, float* x, float* y, float* z);

/* ---- pair counts without device allocation -------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory themselves or let a library do so -- e.g. code inside a framework
 * whose memory pool owns the whole device, or a plugin that must not change its
 * host application's device footprint.  It counts the same pair histogram as
 * tpcf_count with TPCF_PAIR (same loop nests, bit-identical counts) from device
 * arrays x0/y0/z0 (n0 points) and x1/y1/z1 (n1 points), writing nbins counts to
 * the device array hist, and calls no cudaMalloc or cudaFree: its working
 * buffers are one 8 MiB array per device, reserved when the library is loaded
 * and held until the process exits.
 *   - at most 262144 points per catalog (TPCF_ERR_INVALID beyond);
 *   - loop TPCF_LOOP_SAME with identical pointers and sizes counts j >= i of
 *     one catalog; with different arrays it compares loop indices;
 *   - each call looks up that array's device address with the caller's device
 *     current (a host call; valid after a device reset too); the first call on
 *     a device may load the library's device code, so make it before any
 *     stream capture;
 *   - calls share the array: calls that overlap on the GPU (other streams or
 *     host threads) race; the call clears the counter and hist it needs;
 *   - returns TPCF_ERR_CUDA without launching when a CUDA error is already
 *     pending on the calling thread (left pending for its owner);
 *   - a NaN separation is not counted (as the x86-64 build of the reference,
 *     whose int(NaN) is INT_MIN; tpcf_count's pair kernels do the same);
 *   - asynchronous on 'stream' (a cudaStream_t, or NULL for the default stream). */
tpcf_status tpcf_pair_count_noalloc(const float* x0, const float* y0, const float* z0, int64_t n0,
                                    const float* x1, const float* y1, const float* z1, int64_t n1,
                                    int32_t loop, float lo, float hi, int32_t nbins, uint64_t* hist,
                                    void* stream);

/* ---- reference catalog files ---------------------------------------------- */
/* Read a catalog file exactly as the reference's fscanf loops do.
 * format 0: header-count "N" then "x y z" lines, divided by scale_factor in
 *           float (src/3pcf_C_version.cc:311-332);
 * format 1: seven columns "id ra dec z x y z" until EOF, columns 5-7 kept,
 *           at most 1e6 rows (src/3pcf_C_version_triangle_parametrization.cc:364-394).
 * Call with x == NULL to get the count in *n; then with arrays of *n floats. */
tpcf_status tpcf_read_catalog(const char* path, int32_t format, float scale_factor, float* x, float* y,
                              float* z, int64_t* n);

#ifdef __cplusplus
}
#endif
#endif /* TPCF_H */
