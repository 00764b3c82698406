// engine.h -- internal structures shared by the host engine (engine.cpp) and
// the CUDA kernels (kernels.cu).  Not part of the public ABI (include/tpcf.h).
#ifndef TPCF_ENGINE_H
#define TPCF_ENGINE_H

#include <stdint.h>
#include <cuda_runtime.h>

namespace tpcf {

// Points per spatial tile.  A triangle task covers one tile of each role.
constexpr int TILE = 64;

// Per-triangle predicate of a task (how the reference's loop bounds restrict
// the triples of a tile triple).
enum Pred : uint32_t {
    PRED_NONE = 0,   // every triple of the tile triple counts once
    PRED_DDR = 1,    // weight [key_k >= key_i] + [key_k >= key_j]  (loop ONE, roles A == B)
    PRED_SAME = 2,   // key_i <= key_j <= key_k                      (loop SAME, generic arrays)
    PRED_ONE = 3,    // key_j <= key_k                               (loop ONE, generic arrays)
    PRED_RDD = 4     // weight [key_i >= key_j] + [key_i >= key_k]   (loop ONE, roles A == B, in the
                     // role order (C, A, A): the single-array point first; guarded kernel only)
};
// task.x: bits 0..21 job slot, 22..24 Pred, 28/29 diagonal flags, 30/31 reach checks
constexpr uint32_t TASK_SLOT_MASK = 0x3FFFFFu;
constexpr uint32_t MAX_BATCH_JOBS = TASK_SLOT_MASK;  // jobs of one launch
constexpr int TASK_PRED_SHIFT = 22;
constexpr uint32_t TASK_PRED_MASK = 0x7u;
constexpr uint32_t TASK_DIAG_IJ = 1u << 28;  // tiles I and J are the same tile of one view: j > i
constexpr uint32_t TASK_DIAG_JK = 1u << 29;  // tiles J and K are the same tile of one view: k > j
// points of tile A may lie out of reach (>= lmax) of tile B / C: worth
// testing point by point (the guarded triangle kernel; others ignore them)
constexpr uint32_t TASK_CHECK_B = 1u << 30;
constexpr uint32_t TASK_CHECK_C = 1u << 31;
// recheck queue item .x: job slot | weight << 22
constexpr int RECHECK_WEIGHT_SHIFT = 22;

// Per-side word of the triangle kernels: word = code * 128 + class_weight.
// code is the side's s-bin times Q*T (monotone in the side length, so the
// codes of the shortest and middle side are the min and median of the three
// words, >> 7); the special codes below keep that order.  class_weight counts
// side classes so that the sum of a triangle's three weights tells whether any
// permutation can be counted: below s_lo: 4, at/above s_hi (or rounding to bin
// S): 1, in range: 0, zero length or at/above the largest side a counted
// triangle can have: 32 (rejects the triangle).
constexpr int CODE_ZERO = -(1 << 23);   // side length exactly 0
constexpr int CODE_BELOW = -(1 << 22);  // 0 < side < s_lo
constexpr int CODE_ABOVE = (1 << 22);   // side >= s_hi
constexpr int CW_IN = 0, CW_ABOVE = 1, CW_BELOW = 4, CW_REJECT = 32;
constexpr int MAX_TRI_BINS = (1 << 22) - 1;  // S*Q*T limit of the triangle kernel encodings
// The fast (guarded FP32) kernel's side words fit 16 bits, so that its j-k
// table holds them in two bytes: word = code16 * 128 + class_weight with
// code16 the side's s-bin itself (the kernel multiplies by Q*T) and the
// special codes below, in the same order as above.  It takes binnings of at
// most MAX_FAST_S s bins (b == S, rounding at the top edge, stays below
// CODE16_ABOVE).
constexpr int CODE16_ZERO = -2, CODE16_BELOW = -1, CODE16_ABOVE = 255;
constexpr int MAX_FAST_S = 254;
// most tasks in one group of the fast triangle kernel (its shared histogram is
// flushed between groups, at most every 256 tasks)
constexpr int MAX_GROUP_TASKS = 64;
// weight sum (4*nBelow + nAbove, >= 32 if rejected) -> permutation validity
constexpr unsigned VALID_ANY = 0x37u;   // shortest or middle side in range
constexpr unsigned VALID_02 = 0x07u;    // shortest side in range (permutations 0 and 2)
constexpr unsigned VALID_1 = 0x33u;     // middle side in range, no zero side (permutation 1)

// Three-side codes: "at or above hist_max" in clean mode.
constexpr uint32_t CODE3_CLEAN_FAR = 1u << 28;

// A histogram target of one launch.
struct DevJob {
    const float4* pts[3];        // spatially sorted points of roles A, B, C; .w = loop index (int bits)
    const int32_t* tile_start[3];// tile -> first point, ntiles+1 entries
    unsigned long long* hist;    // global uint64 histogram (hist_len entries)
    int32_t weight_pred;         // unused by kernels (kept for stats)
    int32_t pad;
};

// Launch-wide binning constants for the triangle kernels.
struct TriParams {
    int S, Q, T, len;            // len = S*Q*T
    float s_lo, s_hi, s_bw;      // reference float values
    float q_lo, q_hi, q_bw;
    float t_lo, t_hi, t_bw;
    int nan_zero;
    // guarded fast path (all in units of bins)
    float q_scale;               // 1/q_bw
    float q_off;                 // -q_lo/q_bw - 0.5
    float q_thr;                 // 0.5 - guard half-width for q
    float t_coef[6];             // acos(|c|) ~ sqrt(1-|c|) * poly(|c|), scaled by 1/(pi' t_bw)
    float t_half;                // pi/(2 pi' t_bw)
    float t_off0;                // t_half - t_lo/t_bw - 0.5
    float t_thrA;                // 0.5 - fixed guard half-width for theta
    float t_thrB;                // slope of the c-dependent guard half-width
    float t2_off;                // (1 - 3 t_lo)/t_bw - 0.5 - 2*(-0.5) handled in code
    int theta_full;              // theta range covers (0,1): skip range checks
    float lmax;                  // sides >= lmax cannot belong to a counted triangle
    float mid_hi;                // s_hi * q_hi (rounded up): permutation 0 needs two sides below it,
                                 // permutation 1 needs all three below it
    float q_rej;                 // a side ratio at or above it is out of the q range whatever the rounding
};

constexpr int TS_UMAX = 68;  // squared-length thresholds of up to 64 bins

struct ThreeParams {
    int n;                       // nbins
    float lo, hi, bw;
    int clean;
    int len;                     // n^3
    // Side codes from squared lengths (guarded FP32 kernel, when fast != 0):
    // u[v] is the smallest float d2 whose reference bin sqrt(d2) -> v' has
    // v' >= v (v' = nbins + 1 for d >= hi), u[0] = -inf, u[nbins + 2] = NaN;
    // inv_bw ~ 1/bw gives a first guess within one bin of the answer.
    int fast;
    float inv_bw;
    float u[TS_UMAX];
    int zcode;  // bin of a zero-length side (nbins + 1 at or above hist_max)
};

constexpr int PR_UMAX = 704;  // squared-length thresholds of up to 700 pair bins

struct PairParams {
    int n;
    float lo, hi, bw;
    // Bins from squared lengths (guarded FP32 kernel, when fast != 0): the
    // code of a separation d is 0 below lo, bin + 1 inside (up to nbins + 1
    // where rounding gives bin nbins), nbins + 2 at or above hi; u[v] is the
    // smallest float d2 whose code is >= v, u[0] = -inf, u[nbins + 3] = NaN.
    int fast = 0;
    float inv_bw = 0.f;
    float u[PR_UMAX];
};

// Exact glibc-acosf exception table on the device.
struct AcosTable {
    const uint32_t* keys;        // sorted float bit patterns of c
    const uint32_t* vals;        // glibc acosf(c) bit patterns
    const uint32_t* bucket;      // 65537 offsets by key >> 16
    uint32_t n;
};

// Guard-band recheck queue (device scratch).
struct RecheckQueue {
    uint4* items;                // {slot | weight << RECHECK_WEIGHT_SHIFT, ia, ib, ic}
    unsigned int* count;
    unsigned int cap;
    unsigned long long* evaluated;  // triangles of (i,j) pairs the fast kernel walked
};

struct LaunchStats {
    unsigned int* error_flag;    // set by kernels on an internal invariant failure
};

// ---- kernel launchers (kernels.cu) ----
cudaError_t prepare_kernels(int device);  // once per device before any launch
// groups[g] .. groups[g + 1]: the tasks of group g (same job, tiles B and C);
// gbox[6 g ..]: lo/hi of the union of their A tiles; jbj: JBJ binning
cudaError_t launch_triangle_fast(const DevJob* jobs, const uint4* tasks, const uint32_t* groups, const float* gbox,
                                 unsigned int ngroups, unsigned int* group_counter, const TriParams& p,
                                 RecheckQueue q, int grid, int hist_copies, int jbj, cudaStream_t st);
cudaError_t launch_triangle_recheck(const DevJob* jobs, RecheckQueue q, const TriParams& p, AcosTable t,
                                    int grid, cudaStream_t st);
cudaError_t launch_triangle_fp64(const DevJob* jobs, const uint4* tasks, unsigned int ntasks,
                                 unsigned int* task_counter, const TriParams& p, AcosTable t, int grid,
                                 int hist_copies, int mode, cudaStream_t st);  // mode: 0 FP64, 1 geometry, 2 JBJ
cudaError_t launch_three_side(const DevJob* jobs, const uint4* tasks, unsigned int ntasks,
                              unsigned int* task_counter, const ThreeParams& p, int fp64, int grid,
                              int hist_copies, int groups, cudaStream_t st);
cudaError_t launch_pairs(const DevJob* jobs, const uint4* tasks, unsigned int ntasks,
                         unsigned int* task_counter, const PairParams& p, int fp64, int grid,
                         int hist_copies, cudaStream_t st);
cudaError_t launch_acos_check(AcosTable t, uint32_t key_begin, uint32_t count, unsigned int* mismatches,
                              cudaStream_t st);
cudaError_t launch_radecz_to_xyz(const double* ra, const double* dec, const double* redshift, int64_t n,
                                 const double poly[3], float* x, float* y, float* z, cudaStream_t st);

// shared-memory bytes of a launch (for occupancy / admission)
size_t triangle_smem_bytes(int hist_len, int hist_copies);
size_t three_side_smem_bytes(const ThreeParams& p, int hist_copies, int groups);
size_t pair_smem_bytes(int hist_len, int hist_copies);

}  // namespace tpcf
#endif
