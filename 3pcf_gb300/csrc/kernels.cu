// kernels.cu -- sm_103a counting kernels.
//
// All kernels are persistent: a grid of (SM count x resident CTAs) pulls tile
// tasks from a device counter.  A task names one spatial tile (<= 64 points)
// of each role; the CTA stages the tiles' points in shared memory, computes the
// side lengths of the tile pairs once (exactly as the reference does), and then
// walks the triangles with one warp per point of role A, a loop over role B
// and the 32 lanes spanning role C.  Counts go to warp-private shared
// histograms (32-bit) that are flushed with 64-bit global atomics when the
// task's histogram changes, after a bounded number of tasks, and at exit.
//
// Exactness: side lengths and their bins are computed with IEEE
// round-to-nearest intrinsics in the reference's operation order, so they equal
// the reference's floats.  The triangle-parametrization fast path then works
// with approximate reciprocals/arc cosines and sends every triangle whose q or
// theta value lies within a bounded guard band of a bin edge to a recheck
// queue; the recheck kernel recomputes those triangles with the reference's
// exact arithmetic (including glibc's acosf through an exception table).
#include <stdint.h>
#include <limits.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/tpcf.h"
#include "engine.h"
#include "exact_acos.h"

namespace tpcf {

// ---------------------------------------------------------------------------
// Exact reference arithmetic.  FOps<false>: IEEE float intrinsics (never
// contracted).  FOps<true>: each float operation computed in FP64 and rounded
// to float -- identical results for + - * / sqrt (double rounding is innocuous
// when the wide format has at least 2p+2 bits, Figueroa 1995).
template <bool FP64>
struct FOps;
template <>
struct FOps<false> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
};
template <>
struct FOps<true> {
    static __device__ __forceinline__ float add(float a, float b) { return __double2float_rn(__dadd_rn(a, b)); }
    static __device__ __forceinline__ float sub(float a, float b) { return __double2float_rn(__dsub_rn(a, b)); }
    static __device__ __forceinline__ float mul(float a, float b) { return __double2float_rn(__dmul_rn(a, b)); }
    static __device__ __forceinline__ float div(float a, float b) { return __double2float_rn(__ddiv_rn(a, b)); }
    static __device__ __forceinline__ float sqrt(float a) { return __double2float_rn(__dsqrt_rn(a)); }
};

// |p0 - p1| as the reference computes it: sqrt((dx*dx + dy*dy) + dz*dz) in
// float (src/3pcf_C_version.cc:57-60, src/3pcf_C_version_triangle_parametrization.cc:119-122,
// src/2pcf_C_version.cc:92-95).  Symmetric in its arguments bit for bit.
template <bool FP64>
__device__ __forceinline__ float ref_dist(float4 a, float4 b) {
    typedef FOps<FP64> F;
    float dx = F::sub(a.x, b.x), dy = F::sub(a.y, b.y), dz = F::sub(a.z, b.z);
    float s = F::mul(dx, dx);
    s = F::add(s, F::mul(dy, dy));
    s = F::add(s, F::mul(dz, dz));
    return F::sqrt(s);
}

// distance_to_bin of the triangle and pair programs
// (src/3pcf_C_version_triangle_parametrization.cc:84-113, src/2pcf_C_version.cc:57-86).
template <bool FP64>
__device__ __forceinline__ int ref_bin_tp(float v, float lo, float hi, int n, int nan_zero) {
    typedef FOps<FP64> F;
    float bw = F::div(F::sub(hi, lo), (float)n);
    if (v < lo) return -999;
    if (v >= hi) return -999;
    if (v != v) return nan_zero ? 0 : INT_MIN;  // int(NaN): aarch64 0, x86-64 INT_MIN
    return __float2int_rz(F::div(F::sub(v, lo), bw));
}

// glibc acosf reproduced exactly: (float)tpcf_acos_d(c) unless c is listed in
// the exception table built on the host from the host's own libm.
__device__ __forceinline__ float acosf_ref(float c, const AcosTable& t) {
    if (!(c >= -1.0f && c <= 1.0f)) return __int_as_float(0x7fc00000);
    float r = __double2float_rn(tpcf_acos_d((double)c));
    uint32_t key = __float_as_uint(c);
    uint32_t lo = t.bucket[key >> 16], hi = t.bucket[(key >> 16) + 1];
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (t.keys[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    if (lo < t.n && t.keys[lo] == key) r = __uint_as_float(t.vals[lo]);
    return r;
}

// distance() of the triangle program (:116-240) after the side lengths:
// three histogram indices, or -1 for "not counted" (out of range, zero side, or
// an index past the array end, which the reference never prints).
template <bool FP64>
__device__ void tp_exact(float dist0, float dist1, float dist2, const TriParams& p, const AcosTable& t,
                         int out[3]) {
    typedef FOps<FP64> F;
    float shortest, middle, longest;
    if (dist0 > dist1) {
        if (dist0 > dist2) {
            longest = dist0;
            if (dist1 > dist2) { middle = dist1; shortest = dist2; }
            else { middle = dist2; shortest = dist1; }
        } else {
            middle = dist0;
            if (dist1 > dist2) { longest = dist1; shortest = dist2; }
            else { longest = dist2; shortest = dist1; }
        }
    } else {
        if (dist1 > dist2) {
            longest = dist1;
            if (dist0 > dist2) { middle = dist0; shortest = dist2; }
            else { middle = dist2; shortest = dist0; }
        } else {
            middle = dist1; longest = dist2; shortest = dist0;
        }
    }
    float s2 = F::mul(shortest, shortest), m2 = F::mul(middle, middle), l2 = F::mul(longest, longest);
    bool zero = dist0 == 0.f || dist1 == 0.f || dist2 == 0.f;
    float th0 = 0.f, th1 = 0.f;
    for (int k = 0; k < 3; k++) {
        float s, q;
        int i2;
        if (k == 0) {
            s = shortest;
            q = F::div(middle, shortest);
            float c = F::div(F::sub(F::add(s2, m2), l2), F::mul(F::mul(2.f, shortest), middle));
            th0 = __double2float_rn(__ddiv_rn((double)acosf_ref(c, t), 3.14159));
            i2 = ref_bin_tp<FP64>(th0, p.t_lo, p.t_hi, p.T, p.nan_zero);
        } else if (k == 1) {
            s = middle;
            q = F::div(longest, middle);
            float c = F::div(F::sub(F::add(m2, l2), s2), F::mul(F::mul(2.f, middle), longest));
            th1 = __double2float_rn(__ddiv_rn((double)acosf_ref(c, t), 3.14159));
            i2 = ref_bin_tp<FP64>(th1, p.t_lo, p.t_hi, p.T, p.nan_zero);
        } else {
            s = shortest;
            q = F::div(longest, shortest);
            float th2 = __double2float_rn(__dsub_rn(__dsub_rn(1.0, (double)th0), (double)th1));
            i2 = ref_bin_tp<FP64>(th2, p.t_lo, p.t_hi, p.T, p.nan_zero);
        }
        int i0 = ref_bin_tp<FP64>(s, p.s_lo, p.s_hi, p.S, p.nan_zero);
        int i1 = ref_bin_tp<FP64>(q, p.q_lo, p.q_hi, p.Q, p.nan_zero);
        int tot = -1;
        if (!(i0 < 0 || i1 < 0 || i2 < 0) && !zero) {
            long long idx = (long long)p.Q * p.T * i0 + (long long)p.T * i1 + i2;
            if (idx < p.len) tot = (int)idx;
        }
        out[k] = tot;
    }
}

// ---------------------------------------------------------------------------
// The same triangle formulas evaluated in double from the float coordinates,
// acos in double: not the reference's float arithmetic, but the FP64 truth
// the derived correlation function's error is quoted against.  Every
// operation is an explicit round-to-nearest double op (no contraction), so a
// host restatement compiled without FMA contraction agrees except where the
// two acos implementations differ.

__device__ __forceinline__ double geo_dist(float4 a, float4 b) {
    double dx = __dsub_rn((double)a.x, (double)b.x);
    double dy = __dsub_rn((double)a.y, (double)b.y);
    double dz = __dsub_rn((double)a.z, (double)b.z);
    double s = __dmul_rn(dx, dx);
    s = __dadd_rn(s, __dmul_rn(dy, dy));
    s = __dadd_rn(s, __dmul_rn(dz, dz));
    return __dsqrt_rn(s);
}

__device__ __forceinline__ int geo_bin(double v, float lo, float hi, int n, int nan_zero) {
    double bw = __ddiv_rn(__dsub_rn((double)hi, (double)lo), (double)n);
    if (v < (double)lo) return -999;
    if (v >= (double)hi) return -999;
    if (v != v) return nan_zero ? 0 : INT_MIN;
    return __double2int_rz(__ddiv_rn(__dsub_rn(v, (double)lo), bw));
}

__device__ void tp_geom(double d0, double d1, double d2, const TriParams& p, int out[3]) {
    // shortest <= middle <= longest with the reference's tie handling
    double shortest, middle, longest;
    if (d0 > d1) {
        if (d0 > d2) {
            longest = d0;
            if (d1 > d2) { middle = d1; shortest = d2; }
            else { middle = d2; shortest = d1; }
        } else {
            middle = d0;
            if (d1 > d2) { longest = d1; shortest = d2; }
            else { longest = d2; shortest = d1; }
        }
    } else {
        if (d1 > d2) {
            longest = d1;
            if (d0 > d2) { middle = d0; shortest = d2; }
            else { middle = d2; shortest = d0; }
        } else {
            middle = d1; longest = d2; shortest = d0;
        }
    }
    const double s2 = __dmul_rn(shortest, shortest), m2 = __dmul_rn(middle, middle), l2 = __dmul_rn(longest, longest);
    const bool zero = d0 == 0.0 || d1 == 0.0 || d2 == 0.0;
    double c0 = __ddiv_rn(__dsub_rn(__dadd_rn(s2, m2), l2), __dmul_rn(__dmul_rn(2.0, shortest), middle));
    double c1 = __ddiv_rn(__dsub_rn(__dadd_rn(m2, l2), s2), __dmul_rn(__dmul_rn(2.0, middle), longest));
    double th0 = __ddiv_rn(acos(c0), 3.14159), th1 = __ddiv_rn(acos(c1), 3.14159);
    double th2 = __dsub_rn(__dsub_rn(1.0, th0), th1);
    const double sv[3] = {shortest, middle, shortest};
    const double qv[3] = {__ddiv_rn(middle, shortest), __ddiv_rn(longest, middle), __ddiv_rn(longest, shortest)};
    const double tv[3] = {th0, th1, th2};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        int i0 = geo_bin(sv[k], p.s_lo, p.s_hi, p.S, p.nan_zero);
        int i1 = geo_bin(qv[k], p.q_lo, p.q_hi, p.Q, p.nan_zero);
        int i2 = geo_bin(tv[k], p.t_lo, p.t_hi, p.T, p.nan_zero);
        int tot = -1;
        if (!(i0 < 0 || i1 < 0 || i2 < 0) && !zero) {
            long long idx = (long long)p.Q * p.T * i0 + (long long)p.T * i1 + i2;
            if (idx < p.len) tot = (int)idx;
        }
        out[k] = tot;
    }
}

// ---------------------------------------------------------------------------
// Persistent-task plumbing.

constexpr unsigned int FLUSH_EVERY = 256;  // tasks between histogram flushes (u32 safety)
constexpr uint32_t TASK_NONE = 0xFFFFFFFFu;

// Swizzled shared histograms (three-side kernels): bin b of a copy lives at
// word hist_pos(b), its low five bits (the bank) XORed with the next two 5-bit
// groups, so that the lanes of one atomic instruction whose bins differ only
// in higher digits (n^2 i2 + n i1 + i0 with n = 32 puts every lane of a
// three-side row in one bank) spread over the banks.  It permutes each
// aligned group of 32 words, so a copy takes hist_stride(words) words.
__host__ __device__ constexpr int hist_stride(int len) { return (len + 31) & ~31; }
__device__ __forceinline__ unsigned hist_pos(unsigned b) { return b ^ (((b >> 5) ^ (b >> 10)) & 31u); }

// Adds 'copies' shared histograms of len bins (len words apart) into the
// job's 64-bit histogram and clears them.
__device__ __forceinline__ void flush_hist(unsigned int* H, int copies, int len, unsigned long long* g) {
    __syncthreads();
    for (int b = threadIdx.x; b < len; b += blockDim.x) {
        unsigned long long sum = 0;
        for (int c = 0; c < copies; c++) {
            sum += H[c * len + b];
            H[c * len + b] = 0;
        }
        if (sum) atomicAdd(g + b, sum);
    }
    __syncthreads();
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ---------------------------------------------------------------------------
// Triangle parametrization, guarded FP32.

constexpr int TRI_WARPS = 8;
constexpr int TRI_THREADS = TRI_WARPS * 32;
constexpr int TRI_QCAP = 128;  // per-warp candidate queue: up to 63 pending + 64 new
// per j of role B: bit masks over k of the classes of side j-k (B, I, M, H)
// and of key_k >= key_j; held in shared memory as five 64-entry arrays
// (JM_WORDS x TILE, word-major) so that lanes reading different j's do not
// share banks
struct JMasks {
    unsigned long long c[4];
    unsigned long long kge;
};
constexpr int JM_WORDS = 5;
// A tiles resident at once: the tasks of a group (one job, tiles B and C
// shared) are counted up to four at a time, their points i handed out to the
// warps together
#ifndef TRI_GROUP_A_TILES
#define TRI_GROUP_A_TILES 4
#endif
constexpr int TRI_GROUP_A = TRI_GROUP_A_TILES;
// layout: tiles B, C and up to TRI_GROUP_A A tiles | j-class masks | per-warp
// i-j and i-k rows | j-k sides | per-warp candidate queues | j-k side words
// (16 bits) | histogram copies
constexpr size_t TRI_SMEM_FIXED = (2 + TRI_GROUP_A) * TILE * sizeof(float4) +
                                  JM_WORDS * TILE * sizeof(unsigned long long) + 2 * TRI_WARPS * TILE * sizeof(int2) +
                                  TILE * TILE * sizeof(float) + TRI_WARPS * TRI_QCAP * sizeof(uint32_t) +
                                  TILE * TILE * sizeof(short);
// (the plain FP64 kernel's layout -- three tiles, a j-k table of int2 and one
// row per warp -- fits the same allocation)
static_assert(TRI_SMEM_FIXED >= 3 * TILE * sizeof(float4) + TILE * TILE * sizeof(int2) + TRI_WARPS * TILE * sizeof(int2),
              "FP64 triangle layout");

// s-bin code of one side, monotone in the side length, multiplied by Q*T
// (used by the plain FP64 kernel).
template <bool FP64>
__device__ __forceinline__ int tri_side_code(float d, const TriParams& p) {
    typedef FOps<FP64> F;
    if (d == 0.f) return CODE_ZERO;
    if (d < p.s_lo) return CODE_BELOW;
    if (d >= p.s_hi) return CODE_ABOVE;
    return __float2int_rz(F::div(F::sub(d, p.s_lo), p.s_bw)) * (p.Q * p.T);
}

// Side word of the fast kernel: code16 * 128 + class weight, 16 bits (see
// engine.h); code16 is the s-bin itself.
// (A division-free s-bin -- a guess corrected against exact thresholds
// staged in shared memory -- measured slower: 14.19 vs 13.95 ms on the
// default workload.)
__device__ __forceinline__ int tri_side_word(float d, const TriParams& p) {
    int code, w;
    if (d == 0.f) {
        code = CODE16_ZERO;
        w = CW_REJECT;
    } else if (d < p.s_lo) {
        code = CODE16_BELOW;
        w = CW_BELOW;
    } else if (d >= p.s_hi) {
        code = CODE16_ABOVE;
        w = CW_ABOVE;
    } else {
        code = __float2int_rz(__fdiv_rn(__fsub_rn(d, p.s_lo), p.s_bw));
        w = code < p.S ? CW_IN : CW_ABOVE;  // code == S: rounding at the top edge, index past the array
    }
    if (d >= p.lmax) w = CW_REJECT;
    return code * 128 + w;
}

// 1.5 * 2^23: adding it rounds a float in (-2^22, 2^22) to an integer held in
// the low mantissa bits.
#define MAGIC 12582912.0f
#define MAGIC_BITS 0x4B400000

struct GuardedBin {
    int bin;      // floor of the bin coordinate (valid if not near an edge)
    float err;    // signed distance of the coordinate from its bin centre (in [-0.5, 0.5])
};

// f_m = coordinate - 0.5; returns floor(coordinate) and the offset used by the guard
__device__ __forceinline__ GuardedBin magic_floor(float f_m) {
    float tm = __fadd_rn(f_m, MAGIC);
    float dd = __fsub_rn(tm, MAGIC);
    GuardedBin g;
    g.bin = __float_as_int(tm) - MAGIC_BITS;
    g.err = __fsub_rn(f_m, dd);
    return g;
}

// theta coordinate of a cosine (approximate) and its guard threshold
__device__ __forceinline__ void theta_fast(float c, const TriParams& p, float& f_m, float& thr) {
    float x = fabsf(c);
    float t = __fsub_rn(1.0f, x);
    float y = rsqrt_approx(t);
    float sq = __fmul_rn(t, y);
    float P = p.t_coef[5];
    P = __fmaf_rn(P, x, p.t_coef[4]);
    P = __fmaf_rn(P, x, p.t_coef[3]);
    P = __fmaf_rn(P, x, p.t_coef[2]);
    P = __fmaf_rn(P, x, p.t_coef[1]);
    P = __fmaf_rn(P, x, p.t_coef[0]);
    float a = __fmaf_rn(sq, P, -p.t_half);                                     // K*acos(|c|) - K*pi/2
    a = __int_as_float(__float_as_int(a) ^ (__float_as_int(c) & 0x80000000));  // acos(-x) = pi - acos(x)
    f_m = __fadd_rn(a, p.t_off0);
    thr = __fmaf_rn(-p.t_thrB, y, p.t_thrA);
}

__device__ __forceinline__ unsigned weight_index(int wa, int wb, int wc) { return (unsigned)(wa + wb + wc) & 127u; }
__device__ __forceinline__ bool mask_bit(unsigned mask, unsigned idx) { return (__funnelshift_rc(mask, 0u, idx) & 1u) != 0; }

// Two floats in one 64-bit register for the packed FP32 instructions of
// sm_100+ (add/sub/mul/fma .rn .f32x2: two IEEE single operations per
// instruction, each element rounded exactly as the scalar operation).  Unlike
// the scalar __fmul_rn/__fadd_rn intrinsics, a packed product that feeds a
// packed sum is contracted into one fma.f32x2 by ptxas (measured: the packed
// squared side sums differ from the scalar ones in a fifth of the cases), so
// only results whose exact rounding does not matter, or that no contraction
// can reach, are computed packed.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void up2(f32x2 r, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r)); }
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f32x2 splat2(float a) { return pk2(a, a); }

// magic_floor of two coordinates
__device__ __forceinline__ void magic_floor2(f32x2 f_m, int& b0, int& b1, float& e0, float& e1) {
    const f32x2 mg = splat2(MAGIC);
    const f32x2 tm = add2(f_m, mg);
    up2(sub2(f_m, sub2(tm, mg)), e0, e1);
    float t0, t1;
    up2(tm, t0, t1);
    b0 = __float_as_int(t0) - MAGIC_BITS;
    b1 = __float_as_int(t1) - MAGIC_BITS;
}

// theta_fast of two cosines
__device__ __forceinline__ void theta_fast2(f32x2 c, const TriParams& p, f32x2& f_m, f32x2& thr) {
    float c0, c1;
    up2(c, c0, c1);
    const f32x2 x = pk2(fabsf(c0), fabsf(c1));
    const f32x2 t = sub2(splat2(1.0f), x);
    float t0, t1;
    up2(t, t0, t1);
    const f32x2 y = pk2(rsqrt_approx(t0), rsqrt_approx(t1));
    const f32x2 sq = mul2(t, y);
    f32x2 P = splat2(p.t_coef[5]);
    P = fma2(P, x, splat2(p.t_coef[4]));
    P = fma2(P, x, splat2(p.t_coef[3]));
    P = fma2(P, x, splat2(p.t_coef[2]));
    P = fma2(P, x, splat2(p.t_coef[1]));
    P = fma2(P, x, splat2(p.t_coef[0]));
    float a0, a1;
    up2(fma2(sq, P, splat2(-p.t_half)), a0, a1);  // K*acos(|c|) - K*pi/2
    a0 = __int_as_float(__float_as_int(a0) ^ (__float_as_int(c0) & 0x80000000));  // acos(-x) = pi - acos(x)
    a1 = __int_as_float(__float_as_int(a1) ^ (__float_as_int(c1) & 0x80000000));
    f_m = add2(pk2(a0, a1), splat2(p.t_off0));
    thr = fma2(splat2(-p.t_thrB), y, splat2(p.t_thrA));
}

// Full fast path of two triangles at once (each lane's two candidates): sides
// a, b, c with their words; w: multiplicities (0 = none).  The FP32
// arithmetic of the two runs in packed f32x2 instructions.  A triangle whose
// weight index says some permutation may count is binned into Hw, unless a
// permutation that could count has a coordinate inside its guard band: then
// guard[t] is set and the triangle must be recomputed exactly.
template <bool THETA_FULL>
__device__ __forceinline__ void triangle_full2(const float (&a)[2], const int (&wa)[2], const float (&b)[2],
                                               const int (&wb)[2], const float (&c)[2], const int (&wc)[2],
                                               const unsigned (&w)[2], const TriParams& p, unsigned int* Hw,
                                               bool (&guard)[2]) {
    float s[2], m[2], l[2];
    int off_s[2], off_m[2];
    bool v02[2], v1[2];
#pragma unroll
    for (int t = 0; t < 2; t++) {
        const unsigned idx = weight_index(wa[t], wb[t], wc[t]);
        v02[t] = w[t] && mask_bit(VALID_02, idx);
        v1[t] = w[t] && mask_bit(VALID_1, idx);
        const float lo_ab = fminf(a[t], b[t]), hi_ab = fmaxf(a[t], b[t]);
        s[t] = fminf(lo_ab, c[t]);
        l[t] = fmaxf(hi_ab, c[t]);
        m[t] = fmaxf(lo_ab, fminf(hi_ab, c[t]));
        const int wlo = min(wa[t], wb[t]), whi = max(wa[t], wb[t]);
        // s-bins of the shortest and the middle side, times Q
        off_s[t] = (min(wlo, wc[t]) >> 7) * p.Q;
        off_m[t] = (max(wlo, min(whi, wc[t])) >> 7) * p.Q;
    }
    const f32x2 S = pk2(s[0], s[1]), M = pk2(m[0], m[1]), L = pk2(l[0], l[1]);
    // the squares enter the cosine numerators as the reference rounds them:
    // scalar products (ptxas contracts a packed mul.rn.f32x2 feeding an
    // add.rn.f32x2 into fma.f32x2, measured on sm_103a, which would change
    // the numerators' rounding)
    const f32x2 S2 = pk2(__fmul_rn(s[0], s[0]), __fmul_rn(s[1], s[1]));
    const f32x2 M2 = pk2(__fmul_rn(m[0], m[0]), __fmul_rn(m[1], m[1]));
    const f32x2 L2 = pk2(__fmul_rn(l[0], l[0]), __fmul_rn(l[1], l[1]));
    const f32x2 qs = splat2(p.q_scale), qo = splat2(p.q_off);
    const f32x2 rsq = mul2(pk2(rcp_approx(s[0]), rcp_approx(s[1])), qs);
    const f32x2 rmq = mul2(pk2(rcp_approx(m[0]), rcp_approx(m[1])), qs);
    int q0b[2], q1b[2], q2b[2], t0b[2], t1b[2], t2b[2];
    float q0e[2], q1e[2], q2e[2], t0e[2], t1e[2], t2e[2];
    magic_floor2(fma2(M, rsq, qo), q0b[0], q0b[1], q0e[0], q0e[1]);
    magic_floor2(fma2(L, rmq, qo), q1b[0], q1b[1], q1e[0], q1e[1]);
    magic_floor2(fma2(L, rsq, qo), q2b[0], q2b[1], q2e[0], q2e[1]);
    const f32x2 num0 = sub2(add2(S2, M2), L2);
    const f32x2 num1 = sub2(add2(M2, L2), S2);
    float sm0, sm1, ml0, ml1;
    up2(mul2(S, M), sm0, sm1);
    up2(mul2(M, L), ml0, ml1);
    const f32x2 half = splat2(0.5f);
    const f32x2 c0 = mul2(mul2(num0, pk2(rcp_approx(sm0), rcp_approx(sm1))), half);
    const f32x2 c1 = mul2(mul2(num1, pk2(rcp_approx(ml0), rcp_approx(ml1))), half);
    f32x2 f0m, thr0, f1m, thr1;
    theta_fast2(c0, p, f0m, thr0);
    theta_fast2(c1, p, f1m, thr1);
    const f32x2 f2m = sub2(sub2(splat2(p.t2_off), f0m), f1m);
    float thr0v[2], thr1v[2], thr2v[2];
    up2(thr0, thr0v[0], thr0v[1]);
    up2(thr1, thr1v[0], thr1v[1]);
    up2(add2(add2(thr0, thr1), splat2(-0.5f - 1e-6f)), thr2v[0], thr2v[1]);
    magic_floor2(f0m, t0b[0], t0b[1], t0e[0], t0e[1]);
    magic_floor2(f1m, t1b[0], t1b[1], t1e[0], t1e[1]);
    magic_floor2(f2m, t2b[0], t2b[1], t2e[0], t2e[1]);
#pragma unroll
    for (int t = 0; t < 2; t++) {
        // guard: a permutation that could count has a value near a bin edge
        const bool gq0 = !(fabsf(q0e[t]) <= p.q_thr), gq1 = !(fabsf(q1e[t]) <= p.q_thr),
                   gq2 = !(fabsf(q2e[t]) <= p.q_thr);
        const bool gt0 = !(fabsf(t0e[t]) <= thr0v[t]), gt1 = !(fabsf(t1e[t]) <= thr1v[t]),
                   gt2 = !(fabsf(t2e[t]) <= thr2v[t]);
        const bool g = (v02[t] && (gq0 || gt0 || gq2 || gt2)) || (v1[t] && (gq1 || gt1));
        bool ok0 = v02[t] && !g && (unsigned)q0b[t] < (unsigned)p.Q;
        bool ok1 = v1[t] && !g && (unsigned)q1b[t] < (unsigned)p.Q;
        bool ok2 = v02[t] && !g && (unsigned)q2b[t] < (unsigned)p.Q;
        if (!THETA_FULL) {
            ok0 = ok0 && (unsigned)t0b[t] < (unsigned)p.T;
            ok1 = ok1 && (unsigned)t1b[t] < (unsigned)p.T;
            ok2 = ok2 && (unsigned)t2b[t] < (unsigned)p.T;
        }
        if (ok0) atomicAdd(Hw + (off_s[t] + q0b[t]) * p.T + t0b[t], w[t]);
        if (ok1) atomicAdd(Hw + (off_m[t] + q1b[t]) * p.T + t1b[t], w[t]);
        if (ok2) atomicAdd(Hw + (off_s[t] + q2b[t]) * p.T + t2b[t], w[t]);
        guard[t] = g;
    }
}

// JBJ binning of two triangles (src/3pcf_C_version_triangle_parametrization_JBJ.cc
// distance(), :116-229): one permutation, s = shortest, q = s/m and
// theta = (l - m)/s in float, binned as distance_to_bin does.  These are the
// reference's float operations done exactly (IEEE division), so no guard band
// is needed.  The s-bin comes from the shortest side's word; a triangle whose
// weight index says its shortest side is out of range, zero or rejected, or
// whose multiplicity is 0, adds nothing.

// distance_to_bin: -1 outside [lo, hi); the bin as the reference truncates it,
// which rounding can make n at the top edge (the index then runs into the
// next row, as the reference's does, or past the array)
__device__ __forceinline__ int jbj_axis_bin(float v, float lo, float hi, float bw) {
    if (!(v >= lo) || v >= hi) return -1;  // (v is never NaN here: no zero side reaches this)
    return __float2int_rz(__fdiv_rn(__fsub_rn(v, lo), bw));
}

__device__ __forceinline__ void jbj_full2(const float (&a)[2], const int (&wa)[2], const float (&b)[2],
                                          const int (&wb)[2], const float (&c)[2], const int (&wc)[2],
                                          const unsigned (&w)[2], const TriParams& p, unsigned int* Hw) {
#pragma unroll
    for (int t = 0; t < 2; t++) {
        const unsigned idx = weight_index(wa[t], wb[t], wc[t]);
        const bool v = w[t] && mask_bit(VALID_02, idx);
        const float lo_ab = fminf(a[t], b[t]), hi_ab = fmaxf(a[t], b[t]);
        const float s = fminf(lo_ab, c[t]), l = fmaxf(hi_ab, c[t]), m = fmaxf(lo_ab, fminf(hi_ab, c[t]));
        const int code = min(min(wa[t], wb[t]), wc[t]) >> 7;  // s-bin of the shortest side
        const int i1 = jbj_axis_bin(__fdiv_rn(s, m), p.q_lo, p.q_hi, p.q_bw);
        const int i2 = jbj_axis_bin(__fdiv_rn(__fsub_rn(l, m), s), p.t_lo, p.t_hi, p.t_bw);
        const int x = (code * p.Q + i1) * p.T + i2;
        if (v && i1 >= 0 && i2 >= 0 && x < p.len) atomicAdd(Hw + x, w[t]);
    }
}

__device__ __forceinline__ void push_recheck(RecheckQueue& q, uint32_t slot, unsigned w, uint32_t ia, uint32_t ib,
                                             uint32_t ic) {
    unsigned int pos = atomicAdd(q.count, 1u);
    if (pos < q.cap) q.items[pos] = make_uint4(slot | (w << RECHECK_WEIGHT_SHIFT), ia, ib, ic);
}

struct TaskGeom {
    int a0, nA, b0, nB, c0, nC;
};

__device__ __forceinline__ TaskGeom task_geom(const DevJob& J, uint4 task) {
    TaskGeom g;
    g.a0 = J.tile_start[0][task.y];
    g.nA = J.tile_start[0][task.y + 1] - g.a0;
    g.b0 = J.tile_start[1][task.z];
    g.nB = J.tile_start[1][task.z + 1] - g.b0;
    g.c0 = J.tile_start[2][task.w];
    g.nC = J.tile_start[2][task.w + 1] - g.c0;
    return g;
}

__device__ __forceinline__ void load_points(float4* P, const DevJob& J, const TaskGeom& g) {
    for (int t = threadIdx.x; t < 3 * TILE; t += blockDim.x) {
        int role = t / TILE, idx = t % TILE;
        int n = role == 0 ? g.nA : (role == 1 ? g.nB : g.nC);
        int base = role == 0 ? g.a0 : (role == 1 ? g.b0 : g.c0);
        P[t] = idx < n ? J.pts[role][base + idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__device__ __forceinline__ int pkey(float4 p) { return __float_as_int(p.w); }

// Queued candidate triangle of the current i: j (bits 0-5), k (bits 6-11) and
// its weight (bits 12-13).

// Runs the full binning path on n (<= 64) queued candidates, two per lane
// (packed into the f32x2 instructions of one binning path).
template <bool THETA_FULL, bool JBJ>
__device__ __forceinline__ void run_candidates(const uint32_t* cand, int n, const int2* row_ij, const int2* row_ik,
                                               const float* JKd, const short* JKw, const TriParams& p, unsigned int* Hw,
                                               RecheckQueue& q, uint32_t slot, uint32_t ia, int b0, int c0) {
    const int lane = threadIdx.x & 31;
    const uint32_t e0 = lane < n ? cand[lane] : 0u;
    const uint32_t e1 = lane + 32 < n ? cand[lane + 32] : 0u;
    const int j0 = e0 & 63, k0 = (e0 >> 6) & 63, j1 = e1 & 63, k1 = (e1 >> 6) & 63;
    const unsigned w0 = e0 >> 12, w1 = e1 >> 12;
    const int2 ij0 = row_ij[j0], ik0 = row_ik[k0];
    const int2 ij1 = row_ij[j1], ik1 = row_ik[k1];
    const float fa[2] = {__int_as_float(ij0.x), __int_as_float(ij1.x)};
    const float fb[2] = {__int_as_float(ik0.x), __int_as_float(ik1.x)};
    const float fc[2] = {JKd[j0 * TILE + k0], JKd[j1 * TILE + k1]};
    const int wa[2] = {ij0.y, ij1.y}, wb[2] = {ik0.y, ik1.y};
    const int wc[2] = {JKw[j0 * TILE + k0], JKw[j1 * TILE + k1]};
    const unsigned ww[2] = {w0, w1};
    if (JBJ) {
        jbj_full2(fa, wa, fb, wb, fc, wc, ww, p, Hw);
        return;
    }
    bool guard[2];
    triangle_full2<THETA_FULL>(fa, wa, fb, wb, fc, wc, ww, p, Hw, guard);
    const bool g0 = guard[0], g1 = guard[1];
    if (g0) push_recheck(q, slot, w0, ia, (uint32_t)(b0 + j0), (uint32_t)(c0 + k0));
    if (g1) push_recheck(q, slot, w1, ia, (uint32_t)(b0 + j1), (uint32_t)(c0 + k1));
}

// Side class for candidate filtering: 0 none (zero length or too long),
// 1 below s_lo, 2 in the s range, 3 above s_hi but below s_hi*q_hi, 4 from
// s_hi*q_hi up to the largest side a counted triangle can have.
__device__ __forceinline__ int side_class(int word, float d, const TriParams& p) {
    const int w = word & 127;
    if (w >= CW_REJECT) return 0;
    if (w == CW_BELOW) return 1;
    if (w == CW_IN) return 2;
    return d < p.mid_hi ? 3 : 4;
}

__device__ __forceinline__ unsigned long long ballot64(bool lo, bool hi) {
    return (unsigned long long)__ballot_sync(0xffffffffu, lo) | ((unsigned long long)__ballot_sync(0xffffffffu, hi) << 32);
}

// Candidate k's of a pair (i, j) whose side i-j has class cij, from the class
// masks of the sides i-k (n*) and j-k (m*).  A triangle can count only through
// permutation 0/2 (no side below s_lo, one side in the s range, at most one
// side at/above s_hi*q_hi) or permutation 1 (no side at/above s_hi*q_hi, at
// most one below s_lo, at most one in [s_hi, s_hi*q_hi)); these are the
// (class_ik, class_jk) combinations that leave one of the two possible.
__device__ __forceinline__ unsigned long long candidate_mask(int cij, unsigned long long nB, unsigned long long nI,
                                                             unsigned long long nM, unsigned long long nH,
                                                             unsigned long long mB, unsigned long long mI,
                                                             unsigned long long mM, unsigned long long mH) {
    if (cij == 2) return (nB | nI | nM | nH) & (mB | mI | mM | mH) & ~((nB | nH) & (mB | mH));
    if (cij == 3) return (nI & (mB | mI | mM | mH)) | ((nB | nI | nM | nH) & mI);
    return (nI & (mI | mM)) | (nM & mI);  // cij == 1 or 4
}

// The same for the JBJ parametrization: a triangle can count only if its
// shortest side is in the s range, i.e. no side below s_lo and at least one
// in range.
__device__ __forceinline__ unsigned long long candidate_mask_jbj(int cij, unsigned long long nI, unsigned long long nM,
                                                                 unsigned long long nH, unsigned long long mI,
                                                                 unsigned long long mM, unsigned long long mH) {
    if (cij == 1) return 0ull;
    if (cij == 2) return (nI | nM | nH) & (mI | mM | mH);
    return (nI & (mI | mM | mH)) | ((nM | nH) & mI);
}

template <int PRED, bool THETA_FULL, bool JBJ>
__device__ void triangle_group_fast(const DevJob& J, const uint4* __restrict__ gt, int nt, const TriParams& p,
                                    float4* P, float* JKd, short* JKw, int2* IJ, int2* IK, uint32_t* Q,
                                    unsigned long long* JM, float* BX, int4* s_meta, unsigned int* Hw,
                                    RecheckQueue& q, unsigned long long& evaluated, unsigned long long& binned,
                                    int* next_i, const float* abox) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4 *PB = P, *PC = P + TILE, *PA = P + 2 * TILE;
    // every task of the group has the same job and tiles B and C
    const uint4 t0 = gt[0];
    const uint32_t slot = t0.x & TASK_SLOT_MASK;
    const bool diag_jk = t0.x & TASK_DIAG_JK;
    const int tb0 = J.tile_start[1][t0.z], numB = J.tile_start[1][t0.z + 1] - tb0;  // first point, points of B
    const int tc0 = J.tile_start[2][t0.w], numC = J.tile_start[2][t0.w + 1] - tc0;  // ... of C
    // a side that provably reaches lmax is rejected whatever its exact value:
    // points farther than that from a whole tile take no part in the task
    // (the 1e-5 margin covers the rounding of the bound and of the distance)
    const float reach = p.lmax * (1.0f + 1e-5f);
    const float reach2 = reach * reach;
    auto far_from = [&](float4 pt, int role) -> bool {
        const float* bx = BX + role * 12;
        float s2 = 0.f;
        {
            const float lo = fminf(bx[0], bx[6]), hi = fmaxf(bx[3], bx[9]);
            const float gap = fmaxf(0.f, fmaxf(lo - pt.x, pt.x - hi));
            s2 = fmaf(gap, gap, s2);
        }
        {
            const float lo = fminf(bx[1], bx[7]), hi = fmaxf(bx[4], bx[10]);
            const float gap = fmaxf(0.f, fmaxf(lo - pt.y, pt.y - hi));
            s2 = fmaf(gap, gap, s2);
        }
        {
            const float lo = fminf(bx[2], bx[8]), hi = fmaxf(bx[5], bx[11]);
            const float gap = fmaxf(0.f, fmaxf(lo - pt.z, pt.z - hi));
            s2 = fmaf(gap, gap, s2);
        }
        return s2 >= reach2;
    };
    int2* row_ij = IJ + warp * TILE;
    int2* row_ik = IK + warp * TILE;
    uint32_t* cand = Q + warp * TRI_QCAP;
    int key_k0 = 0, key_k1 = 0;
    unsigned ev = 0, bn = 0;
    for (int ch = 0; ch < nt; ch += TRI_GROUP_A) {
        const int nr = min(TRI_GROUP_A, nt - ch);
        if (ch > 0) __syncthreads();  // the previous chunk's i loops are done with its A tiles
        // tiles B and C (first chunk) and the chunk's A tiles; A tile r of
        // the chunk at PA + r * TILE
        for (int tt = (ch == 0 ? 0 : 2 * TILE) + threadIdx.x; tt < (2 + nr) * TILE; tt += blockDim.x) {
            const int idx = tt % TILE;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (tt < TILE) {
                if (idx < numB) v = J.pts[1][tb0 + idx];
            } else if (tt < 2 * TILE) {
                if (idx < numC) v = J.pts[2][tc0 + idx];
            } else {
                const uint32_t at = gt[ch + tt / TILE - 2].y;
                const int a0 = J.tile_start[0][at];
                if (idx < J.tile_start[0][at + 1] - a0) v = J.pts[0][a0 + idx];
            }
            P[tt] = v;
        }
        if (threadIdx.x < nr) {
            const uint4 t = gt[ch + threadIdx.x];
            const int a0 = J.tile_start[0][t.y];
            s_meta[threadIdx.x] = make_int4(a0, J.tile_start[0][t.y + 1] - a0, (int)t.x, 0);
        }
        if (threadIdx.x == 0) *next_i = 0;
        __syncthreads();
        if (ch == 0) {
            // bounding boxes of tiles B and C (two 32-point halves each), for
            // the points of A out of reach of a whole tile
            if (warp >= 2 && warp < 6) {
                const int role = warp >> 1, idx = (warp & 1) * 32 + lane;
                const int n = role == 1 ? numB : numC;
                const float4 pt = P[(role - 1) * TILE + idx];
                const bool valid = idx < n;
                float lo[3] = {valid ? pt.x : INFINITY, valid ? pt.y : INFINITY, valid ? pt.z : INFINITY};
                float hi[3] = {valid ? pt.x : -INFINITY, valid ? pt.y : -INFINITY, valid ? pt.z : -INFINITY};
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
                        hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
                    }
                if (lane == 0) {
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        BX[warp * 6 + a] = lo[a];
                        BX[warp * 6 + 3 + a] = hi[a];
                    }
                }
            }
            key_k0 = pkey(PC[lane]);
            key_k1 = pkey(PC[lane + 32]);
            // rows j of the j-k side table and their class masks, one warp per row;
            // abox: the box of every A tile of the group
            for (int j = warp; j < numB; j += TRI_WARPS) {
                const float4 pj = PB[j];
                float a2 = 0.f;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const float v = a == 0 ? pj.x : (a == 1 ? pj.y : pj.z);
                    const float gap = fmaxf(0.f, fmaxf(abox[a] - v, v - abox[3 + a]));
                    a2 = fmaf(gap, gap, a2);
                }
                if (a2 >= reach2) {  // no i of the group reaches j: empty masks, the row is never read
                    if (lane < JM_WORDS) JM[lane * TILE + j] = 0ull;
                    continue;
                }
                int c0 = 0, c1 = 0;
                if (lane < numC) {
                    float d = ref_dist<false>(pj, PC[lane]);
                    int w = tri_side_word(d, p);
                    JKd[j * TILE + lane] = d;
                    JKw[j * TILE + lane] = (short)w;
                    c0 = side_class(w, d, p);
                }
                if (lane + 32 < numC) {
                    float d = ref_dist<false>(pj, PC[lane + 32]);
                    int w = tri_side_word(d, p);
                    JKd[j * TILE + lane + 32] = d;
                    JKw[j * TILE + lane + 32] = (short)w;
                    c1 = side_class(w, d, p);
                }
                JMasks m;
#pragma unroll
                for (int c = 0; c < 4; c++) m.c[c] = ballot64(c0 == c + 1, c1 == c + 1);
                const int kj = pkey(pj);
                m.kge = ballot64(lane < numC && key_k0 >= kj, lane + 32 < numC && key_k1 >= kj);
                if (lane == 0) {
#pragma unroll
                    for (int c = 0; c < 4; c++) JM[c * TILE + j] = m.c[c];
                    JM[4 * TILE + j] = m.kge;
                }
            }
            __syncthreads();
        }
        for (;;) {
            // points of the chunk's A tiles are handed out to warps
            // dynamically (balances the very uneven work per point)
            int ii = 0;
            if (lane == 0) ii = atomicAdd(next_i, 1);
            ii = __shfl_sync(0xffffffffu, ii, 0);
            if (ii >= nr * TILE) break;
            const int4 meta = s_meta[ii / TILE];  // first point, points, task flags
            const int i = ii % TILE;
            if (i >= meta.y) continue;
            const bool diag_ij = meta.z & TASK_DIAG_IJ;
            const bool chk_b = meta.z & TASK_CHECK_B, chk_c = meta.z & TASK_CHECK_C;
            const float4 pi = PA[ii];
            if ((chk_b && far_from(pi, 1)) || (chk_c && far_from(pi, 2))) continue;
            const int ki = pkey(pi);
            // i-k sides: words for the binning path, class masks for the filter
            int c0 = 0, c1 = 0;
            if (lane < numC) {
                float d = ref_dist<false>(pi, PC[lane]);
                int w = tri_side_word(d, p);
                row_ik[lane] = make_int2(__float_as_int(d), w);
                c0 = side_class(w, d, p);
            }
            if (lane + 32 < numC) {
                float d = ref_dist<false>(pi, PC[lane + 32]);
                int w = tri_side_word(d, p);
                row_ik[lane + 32] = make_int2(__float_as_int(d), w);
                c1 = side_class(w, d, p);
            }
            const unsigned long long nB = ballot64(c0 == 1, c1 == 1), nI = ballot64(c0 == 2, c1 == 2);
            const unsigned long long nM = ballot64(c0 == 3, c1 == 3), nH = ballot64(c0 == 4, c1 == 4);
            const unsigned long long any_k = nB | nI | nM | nH;
            if (!any_k) continue;  // no k within reach of i (warp-uniform)
            unsigned long long kge_i = 0;  // PRED_DDR: key_k >= key_i; PRED_RDD: key_k <= key_i
            if (PRED == PRED_DDR) kge_i = ballot64(lane < numC && key_k0 >= ki, lane + 32 < numC && key_k1 >= ki);
            if (PRED == PRED_RDD) kge_i = ballot64(lane < numC && key_k0 <= ki, lane + 32 < numC && key_k1 <= ki);
            // i-j sides: words for the binning path; each lane then forms the
            // candidate-k mask of its own two j's (the scan over j is lane-parallel)
            // mask of candidate k's (and of weight-2 k's) of the pair (i, j)
            auto scan_j = [&](int j, unsigned long long& cm, unsigned long long& w2) -> bool {
                cm = 0;
                w2 = 0;
                if (j >= numB) return false;
                float d = ref_dist<false>(pi, PB[j]);
                int w = tri_side_word(d, p);
                row_ij[j] = make_int2(__float_as_int(d), w);
                const int c = side_class(w, d, p);
                bool ok = c != 0 && any_k && (!diag_ij || j > i);
                if (PRED == PRED_SAME) ok = ok && ki <= pkey(PB[j]);
                if (!ok) return false;
                cm = JBJ ? candidate_mask_jbj(c, nI, nM, nH, JM[TILE + j], JM[2 * TILE + j], JM[3 * TILE + j])
                         : candidate_mask(c, nB, nI, nM, nH, JM[j], JM[TILE + j], JM[2 * TILE + j], JM[3 * TILE + j]);
                if (diag_jk) cm &= j >= 63 ? 0ull : (~0ull << (j + 1));
                if (PRED == PRED_RDD) {
                    // weight [key_j <= key_i] + [key_k <= key_i]
                    if (pkey(PB[j]) <= ki) {
                        w2 = cm & kge_i;
                    } else {
                        cm &= kge_i;
                    }
                } else if (PRED != PRED_NONE) {
                    const unsigned long long kge_j = JM[4 * TILE + j];
                    if (PRED == PRED_DDR) {
                        w2 = cm & kge_i & kge_j;  // weight 2: k >= i and k >= j
                        cm &= kge_i | kge_j;      // weight 0 otherwise
                    } else {
                        cm &= kge_j;              // key_j <= key_k
                    }
                }
                return true;
            };
            unsigned long long cm0, w20, cm1, w21;
            const bool ok0 = scan_j(lane, cm0, w20);
            const bool ok1 = scan_j(lane + 32, cm1, w21);
            // walked (i, j, k): every k with a usable i-k side, for every usable j
            ev += (unsigned)__popcll(any_k) *
                  (unsigned)(__popc(__ballot_sync(0xffffffffu, ok0)) + __popc(__ballot_sync(0xffffffffu, ok1)));
            __syncwarp();
            const uint32_t ia = (uint32_t)(meta.x + i);
            // Candidates of this i: every j with a non-empty mask in turn, expanded
            // by the whole warp (lanes over k), queued and binned 64 at a time.
            // (A lane-parallel compaction of the j's with few candidates, through
            // a prefix sum of per-lane counts, measured slower on clustered data:
            // its scattered j/k break the conflict-free table reads of binning.)
            const unsigned lbit = 1u << lane, lt = lbit - 1u;
            // queue entries of this lane's k = lane and k = lane + 32 (weight 1;
            // plus j and the weight bit of two-array jobs)
            const uint32_t klo = ((uint32_t)lane << 6) | (1u << 12), khi = ((uint32_t)(lane + 32) << 6) | (1u << 12);
            int qn = 0;  // queued candidates (warp-uniform)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                unsigned live = __ballot_sync(0xffffffffu, (h ? cm1 : cm0) != 0ull);
                const unsigned long long cmv = h ? cm1 : cm0, w2v = h ? w21 : w20;
                while (live) {
                    const int src = __ffs(live) - 1;
                    live &= live - 1u;
                    const uint32_t j = (uint32_t)(src + 32 * h);
                    const unsigned lo = __shfl_sync(0xffffffffu, (unsigned)cmv, src);
                    const unsigned hi = __shfl_sync(0xffffffffu, (unsigned)(cmv >> 32), src);
                    uint32_t vlo = klo + j, vhi = khi + j;
                    if (PRED == PRED_DDR || PRED == PRED_RDD) {
                        const unsigned w2lo = __shfl_sync(0xffffffffu, (unsigned)w2v, src);
                        const unsigned w2hi = __shfl_sync(0xffffffffu, (unsigned)(w2v >> 32), src);
                        vlo += (w2lo & lbit) ? (1u << 12) : 0u;
                        vhi += (w2hi & lbit) ? (1u << 12) : 0u;
                    }
                    const int nlo = __popc(lo);
                    if (lo & lbit) cand[qn + __popc(lo & lt)] = vlo;
                    if (hi & lbit) cand[qn + nlo + __popc(hi & lt)] = vhi;
                    qn += nlo + __popc(hi);
                    if (qn >= 64) {
                        __syncwarp();
                        qn -= 64;
                        run_candidates<THETA_FULL, JBJ>(cand + qn, 64, row_ij, row_ik, JKd, JKw, p, Hw, q, slot, ia, tb0, tc0);
                        bn += 64;
                        __syncwarp();
                    }
                }
            }
            __syncwarp();
            if (qn > 0) {
                run_candidates<THETA_FULL, JBJ>(cand, qn, row_ij, row_ik, JKd, JKw, p, Hw, q, slot, ia, tb0, tc0);
                bn += qn;
            }
            __syncwarp();
        }
    }
    // (per-warp totals into the CTA's counters: no 64-bit accumulators live
    // in registers across the kernel)
    if (lane == 0) {
        atomicAdd(&evaluated, (unsigned long long)ev);
        atomicAdd(&binned, (unsigned long long)bn);
    }
}

template <bool THETA_FULL, bool JBJ>
__device__ __forceinline__ void triangle_dispatch(const DevJob& J, const uint4* gt, int nt, const TriParams& p,
                                                  float4* P, float* JKd, short* JKw, int2* IJ, int2* IK, uint32_t* Q,
                                                  unsigned long long* JM, float* BX, int4* s_meta, unsigned int* Hw,
                                                  RecheckQueue& q, unsigned long long& ev, unsigned long long& bn,
                                                  int* next_i, const float* abox) {
#define TRI_GROUP_ARGS J, gt, nt, p, P, JKd, JKw, IJ, IK, Q, JM, BX, s_meta, Hw, q, ev, bn, next_i, abox
    switch ((gt[0].x >> TASK_PRED_SHIFT) & TASK_PRED_MASK) {
        case PRED_NONE: triangle_group_fast<PRED_NONE, THETA_FULL, JBJ>(TRI_GROUP_ARGS); break;
        case PRED_DDR: triangle_group_fast<PRED_DDR, THETA_FULL, JBJ>(TRI_GROUP_ARGS); break;
        case PRED_RDD: triangle_group_fast<PRED_RDD, THETA_FULL, JBJ>(TRI_GROUP_ARGS); break;
        case PRED_SAME: triangle_group_fast<PRED_SAME, THETA_FULL, JBJ>(TRI_GROUP_ARGS); break;
        default: triangle_group_fast<PRED_ONE, THETA_FULL, JBJ>(TRI_GROUP_ARGS); break;
    }
#undef TRI_GROUP_ARGS
}

#ifndef TRI_MIN_BLOCKS
#define TRI_MIN_BLOCKS 4
#endif
// Persistent over groups of tasks: group g is tasks [groups[g], groups[g+1]),
// which share the job, tile B and tile C; gbox[6 g ..] is the box (lo, hi) of
// all their A tiles.
template <bool THETA_FULL, bool JBJ>
__global__ void __launch_bounds__(TRI_THREADS, TRI_MIN_BLOCKS)
triangle_fast_kernel(const DevJob* __restrict__ jobs, const uint4* __restrict__ tasks, const uint32_t* __restrict__ groups,
                     const float* __restrict__ gbox, unsigned int ngroups, unsigned int* group_counter, TriParams p,
                     RecheckQueue q, int copies) {
    extern __shared__ __align__(16) unsigned char smem[];
    float4* P = reinterpret_cast<float4*>(smem);
    unsigned long long* JM = reinterpret_cast<unsigned long long*>(P + (2 + TRI_GROUP_A) * TILE);
    int2* IJ = reinterpret_cast<int2*>(JM + JM_WORDS * TILE);
    int2* IK = IJ + TRI_WARPS * TILE;
    float* JKd = reinterpret_cast<float*>(IK + TRI_WARPS * TILE);
    uint32_t* Q = reinterpret_cast<uint32_t*>(JKd + TILE * TILE);
    short* JKw = reinterpret_cast<short*>(Q + TRI_WARPS * TRI_QCAP);
    unsigned int* H = reinterpret_cast<unsigned int*>(JKw + TILE * TILE);
    __shared__ unsigned int s_group;
    __shared__ int s_next_i;
    __shared__ float s_box[6 * 6];  // tile bounding boxes: 6 half-tiles x {lo, hi}
    __shared__ float s_abox[6];
    __shared__ int4 s_meta[TRI_GROUP_A];  // A tiles of the chunk: first point, points, task flags
    for (int b = threadIdx.x; b < copies * p.len; b += blockDim.x) H[b] = 0;
    unsigned int* Hw = H + ((threadIdx.x >> 5) % copies) * p.len;
    int cur = -1;
    unsigned int since = 0;
    __shared__ unsigned long long ev, bn;  // triangles walked and binned by this CTA
    if (threadIdx.x == 0) ev = bn = 0;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_group = atomicAdd(group_counter, 1u);
        __syncthreads();
        const unsigned int gi = s_group;
        if (gi >= ngroups) break;
        if (threadIdx.x < 6) s_abox[threadIdx.x] = gbox[6 * (size_t)gi + threadIdx.x];
        const uint32_t t0 = groups[gi], t1 = groups[gi + 1];
        const int slot = (int)(tasks[t0].x & TASK_SLOT_MASK);
        // (groups hold at most MAX_GROUP_TASKS <= FLUSH_EVERY tasks)
        if ((slot != cur || since + (t1 - t0) > FLUSH_EVERY) && cur >= 0) {
            flush_hist(H, copies, p.len, jobs[cur].hist);
            since = 0;
        }
        cur = slot;
        since += t1 - t0;
        triangle_dispatch<THETA_FULL, JBJ>(jobs[slot], tasks + t0, (int)(t1 - t0), p, P, JKd, JKw, IJ, IK, Q, JM,
                                           s_box, s_meta, Hw, q, ev, bn, &s_next_i, s_abox);
    }
    if (cur >= 0) flush_hist(H, copies, p.len, jobs[cur].hist);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (ev) atomicAdd(q.evaluated, ev);
        if (bn) atomicAdd(q.evaluated + 1, bn);
    }
}

// Exact recomputation of queued guard-band triangles.
__global__ void triangle_recheck_kernel(const DevJob* __restrict__ jobs, RecheckQueue q, TriParams p, AcosTable t) {
    unsigned int n = *q.count;
    if (n > q.cap) n = q.cap;
    for (unsigned int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        uint4 it = q.items[e];
        const DevJob& J = jobs[it.x & TASK_SLOT_MASK];
        unsigned w = it.x >> RECHECK_WEIGHT_SHIFT;
        float4 pa = J.pts[0][it.y], pb = J.pts[1][it.z], pc = J.pts[2][it.w];
        int out[3];
        tp_exact<false>(ref_dist<false>(pa, pb), ref_dist<false>(pa, pc), ref_dist<false>(pb, pc), p, t, out);
        for (int k = 0; k < 3; k++)
            if (out[k] >= 0) atomicAdd(J.hist + out[k], (unsigned long long)w);
    }
}

// ---------------------------------------------------------------------------
// Triangle parametrization, plain FP64: every triangle through the exact
// reference arithmetic with each float operation done in FP64.

// JBJ shape parametrization (src/3pcf_C_version_triangle_parametrization_JBJ.cc
// distance(), :116-229): one permutation, s = shortest, q = shortest/middle,
// theta = (longest - middle)/shortest, in float, binned like the triangle
// program; -1 if not counted (zero side, out of range, past the array).
__device__ __forceinline__ int jbj_index(float dist0, float dist1, float dist2, const TriParams& p) {
    float shortest, middle, longest;
    if (dist0 > dist1) {
        if (dist0 > dist2) {
            longest = dist0;
            if (dist1 > dist2) { middle = dist1; shortest = dist2; }
            else { middle = dist2; shortest = dist1; }
        } else {
            middle = dist0;
            if (dist1 > dist2) { longest = dist1; shortest = dist2; }
            else { longest = dist2; shortest = dist1; }
        }
    } else {
        if (dist1 > dist2) {
            longest = dist1;
            if (dist0 > dist2) { middle = dist0; shortest = dist2; }
            else { middle = dist2; shortest = dist0; }
        } else {
            middle = dist1; longest = dist2; shortest = dist0;
        }
    }
    if (dist0 == 0.f || dist1 == 0.f || dist2 == 0.f) return -1;
    const float q = __fdiv_rn(shortest, middle);
    const float th = __fdiv_rn(__fsub_rn(longest, middle), shortest);
    const int i0 = ref_bin_tp<false>(shortest, p.s_lo, p.s_hi, p.S, p.nan_zero);
    const int i1 = ref_bin_tp<false>(q, p.q_lo, p.q_hi, p.Q, p.nan_zero);
    const int i2 = ref_bin_tp<false>(th, p.t_lo, p.t_hi, p.T, p.nan_zero);
    if (i0 < 0 || i1 < 0 || i2 < 0) return -1;
    const long long idx = (long long)p.Q * p.T * i0 + (long long)p.T * i1 + i2;
    return idx < p.len ? (int)idx : -1;
}

// Arithmetic of the exact per-triangle kernel.
enum ExactMode : int {
    MODE_FP64 = 0,  // the reference's float arithmetic done in FP64 (identical histograms)
    MODE_GEOM = 1,  // the FP64-geometry truth (tp_geom)
    MODE_JBJ = 2    // the JBJ parametrization in the reference's float arithmetic
};

template <int MODE> struct SideReal { typedef float type; };
template <> struct SideReal<MODE_GEOM> { typedef double type; };

template <int MODE>
__device__ __forceinline__ typename SideReal<MODE>::type side_fp64(float4 a, float4 b) {
    if constexpr (MODE == MODE_GEOM) return geo_dist(a, b);
    else if constexpr (MODE == MODE_JBJ) return ref_dist<false>(a, b);
    else return ref_dist<true>(a, b);
}

template <int PRED, int MODE>
__device__ void triangle_task_fp64(const DevJob& J, uint4 task, const TriParams& p, const AcosTable& t,
                                   float4* P, int2* JK, int2* IJ, unsigned int* Hw) {
    typedef typename SideReal<MODE>::type R;  // at most 8 bytes: fits the int2 slots
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const TaskGeom g = task_geom(J, task);
    const bool diag_ij = task.x & TASK_DIAG_IJ, diag_jk = task.x & TASK_DIAG_JK;
    R* jk = reinterpret_cast<R*>(JK);
    load_points(P, J, g);
    __syncthreads();
    for (int e = threadIdx.x; e < TILE * TILE; e += blockDim.x) {
        int j = e / TILE, k = e % TILE;
        if (j < g.nB && k < g.nC) jk[e] = side_fp64<MODE>(P[TILE + j], P[2 * TILE + k]);
    }
    __syncthreads();
    R* row = reinterpret_cast<R*>(IJ + warp * TILE);
    for (int i = warp; i < g.nA; i += TRI_WARPS) {
        const float4 pi = P[i];
        R dik[2];
#pragma unroll
        for (int r = 0; r < 2; r++) {
            int k = lane + 32 * r;
            dik[r] = k < g.nC ? side_fp64<MODE>(pi, P[2 * TILE + k]) : (R)0;
            if (k < g.nB) row[k] = side_fp64<MODE>(pi, P[TILE + k]);
        }
        __syncwarp();
        const int ki = pkey(pi);
        for (int j = diag_ij ? i + 1 : 0; j < g.nB; j++) {
            const R dij = row[j];
            const int kj = pkey(P[TILE + j]);
            if (PRED == PRED_SAME && !(ki <= kj)) continue;
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int k = lane + 32 * r;
                if (k >= g.nC || (diag_jk && k <= j)) continue;
                unsigned w = 1u;
                const int kkey = pkey(P[2 * TILE + k]);
                if (PRED == PRED_DDR) w = (unsigned)(kkey >= ki) + (unsigned)(kkey >= kj);
                if (PRED == PRED_SAME || PRED == PRED_ONE) w = kj <= kkey ? 1u : 0u;
                if (!w) continue;
                if constexpr (MODE == MODE_JBJ) {
                    const int b = jbj_index(dij, dik[r], jk[j * TILE + k], p);
                    if (b >= 0) atomicAdd(Hw + b, w);
                    continue;
                }
                int out[3];
                if constexpr (MODE == MODE_GEOM) tp_geom(dij, dik[r], jk[j * TILE + k], p, out);
                else tp_exact<true>(dij, dik[r], jk[j * TILE + k], p, t, out);
                for (int b = 0; b < 3; b++)
                    if (out[b] >= 0) atomicAdd(Hw + out[b], w);
            }
        }
        __syncwarp();
    }
}

template <int MODE>
__global__ void __launch_bounds__(TRI_THREADS, 1)
triangle_fp64_kernel(const DevJob* __restrict__ jobs, const uint4* __restrict__ tasks, unsigned int ntasks,
                     unsigned int* task_counter, TriParams p, AcosTable t, int copies) {
    extern __shared__ __align__(16) unsigned char smem[];
    float4* P = reinterpret_cast<float4*>(smem);
    int2* JK = reinterpret_cast<int2*>(smem + 3 * TILE * sizeof(float4));
    int2* IJ = JK + TILE * TILE;
    unsigned int* H = reinterpret_cast<unsigned int*>(IJ + TRI_WARPS * TILE);
    __shared__ uint4 s_task;
    for (int b = threadIdx.x; b < copies * p.len; b += blockDim.x) H[b] = 0;
    unsigned int* Hw = H + ((threadIdx.x >> 5) % copies) * p.len;
    int cur = -1;
    unsigned int since = 0;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int tt = atomicAdd(task_counter, 1u);
            s_task = tt < ntasks ? tasks[tt] : make_uint4(TASK_NONE, 0, 0, 0);
        }
        __syncthreads();
        const uint4 task = s_task;
        const int slot = task.x == TASK_NONE ? -1 : (int)(task.x & TASK_SLOT_MASK);
        if ((slot != cur || since >= FLUSH_EVERY) && cur >= 0) {
            flush_hist(H, copies, p.len, jobs[cur].hist);
            since = 0;
        }
        cur = slot;
        if (slot < 0) break;
        since++;
        const DevJob& J = jobs[slot];
        switch ((task.x >> TASK_PRED_SHIFT) & TASK_PRED_MASK) {
            case PRED_NONE: triangle_task_fp64<PRED_NONE, MODE>(J, task, p, t, P, JK, IJ, Hw); break;
            case PRED_DDR: triangle_task_fp64<PRED_DDR, MODE>(J, task, p, t, P, JK, IJ, Hw); break;
            case PRED_SAME: triangle_task_fp64<PRED_SAME, MODE>(J, task, p, t, P, JK, IJ, Hw); break;
            default: triangle_task_fp64<PRED_ONE, MODE>(J, task, p, t, P, JK, IJ, Hw); break;
        }
    }
}

// ---------------------------------------------------------------------------
// Three-side histogram (src/3pcf_C_version.cc): every ordered triple, sides in
// source order d01 -> i0, d02 -> i1, d12 -> i2, index n^2 i2 + n i1 + i0.

constexpr int TS_WARPS = 8;  // warps per CTA, or per group of the grouped kernel
constexpr int TS_GROUP_THREADS = TS_WARPS * 32;
constexpr int TS_GROUPS_MAX = 4;
constexpr uint32_t TS_FAR = 1u << 30;
// A copy receives at most 64^3 = 2^18 counts per task, so 8192 tasks keep
// every 32-bit shared counter below 2^31.
constexpr unsigned int TS_FLUSH_EVERY = 8192;

// Per warp: the i-k and i-j code rows of its point i and a queue of (j, k)
// candidates (up to 31 left over plus 64 from one j).
constexpr int TS_QCAP = 96;
constexpr int TS_ROW = 2 * TILE + TS_QCAP;

// Shared memory of one task pipeline (an 8-warp CTA, or one group of the
// grouped kernel): point tiles, j-k table, per-warp rows, j-k masks, boxes,
// next point.  The j-k table holds 32-bit codes; in clean mode it holds the
// bins alone (only sides below hist_max are ever read), one byte each up to
// 255 bins.
struct TsLayout {
    size_t jk, rows, jkm, box, flags, next, bytes;
};
__host__ __device__ constexpr bool ts_byte_jk(const ThreeParams& p) { return p.clean && p.n <= 255; }
__host__ __device__ constexpr TsLayout ts_layout(bool byte_jk) {
    const size_t jk = 3 * TILE * sizeof(float4);
    const size_t rows = jk + (byte_jk ? TILE * TILE : TILE * TILE * sizeof(uint32_t));
    const size_t jkm = rows + TS_WARPS * TS_ROW * sizeof(uint32_t);
    const size_t box = jkm + TILE * sizeof(unsigned long long);
    const size_t flags = box + 36 * sizeof(float);  // reach flags of the points of tiles B and A
    const size_t next = flags + 2 * TILE;
    return TsLayout{jk, rows, jkm, box, flags, next, (next + sizeof(int) + 127) & ~(size_t)127};
}

// distance_to_bin of src/3pcf_C_version.cc:23-51, times 'scale'; sides at or
// above hist_max give nbins+1 (reference) or, in clean mode, a value that
// pushes every derived index out of range.
template <bool FP64>
__device__ __forceinline__ uint32_t side_code3(float d, const ThreeParams& p, uint32_t scale) {
    typedef FOps<FP64> F;
    if (d < p.lo) return 0u;
    if (d >= p.hi) return p.clean ? TS_FAR : (uint32_t)(p.n + 1) * scale;
    return (uint32_t)__float2int_rz(F::div(F::sub(d, p.lo), p.bw)) * scale;
}

// Three-side code of the side a-b.  The guarded FP32 kernel skips the square
// root and the division: the bin is a non-decreasing step function of the
// squared length, so a first guess from an approximate square root (within one
// bin) is corrected against the exact thresholds U of the two neighbouring
// steps.  The plain FP64 kernel evaluates the reference's formula.
template <bool FP64>
__device__ __forceinline__ uint32_t side_code3_pts(float4 a, float4 b, const ThreeParams& p, const float* U,
                                                   uint32_t scale) {
    if (!FP64 && p.fast) {
        const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
        float d2 = __fmul_rn(dx, dx);
        d2 = __fadd_rn(d2, __fmul_rn(dy, dy));
        d2 = __fadd_rn(d2, __fmul_rn(dz, dz));
        float da;
        asm("sqrt.approx.f32 %0, %1;" : "=f"(da) : "f"(d2));
        // the guess rounds to nearest: where d reaches hi the code jumps over
        // nbins (unless rounding gives bin nbins), and a truncated guess just
        // below hi would be two steps short
        int v = __float2int_rn(__fmul_rn(__fsub_rn(da, p.lo), p.inv_bw));
        v = min(max(v, 0), p.n + 1);
        v = v - 1 + (d2 >= U[v] ? 1 : 0) + (d2 >= U[v + 1] ? 1 : 0);
        if (v > p.n) return p.clean ? TS_FAR : (uint32_t)(p.n + 1) * scale;
        return (uint32_t)v * scale;
    }
    return side_code3<FP64>(ref_dist<FP64>(a, b), p, scale);
}

// Symmetric three-side tasks (one catalog in all roles) visit each multiset
// {i <= j <= k} once.  With a shared histogram they count it once in a
// multiset accumulator (m = nbins + 2 codes per side, so no index aliases):
//   U[v_jk m^2 + v_ik m + v_ij]   three distinct points,
//   U2[v]                         two equal indices (sides 0, v, v),
//   U6                            i == j == k,
// which ts_flush expands into the reference's ordered histogram.  The
// accumulator is ts_acc_words(p) words, U2 from word ts_u2(p).
__host__ __device__ inline int ts_u2(const ThreeParams& p) {
    const int m = p.n + 2;
    return hist_stride(m * m * m);
}
__host__ __device__ inline int ts_acc_words(const ThreeParams& p) {
    const int acc = ts_u2(p) + p.n + 3;
    return acc > p.len ? acc : p.len;
}

// Adds one ordering (sides d01, d02, d12 with codes x0, x1, x2) of a triple
// to the reference's histogram (an index at or past its end is dropped).
__device__ __forceinline__ void ts_put(unsigned long long* g, uint32_t x0, uint32_t x1, uint32_t x2,
                                       const ThreeParams& p, unsigned long long u) {
    const uint32_t t = x2 * (uint32_t)p.n * (uint32_t)p.n + x1 * (uint32_t)p.n + x0;
    if (t < (uint32_t)p.len) atomicAdd(g + t, u);
}

// The distinct orderings of a multiset with side codes (v_ij, v_ik, v_jk):
// (i,j,k) (ij,ik,jk), (i,k,j) (ik,ij,jk), (j,i,k) (ij,jk,ik), (j,k,i) (jk,ij,ik),
// (k,i,j) (ik,jk,ij), (k,j,i) (jk,ik,ij); with i == j or j == k three of them.
__device__ __forceinline__ void ts_put_orderings(unsigned long long* g, uint32_t vij, uint32_t vik, uint32_t vjk,
                                                 bool eij, bool ejk, const ThreeParams& p, unsigned long long u) {
    ts_put(g, vij, vik, vjk, p, u);
    if (!ejk) ts_put(g, vik, vij, vjk, p, u);
    if (!eij) ts_put(g, vij, vjk, vik, p, u);
    if (!eij) ts_put(g, vjk, vij, vik, p, u);
    if (!ejk) ts_put(g, vik, vjk, vij, p, u);
    if (!eij && !ejk) ts_put(g, vjk, vik, vij, p, u);
}

// Flushes 'copies' shared copies (hist_stride(ts_acc_words(p)) words apart)
// into the job's 64-bit histogram: the swizzled ordered histogram, or the
// multiset accumulator of a symmetric job expanded into its orderings.
__device__ void ts_flush(unsigned int* H, int copies, const ThreeParams& p, unsigned long long* g, bool sym) {
    const int stride = hist_stride(ts_acc_words(p));
    __syncthreads();
    if (!sym) {
        for (int b = threadIdx.x; b < p.len; b += blockDim.x) {
            const int at = (int)hist_pos((unsigned)b);
            unsigned long long u = 0;
            for (int c = 0; c < copies; c++) {
                u += H[c * stride + at];
                H[c * stride + at] = 0;
            }
            if (u) atomicAdd(g + b, u);
        }
    } else {
        const int m = p.n + 2, m3 = m * m * m, u2 = ts_u2(p);
        const uint32_t z = (uint32_t)p.zcode;
        for (int b = threadIdx.x; b < m3 + m + 1; b += blockDim.x) {
            const int at = b < m3 ? (int)hist_pos((unsigned)b) : u2 + (b - m3);
            unsigned long long u = 0;
            for (int c = 0; c < copies; c++) {
                u += H[c * stride + at];
                H[c * stride + at] = 0;
            }
            if (!u) continue;
            if (b < m3) {
                const uint32_t vij = b % m, vik = (b / m) % m, vjk = b / (m * m);
                ts_put_orderings(g, vij, vik, vjk, false, false, p, u);
            } else if (b < m3 + m) {
                const uint32_t v = b - m3;  // (i, i, k) or (i, k, k): sides 0, v, v
                ts_put(g, z, v, v, p, u);
                ts_put(g, v, z, v, p, u);
                ts_put(g, v, v, z, p, u);
            } else {
                ts_put(g, z, z, z, p, u);
            }
        }
    }
    __syncthreads();
}

// One task pipeline: its threads (tid in [0, 256)), and its barrier (0: the
// CTA's, else a named barrier of its 256 threads).
struct TsPipe {
    int tid, warp, lane, bar;
    __device__ __forceinline__ void sync() const {
        if (bar == 0) __syncthreads();
        else asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(TS_GROUP_THREADS) : "memory");
    }
};

// Bounding boxes of the three tiles (two 32-point halves each) into BX, one
// warp per half; the caller synchronises.
__device__ __forceinline__ void tile_boxes(const float4* P, const TaskGeom& g, float* BX, int warp, int lane) {
    if (warp >= 6) return;
    const int role = warp >> 1, idx = (warp & 1) * 32 + lane;
    const int n = role == 0 ? g.nA : (role == 1 ? g.nB : g.nC);
    const float4 pt = P[role * TILE + idx];
    const bool valid = idx < n;
    float lo[3] = {valid ? pt.x : INFINITY, valid ? pt.y : INFINITY, valid ? pt.z : INFINITY};
    float hi[3] = {valid ? pt.x : -INFINITY, valid ? pt.y : -INFINITY, valid ? pt.z : -INFINITY};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int a = 0; a < 3; a++) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    if (lane == 0) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            BX[warp * 6 + a] = lo[a];
            BX[warp * 6 + 3 + a] = hi[a];
        }
    }
}

// True if every point of half-tile box 'b' (role * 2 + half) is at least
// 'reach' from pt; an empty half (inverted box) is far from everything.
__device__ __forceinline__ bool far_from_box(const float* BX, float4 pt, int b, float reach2) {
    const float* b0 = BX + b * 6;
    const float gx = fmaxf(0.f, fmaxf(b0[0] - pt.x, pt.x - b0[3]));
    const float gy = fmaxf(0.f, fmaxf(b0[1] - pt.y, pt.y - b0[4]));
    const float gz = fmaxf(0.f, fmaxf(b0[2] - pt.z, pt.z - b0[5]));
    return fmaf(gz, gz, fmaf(gy, gy, gx * gx)) >= reach2;
}

// One task (tiles A, B, C) of the three-side histogram on one pipeline whose
// shared memory starts at 'base'; counts go to the shared copy Hw (swizzled)
// or, with GLOBAL_HIST, straight to the job's 64-bit histogram.
template <bool FP64, bool GLOBAL_HIST>
__device__ void three_side_task(const DevJob& J, uint4 task, const ThreeParams& p, const float* U,
                                unsigned char* base, unsigned int* Hw, const TsPipe& pp) {
    float4* P = reinterpret_cast<float4*>(base);
    const bool byte_jk = ts_byte_jk(p);
    const TsLayout L = ts_layout(byte_jk);
    uint8_t* FJ = base + L.flags;  // per j of tile B: 1 reaches tile A, 2 / 4 reaches half 0 / 1 of tile C
    uint8_t* FI = FJ + TILE;       // per i of tile A: 1 / 2 reaches half 0 / 1 of B, 4 / 8 of C
    uint32_t* JK = reinterpret_cast<uint32_t*>(base + L.jk);
    uint8_t* JK8 = base + L.jk;
    uint32_t* ROWS = reinterpret_cast<uint32_t*>(base + L.rows);
    unsigned long long* JKM = reinterpret_cast<unsigned long long*>(base + L.jkm);
    float* BX = reinterpret_cast<float*>(base + L.box);
    int* next_i = reinterpret_cast<int*>(base + L.next);
    const int warp = pp.warp, lane = pp.lane;
    const TaskGeom g = task_geom(J, task);
    const uint32_t n = p.n, n2 = (uint32_t)p.n * p.n, len = (uint32_t)p.len;
    const uint32_t m = n + 2, mm = m * m, u2 = (uint32_t)ts_u2(p);  // multiset accumulator
    // Symmetric tasks (one catalog in all three roles): tiles a <= b <= c and,
    // on diagonal tile pairs, positions i <= j <= k, so that every multiset
    // {i, j, k} is visited once and counted for all its orderings.
    const bool sym = ((task.x >> TASK_PRED_SHIFT) & TASK_PRED_MASK) == PRED_SAME;
    const bool diag_ij = task.x & TASK_DIAG_IJ, diag_jk = task.x & TASK_DIAG_JK;
    for (int t = pp.tid; t < 3 * TILE; t += TS_GROUP_THREADS) {
        const int role = t / TILE, idx = t % TILE;
        const int nr = role == 0 ? g.nA : (role == 1 ? g.nB : g.nC);
        const int b0 = role == 0 ? g.a0 : (role == 1 ? g.b0 : g.c0);
        P[t] = idx < nr ? J.pts[role][b0 + idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (pp.tid == 0) *next_i = 0;
    pp.sync();
    if (p.clean) {
        // Clean mode drops every triple with a side >= hist_max, so a point
        // farther than that from a whole tile takes no part in the task (the
        // 1e-5 margin covers the rounding of the bound and of the distance).
        // (The planner flags tile pairs A-B and A-C that are not wholly within
        // reach; B-C pairs are checked here on the half-tile boxes.)
        const bool chk_b = task.x & TASK_CHECK_B, chk_c = task.x & TASK_CHECK_C;
        tile_boxes(P, g, BX, warp, lane);
        pp.sync();
        const float reach = p.hi * (1.0f + 1e-5f), reach2 = reach * reach;
        // reach flags of every point against the half-tile boxes, lane-parallel
        if (warp == 0) {
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int j = lane + 32 * r;
                const float4 pj = P[TILE + j];
                unsigned f = 0;
                if (!chk_b || !far_from_box(BX, pj, 0, reach2) || !far_from_box(BX, pj, 1, reach2)) f |= 1u;
                if (!far_from_box(BX, pj, 4, reach2)) f |= 2u;
                if (!far_from_box(BX, pj, 5, reach2)) f |= 4u;
                FJ[j] = (uint8_t)f;
            }
        } else if (warp == 1) {
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int i = lane + 32 * r;
                const float4 pi = P[i];
                unsigned f = 0;
                if (!chk_b || !far_from_box(BX, pi, 2, reach2)) f |= 1u;
                if (!chk_b || !far_from_box(BX, pi, 3, reach2)) f |= 2u;
                if (!chk_c || !far_from_box(BX, pi, 4, reach2)) f |= 4u;
                if (!chk_c || !far_from_box(BX, pi, 5, reach2)) f |= 8u;
                FI[i] = (uint8_t)f;
            }
        }
        pp.sync();
        // j-k codes, one warp per row j, and JKM[j]: the k's whose side is
        // below hist_max (halves of tile C out of reach of j are skipped)
        for (int j = warp; j < g.nB; j += TS_WARPS) {
            const float4 pj = P[TILE + j];
            const unsigned f = FJ[j];
            if (!(f & 1u) || !(f & 6u)) {  // no i, or no k, reaches j: the row is never read
                if (lane == 0) JKM[j] = 0ull;
                continue;
            }
            uint32_t c0 = TS_FAR, c1 = TS_FAR;
            if ((f & 2u) && lane < g.nC) c0 = side_code3_pts<FP64>(pj, P[2 * TILE + lane], p, U, 1u);
            if ((f & 4u) && lane + 32 < g.nC) c1 = side_code3_pts<FP64>(pj, P[2 * TILE + lane + 32], p, U, 1u);
            if (byte_jk) {  // bins <= nbins <= 255 where read
                JK8[j * TILE + lane] = (uint8_t)c0;
                JK8[j * TILE + lane + 32] = (uint8_t)c1;
            } else {
                JK[j * TILE + lane] = c0;
                JK[j * TILE + lane + 32] = c1;
            }
            unsigned long long m = ballot64(c0 < TS_FAR, c1 < TS_FAR);
            if (sym && diag_jk) m &= ~0ull << j;  // k >= j
            if (lane == 0) JKM[j] = m;
        }
        pp.sync();
        uint32_t* row_ik = ROWS + warp * TS_ROW;
        uint32_t* row_ij = row_ik + TILE;
        uint32_t* cq = row_ij + TILE;
        const unsigned lt = (1u << lane) - 1u;
        auto add = [&](uint32_t idx) {
            if (idx < len) {  // a side rounded to bin nbins aliases as in the reference
                if (GLOBAL_HIST) atomicAdd(J.hist + idx, 1ull);
                else atomicAdd(Hw + hist_pos(idx), 1u);
            }
        };
        int i = 0;
        auto count_candidates = [&](const uint32_t* e, int cnt) {
            if (lane < cnt) {
                const uint32_t c = e[lane];
                const int j = c & 63, k = c >> 6;
                const uint32_t vjk = byte_jk ? (uint32_t)JK8[j * TILE + k] : JK[j * TILE + k];
                const uint32_t vik = row_ik[k], vij = row_ij[j];
                if (!sym) {
                    add(vjk * n2 + vik * n + vij);
                } else {
                    const bool eij = diag_ij && i == j, ejk = diag_jk && j == k;
                    if (GLOBAL_HIST) ts_put_orderings(J.hist, vij, vik, vjk, eij, ejk, p, 1ull);
                    else if (!eij && !ejk) atomicAdd(Hw + hist_pos(vjk * mm + vik * m + vij), 1u);
                    else atomicAdd(Hw + u2 + (eij && ejk ? m : (eij ? vik : vij)), 1u);
                }
            }
        };
        for (;;) {
            // points of tile A go to warps one at a time (their work is uneven)
            i = 0;
            if (lane == 0) i = atomicAdd(next_i, 1);
            i = __shfl_sync(0xffffffffu, i, 0);
            if (i >= g.nA) break;
            const float4 pi = P[i];
            const unsigned fi = FI[i];
            if (!(fi & 3u) || !(fi & 12u)) continue;  // out of reach of tile B or tile C (warp-uniform)
            uint32_t cik[2], cij[2];
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int k = lane + 32 * r;
                cik[r] = ((fi >> (2 + r)) & 1u) && k < g.nC ? side_code3_pts<FP64>(pi, P[2 * TILE + k], p, U, 1u)
                                                             : TS_FAR;
            }
            const unsigned long long mk = ballot64(cik[0] < TS_FAR, cik[1] < TS_FAR);
            if (!mk) continue;  // warp-uniform
            // j's with a usable i-j side and a k usable with both i and j
            bool vj[2];
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int j = lane + 32 * r;
                cij[r] = TS_FAR;
                vj[r] = false;
                if (((fi >> r) & 1u) && j < g.nB && (JKM[j] & mk) && !(sym && diag_ij && j < i)) {
                    cij[r] = side_code3_pts<FP64>(pi, P[TILE + j], p, U, 1u);
                    vj[r] = cij[r] < TS_FAR;
                }
            }
            unsigned long long mj = ballot64(vj[0], vj[1]);
            // Candidates (j, k) of this i, every j in turn, queued by the
            // whole warp and counted 32 at a time.
            row_ik[lane] = cik[0];
            row_ik[lane + 32] = cik[1];
            row_ij[lane] = cij[0];
            row_ij[lane + 32] = cij[1];
            int qn = 0;  // warp-uniform
            while (mj) {
                const int j = __ffsll((long long)mj) - 1;
                mj &= mj - 1ull;
                const unsigned long long cm = mk & JKM[j];
                const unsigned lo = (unsigned)cm, hi = (unsigned)(cm >> 32);
                const int nlo = __popc(lo);
                if ((lo >> lane) & 1u) cq[qn + __popc(lo & lt)] = (uint32_t)j | ((uint32_t)lane << 6);
                if ((hi >> lane) & 1u) cq[qn + nlo + __popc(hi & lt)] = (uint32_t)j | ((uint32_t)(lane + 32) << 6);
                qn += nlo + __popc(hi);
                __syncwarp();
                while (qn >= 32) {
                    qn -= 32;
                    count_candidates(cq + qn, 32);
                    __syncwarp();
                }
            }
            if (qn > 0) count_candidates(cq, qn);
            __syncwarp();
        }
        return;
    }
    if (sym) {
        // every multiset {i <= j <= k} of the task (codes 0 .. nbins + 1)
        for (int e = pp.tid; e < TILE * TILE; e += TS_GROUP_THREADS) {
            const int j = e / TILE, k = e % TILE;
            JK[e] = (j < g.nB && k < g.nC) ? side_code3_pts<FP64>(P[TILE + j], P[2 * TILE + k], p, U, 1u) : 0u;
        }
        pp.sync();
        uint32_t* row = ROWS + warp * TS_ROW;
        for (int i = warp; i < g.nA; i += TS_WARPS) {
            const float4 pi = P[i];
            uint32_t vik[2];
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int k = lane + 32 * r;
                vik[r] = k < g.nC ? side_code3_pts<FP64>(pi, P[2 * TILE + k], p, U, 1u) : 0u;
                if (lane + 32 * r < g.nB) row[lane + 32 * r] = side_code3_pts<FP64>(pi, P[TILE + lane + 32 * r], p, U, 1u);
            }
            __syncwarp();
            if (!GLOBAL_HIST && !diag_ij && !diag_jk) {
                // three tiles apart: every (j, k) is a multiset of distinct points
                const uint32_t vikm0 = vik[0] * m, vikm1 = vik[1] * m;
                const bool k0 = lane < g.nC, k1 = lane + 32 < g.nC;
#pragma unroll 4
                for (int j = 0; j < g.nB; j++) {
                    const uint32_t vij = row[j];
                    if (k0) atomicAdd(Hw + hist_pos(JK[j * TILE + lane] * mm + vikm0 + vij), 1u);
                    if (k1) atomicAdd(Hw + hist_pos(JK[j * TILE + lane + 32] * mm + vikm1 + vij), 1u);
                }
                __syncwarp();
                continue;
            }
            for (int j = diag_ij ? i : 0; j < g.nB; j++) {
                const uint32_t vij = row[j];
                const bool eij = diag_ij && j == i;
#pragma unroll
                for (int r = 0; r < 2; r++) {
                    const int k = lane + 32 * r;
                    if (k >= g.nC || (diag_jk && k < j)) continue;
                    const bool ejk = diag_jk && k == j;
                    const uint32_t vjk = JK[j * TILE + k];
                    if (GLOBAL_HIST) ts_put_orderings(J.hist, vij, vik[r], vjk, eij, ejk, p, 1ull);
                    else if (!eij && !ejk) atomicAdd(Hw + hist_pos(vjk * mm + vik[r] * m + vij), 1u);
                    else atomicAdd(Hw + u2 + (eij && ejk ? m : (eij ? vik[r] : vij)), 1u);
                }
            }
            __syncwarp();
        }
        return;
    }
    for (int e = pp.tid; e < TILE * TILE; e += TS_GROUP_THREADS) {
        const int j = e / TILE, k = e % TILE;
        JK[e] = (j < g.nB && k < g.nC) ? side_code3_pts<FP64>(P[TILE + j], P[2 * TILE + k], p, U, n2)
                                       : TS_FAR;
    }
    pp.sync();
    uint32_t* row = ROWS + warp * TS_ROW;
    for (int i = warp; i < g.nA; i += TS_WARPS) {
        const float4 pi = P[i];
        uint32_t cik[2];
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const int k = lane + 32 * r;
            cik[r] = k < g.nC ? side_code3_pts<FP64>(pi, P[2 * TILE + k], p, U, n) : TS_FAR;
        }
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const int k = lane + 32 * r;
            if (k < g.nB) row[k] = side_code3_pts<FP64>(pi, P[TILE + k], p, U, 1u);
        }
        __syncwarp();
#pragma unroll 4
        for (int j = 0; j < g.nB; j++) {
            const uint32_t cij = row[j];
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int k = lane + 32 * r;
                const uint32_t idx = JK[j * TILE + k] + cik[r] + cij;
                if (idx < len) {
                    if (GLOBAL_HIST) atomicAdd(J.hist + idx, 1ull);
                    else atomicAdd(Hw + hist_pos(idx), 1u);
                }
            }
        }
        __syncwarp();
    }
}

// 8-warp CTAs, several per SM: warp-private shared histogram copies (copies
// > 0) or the global histogram.
template <bool FP64, bool GLOBAL_HIST>
__global__ void __launch_bounds__(TS_GROUP_THREADS, 4)
three_side_kernel(const DevJob* __restrict__ jobs, const uint4* __restrict__ tasks, unsigned int ntasks,
                  unsigned int* task_counter, ThreeParams p, int copies) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned int* H = reinterpret_cast<unsigned int*>(smem + ts_layout(ts_byte_jk(p)).bytes);
    __shared__ uint4 s_task;
    __shared__ float s_u[TS_UMAX];
    for (int v = threadIdx.x; v < TS_UMAX; v += blockDim.x) s_u[v] = p.u[v];
    const int stride = hist_stride(ts_acc_words(p));
    if (!GLOBAL_HIST)
        for (int b = threadIdx.x; b < copies * stride; b += blockDim.x) H[b] = 0;
    unsigned int* Hw = H + (GLOBAL_HIST ? 0 : ((threadIdx.x >> 5) % copies) * stride);
    bool cur_sym = false;
    const TsPipe pp{(int)threadIdx.x, (int)(threadIdx.x >> 5), (int)(threadIdx.x & 31), 0};
    int cur = -1;
    unsigned int since = 0;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int t = atomicAdd(task_counter, 1u);
            s_task = t < ntasks ? tasks[t] : make_uint4(TASK_NONE, 0, 0, 0);
        }
        __syncthreads();
        const uint4 task = s_task;
        const int slot = task.x == TASK_NONE ? -1 : (int)(task.x & TASK_SLOT_MASK);
        if (!GLOBAL_HIST && (slot != cur || since >= TS_FLUSH_EVERY) && cur >= 0) {
            ts_flush(H, copies, p, jobs[cur].hist, cur_sym);
            since = 0;
        }
        cur = slot;
        cur_sym = ((task.x >> TASK_PRED_SHIFT) & TASK_PRED_MASK) == PRED_SAME;
        if (slot < 0) break;
        since++;
        three_side_task<FP64, GLOBAL_HIST>(jobs[slot], task, p, s_u, smem, Hw, pp);
    }
}

// One CTA per SM of 'groups' independent 8-warp task pipelines (named
// barriers 1..groups) around one shared histogram too large for several
// CTAs per SM.  A pipeline runs tasks of the current job until it draws a
// task of another job (or none), or the CTA has run TS_FLUSH_EVERY tasks since
// the last flush; then it waits for the others at a CTA barrier, where the
// histogram is flushed and the next current job is the smallest one held.
// Every pipeline reaches that barrier: each runs finitely many tasks of the
// current job.  At most TS_FLUSH_EVERY + groups - 1 tasks are counted between
// two flushes, each at most 2^18 per bin, so the 32-bit counters cannot wrap.
template <bool FP64>
__global__ void __launch_bounds__(TS_GROUPS_MAX * TS_GROUP_THREADS, 1)
three_side_grouped_kernel(const DevJob* __restrict__ jobs, const uint4* __restrict__ tasks, unsigned int ntasks,
                          unsigned int* task_counter, ThreeParams p, int groups) {
    extern __shared__ __align__(16) unsigned char smem[];
    const size_t pipe_bytes = ts_layout(ts_byte_jk(p)).bytes;
    unsigned int* H = reinterpret_cast<unsigned int*>(smem + (size_t)groups * pipe_bytes);
    __shared__ uint4 s_task[TS_GROUPS_MAX];
    __shared__ unsigned int s_stop[TS_GROUPS_MAX];  // the pipeline leaves the job to flush
    __shared__ unsigned int s_since;                // tasks run since the last flush
    __shared__ float s_u[TS_UMAX];
    for (int v = threadIdx.x; v < TS_UMAX; v += blockDim.x) s_u[v] = p.u[v];
    const int gi = threadIdx.x / TS_GROUP_THREADS, gt = threadIdx.x % TS_GROUP_THREADS;
    const TsPipe pp{gt, gt >> 5, gt & 31, 1 + gi};
    unsigned char* base = smem + (size_t)gi * pipe_bytes;
    for (int b = threadIdx.x; b < hist_stride(ts_acc_words(p)); b += blockDim.x) H[b] = 0;
    if (threadIdx.x == 0) s_since = 0;
    auto draw = [&]() {
        if (gt == 0) {
            unsigned int t = atomicAdd(task_counter, 1u);
            s_task[gi] = t < ntasks ? tasks[t] : make_uint4(TASK_NONE, 0, 0, 0);
        }
    };
    draw();
    int cur = -1;
    bool cur_sym = false;
    for (;;) {
        __syncthreads();  // every pipeline waits here with a task of another job, or none
        if (cur >= 0) ts_flush(H, 1, p, jobs[cur].hist, cur_sym);
        uint32_t next = TASK_NONE;
        for (int g2 = 0; g2 < groups; g2++) {
            const uint32_t x = s_task[g2].x;
            if (x != TASK_NONE) next = min(next, x & TASK_SLOT_MASK);
        }
        if (next == TASK_NONE) break;  // uniform: every thread read the same words
        for (int g2 = 0; g2 < groups; g2++) {  // all tasks of a job are alike
            const uint32_t x = s_task[g2].x;
            if (x != TASK_NONE && (x & TASK_SLOT_MASK) == next)
                cur_sym = ((x >> TASK_PRED_SHIFT) & TASK_PRED_MASK) == PRED_SAME;
        }
        if (threadIdx.x < TS_GROUPS_MAX) s_stop[threadIdx.x] = 0;
        if (threadIdx.x == 0) s_since = 0;
        __syncthreads();
        cur = (int)next;
        for (;;) {
            // s_task[gi] and s_stop[gi] change only between this pipeline's barriers
            const uint4 task = s_task[gi];
            if (task.x == TASK_NONE || (int)(task.x & TASK_SLOT_MASK) != cur || s_stop[gi]) break;
            three_side_task<FP64, false>(jobs[cur], task, p, s_u, base, H, pp);
            pp.sync();  // the pipeline is done with s_task[gi] and its buffers
            if (gt == 0) s_stop[gi] = atomicAdd(&s_since, 1u) + 1 >= TS_FLUSH_EVERY;
            draw();
            pp.sync();
        }
    }
}

// ---------------------------------------------------------------------------
// Pair counts (src/2pcf_C_version.cc).  Tasks name a tile of each role (w unused).

constexpr int PR_WARPS = 8;
constexpr int PR_THREADS = PR_WARPS * 32;
constexpr size_t PR_SMEM_FIXED = 2 * TILE * sizeof(float4);

// Pair bin of the separation a-b, -1 if not counted.  The guarded FP32
// kernel works on the squared separation: a first guess from an approximate
// square root (within one step) corrected against the exact thresholds U of
// the neighbouring steps of the code (0 below lo, bin + 1, nbins + 2 at or
// above hi); the plain FP64 kernel evaluates the reference's formula.
template <bool FP64>
__device__ __forceinline__ int pair_bin(float4 a, float4 b, const PairParams& p, const float* U) {
    if (!FP64 && p.fast) {
        const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
        float d2 = __fmul_rn(dx, dx);
        d2 = __fadd_rn(d2, __fmul_rn(dy, dy));
        d2 = __fadd_rn(d2, __fmul_rn(dz, dz));
        float da;
        asm("sqrt.approx.f32 %0, %1;" : "=f"(da) : "f"(d2));
        // rounded guess (as for the three-side codes: the code jumps over
        // nbins + 1 where d reaches hi)
        int v = __float2int_rn(__fmul_rn(__fsub_rn(da, p.lo), p.inv_bw)) + 1;
        v = min(max(v, 0), p.n + 2);
        v = v - 1 + (d2 >= U[v] ? 1 : 0) + (d2 >= U[v + 1] ? 1 : 0);
        return v >= 1 && v <= p.n ? v - 1 : -1;
    }
    const int bn = ref_bin_tp<FP64>(ref_dist<FP64>(a, b), p.lo, p.hi, p.n, 0);
    return bn >= 0 && bn < p.n ? bn : -1;
}

template <bool FP64, int PRED>
__device__ void pair_task(const DevJob& J, uint4 task, const PairParams& p, const float* U, float4* P,
                          unsigned int* Hw) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a0 = J.tile_start[0][task.y], nA = J.tile_start[0][task.y + 1] - a0;
    const int b0 = J.tile_start[1][task.z], nB = J.tile_start[1][task.z + 1] - b0;
    const bool diag = task.x & TASK_DIAG_IJ;
    for (int t = threadIdx.x; t < 2 * TILE; t += blockDim.x) {
        int role = t / TILE, idx = t % TILE;
        int nn = role == 0 ? nA : nB, base = role == 0 ? a0 : b0;
        P[t] = idx < nn ? J.pts[role][base + idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    // each lane keeps its two points of tile B in registers for the whole task
    const float4 pj[2] = {P[TILE + lane], P[TILE + lane + 32]};
    for (int i = warp; i < nA; i += PR_WARPS) {
        const float4 pi = P[i];
        const int ki = pkey(pi);
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const int j = lane + 32 * r;
            if (j >= nB) continue;
            if (diag && j < i) continue;  // self pairs (j == i) are counted, as the reference's j >= i
            if (PRED == PRED_SAME && pkey(pj[r]) < ki) continue;
            const int b = pair_bin<FP64>(pi, pj[r], p, U);
            if (b >= 0) atomicAdd(Hw + b, 1u);
        }
    }
    __syncthreads();
}

template <bool FP64>
__global__ void __launch_bounds__(PR_THREADS)
pair_kernel(const DevJob* __restrict__ jobs, const uint4* __restrict__ tasks, unsigned int ntasks,
            unsigned int* task_counter, PairParams p, int copies) {
    extern __shared__ __align__(16) unsigned char smem[];
    float4* P = reinterpret_cast<float4*>(smem);
    unsigned int* H = reinterpret_cast<unsigned int*>(smem + PR_SMEM_FIXED);
    __shared__ uint4 s_task;
    __shared__ float s_u[PR_UMAX];
    if (!FP64 && p.fast)
        for (int v = threadIdx.x; v < PR_UMAX; v += blockDim.x) s_u[v] = p.u[v];
    for (int b = threadIdx.x; b < copies * p.n; b += blockDim.x) H[b] = 0;
    unsigned int* Hw = H + ((threadIdx.x >> 5) % copies) * p.n;
    int cur = -1;
    unsigned int since = 0;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int t = atomicAdd(task_counter, 1u);
            s_task = t < ntasks ? tasks[t] : make_uint4(TASK_NONE, 0, 0, 0);
        }
        __syncthreads();
        const uint4 task = s_task;
        const int slot = task.x == TASK_NONE ? -1 : (int)(task.x & TASK_SLOT_MASK);
        if ((slot != cur || since >= 4096) && cur >= 0) {
            flush_hist(H, copies, p.n, jobs[cur].hist);
            since = 0;
        }
        cur = slot;
        if (slot < 0) break;
        since++;
        if (((task.x >> TASK_PRED_SHIFT) & TASK_PRED_MASK) == PRED_SAME)
            pair_task<FP64, PRED_SAME>(jobs[slot], task, p, s_u, P, Hw);
        else
            pair_task<FP64, PRED_NONE>(jobs[slot], task, p, s_u, P, Hw);
    }
}

// ---------------------------------------------------------------------------
// Self-check of the exception table: counts floats whose table-driven value
// differs from the table entry (should be 0) -- used by tests.
__global__ void acos_check_kernel(AcosTable t, uint32_t key_begin, uint32_t count, unsigned int* mismatches) {
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
        uint32_t idx = key_begin + e;
        if (idx >= t.n) break;
        float c = __uint_as_float(t.keys[idx]);
        if (__float_as_uint(acosf_ref(c, t)) != t.vals[idx]) atomicAdd(mismatches, 1u);
    }
}

// ---------------------------------------------------------------------------
// Launchers

size_t triangle_smem_bytes(int hist_len, int copies) { return TRI_SMEM_FIXED + (size_t)hist_len * copies * 4; }
size_t three_side_smem_bytes(const ThreeParams& p, int copies, int groups) {
    // groups > 0: the grouped kernel (one histogram); else 8-warp CTAs with
    // 'copies' copies (0: the global histogram)
    const size_t pipe = ts_layout(ts_byte_jk(p)).bytes;
    const int words = groups > 0 || copies > 0 ? hist_stride(ts_acc_words(p)) : 0;
    if (groups > 0) return (size_t)groups * pipe + (size_t)words * 4;
    return pipe + (size_t)words * copies * 4;
}
size_t pair_smem_bytes(int hist_len, int copies) { return PR_SMEM_FIXED + (size_t)hist_len * copies * 4; }

// Every counting kernel may use the device's whole opt-in shared memory per
// block.  Set once per device, before any launch or graph capture, and never
// lowered: a launch (or a captured graph replayed later) is then valid for
// any histogram size the launch shape allows.
cudaError_t prepare_kernels(int device) {
    int optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e != cudaSuccess) return e;
    const void* fns[] = {(const void*)triangle_fast_kernel<true, false>, (const void*)triangle_fast_kernel<false, false>,
                         (const void*)triangle_fast_kernel<false, true>,
                         (const void*)triangle_fp64_kernel<MODE_FP64>, (const void*)triangle_fp64_kernel<MODE_GEOM>,
                         (const void*)triangle_fp64_kernel<MODE_JBJ>, (const void*)three_side_kernel<true, true>,
                         (const void*)three_side_kernel<true, false>, (const void*)three_side_kernel<false, true>,
                         (const void*)three_side_kernel<false, false>, (const void*)three_side_grouped_kernel<true>,
                         (const void*)three_side_grouped_kernel<false>, (const void*)pair_kernel<true>,
                         (const void*)pair_kernel<false>};
    for (const void* f : fns) {
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, f);
        if (e != cudaSuccess) return e;
        // dynamic plus static shared memory may not exceed the opt-in limit
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_triangle_fast(const DevJob* jobs, const uint4* tasks, const uint32_t* groups, const float* gbox,
                                 unsigned int ngroups, unsigned int* group_counter, const TriParams& p, RecheckQueue q,
                                 int grid, int copies, int jbj, cudaStream_t st) {
    size_t smem = triangle_smem_bytes(p.len, copies);
    if (jbj)
        triangle_fast_kernel<false, true><<<grid, TRI_THREADS, smem, st>>>(jobs, tasks, groups, gbox, ngroups,
                                                                           group_counter, p, q, copies);
    else if (p.theta_full)
        triangle_fast_kernel<true, false><<<grid, TRI_THREADS, smem, st>>>(jobs, tasks, groups, gbox, ngroups,
                                                                           group_counter, p, q, copies);
    else
        triangle_fast_kernel<false, false><<<grid, TRI_THREADS, smem, st>>>(jobs, tasks, groups, gbox, ngroups,
                                                                            group_counter, p, q, copies);
    return cudaGetLastError();
}

cudaError_t launch_triangle_recheck(const DevJob* jobs, RecheckQueue q, const TriParams& p, AcosTable t, int grid,
                                    cudaStream_t st) {
    triangle_recheck_kernel<<<grid, 128, 0, st>>>(jobs, q, p, t);
    return cudaGetLastError();
}

cudaError_t launch_triangle_fp64(const DevJob* jobs, const uint4* tasks, unsigned int ntasks,
                                 unsigned int* task_counter, const TriParams& p, AcosTable t, int grid, int copies,
                                 int mode, cudaStream_t st) {
    size_t smem = triangle_smem_bytes(p.len, copies);
    auto kern = mode == MODE_GEOM ? triangle_fp64_kernel<MODE_GEOM>
                : mode == MODE_JBJ  ? triangle_fp64_kernel<MODE_JBJ>
                                    : triangle_fp64_kernel<MODE_FP64>;
    kern<<<grid, TRI_THREADS, smem, st>>>(jobs, tasks, ntasks, task_counter, p, t, copies);
    return cudaGetLastError();
}

cudaError_t launch_three_side(const DevJob* jobs, const uint4* tasks, unsigned int ntasks,
                              unsigned int* task_counter, const ThreeParams& p, int fp64, int grid, int copies,
                              int groups, cudaStream_t st) {
    if (groups > 0) {
        if (groups > TS_GROUPS_MAX) return cudaErrorInvalidValue;
        const size_t smem = three_side_smem_bytes(p, 1, groups);
        const int threads = groups * TS_GROUP_THREADS;
        if (fp64)
            three_side_grouped_kernel<true><<<grid, threads, smem, st>>>(jobs, tasks, ntasks, task_counter, p, groups);
        else
            three_side_grouped_kernel<false><<<grid, threads, smem, st>>>(jobs, tasks, ntasks, task_counter, p, groups);
        return cudaGetLastError();
    }
    const bool global = copies == 0;
    const size_t smem = three_side_smem_bytes(p, global ? 0 : copies, 0);
#define TS_LAUNCH(FP, GL) \
    three_side_kernel<FP, GL><<<grid, TS_GROUP_THREADS, smem, st>>>(jobs, tasks, ntasks, task_counter, p, copies > 0 ? copies : 1);
    if (fp64) {
        if (global) { TS_LAUNCH(true, true) } else { TS_LAUNCH(true, false) }
    } else {
        if (global) { TS_LAUNCH(false, true) } else { TS_LAUNCH(false, false) }
    }
#undef TS_LAUNCH
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Catalog conversion (sample_data/gen_flat_MICE_data.py:53-99): comoving
// distance from redshift by the quadratic fit r = p0 + p1 z + p2 z^2, then
//   x = r sin(rad (90 - dec)) sin(rad ra), y = r sin(rad (90 - dec)) cos(rad ra),
//   z = r cos(rad (90 - dec)),  rad = pi/180,
// in double with the script's order of operations (no contraction), rounded
// to the float coordinates the counting kernels use.
__global__ void radecz_kernel(const double* __restrict__ ra, const double* __restrict__ dec,
                              const double* __restrict__ zr, int64_t n, double p0, double p1, double p2,
                              float* __restrict__ x, float* __restrict__ y, float* __restrict__ z) {
    const double rad = 3.141592653589793 / 180.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double zz = zr[i];
        const double r = __dadd_rn(__dadd_rn(p0, __dmul_rn(p1, zz)), __dmul_rn(__dmul_rn(p2, zz), zz));
        const double polar = __dmul_rn(rad, __dsub_rn(90.0, dec[i]));
        const double az = __dmul_rn(rad, ra[i]);
        double sp, cp, sa, ca;
        sincos(polar, &sp, &cp);
        sincos(az, &sa, &ca);
        const double rs = __dmul_rn(r, sp);
        x[i] = __double2float_rn(__dmul_rn(rs, sa));
        y[i] = __double2float_rn(__dmul_rn(rs, ca));
        z[i] = __double2float_rn(__dmul_rn(r, cp));
    }
}

cudaError_t launch_radecz_to_xyz(const double* ra, const double* dec, const double* redshift, int64_t n,
                                 const double poly[3], float* x, float* y, float* z, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
    radecz_kernel<<<(unsigned)blocks, 256, 0, st>>>(ra, dec, redshift, n, poly[0], poly[1], poly[2], x, y, z);
    return cudaGetLastError();
}

cudaError_t launch_pairs(const DevJob* jobs, const uint4* tasks, unsigned int ntasks, unsigned int* task_counter,
                         const PairParams& p, int fp64, int grid, int copies, cudaStream_t st) {
    size_t smem = pair_smem_bytes(p.n, copies);
    if (fp64)
        pair_kernel<true><<<grid, PR_THREADS, smem, st>>>(jobs, tasks, ntasks, task_counter, p, copies);
    else
        pair_kernel<false><<<grid, PR_THREADS, smem, st>>>(jobs, tasks, ntasks, task_counter, p, copies);
    return cudaGetLastError();
}

cudaError_t launch_acos_check(AcosTable t, uint32_t key_begin, uint32_t count, unsigned int* mismatches,
                              cudaStream_t st) {
    acos_check_kernel<<<1024, 256, 0, st>>>(t, key_begin, count, mismatches);
    return cudaGetLastError();
}

}  // namespace tpcf

// ===========================================================================
// Pair counts without any device allocation.
//
// For callers that cannot call cudaMalloc -- code running inside a framework
// that owns all device memory through its own pool, or a library that must not
// grow the process's footprint behind its host application's back.  They pass
// device pointers to their catalogs and to the output histogram; every other
// buffer the count needs (packed points, tile table, job descriptor, task
// counter) is the file-scope array below, which exists on every device that
// loads this library until the process exits.
//
// Limits and sharing: at most NOALLOC_MAX_POINTS points per catalog; all calls
// on a device share the array, so calls whose work overlaps on the GPU (two
// streams, or two host threads) race and must be serialised by the caller.
// The array keeps the previous call's contents; everything that must start
// from zero (task counter, output histogram) is cleared by the call itself.
// ===========================================================================

namespace tpcf {

constexpr int64_t NOALLOC_MAX_POINTS = 1 << 18;             // per catalog
constexpr int NOALLOC_MAX_TILES = (int)(NOALLOC_MAX_POINTS / TILE);

struct NoAllocScratch {
    float4 pts[2][NOALLOC_MAX_POINTS];        // 2 x 4 MiB
    int32_t tile_start[2][NOALLOC_MAX_TILES + 1];
    DevJob job;
    unsigned int task_counter;
};
static __device__ __align__(256) NoAllocScratch g_noalloc;  // 8 MiB per device

// packs SoA catalogs into the scratch points (.w = loop index), fills the tile
// table, resets the task counter
__global__ void noalloc_prepare(const float* x0, const float* y0, const float* z0, int n0, const float* x1,
                                const float* y1, const float* z1, int n1, unsigned long long* hist) {
    NoAllocScratch* S = &g_noalloc;
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = tid; i < n0; i += stride) S->pts[0][i] = make_float4(x0[i], y0[i], z0[i], __int_as_float(i));
    for (int i = tid; i < n1; i += stride) S->pts[1][i] = make_float4(x1[i], y1[i], z1[i], __int_as_float(i));
    const int t0 = (n0 + TILE - 1) / TILE, t1 = (n1 + TILE - 1) / TILE;
    for (int t = tid; t <= t0; t += stride) S->tile_start[0][t] = min(t * TILE, n0);
    for (int t = tid; t <= t1; t += stride) S->tile_start[1][t] = min(t * TILE, n1);
    if (tid == 0) {
        S->job.pts[0] = S->pts[0];
        S->job.pts[1] = S->pts[1];
        S->job.pts[2] = S->pts[1];
        S->job.tile_start[0] = S->tile_start[0];
        S->job.tile_start[1] = S->tile_start[1];
        S->job.tile_start[2] = S->tile_start[1];
        S->job.hist = hist;
        S->task_counter = 0u;
    }
}

// pair_kernel with tile-pair tasks computed from the counter value (no task
// list): task t is tile pair (t / ntB, t % ntB); 'same' enumerates only a <= b
// of one catalog with j >= i inside the diagonal tile
template <bool FP64>
__global__ void __launch_bounds__(PR_THREADS)
pair_kernel_noalloc(unsigned int* task_counter, int ntA, int ntB, int same, int pred_same, PairParams p, int copies) {
    extern __shared__ __align__(16) unsigned char smem[];
    float4* P = reinterpret_cast<float4*>(smem);
    unsigned int* H = reinterpret_cast<unsigned int*>(smem + PR_SMEM_FIXED);
    __shared__ unsigned int s_t;
    const DevJob& J = g_noalloc.job;
    for (int b = threadIdx.x; b < copies * p.n; b += blockDim.x) H[b] = 0;
    unsigned int* Hw = H + ((threadIdx.x >> 5) % copies) * p.n;
    const unsigned int ntasks = (unsigned int)ntA * (unsigned int)ntB;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_t = atomicAdd(task_counter, 1u);
        __syncthreads();
        const unsigned int t = s_t;
        if (t >= ntasks) break;
        const unsigned int a = t / (unsigned int)ntB, b = t % (unsigned int)ntB;
        if (same && b < a) continue;
        uint4 task = make_uint4((same && a == b ? TASK_DIAG_IJ : 0u), a, b, 0u);
        if (pred_same) pair_task<FP64, PRED_SAME>(J, task, p, nullptr, P, Hw);
        else pair_task<FP64, PRED_NONE>(J, task, p, nullptr, P, Hw);
    }
    flush_hist(H, copies, p.n, J.hist);
}

}  // namespace tpcf

// Declared in include/tpcf.h.  Every call looks up the device address of the
// scratch array (cudaGetSymbolAddress) with the caller's device current: a
// host call, so the address is never stale (a device reset reloads the
// module).  The first call on a device may load the library's device code:
// make it outside any stream capture.
extern "C" int32_t tpcf_pair_count_noalloc(const float* x0, const float* y0, const float* z0, int64_t n0,
                                           const float* x1, const float* y1, const float* z1, int64_t n1,
                                           int32_t loop, float lo, float hi, int32_t nbins, uint64_t* hist_out,
                                           void* stream) {
    using namespace tpcf;
    unsigned long long* hist = reinterpret_cast<unsigned long long*>(hist_out);
    if (n0 < 0 || n1 < 0 || n0 > NOALLOC_MAX_POINTS || n1 > NOALLOC_MAX_POINTS) return TPCF_ERR_INVALID;
    if (!hist || nbins <= 0 || !(hi > lo)) return TPCF_ERR_INVALID;
    if ((n0 > 0 && (!x0 || !y0 || !z0)) || (n1 > 0 && (!x1 || !y1 || !z1))) return TPCF_ERR_INVALID;
    if (loop != TPCF_LOOP_ALL && loop != TPCF_LOOP_SAME && loop != TPCF_LOOP_ONE) return TPCF_ERR_INVALID;
    int copies = 8;
    while (copies > 1 && pair_smem_bytes(nbins, copies) > 200 * 1024) copies /= 2;
    if (pair_smem_bytes(nbins, copies) > 227 * 1024) return TPCF_ERR_INVALID;
    // an error left by the caller's earlier work is reported, not consumed
    if (cudaPeekAtLastError() != cudaSuccess) return TPCF_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TPCF_ERR_NO_DEVICE;
    void* scratch = nullptr;
    if (cudaGetSymbolAddress(&scratch, g_noalloc) != cudaSuccess || !scratch) {
        (void)cudaGetLastError();
        return TPCF_ERR_CUDA;
    }
    cudaStream_t st = (cudaStream_t)stream;
    NoAllocScratch* S = (NoAllocScratch*)scratch;
    unsigned int* counter = &S->task_counter;
    // (an error of this call's own CUDA calls is consumed before returning, so
    // that it does not stay pending for the caller's next CUDA call)
    auto own_error = []() {
        (void)cudaGetLastError();
        return (int32_t)TPCF_ERR_CUDA;
    };
    if (cudaMemsetAsync(hist, 0, sizeof(unsigned long long) * (size_t)nbins, st) != cudaSuccess) return own_error();
    noalloc_prepare<<<256, 256, 0, st>>>(x0, y0, z0, (int)n0, x1, y1, z1, (int)n1, hist);
    if (cudaGetLastError() != cudaSuccess) return TPCF_ERR_CUDA;  // (consumed by the check itself)
    const bool same = loop == TPCF_LOOP_SAME && x0 == x1 && y0 == y1 && z0 == z1 && n0 == n1;
    const int pred_same = loop == TPCF_LOOP_SAME && !same;
    const int ntA = (int)((n0 + TILE - 1) / TILE), ntB = (int)((n1 + TILE - 1) / TILE);
    if (ntA > 0 && ntB > 0) {
        PairParams p;
        p.n = nbins;
        p.lo = lo;
        p.hi = hi;
        volatile float span = hi - lo;
        p.bw = span / (float)nbins;
        size_t smem = pair_smem_bytes(nbins, copies);
        // the kernel's dynamic shared memory limit: always the device's opt-in
        // maximum, never lowered (a lower per-call value would invalidate
        // launches recorded earlier with a larger size)
        // (dynamic plus the kernel's static shared memory within the opt-in limit)
        int optin = 0, sms = 0;
        cudaFuncAttributes fa;
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, pair_kernel_noalloc<false>) != cudaSuccess)
            return own_error();
        const int smem_max = optin - (int)fa.sharedSizeBytes;
        if ((size_t)smem_max < smem) return TPCF_ERR_INVALID;
        if (cudaFuncSetAttribute(pair_kernel_noalloc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max) !=
            cudaSuccess)
            return own_error();
        long long tasks = (long long)ntA * ntB;
        int grid = (int)std::min<long long>(tasks, (long long)sms * 4);
        pair_kernel_noalloc<false><<<grid, PR_THREADS, smem, st>>>(counter, ntA, ntB, same ? 1 : 0, pred_same, p, copies);
        if (cudaGetLastError() != cudaSuccess) return TPCF_ERR_CUDA;
    }
    return TPCF_OK;
}
