// exact_acos.h -- a double-precision arc cosine whose every step is an explicit
// IEEE-754 operation (fma, add, multiply, sqrt), so that the host and the device
// compute bit-identical results.
//
// Why: the triangle-parametrization program calls glibc's acosf
// (src/3pcf_C_version_triangle_parametrization.cc:197,202), which is not
// correctly rounded.  The engine reproduces it exactly as
//     acosf_ref(c) = table[c] if c is in the exception table, else (float)tpcf_acos_d(c)
// where the exception table lists every float c in [-1, 1] for which the host's
// glibc acosf differs from (float)tpcf_acos_d(c).  The table is built on the
// host by an exhaustive scan, which is exact only if the device evaluates
// tpcf_acos_d bit-identically -- hence no contraction and no library acos here.
//
// Method: acos(x) = pi/2 - asin(x) for |x| <= 1/2, and
//         acos(x) = 2 asin(sqrt((1-x)/2)), acos(-x) = pi - acos(x) for |x| > 1/2,
// with asin(t) = t + t*u*P(u), u = t^2 in [0, 1/4], P a degree-16 least-squares
// fit on Chebyshev nodes of (asin(sqrt u) - sqrt u)/u^1.5 (max relative error
// of asin about 1.2e-16 on [0, 1/2]).
#ifndef TPCF_EXACT_ACOS_H
#define TPCF_EXACT_ACOS_H

#include <math.h>

#if defined(__CUDACC__)
#define TPCF_HD __host__ __device__ __forceinline__
#else
#define TPCF_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define TPCF_DADD(a, b) __dadd_rn((a), (b))
#define TPCF_DMUL(a, b) __dmul_rn((a), (b))
#define TPCF_DFMA(a, b, c) __fma_rn((a), (b), (c))
#define TPCF_DSQRT(a) __dsqrt_rn(a)
#else
// host translation units are compiled with -ffp-contract=off
#define TPCF_DADD(a, b) ((a) + (b))
#define TPCF_DMUL(a, b) ((a) * (b))
#define TPCF_DFMA(a, b, c) fma((a), (b), (c))
#define TPCF_DSQRT(a) sqrt(a)
#endif

TPCF_HD double tpcf_asin_poly(double u) {
    double p = 0.033828873395440925;
    p = TPCF_DFMA(p, u, -0.035444145756186374);
    p = TPCF_DFMA(p, u, 0.03176524412107469);
    p = TPCF_DFMA(p, u, -0.006588625898530745);
    p = TPCF_DFMA(p, u, 0.009252028847581322);
    p = TPCF_DFMA(p, u, 0.0056906520430134305);
    p = TPCF_DFMA(p, u, 0.007432427801322617);
    p = TPCF_DFMA(p, u, 0.008376241422328857);
    p = TPCF_DFMA(p, u, 0.009762836199034244);
    p = TPCF_DFMA(p, u, 0.01155172271071856);
    p = TPCF_DFMA(p, u, 0.013964847323925408);
    p = TPCF_DFMA(p, u, 0.017352764309798544);
    p = TPCF_DFMA(p, u, 0.022372159093271924);
    p = TPCF_DFMA(p, u, 0.03038194444441459);
    p = TPCF_DFMA(p, u, 0.04464285714285734);
    p = TPCF_DFMA(p, u, 0.075);
    p = TPCF_DFMA(p, u, 0.16666666666666666);
    return p;
}

// asin(t) for t in [0, 1/2]
TPCF_HD double tpcf_asin_small(double t) {
    double u = TPCF_DMUL(t, t);
    return TPCF_DFMA(TPCF_DMUL(t, u), tpcf_asin_poly(u), t);
}

// acos(x) in double for x in [-1, 1]; NaN outside.
TPCF_HD double tpcf_acos_d(double x) {
    const double pio2_hi = 1.5707963267948966;   // nearest double to pi/2
    const double pio2_lo = 6.123233995736766e-17; // pi/2 - pio2_hi
    const double pi_hi = 3.141592653589793;
    const double pi_lo = 1.2246467991473532e-16;
    if (!(x >= -1.0 && x <= 1.0)) return (x - x) / (x - x);  // NaN
    double ax = x < 0 ? -x : x;
    if (ax <= 0.5) {
        double a = ax > 0 ? tpcf_asin_small(ax) : 0.0;
        if (x < 0) a = -a;
        // pi/2 - asin(x) = pio2_hi - (asin(x) - pio2_lo)
        return TPCF_DADD(pio2_hi, -TPCF_DADD(a, -pio2_lo));
    }
    // (1 - |x|)/2 is exact (Sterbenz); sqrt correctly rounded
    double t = TPCF_DSQRT(TPCF_DMUL(TPCF_DADD(1.0, -ax), 0.5));
    double a2 = TPCF_DMUL(2.0, tpcf_asin_small(t));
    if (x > 0) return a2;
    return TPCF_DADD(pi_hi, -TPCF_DADD(a2, -pi_lo));
}

#endif
