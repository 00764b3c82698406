/*
 * tpcf_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of the reference's three counting algorithms, used by the
 * test-suite and by the CPU-baseline leg of bench.py as the CHECKER.  Nothing in
 * the product links, loads or calls this file; the product path is the CUDA
 * engine in 3pcf_gb300/ and fails loudly when that is missing.
 *
 * Semantics follow the reference C programs (citations are paths inside the
 * mattbellis/3pcf project):
 *   three-side histogram   src/3pcf_C_version.cc
 *   triangle parametrization src/3pcf_C_version_triangle_parametrization.cc
 *   2pcf pair counts       src/2pcf_C_version.cc
 *
 * Every floating-point step is written as the same sequence of IEEE single
 * operations the reference performs.  Build with -ffp-contract=off (no FMA
 * contraction) so that the result matches an x86-64 SSE build of the reference.
 * The one platform-dependent step of the reference, converting a NaN to int in
 * distance_to_bin (x86 cvttss2si gives INT_MIN, aarch64 fcvtzs gives 0), is an
 * explicit parameter (nan_zero).
 *
 * Pinning: tests/test_oracle.py checks this code against the reference's own
 * golden outputs (the examples/sandbox histogram files, copied to tests/golden/) and against
 * outputs of the reference programs compiled from source (oracle/ref_build.py).
 *
 * Loops are split over the outermost index across POSIX threads; every thread
 * owns a private integer histogram, so the result is independent of the
 * schedule.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>

typedef struct {
    const float* x;
    const float* y;
    const float* z;
    long n;
} ocat_t;

/* ------------------------------------------------------------------------- */
/* distance of two points exactly as the reference: sqrt(dx*dx+dy*dy+dz*dz) in */
/* float, left-to-right sums (src/3pcf_C_version.cc:57-60,                     */
/* src/3pcf_C_version_triangle_parametrization.cc:119-132,                     */
/* src/2pcf_C_version.cc:92-95).                                               */
static inline float ref_dist(float x0, float y0, float z0, float x1, float y1, float z1) {
    float xdiff = x0 - x1;
    float ydiff = y0 - y1;
    float zdiff = z0 - z1;
    float s = xdiff * xdiff;
    s = s + ydiff * ydiff;
    s = s + zdiff * zdiff;
    return sqrtf(s);
}

/* ------------------------------------------------------------------------- */
/* Three-side histogram: src/3pcf_C_version.cc                                 */

/* distance_to_bin, src/3pcf_C_version.cc:23-51 (flag == 0, linear bins):
 * below hist_min -> 0, at or above hist_max -> nbins+1, else int((d-lo)/w). */
static inline int o3_bin(float dist, float lo, float hi, int nbins, float bw) {
    if (dist < lo) return 0;
    if (dist >= hi) return nbins + 1;
    return (int)((dist - lo) / bw);
}

typedef struct {
    const ocat_t* c;
    float lo, hi, bw;
    int nbins, clean;
    long i_next;
    pthread_mutex_t* mu;
} o3_task_t;

static long grab(long* next, pthread_mutex_t* mu, long chunk) {
    pthread_mutex_lock(mu);
    long v = *next;
    *next += chunk;
    pthread_mutex_unlock(mu);
    return v;
}

typedef struct {
    o3_task_t* shared;
    unsigned long long* hist;
    unsigned long long ncalc;
} o3_worker_t;

static void* o3_worker(void* arg) {
    o3_worker_t* w = (o3_worker_t*)arg;
    o3_task_t* t = w->shared;
    const ocat_t* c = t->c;
    const long size = (long)t->nbins * t->nbins * t->nbins;
    const int n = t->nbins;
    /* bins of d02 for the current i, cached (same float operations) */
    int* b1k = (int*)malloc(sizeof(int) * (c[2].n > 0 ? c[2].n : 1));
    unsigned char* far1 = (unsigned char*)malloc(c[2].n > 0 ? c[2].n : 1);
    for (;;) {
        long i0 = grab(&t->i_next, t->mu, 1);
        if (i0 >= c[0].n) break;
        long i = i0;
        for (long k = 0; k < c[2].n; k++) {
            float d1 = ref_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[2].x[k], c[2].y[k], c[2].z[k]);
            b1k[k] = o3_bin(d1, t->lo, t->hi, n, t->bw);
            far1[k] = d1 >= t->hi;
        }
        /* hot loop over every ordered (i,j,k): src/3pcf_C_version.cc:363-432
         * (jmin/kmin are computed there but not used by the loops). */
        for (long j = 0; j < c[1].n; j++) {
            float d0 = ref_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[1].x[j], c[1].y[j], c[1].z[j]);
            int b0 = o3_bin(d0, t->lo, t->hi, n, t->bw);
            int far0 = d0 >= t->hi;
            for (long k = 0; k < c[2].n; k++) {
                /* distance(), src/3pcf_C_version.cc:54-142: sides in source
                 * order d01 -> i0, d02 -> i1, d12 -> i2, unsorted. */
                float d2 = ref_dist(c[1].x[j], c[1].y[j], c[1].z[j], c[2].x[k], c[2].y[k], c[2].z[k]);
                w->ncalc++;
                if (t->clean && (far0 || far1[k] || d2 >= t->hi)) continue;
                int b2 = o3_bin(d2, t->lo, t->hi, n, t->bw);
                long idx = (long)n * n * b2 + (long)n * b1k[k] + b0;  /* :137-139 */
                /* An index at or past nbins^3 is a write past the end of the
                 * reference's array (undefined); it never reaches the printed
                 * histogram, so it is not counted here. */
                if (idx < size) w->hist[idx]++;
            }
        }
    }
    free(b1k);
    free(far1);
    return NULL;
}

/* Three-side histogram of every ordered triple (i in c[0], j in c[1], k in c[2]).
 * hist has nbins^3 entries in the reference's index layout n^2*i2 + n*i1 + i0.
 * clean != 0 additionally skips triples with any side >= hist_max.
 * Returns the number of triples visited (the reference's fake_tot, :429). */
unsigned long long oracle_three_side(const ocat_t* cats, float hist_min, float hist_max, int nbins,
                                     int clean, unsigned long long* hist, int nthreads) {
    const long size = (long)nbins * nbins * nbins;
    memset(hist, 0, sizeof(unsigned long long) * size);
    if (nthreads < 1) nthreads = 1;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    o3_task_t task;
    task.c = cats;
    task.lo = hist_min;
    task.hi = hist_max;
    task.bw = (hist_max - hist_min) / nbins; /* float, src/3pcf_C_version.cc:174 */
    task.nbins = nbins;
    task.clean = clean;
    task.i_next = 0;
    task.mu = &mu;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    o3_worker_t* ws = (o3_worker_t*)calloc(nthreads, sizeof(o3_worker_t));
    for (int t = 0; t < nthreads; t++) {
        ws[t].shared = &task;
        ws[t].hist = (unsigned long long*)calloc(size, sizeof(unsigned long long));
        pthread_create(&th[t], NULL, o3_worker, &ws[t]);
    }
    unsigned long long ncalc = 0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        for (long b = 0; b < size; b++) hist[b] += ws[t].hist[b];
        ncalc += ws[t].ncalc;
        free(ws[t].hist);
    }
    free(ws);
    free(th);
    return ncalc;
}

/* ------------------------------------------------------------------------- */
/* Triangle parametrization: src/3pcf_C_version_triangle_parametrization.cc    */

/* distance_to_bin, :84-113 (flag == 0): the bin width is recomputed in float
 * from the float-converted limits; out of range returns -999.  A NaN input
 * reaches int(NaN), whose value is platform-defined (see file header). */
static inline int tp_bin(float v, float lo, float hi, int nbins, int nan_zero) {
    float bw = (hi - lo) / nbins;
    if (v < lo) return -999;
    if (v >= hi) return -999;
    if (v != v) return nan_zero ? 0 : INT_MIN;
    return (int)((v - lo) / bw);
}

typedef struct {
    float lo[3], hi[3];
    int nb[3];
    int nan_zero;
} tp_spec_t;

/* distance(), :116-240, after the three side lengths dist0 = |p0-p1|,
 * dist1 = |p0-p2|, dist2 = |p1-p2| (each a symmetric function of its two
 * points, so callers may cache them).  Writes the three indices or -999. */
static inline void tp_core(float dist0, float dist1, float dist2, const tp_spec_t* sp, int totbins[3]) {
    float shortest, middle, longest;
    /* three-way sort, :146-181 */
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
    float shortest2 = shortest * shortest;  /* :188-190 */
    float middle2 = middle * middle;
    float longest2 = longest * longest;
    float theta0 = 0.f, theta1 = 0.f, theta2, s, q;
    int i0, i1, i2;
    const int QT = sp->nb[1] * sp->nb[2];
    const int T = sp->nb[2];
    for (int k = 0; k < 3; k++) {
        if (k == 0) {
            s = shortest;
            q = middle / shortest;
            /* (acosf(c))*INVPI with INVPI = 1.0/PI, PI = 3.14159 (:10-11):
             * the product and quotient are evaluated in double, then stored. */
            float c = (shortest2 + middle2 - longest2) / (2 * shortest * middle);
            theta0 = (float)(((double)acosf(c) * 1.0) / 3.14159);
            i2 = tp_bin(theta0, sp->lo[2], sp->hi[2], sp->nb[2], sp->nan_zero);
        } else if (k == 1) {
            s = middle;
            q = longest / middle;
            float c = (middle2 + longest2 - shortest2) / (2 * middle * longest);
            theta1 = (float)(((double)acosf(c) * 1.0) / 3.14159);
            i2 = tp_bin(theta1, sp->lo[2], sp->hi[2], sp->nb[2], sp->nan_zero);
        } else {
            s = shortest;
            q = longest / shortest;
            theta2 = (float)(1.0 - (double)theta0 - (double)theta1);  /* :208 */
            i2 = tp_bin(theta2, sp->lo[2], sp->hi[2], sp->nb[2], sp->nan_zero);
        }
        i0 = tp_bin(s, sp->lo[0], sp->hi[0], sp->nb[0], sp->nan_zero);
        i1 = tp_bin(q, sp->lo[1], sp->hi[1], sp->nb[1], sp->nan_zero);
        int tot;
        if (i0 < 0 || i1 < 0 || i2 < 0) tot = -999;
        else tot = QT * i0 + T * i1 + i2;  /* :226 */
        if (dist0 == 0 || dist1 == 0 || dist2 == 0) tot = -999;  /* :230-234 */
        totbins[k] = tot;
    }
}

static inline void tp_distance(float x0, float y0, float z0, float x1, float y1, float z1,
                               float x2, float y2, float z2, const tp_spec_t* sp, int totbins[3]) {
    tp_core(ref_dist(x0, y0, z0, x1, y1, z1), ref_dist(x0, y0, z0, x2, y2, z2),
            ref_dist(x1, y1, z1, x2, y2, z2), sp, totbins);
}

typedef struct {
    const ocat_t* c;
    tp_spec_t sp;
    int which;
    long i_next;
    pthread_mutex_t* mu;
} tp_task_t;

typedef struct {
    tp_task_t* shared;
    unsigned long long* hist;
    unsigned long long ncalc;
} tp_worker_t;

static void* tp_worker(void* arg) {
    tp_worker_t* w = (tp_worker_t*)arg;
    tp_task_t* t = w->shared;
    const ocat_t* c = t->c;
    const long size = (long)t->sp.nb[0] * t->sp.nb[1] * t->sp.nb[2];
    float* d02 = (float*)malloc(sizeof(float) * (c[2].n > 0 ? c[2].n : 1));
    for (;;) {
        long i = grab(&t->i_next, t->mu, 1);
        if (i >= c[0].n) break;
        for (long k = 0; k < c[2].n; k++)
            d02[k] = ref_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[2].x[k], c[2].y[k], c[2].z[k]);
        /* loop bounds, :484-509.  The mode is stored in a bool, so the
         * "which == 2" value collapses to 1 and the DRD branch is dead:
         * which 0 -> jmin = i, kmin = j;  which 1 -> jmin = 0, kmin = j. */
        long jmin = (t->which == 0) ? i : 0;
        for (long j = jmin; j < c[1].n; j++) {
            float d01 = ref_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[1].x[j], c[1].y[j], c[1].z[j]);
            for (long k = j; k < c[2].n; k++) {
                int tb[3];
                float d12 = ref_dist(c[1].x[j], c[1].y[j], c[1].z[j], c[2].x[k], c[2].y[k], c[2].z[k]);
                tp_core(d01, d02[k], d12, &t->sp, tb);
                w->ncalc++;
                for (int b = 0; b < 3; b++) {
                    /* :522-530; an index past the array end is undefined in the
                     * reference and never printed, so it is not counted. */
                    if (tb[b] >= 0 && tb[b] < size) w->hist[tb[b]]++;
                }
            }
        }
    }
    free(d02);
    return NULL;
}

/* Triangle-parametrization histogram with the reference's loop nest for the
 * given mode (which = 0 or 1, after the bool collapse).  lohi = {s_lo, s_hi,
 * q_lo, q_hi, theta_lo, theta_hi} as floats, nb = {S, Q, T}.  hist has S*Q*T
 * 64-bit entries (the reference stores unsigned int and wraps; callers apply
 * the wrap when writing).  Returns the reference's numcalc. */
unsigned long long oracle_triangle(const ocat_t* cats, int which, const float* lohi, const int* nb,
                                   int nan_zero, unsigned long long* hist, int nthreads) {
    const long size = (long)nb[0] * nb[1] * nb[2];
    memset(hist, 0, sizeof(unsigned long long) * size);
    if (nthreads < 1) nthreads = 1;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    tp_task_t task;
    task.c = cats;
    for (int a = 0; a < 3; a++) {
        task.sp.lo[a] = lohi[2 * a];
        task.sp.hi[a] = lohi[2 * a + 1];
        task.sp.nb[a] = nb[a];
    }
    task.sp.nan_zero = nan_zero;
    task.which = which ? 1 : 0;
    task.i_next = 0;
    task.mu = &mu;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    tp_worker_t* ws = (tp_worker_t*)calloc(nthreads, sizeof(tp_worker_t));
    for (int t = 0; t < nthreads; t++) {
        ws[t].shared = &task;
        ws[t].hist = (unsigned long long*)calloc(size, sizeof(unsigned long long));
        pthread_create(&th[t], NULL, tp_worker, &ws[t]);
    }
    unsigned long long ncalc = 0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        for (long b = 0; b < size; b++) hist[b] += ws[t].hist[b];
        ncalc += ws[t].ncalc;
        free(ws[t].hist);
    }
    free(ws);
    free(th);
    return ncalc;
}

/* ------------------------------------------------------------------------- */
/* JBJ shape parametrization: src/3pcf_C_version_triangle_parametrization_JBJ.cc
 * distance(), :116-229: one permutation only, s = shortest, q = shortest /
 * middle, theta = (longest - middle) / shortest, binned by the same
 * distance_to_bin (:84-113); zero sides drop the triangle.  main() passes a
 * three-entry bins array initialised to {0, 0, 0} (:455) of which distance()
 * only writes entry 0, so every visited triangle also adds 2 to hist[0]
 * (:511-518); compat = 1 reproduces that, 0 leaves it out. */

static inline int jbj_core(float dist0, float dist1, float dist2, const tp_spec_t* sp) {
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
    float s = shortest;
    float q = shortest / middle;
    float theta = (longest - middle) / shortest;
    int i2 = tp_bin(theta, sp->lo[2], sp->hi[2], sp->nb[2], sp->nan_zero);
    int i0 = tp_bin(s, sp->lo[0], sp->hi[0], sp->nb[0], sp->nan_zero);
    int i1 = tp_bin(q, sp->lo[1], sp->hi[1], sp->nb[1], sp->nan_zero);
    int tot = (i0 < 0 || i1 < 0 || i2 < 0) ? -999 : sp->nb[1] * sp->nb[2] * i0 + sp->nb[2] * i1 + i2;
    if (dist0 == 0 || dist1 == 0 || dist2 == 0) tot = -999;
    return tot;
}

static void* jbj_worker(void* arg) {
    tp_worker_t* w = (tp_worker_t*)arg;
    tp_task_t* t = w->shared;
    const ocat_t* c = t->c;
    const long size = (long)t->sp.nb[0] * t->sp.nb[1] * t->sp.nb[2];
    for (;;) {
        long i = grab(&t->i_next, t->mu, 1);
        if (i >= c[0].n) break;
        long jmin = (t->which == 0) ? i : 0;
        for (long j = jmin; j < c[1].n; j++) {
            float d01 = ref_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[1].x[j], c[1].y[j], c[1].z[j]);
            for (long k = j; k < c[2].n; k++) {
                float d02 = ref_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[2].x[k], c[2].y[k], c[2].z[k]);
                float d12 = ref_dist(c[1].x[j], c[1].y[j], c[1].z[j], c[2].x[k], c[2].y[k], c[2].z[k]);
                int b = jbj_core(d01, d02, d12, &t->sp);
                w->ncalc++;
                if (b >= 0 && b < size) w->hist[b]++;
            }
        }
    }
    return NULL;
}

unsigned long long oracle_triangle_jbj(const ocat_t* cats, int which, const float* lohi, const int* nb,
                                       int compat, unsigned long long* hist, int nthreads) {
    const long size = (long)nb[0] * nb[1] * nb[2];
    memset(hist, 0, sizeof(unsigned long long) * size);
    if (nthreads < 1) nthreads = 1;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    tp_task_t task;
    task.c = cats;
    for (int a = 0; a < 3; a++) {
        task.sp.lo[a] = lohi[2 * a];
        task.sp.hi[a] = lohi[2 * a + 1];
        task.sp.nb[a] = nb[a];
    }
    task.sp.nan_zero = 0;
    task.which = which ? 1 : 0;
    task.i_next = 0;
    task.mu = &mu;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    tp_worker_t* ws = (tp_worker_t*)calloc(nthreads, sizeof(tp_worker_t));
    for (int t = 0; t < nthreads; t++) {
        ws[t].shared = &task;
        ws[t].hist = (unsigned long long*)calloc(size, sizeof(unsigned long long));
        pthread_create(&th[t], NULL, jbj_worker, &ws[t]);
    }
    unsigned long long ncalc = 0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        for (long b = 0; b < size; b++) hist[b] += ws[t].hist[b];
        ncalc += ws[t].ncalc;
        free(ws[t].hist);
    }
    free(ws);
    free(th);
    if (compat && size > 0) hist[0] += 2 * ncalc;
    return ncalc;
}

/* ------------------------------------------------------------------------- */
/* FP64 geometry: the triangle formulas of :116-240 evaluated in double from
 * the float coordinates, acos in double.  Not the reference's counts; the FP64
 * truth that the error of the derived correlation function is measured
 * against.  Same loop nest and counting rules as oracle_triangle. */

static inline double geo_dist(float x0, float y0, float z0, float x1, float y1, float z1) {
    double dx = (double)x0 - (double)x1, dy = (double)y0 - (double)y1, dz = (double)z0 - (double)z1;
    return sqrt(dx * dx + dy * dy + dz * dz);
}

static inline int geo_bin(double v, float lo, float hi, int nbins, int nan_zero) {
    double bw = ((double)hi - (double)lo) / nbins;
    if (v < lo) return -999;
    if (v >= hi) return -999;
    if (v != v) return nan_zero ? 0 : INT_MIN;
    return (int)((v - lo) / bw);
}

static inline void geo_core(double d0, double d1, double d2, const tp_spec_t* sp, int totbins[3]) {
    double a = d0, b = d1, c = d2, t;
    /* ascending order; ties do not matter here (equal values) */
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
    const double th0 = acos((a * a + b * b - c * c) / (2 * a * b)) / 3.14159;
    const double th1 = acos((b * b + c * c - a * a) / (2 * b * c)) / 3.14159;
    const double sv[3] = {a, b, a}, qv[3] = {b / a, c / b, c / a}, tv[3] = {th0, th1, 1.0 - th0 - th1};
    for (int k = 0; k < 3; k++) {
        int i0 = geo_bin(sv[k], sp->lo[0], sp->hi[0], sp->nb[0], sp->nan_zero);
        int i1 = geo_bin(qv[k], sp->lo[1], sp->hi[1], sp->nb[1], sp->nan_zero);
        int i2 = geo_bin(tv[k], sp->lo[2], sp->hi[2], sp->nb[2], sp->nan_zero);
        int tot = (i0 < 0 || i1 < 0 || i2 < 0) ? -999 : sp->nb[1] * sp->nb[2] * i0 + sp->nb[2] * i1 + i2;
        if (d0 == 0 || d1 == 0 || d2 == 0) tot = -999;
        totbins[k] = tot;
    }
}

static void* geo_worker(void* arg) {
    tp_worker_t* w = (tp_worker_t*)arg;
    tp_task_t* t = w->shared;
    const ocat_t* c = t->c;
    const long size = (long)t->sp.nb[0] * t->sp.nb[1] * t->sp.nb[2];
    for (;;) {
        long i = grab(&t->i_next, t->mu, 1);
        if (i >= c[0].n) break;
        long jmin = (t->which == 0) ? i : 0;
        for (long j = jmin; j < c[1].n; j++) {
            double d01 = geo_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[1].x[j], c[1].y[j], c[1].z[j]);
            for (long k = j; k < c[2].n; k++) {
                int tb[3];
                double d02 = geo_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[2].x[k], c[2].y[k], c[2].z[k]);
                double d12 = geo_dist(c[1].x[j], c[1].y[j], c[1].z[j], c[2].x[k], c[2].y[k], c[2].z[k]);
                geo_core(d01, d02, d12, &t->sp, tb);
                w->ncalc++;
                for (int b = 0; b < 3; b++)
                    if (tb[b] >= 0 && tb[b] < size) w->hist[tb[b]]++;
            }
        }
    }
    return NULL;
}

unsigned long long oracle_triangle_geom64(const ocat_t* cats, int which, const float* lohi, const int* nb,
                                          int nan_zero, unsigned long long* hist, int nthreads) {
    const long size = (long)nb[0] * nb[1] * nb[2];
    memset(hist, 0, sizeof(unsigned long long) * size);
    if (nthreads < 1) nthreads = 1;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    tp_task_t task;
    task.c = cats;
    for (int a = 0; a < 3; a++) {
        task.sp.lo[a] = lohi[2 * a];
        task.sp.hi[a] = lohi[2 * a + 1];
        task.sp.nb[a] = nb[a];
    }
    task.sp.nan_zero = nan_zero;
    task.which = which ? 1 : 0;
    task.i_next = 0;
    task.mu = &mu;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    tp_worker_t* ws = (tp_worker_t*)calloc(nthreads, sizeof(tp_worker_t));
    for (int t = 0; t < nthreads; t++) {
        ws[t].shared = &task;
        ws[t].hist = (unsigned long long*)calloc(size, sizeof(unsigned long long));
        pthread_create(&th[t], NULL, geo_worker, &ws[t]);
    }
    unsigned long long ncalc = 0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        for (long b = 0; b < size; b++) hist[b] += ws[t].hist[b];
        ncalc += ws[t].ncalc;
        free(ws[t].hist);
    }
    free(ws);
    free(th);
    return ncalc;
}

/* Exact triangle-parametrization indices of one triangle (for tests of edge
 * cases).  Returns the three histogram indices or -999. */
void oracle_triangle_one(const float* p0, const float* p1, const float* p2, const float* lohi,
                         const int* nb, int nan_zero, int* out3) {
    tp_spec_t sp;
    for (int a = 0; a < 3; a++) {
        sp.lo[a] = lohi[2 * a];
        sp.hi[a] = lohi[2 * a + 1];
        sp.nb[a] = nb[a];
    }
    sp.nan_zero = nan_zero;
    tp_distance(p0[0], p0[1], p0[2], p1[0], p1[1], p1[2], p2[0], p2[1], p2[2], &sp, out3);
}

/* glibc acosf, exposed so tests can compare the engine's table-driven exact
 * acosf with the host libm the reference links against. */
float oracle_acosf(float c) { return acosf(c); }

/* ------------------------------------------------------------------------- */
/* 2pcf pair counts: src/2pcf_C_version.cc                                     */

typedef struct {
    const ocat_t* c;
    float lo, hi;
    int nbins, which;
    long i_next;
    pthread_mutex_t* mu;
} pr_task_t;

typedef struct {
    pr_task_t* shared;
    unsigned long long* hist;
    unsigned long long ncalc;
} pr_worker_t;

static void* pr_worker(void* arg) {
    pr_worker_t* w = (pr_worker_t*)arg;
    pr_task_t* t = w->shared;
    const ocat_t* c = t->c;
    for (;;) {
        long i0 = grab(&t->i_next, t->mu, 16);
        if (i0 >= c[0].n) break;
        long i1 = i0 + 16 < c[0].n ? i0 + 16 : c[0].n;
        for (long i = i0; i < i1; i++) {
            long jmin = (t->which == 0) ? i : 0; /* :365-370 */
            for (long j = jmin; j < c[1].n; j++) {
                float d = ref_dist(c[0].x[i], c[0].y[i], c[0].z[i], c[1].x[j], c[1].y[j], c[1].z[j]);
                w->ncalc++;
                int b = tp_bin(d, t->lo, t->hi, t->nbins, 0); /* distance_to_bin :57-86 */
                if (b >= 0 && b < t->nbins) w->hist[b]++;
            }
        }
    }
    return NULL;
}

/* Pair histogram with the reference loop (which = 0: j >= i, self pairs
 * included; which = 1: every ordered pair).  Returns the pairs visited. */
unsigned long long oracle_pair(const ocat_t* cats, int which, float lo, float hi, int nbins,
                               unsigned long long* hist, int nthreads) {
    memset(hist, 0, sizeof(unsigned long long) * nbins);
    if (nthreads < 1) nthreads = 1;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    pr_task_t task;
    task.c = cats;
    task.lo = lo;
    task.hi = hi;
    task.nbins = nbins;
    task.which = which ? 1 : 0;
    task.i_next = 0;
    task.mu = &mu;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    pr_worker_t* ws = (pr_worker_t*)calloc(nthreads, sizeof(pr_worker_t));
    for (int t = 0; t < nthreads; t++) {
        ws[t].shared = &task;
        ws[t].hist = (unsigned long long*)calloc(nbins, sizeof(unsigned long long));
        pthread_create(&th[t], NULL, pr_worker, &ws[t]);
    }
    unsigned long long ncalc = 0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        for (long b = 0; b < nbins; b++) hist[b] += ws[t].hist[b];
        ncalc += ws[t].ncalc;
        free(ws[t].hist);
    }
    free(ws);
    free(th);
    return ncalc;
}

/* ------------------------------------------------------------------------- */
/* Catalog readers with the reference's own fscanf loops.                      */
#include <stdio.h>

/* Header-count format, src/3pcf_C_version.cc:311-332: "%d" count, then count
 * lines "%f %f %f", each coordinate divided by scale_factor in float.
 * Returns the count read from the header, or -1 if the file cannot be opened.
 * At most cap points are stored. */
long oracle_read_header(const char* path, float scale_factor, float* x, float* y, float* z, long cap) {
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    int n = 0;
    if (fscanf(f, "%d", &n) != 1) n = 0;
    float t0 = 0, t1 = 0, t2 = 0;
    for (int j = 0; j < n; j++) {
        if (fscanf(f, "%f %f %f", &t0, &t1, &t2) == EOF) { /* values stay as last read */ }
        if (j < cap) {
            x[j] = t0 / scale_factor;
            y[j] = t1 / scale_factor;
            z[j] = t2 / scale_factor;
        }
    }
    fclose(f);
    return n;
}

/* Seven-column format, src/3pcf_C_version_triangle_parametrization.cc:364-394
 * (same loop in src/2pcf_C_version.cc:235-267): rows "%d %f %f %f %f %f %f"
 * until fscanf returns EOF; columns 5-7 are kept.  More than max_ngals rows is
 * a fatal error in the reference (returns -2 here); -1 if unopenable. */
long oracle_read_7col(const char* path, float* x, float* y, float* z, long cap) {
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    const long max_ngals = 1000000;
    long n = 0;
    int idummy;
    float dummy, t0 = 0, t1 = 0, t2 = 0;
    while (fscanf(f, "%d %f %f %f %f %f %f", &idummy, &dummy, &dummy, &dummy, &t0, &t1, &t2) != EOF) {
        if (n < cap) { x[n] = t0; y[n] = t1; z[n] = t2; }
        if (n >= max_ngals) { fclose(f); return -2; }
        n += 1;
    }
    fclose(f);
    return n;
}
