// cli.cpp -- command-line shims with the reference programs' interface.
//
// Built four times (TPCF_PROGRAM = 0, 1, 2, 3) as
//   tpcf_3side  <- src/3pcf_C_version.cc main()                       (:147-466)
//   tpcf_tp     <- src/3pcf_C_version_triangle_parametrization.cc main() (:245-571)
//   tpcf_2pcf   <- src/2pcf_C_version.cc main()                       (:118-410)
//   tpcf_jbj    <- src/3pcf_C_version_triangle_parametrization_JBJ.cc main() (:240-560)
// Same short options (GNU getopt, so options may follow the catalogs as the
// reference's csh drivers pass them), same positional catalogs, same loop mode
// from argv string identity, same -X/-x index chunks, same default output name
// and byte-identical output files.  The binning, fixed by #define in the
// reference, defaults to the reference's values and can be changed with long
// options.  Counting runs on the GPU through include/tpcf.h.
#include "../../include/tpcf.h"

#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <string>
#include <vector>

#ifndef TPCF_PROGRAM
#define TPCF_PROGRAM 1
#endif

namespace {

struct Axis {
    int n;
    double lo, hi;  // the reference's macro values (double), converted to float for counting
};

enum {
    OPT_NBINS = 1000,
    OPT_HMIN,
    OPT_HMAX,
    OPT_CLEAN,
    OPT_S,
    OPT_Q,
    OPT_T,
    OPT_FP64,
    OPT_NOPRUNE,
    OPT_NAN,
    OPT_DEVICE,
    OPT_QUIET
};

bool parse_axis(const char* s, Axis* a) {
    // "nbins,lo,hi"
    int n;
    double lo, hi;
    if (sscanf(s, "%d,%lf,%lf", &n, &lo, &hi) != 3) return false;
    a->n = n;
    a->lo = lo;
    a->hi = hi;
    return true;
}

void die(tpcf_ctx* ctx, tpcf_status s, const char* what) {
    fprintf(stderr, "%s: %s (%s)\n", what, tpcf_status_string(s), tpcf_last_error(ctx));
    exit(2);
}

struct Loaded {
    uint64_t handle;
    int64_t n;
};

}  // namespace

int main(int argc, char** argv) {
    const int program = TPCF_PROGRAM;  // 0 three-side, 1 triangle, 2 pairs, 3 JBJ
    char* outfilename = nullptr;
    char defaultout[256];
    snprintf(defaultout, sizeof(defaultout), program == 2 ? "default_out_2pcf.dat" : "default_out.dat");
    float scale_factor = 1.0f;
    int voxel_division = -999, vtemp = -999;
    // reference binning defaults
    Axis three{64, 0.0, sqrt(3 * 24 * 24)};              // src/3pcf_C_version.cc:169-173
    Axis S{50, 2.0, 12.0}, Q{16, 0.9, 4.1}, T{32, 0., 1.};  // :31-42
    Axis P{700, 0.0, 70.0};                               // src/2pcf_C_version.cc:14-16
    int clean = 0, fp64 = 0, prune = 1, device = 0, quiet = 0;
#if defined(__aarch64__)
    int nan_policy = TPCF_NAN_ZERO;  // what int(NaN) gives where this binary runs
#else
    int nan_policy = TPCF_NAN_INT_MIN;
#endif
    static struct option longopts[] = {
        {"nbins", required_argument, 0, OPT_NBINS},   {"hist-min", required_argument, 0, OPT_HMIN},
        {"hist-max", required_argument, 0, OPT_HMAX}, {"clean", no_argument, 0, OPT_CLEAN},
        {"s-axis", required_argument, 0, OPT_S},      {"q-axis", required_argument, 0, OPT_Q},
        {"theta-axis", required_argument, 0, OPT_T},  {"pair-axis", required_argument, 0, OPT_S},
        {"fp64", no_argument, 0, OPT_FP64},           {"no-prune", no_argument, 0, OPT_NOPRUNE},
        {"nan-policy", required_argument, 0, OPT_NAN}, {"device", required_argument, 0, OPT_DEVICE},
        {"quiet", no_argument, 0, OPT_QUIET},         {0, 0, 0, 0}};
    const char* shortopts = program == 0 ? "ao:L:l:w:sm" : "ao:l:x:X:";
    int c;
    while ((c = getopt_long(argc, argv, shortopts, longopts, nullptr)) != -1) {
        switch (c) {
            case 'o': outfilename = optarg; break;
            case 's': scale_factor = 206264.0f; break;        // arcseconds, :195-201
            case 'm': scale_factor = 3437.74677f; break;      // arcminutes, :202-208
            case 'L': case 'w': case 'l': case 'a': break;    // parsed, no effect on binning (:183-194)
            case 'X': voxel_division = atoi(optarg); break;
            case 'x': vtemp = atoi(optarg); break;
            case OPT_NBINS: three.n = atoi(optarg); break;
            case OPT_HMIN: three.lo = atof(optarg); break;
            case OPT_HMAX: three.hi = atof(optarg); break;
            case OPT_CLEAN: clean = 1; break;
            case OPT_S:
                if (!parse_axis(optarg, program == 2 ? &P : &S)) { fprintf(stderr, "bad axis %s\n", optarg); return 1; }
                break;
            case OPT_Q:
                if (!parse_axis(optarg, &Q)) { fprintf(stderr, "bad axis %s\n", optarg); return 1; }
                break;
            case OPT_T:
                if (!parse_axis(optarg, &T)) { fprintf(stderr, "bad axis %s\n", optarg); return 1; }
                break;
            case OPT_FP64: fp64 = 1; break;
            case OPT_NOPRUNE: prune = 0; break;
            case OPT_NAN:
                nan_policy = strcmp(optarg, "zero") == 0 ? TPCF_NAN_ZERO : TPCF_NAN_INT_MIN;
                break;
            case OPT_DEVICE: device = atoi(optarg); break;
            case OPT_QUIET: quiet = 1; break;
            case '?': printf("unknown arg %c\n", optopt); break;
        }
    }
    const int ncat = program == 2 ? 2 : 3;
    if (argc < (program == 2 ? 2 : 3)) {
        printf("\nMust pass in at least %s input files on command line!\n", program == 2 ? "two" : "three");
        printf("\nUsage: ");
        exit(1);
    }
    if (argc - optind < ncat) {
        fprintf(stderr, "need %d catalog files\n", ncat);
        return 1;
    }
    if (!outfilename) outfilename = defaultout;
    const char* names[3] = {argv[optind], argv[optind + 1], ncat == 3 ? argv[optind + 2] : argv[optind + 1]};
    int voxel_index[3] = {0, 0, 0};
    if (program != 0 && voxel_division > 0) {
        voxel_index[0] = vtemp / 1000000;
        voxel_index[1] = (vtemp / 1000) % 1000;
        voxel_index[2] = vtemp % 1000;
    }
    // loop mode from argv string identity (the reference's which_three_input_files,
    // kept in a bool), :333-353 and src/2pcf_C_version.cc:214-224
    int which = 0;
    if (ncat == 3) {
        int w = 0;
        if (strcmp(names[0], names[1]) == 0 && strcmp(names[0], names[2]) == 0) w = 0;
        else if (strcmp(names[0], names[1]) != 0 && strcmp(names[1], names[2]) == 0) w = 1;
        else if (strcmp(names[0], names[1]) == 0 && strcmp(names[0], names[2]) != 0) w = 2;
        which = w ? 1 : 0;
    } else {
        which = strcmp(names[0], names[1]) == 0 ? 0 : 1;
    }

    tpcf_ctx* ctx = nullptr;
    tpcf_status st = tpcf_create(&ctx, device);
    if (st != TPCF_OK) die(nullptr, st, "tpcf_create");
    std::map<std::string, Loaded> loaded;
    int64_t ngal[3] = {0, 0, 0};
    tpcf_job job;
    memset(&job, 0, sizeof(job));
    for (int r = 0; r < ncat; r++) {
        std::string name = names[r];
        if (!loaded.count(name)) {
            int64_t n = 0;
            int fmt = program == 0 ? 0 : 1;
            st = tpcf_read_catalog(name.c_str(), fmt, scale_factor, nullptr, nullptr, nullptr, &n);
            if (st == TPCF_ERR_INVALID && fmt == 1) {
                printf("Exceeded max num galaxies");
                exit(-1);
            }
            if (st != TPCF_OK) {
                fprintf(stderr, "cannot read %s\n", name.c_str());
                return 1;
            }
            std::vector<float> x(n > 0 ? n : 1), y(n > 0 ? n : 1), z(n > 0 ? n : 1);
            st = tpcf_read_catalog(name.c_str(), fmt, scale_factor, x.data(), y.data(), z.data(), &n);
            if (st != TPCF_OK) die(ctx, st, "read");
            uint64_t h = 0;
            st = tpcf_catalog_create(ctx, x.data(), y.data(), z.data(), n, &h);
            if (st != TPCF_OK) die(ctx, st, "tpcf_catalog_create");
            loaded[name] = Loaded{h, n};
        }
        const Loaded& L = loaded[name];
        ngal[r] = L.n;
        job.catalog[r] = L.handle;
        job.begin[r] = 0;
        job.end[r] = L.n;
        if (program != 0 && voxel_division > 0 && vtemp >= 0) {
            // vox2gal, :52-80
            int per = (int)(L.n / voxel_division);
            if (per == 0) {
                printf("Voxel chunks are bigger than the number of galaxies!");
                exit(-1);
            }
            int lo = per * voxel_index[r];
            int hi = per * (voxel_index[r] + 1);
            if (voxel_index[r] == voxel_division - 1) hi += (int)(L.n % voxel_division);
            job.begin[r] = lo;
            job.end[r] = hi;
        }
    }
    if (ncat == 2) {
        job.catalog[2] = job.catalog[1];
        job.begin[2] = job.begin[1];
        job.end[2] = job.end[1];
    }
    tpcf_spec spec;
    memset(&spec, 0, sizeof(spec));
    spec.precision = fp64 ? TPCF_PLAIN_FP64 : TPCF_GUARDED_FP32;
    spec.nan_policy = nan_policy;
    spec.prune = prune;
    if (program == 0) {
        spec.kind = TPCF_THREE_SIDE;
        spec.loop = TPCF_LOOP_ALL;
        spec.overflow = clean ? TPCF_OVERFLOW_CLEAN : TPCF_OVERFLOW_COMPAT;
        spec.axis[0] = tpcf_axis{(float)three.lo, (float)three.hi, three.n};
    } else if (program == 1 || program == 3) {
        spec.kind = program == 1 ? TPCF_TRIANGLE : TPCF_TRIANGLE_JBJ;
        spec.loop = which ? TPCF_LOOP_ONE : TPCF_LOOP_SAME;
        spec.overflow = clean ? TPCF_OVERFLOW_CLEAN : TPCF_OVERFLOW_COMPAT;  // JBJ: bin-0 extra counts
        spec.axis[0] = tpcf_axis{(float)S.lo, (float)S.hi, S.n};
        spec.axis[1] = tpcf_axis{(float)Q.lo, (float)Q.hi, Q.n};
        spec.axis[2] = tpcf_axis{(float)T.lo, (float)T.hi, T.n};
    } else {
        spec.kind = TPCF_PAIR;
        spec.loop = which ? TPCF_LOOP_ONE : TPCF_LOOP_SAME;
        spec.axis[0] = tpcf_axis{(float)P.lo, (float)P.hi, P.n};
    }
    int64_t len = 0;
    tpcf_hist_len(&spec, &len);
    std::vector<uint64_t> hist(len > 0 ? len : 1);
    st = tpcf_count(ctx, &spec, &job, hist.data(), len);
    if (st != TPCF_OK) die(ctx, st, "tpcf_count");
    if (!quiet) {
        tpcf_stats stats;
        tpcf_last_stats(ctx, &stats);
        printf("triangles(loop)=%llu evaluated=%llu rechecked=%llu kernel_ms=%.3f\n",
               (unsigned long long)stats.loop_units, (unsigned long long)stats.evaluated_units,
               (unsigned long long)stats.recheck_units, stats.kernel_ms);
    }
    FILE* out = fopen(outfilename, "w");
    if (!out) {
        fprintf(stderr, "cannot write %s\n", outfilename);
        return 1;
    }
    if (program == 0) {
        // :440-460
        int n = three.n;
        fprintf(out, "%d %d %d\n", n, n, n);
        for (int i = 0; i < n; i++) {
            fprintf(out, "%d\n", i);
            for (int j = 0; j < n; j++) {
                for (int k = 0; k < n; k++) fprintf(out, "%llu ", (unsigned long long)hist[(size_t)n * n * k + (size_t)n * j + i]);
                fprintf(out, "\n");
            }
        }
    } else if (program == 1 || program == 3) {
        // :537-569 (JBJ: :527-553); counts are the reference's unsigned int (wrap mod 2^32)
        fprintf(out, "%lld\n%lld\n%lld\n", (long long)ngal[0], (long long)ngal[1], (long long)ngal[2]);
        fprintf(out, "%d %d %d\n", S.n, Q.n, T.n);
        fprintf(out, "%-6.3f %-6.3f %-6.3f\n", S.lo, S.hi, (S.hi - S.lo) / S.n);
        fprintf(out, "%-6.3f %-6.3f %-6.3f\n", Q.lo, Q.hi, (Q.hi - Q.lo) / Q.n);
        fprintf(out, "%-6.3f %-6.3f %-6.3f\n", T.lo, T.hi, (T.hi - T.lo) / T.n);
        for (int i = 0; i < S.n; i++)
            for (int j = 0; j < Q.n; j++) {
                for (int k = 0; k < T.n; k++)
                    fprintf(out, "%u ", (unsigned)(uint32_t)hist[(size_t)Q.n * T.n * i + (size_t)T.n * j + k]);
                fprintf(out, "\n");
            }
    } else {
        // src/2pcf_C_version.cc:391-404
        fprintf(out, "%lld\n%lld\n%d\n", (long long)ngal[0], (long long)ngal[1], P.n);
        fprintf(out, "%-6.3f %-6.3f %-6.3f\n", P.lo, P.hi, (P.hi - P.lo) / P.n);
        for (int i = 0; i < P.n; i++) fprintf(out, "%u\n", (unsigned)(uint32_t)hist[i]);
    }
    fclose(out);
    tpcf_destroy(ctx);
    return 0;
}
