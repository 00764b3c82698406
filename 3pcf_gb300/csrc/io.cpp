// io.cpp -- reference catalog files (tpcf_read_catalog of include/tpcf.h).
//
// Reads with the same fscanf conversions as the reference programs, so that the
// floats (and the row count, including the reference's handling of short or
// malformed rows) are identical:
//   header-count format  src/3pcf_C_version.cc:311-332
//   seven-column format  src/3pcf_C_version_triangle_parametrization.cc:364-394,
//                        src/2pcf_C_version.cc:235-267
#include "../../include/tpcf.h"

#include <stdio.h>

extern "C" tpcf_status tpcf_read_catalog(const char* path, int32_t format, float scale_factor, float* x, float* y,
                                         float* z, int64_t* n) {
    if (!path || !n) return TPCF_ERR_INVALID;
    FILE* f = fopen(path, "r");
    if (!f) return TPCF_ERR_IO;
    const bool store = x && y && z;
    const int64_t cap = store ? *n : 0;
    if (format == 0) {
        int count = 0;
        if (fscanf(f, "%d", &count) != 1 || count < 0) count = 0;
        float t0 = 0, t1 = 0, t2 = 0;
        for (int j = 0; j < count; j++) {
            if (fscanf(f, "%f %f %f", &t0, &t1, &t2) == EOF) {
                // the reference keeps the previous values
            }
            if (store && j < cap) {
                x[j] = t0 / scale_factor;
                y[j] = t1 / scale_factor;
                z[j] = t2 / scale_factor;
            }
        }
        fclose(f);
        *n = count;
        return TPCF_OK;
    }
    if (format == 1) {
        const int64_t max_ngals = 1000000;
        int64_t rows = 0;
        int idummy;
        float dummy, t0 = 0, t1 = 0, t2 = 0;
        while (fscanf(f, "%d %f %f %f %f %f %f", &idummy, &dummy, &dummy, &dummy, &t0, &t1, &t2) != EOF) {
            if (rows >= max_ngals) {  // "Exceeded max num galaxies", :382-386
                fclose(f);
                return TPCF_ERR_INVALID;
            }
            if (store && rows < cap) {
                x[rows] = t0;
                y[rows] = t1;
                z[rows] = t2;
            }
            rows++;
        }
        fclose(f);
        *n = rows;
        return TPCF_OK;
    }
    fclose(f);
    return TPCF_ERR_INVALID;
}
