// Fixture generator (test infrastructure only): the sum over every -X V
// index-chunk run of the triangle-parametrization program on one catalog in
// all three roles (DDD or RRR), with each triangle binned by the reference's
// own distance() function.
//
// Built by tests/golden/make_lrg_rrr.py with
//   g++ -O1 -ffp-contract=off -fopenmp -Dmain=ref_main -include <configured copy> chunk_sum_driver.cc
// where the configured copy is oracle/_ref/src/<variant>.cc (oracle/ref_build.py),
// so that distance(), distance_to_bin() and the binning macros are the
// reference's, compiled here exactly as the reference binaries are.
//
// Why not run the reference binary 1000 times: one -X 10 chunk job of a
// 21,056-point catalog visits 1.56e9 triangles (~130 s), 36 CPU hours in all.
// The sum is the same when only triangles that can be counted are visited:
//  * chunk run (a, b, c) of src/3pcf_C_version_triangle_parametrization.cc:477-533
//    (which == 0) counts the ordered triple (p, q, r), p in chunk a, q in b,
//    r in c, when loc(q) >= loc(p) and loc(r) >= loc(q), loc being the index
//    inside the point's chunk (vox2gal, :52-80).  Over all V^3 chunk runs an
//    unordered triangle {p, q, r} is therefore counted once for each of its
//    six orderings whose chunk-local indices are non-decreasing;
//  * a permutation is counted only if s < S_HI and q < Q_HI, so every side of
//    a counted triangle is below S_HI * (1 + Q_HI) (triangle inequality);
//    triangles with a longer side add nothing and are skipped;
//  * triples with a repeated point have a zero side and add nothing.
#undef main
#include <omp.h>
#include <stdint.h>
#include <vector>

static float *PX, *PY, *PZ;
static int NP;

static int local_index(int p, int div)
{
    if (div <= 0) return p;
    int per = NP / div;
    int c = p / per;
    if (c >= div) c = div - 1;
    return p - per * c;
}

static float side(int a, int b)
{
    float dx = PX[a] - PX[b], dy = PY[a] - PY[b], dz = PZ[a] - PZ[b];
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s points.f32 division\n", argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    fseek(f, 0, SEEK_END);
    long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    NP = (int)(bytes / 12);
    std::vector<float> xyz(3 * (size_t)NP);
    if (fread(xyz.data(), 12, NP, f) != (size_t)NP) return 2;
    fclose(f);
    std::vector<float> X(NP), Y(NP), Z(NP);
    for (int i = 0; i < NP; i++) {
        X[i] = xyz[3 * i];
        Y[i] = xyz[3 * i + 1];
        Z[i] = xyz[3 * i + 2];
    }
    PX = X.data();
    PY = Y.data();
    PZ = Z.data();
    const int div = atoi(argv[2]);
    const int nbins = S_NBINS * Q_NBINS * THETA_NBINS;
    const float reach = (float)(S_HI * (1.0 + Q_HI) * 1.001);
    const int nthreads = omp_get_max_threads();
    std::vector<uint64_t> hist((size_t)nthreads * nbins, 0);
    static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

#pragma omp parallel
    {
        uint64_t *h = &hist[(size_t)omp_get_thread_num() * nbins];
        std::vector<int> near;
#pragma omp for schedule(dynamic, 16)
        for (int a = 0; a < NP; a++) {
            near.clear();
            for (int b = a + 1; b < NP; b++) {
                if (fabsf(PY[b] - PY[a]) >= reach) continue;
                if (side(a, b) < reach) near.push_back(b);
            }
            for (size_t u = 0; u < near.size(); u++) {
                for (size_t v = u + 1; v < near.size(); v++) {
                    int b = near[u], c = near[v];
                    if (side(b, c) >= reach) continue;
                    int id[3] = {a, b, c};
                    int mult = 0;
                    for (int t = 0; t < 6; t++) {
                        int li = local_index(id[perm[t][0]], div);
                        int lj = local_index(id[perm[t][1]], div);
                        int lk = local_index(id[perm[t][2]], div);
                        if (lj >= li && lk >= lj) mult++;
                    }
                    if (!mult) continue;
                    int bins[3];
                    distance(PX[a], PY[a], PZ[a], PX[b], PY[b], PZ[b], PX[c], PY[c], PZ[c], 0, bins);
                    for (int k = 0; k < 3; k++)
                        if (bins[k] >= 0) h[bins[k]] += mult;
                }
            }
        }
    }
    for (int b = 0; b < nbins; b++) {
        uint64_t s = 0;
        for (int t = 0; t < nthreads; t++) s += hist[(size_t)t * nbins + b];
        printf("%llu\n", (unsigned long long)s);
    }
    return 0;
}
