// sum_voxels.cpp -- adds triangle-parametrization histogram files of voxel
// jobs, with the output of examples/sum_voxels.py (:1-56) byte for byte:
//   * every file is read as whitespace-separated tokens; the galaxy counts
//     (tokens 0-2), bin counts (3-5) and axis lines (6-14) of the LAST file are
//     printed; the counts (15...) of all files are added as doubles;
//   * "%d\n" per galaxy count, "%d %d %d\n", "%-6.3f %-6.3f %-6.3f\n" per axis,
//     then S*Q rows of T "%d " values each ending in "\n", and the newline
//     Python's print statement appends.
// Host-only tool (no GPU).  Usage: tpcf_sum_voxels FILE... > merged.dat
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <vector>

namespace {

bool read_tokens(const char* path, std::vector<std::string>& tok) {
    FILE* f = fopen(path, "r");
    if (!f) return false;
    tok.clear();
    std::string cur;
    int c;
    while ((c = fgetc(f)) != EOF) {
        if (c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f') {
            if (!cur.empty()) tok.push_back(cur);
            cur.clear();
        } else {
            cur.push_back((char)c);
        }
    }
    if (!cur.empty()) tok.push_back(cur);
    fclose(f);
    return true;
}

bool to_long(const std::string& s, long long* v) {
    char* end = nullptr;
    *v = strtoll(s.c_str(), &end, 10);
    return end && *end == 0;
}

bool to_double(const std::string& s, double* v) {
    char* end = nullptr;
    *v = strtod(s.c_str(), &end);
    return end && *end == 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s FILE...\n", argv[0]);
        return 1;
    }
    long long ngals[3] = {0, 0, 0}, nbins[3] = {0, 0, 0};
    double hv[3][3] = {{0}};
    std::vector<double> tot;
    std::vector<std::string> tok;
    for (int a = 1; a < argc; a++) {
        if (!read_tokens(argv[a], tok)) {
            fprintf(stderr, "cannot read %s\n", argv[a]);
            return 1;
        }
        if (tok.size() < 15) {
            fprintf(stderr, "%s: not a histogram file\n", argv[a]);
            return 1;
        }
        for (int i = 0; i < 3; i++)
            if (!to_long(tok[i], &ngals[i]) || !to_long(tok[3 + i], &nbins[i])) {
                fprintf(stderr, "%s: bad header\n", argv[a]);
                return 1;
            }
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++)
                if (!to_double(tok[6 + 3 * i + k], &hv[i][k])) {
                    fprintf(stderr, "%s: bad axis line\n", argv[a]);
                    return 1;
                }
        const size_t n = tok.size() - 15;
        if (a == 1) tot.assign(n, 0.0);
        if (n != tot.size()) {
            fprintf(stderr, "%s: %zu counts, expected %zu\n", argv[a], n, tot.size());
            return 1;
        }
        for (size_t b = 0; b < n; b++) {
            double v;
            if (!to_double(tok[15 + b], &v)) {
                fprintf(stderr, "%s: bad count\n", argv[a]);
                return 1;
            }
            tot[b] += v;
        }
    }
    if ((long long)tot.size() != nbins[0] * nbins[1] * nbins[2]) {
        fprintf(stderr, "counts do not match the bin numbers\n");
        return 1;
    }
    for (int i = 0; i < 3; i++) printf("%lld\n", ngals[i]);
    printf("%lld %lld %lld\n", nbins[0], nbins[1], nbins[2]);
    for (int i = 0; i < 3; i++) printf("%-6.3f %-6.3f %-6.3f\n", hv[i][0], hv[i][1], hv[i][2]);
    size_t b = 0;
    for (long long i = 0; i < nbins[0]; i++)
        for (long long j = 0; j < nbins[1]; j++) {
            for (long long k = 0; k < nbins[2]; k++) printf("%lld ", (long long)tot[b++]);
            printf("\n");
        }
    printf("\n");
    return 0;
}
