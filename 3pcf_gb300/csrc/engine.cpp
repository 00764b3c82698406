// engine.cpp -- host side of the counting engine: the C ABI of include/tpcf.h.
//
// Responsibilities
//   * catalogs: host copy + device-resident float4 points;
//   * spatial views: a catalog range is reordered by a balanced k-d split into
//     tiles of exactly TILE points (last tile partial), each with an
//     axis-aligned bounding box; cached per (catalog, range);
//   * task planning: the reference's loop nest becomes a list of tile triples
//     (pairs).  Symmetric loop nests (DDD/RRR: i<=j<=k over one array; DRR: j<=k
//     over one array; DDR: i,j over one array) are enumerated canonically so
//     that each unordered set of points is visited once; everything else is
//     enumerated as ordered tile triples with the reference's index predicate
//     evaluated per triangle.  Tile triples whose bounding boxes prove that no
//     triangle can reach a counted bin are skipped (exact: a rigorous lower
//     bound on every side is compared with the largest side any counted
//     triangle can have);
//   * launches: one persistent kernel per (kind, binning, precision) group,
//     then the exact recheck of guard-band triangles, then D2H of the counts;
//   * glibc acosf exception table for exact theta (built from the host libm by
//     an exhaustive scan of [-1, 1], cached on disk);
//   * serving: submit/wait with a worker thread that batches every pending job
//     of compatible binning into the next launch (continuous batching), with
//     admission by device-memory footprint.
#include "../../include/tpcf.h"
#include "engine.h"
#include "exact_acos.h"

#include <cuda_runtime.h>
#include <dlfcn.h>
#include <gnu/libc-version.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <climits>
#include <cstdint>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <functional>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

using namespace tpcf;

namespace {

thread_local std::string g_tls_error;

struct CudaError {
    cudaError_t e;
};

#define CK(x)                                             \
    do {                                                  \
        cudaError_t _e = (x);                             \
        if (_e != cudaSuccess) throw CudaError{_e};       \
    } while (0)

struct InvalidArg {
    std::string msg;
};

// ---------------------------------------------------------------------------
// device buffers

// Freed device blocks up to 64 MiB are kept per device and power-of-two size
// class for reuse (at most 2 GiB in all), so that the catalogs, views and
// task lists of a repeated upload-count-release cycle cost no cudaMalloc /
// cudaFree (each of which also synchronises the device).  A block is only
// freed once nothing can still use it: views and scratch buffers are released
// after the work that read them has completed on its stream.
class DeviceBlocks {
  public:
    static DeviceBlocks& get() {
        static DeviceBlocks* d = new DeviceBlocks();  // never destroyed: blocks live until the process ends
        return *d;
    }
    void* alloc(size_t bytes, size_t* cap) {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        size_t cls = 256;
        while (cls < bytes) cls <<= 1;
        if (cls > kMaxCached) {
            void* p = nullptr;
            CK(cudaMalloc(&p, bytes));
            *cap = bytes;
            return p;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto& v = free_[std::make_pair(dev, cls)];
            if (!v.empty()) {
                void* p = v.back();
                v.pop_back();
                cached_ -= cls;
                *cap = cls;
                return p;
            }
        }
        void* p = nullptr;
        if (cudaMalloc(&p, cls) != cudaSuccess) {
            // out of memory: give the kept blocks back and try once more
            (void)cudaGetLastError();
            trim();
            CK(cudaMalloc(&p, cls));
        }
        *cap = cls;
        return p;
    }
    void trim() {
        std::lock_guard<std::mutex> lk(mu_);
        int dev = 0;
        cudaGetDevice(&dev);
        for (auto& kv : free_) {
            if (kv.first.first != dev) continue;
            for (void* q : kv.second) cudaFree(q);
            cached_ -= kv.first.second * kv.second.size();
            kv.second.clear();
        }
    }
    void release(void* p, size_t cap) {
        if (!p) return;
        int dev = 0;
        if (cap <= kMaxCached && cudaGetDevice(&dev) == cudaSuccess) {
            std::lock_guard<std::mutex> lk(mu_);
            if (cached_ + cap <= kMaxTotal) {
                free_[std::make_pair(dev, cap)].push_back(p);
                cached_ += cap;
                return;
            }
        }
        cudaFree(p);
    }

  private:
    static constexpr size_t kMaxCached = (size_t)64 << 20, kMaxTotal = (size_t)2 << 30;
    std::mutex mu_;
    std::map<std::pair<int, size_t>, std::vector<void*>> free_;
    size_t cached_ = 0;
};

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    size_t cap = 0;  // bytes of the block
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        DeviceBlocks::get().release(p, cap);
        p = nullptr;
        n = 0;
        cap = 0;
    }
    void reserve(size_t m) {
        if (m <= n) return;
        release();
        p = (T*)DeviceBlocks::get().alloc(std::max<size_t>(m, 1) * sizeof(T), &cap);
        n = m;
    }
    size_t bytes() const { return n * sizeof(T); }
    void swap(DevBuf& o) {
        std::swap(p, o.p);
        std::swap(n, o.n);
        std::swap(cap, o.cap);
    }
};

// Page-locked host buffer (device-to-host copies inside captured graphs need one).
template <typename T>
struct PinnedBuf {
    T* p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { release(); }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
    // grows to a power of two: cudaFreeHost waits for all work on the device,
    // so a serving lane that reallocated for every new batch size would wait
    // for the other lanes' kernels
    void reserve(size_t m) {
        if (m <= n) return;
        release();
        size_t c = 4096;
        while (c < m) c <<= 1;
        CK(cudaMallocHost((void**)&p, c * sizeof(T)));
        n = c;
    }
};

struct Box {
    float lo[3], hi[3];
};

struct Catalog {
    std::vector<float> x, y, z;
    int64_t n = 0;
};

struct View {
    uint64_t id = 0;  // unique per view object (plan cache key)
    int64_t n = 0;
    int ntiles = 0;
    DevBuf<float4> pts;          // sorted points, .w = loop index (int bits)
    DevBuf<int32_t> tile_start;  // ntiles + 1
    std::vector<int32_t> h_tile_start;
    std::vector<Box> boxes;
    size_t upload_bytes = 0;  // host-to-device bytes of its construction
    size_t bytes() const { return pts.bytes() + tile_start.bytes(); }
};

// One split of order[lo, hi): along the widest axis, so that the left part
// holds a multiple of `tile` points.  Returns the split point, or -1 for a
// part of at most `tile` points (a leaf).
int64_t kd_split(const float* xyz, std::vector<int32_t>& order, int64_t lo, int64_t hi, int tile) {
    int64_t n = hi - lo;
    if (n <= tile) return -1;
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = lo; i < hi; i++)
        for (int a = 0; a < 3; a++) {
            float v = xyz[3 * (int64_t)order[i] + a];
            mn[a] = std::min(mn[a], v);
            mx[a] = std::max(mx[a], v);
        }
    int ax = 0;
    for (int a = 1; a < 3; a++)
        if (mx[a] - mn[a] > mx[ax] - mn[ax]) ax = a;
    int64_t ntile = (n + tile - 1) / tile;
    int64_t left = ((ntile + 1) / 2) * tile;
    if (left >= n) left = n - tile;
    // the split coordinate beside each index, contiguous, so that the
    // selection compares without gathering from xyz (a NaN coordinate sorts
    // as +inf: the order stays a strict weak one)
    static thread_local std::vector<std::pair<float, int32_t>> keys;
    keys.resize((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        const float v = xyz[3 * (int64_t)order[lo + i] + ax];
        keys[i] = {std::isnan(v) ? INFINITY : v, order[lo + i]};
    }
    std::nth_element(keys.begin(), keys.begin() + left, keys.begin() + n);  // (coordinate, index) order
    for (int64_t i = 0; i < n; i++) order[lo + i] = keys[i].second;
    return lo + left;
}

void parallel_items(size_t n, const std::function<void(size_t)>& fn);

// Balanced k-d split of order[0, n) until parts hold at most `tile` points;
// leaves appear in order, giving spatially compact tiles.  Level by level,
// the parts of a level split in parallel (each split is deterministic, so the
// order does not depend on the threads).
void kd_order(const float* xyz, std::vector<int32_t>& order, int64_t n, int tile) {
    std::vector<std::pair<int64_t, int64_t>> level{{0, n}};
    while (!level.empty()) {
        std::vector<int64_t> mids(level.size(), -1);
        auto split = [&](size_t i) { mids[i] = kd_split(xyz, order, level[i].first, level[i].second, tile); };
        if (level.size() < 4 || n < 4096) {
            for (size_t i = 0; i < level.size(); i++) split(i);
        } else {
            parallel_items(level.size(), split);
        }
        std::vector<std::pair<int64_t, int64_t>> next;
        for (size_t i = 0; i < level.size(); i++)
            if (mids[i] >= 0) {
                next.push_back({level[i].first, mids[i]});
                next.push_back({mids[i], level[i].second});
            }
        level.swap(next);
    }
}

// Lower bound on the reference's float side length between any point of box
// a and any point of box b (computed in double, then reduced by a relative
// margin that covers the float rounding of the reference's distance).
double box_lower_bound(const Box& a, const Box& b) {
    double s = 0;
    for (int k = 0; k < 3; k++) {
        double g = std::max({0.0, (double)a.lo[k] - (double)b.hi[k], (double)b.lo[k] - (double)a.hi[k]});
        s += g * g;
    }
    return sqrt(s) * (1.0 - 1e-5);
}

// Upper bound on the reference's float side length between box a and box b.
double box_upper_bound(const Box& a, const Box& b) {
    double s = 0;
    for (int k = 0; k < 3; k++) {
        double g = std::max((double)a.hi[k] - (double)b.lo[k], (double)b.hi[k] - (double)a.lo[k]);
        s += g * g;
    }
    return sqrt(s) * (1.0 + 1e-5) + 1e-30;
}

// ---------------------------------------------------------------------------
// exact glibc acosf exception table

struct AcosHost {
    std::vector<uint32_t> keys, vals, bucket;
};

std::string cache_dir() {
    const char* env = getenv("TPCF_CACHE_DIR");
    if (env && *env) return env;
    Dl_info info;
    if (dladdr((void*)&cache_dir, &info) && info.dli_fname) {
        std::string p = info.dli_fname;
        size_t s = p.rfind('/');
        std::string dir = s == std::string::npos ? "." : p.substr(0, s);
        return dir + "/../_cache";
    }
    return "/tmp/tpcf_cache";
}

void mkdirs(const std::string& d) {
    std::string cur;
    for (size_t i = 0; i < d.size(); i++) {
        cur += d[i];
        if (d[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
    }
    mkdir(d.c_str(), 0755);
}

uint32_t fbits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
float ffrom(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Exhaustive scan of every float c in [-1, 1]: record where the host libm's
// acosf differs from (float)tpcf_acos_d(c).
AcosHost build_acos_table() {
    const uint32_t spans[2][2] = {{0x00000000u, 0x3f800001u}, {0x80000000u, 0xbf800001u}};
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    const uint32_t chunks = 512;
    struct Part {
        std::vector<uint32_t> k, v;
    };
    std::vector<Part> parts(2 * chunks);
    std::atomic<uint32_t> next(0);
    auto work = [&]() {
        for (;;) {
            uint32_t c = next.fetch_add(1);
            if (c >= 2 * chunks) break;
            uint32_t side = c / chunks, part = c % chunks;
            uint64_t lo = spans[side][0], hi = spans[side][1];
            uint64_t len = hi - lo;
            uint64_t a = lo + len * part / chunks, b = lo + len * (part + 1) / chunks;
            Part& P = parts[c];
            for (uint64_t u = a; u < b; u++) {
                float x = ffrom((uint32_t)u);
                float g = acosf(x);
                float r = (float)tpcf_acos_d((double)x);
                if (fbits(g) != fbits(r)) {
                    P.k.push_back((uint32_t)u);
                    P.v.push_back(fbits(g));
                }
            }
        }
    };
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++) th.emplace_back(work);
    for (auto& t : th) t.join();
    AcosHost h;
    for (auto& P : parts) {
        h.keys.insert(h.keys.end(), P.k.begin(), P.k.end());
        h.vals.insert(h.vals.end(), P.v.begin(), P.v.end());
    }
    h.bucket.assign(65537, 0);
    size_t i = 0;
    for (uint32_t b = 0; b <= 65536; b++) {
        while (i < h.keys.size() && (h.keys[i] >> 16) < b) i++;
        h.bucket[b] = (uint32_t)i;
    }
    return h;
}

std::string acos_cache_path() {
    char name[256];
    // the table depends on the C library's acosf, the architecture and this
    // file's tpcf_acos_d; a probe value keys the latter
    uint32_t probe = fbits((float)tpcf_acos_d(0.3)) ^ fbits((float)tpcf_acos_d(-0.87));
#if defined(__aarch64__)
    const char* arch = "aarch64";
#elif defined(__x86_64__)
    const char* arch = "x86_64";
#else
    const char* arch = "other";
#endif
    snprintf(name, sizeof(name), "/acosf_exc_v1_%s_glibc%s_%08x.bin", arch, gnu_get_libc_version(), probe);
    return cache_dir() + name;
}

AcosHost load_or_build_acos_table() {
    std::string path = acos_cache_path();
    FILE* f = fopen(path.c_str(), "rb");
    if (f) {
        AcosHost h;
        uint32_t n = 0;
        bool ok = fread(&n, 4, 1, f) == 1 && n < (1u << 28);
        if (ok) {
            h.keys.resize(n);
            h.vals.resize(n);
            h.bucket.resize(65537);
            ok = fread(h.keys.data(), 4, n, f) == n && fread(h.vals.data(), 4, n, f) == n &&
                 fread(h.bucket.data(), 4, 65537, f) == 65537;
        }
        fclose(f);
        if (ok) return h;
    }
    AcosHost h = build_acos_table();
    mkdirs(cache_dir());
    std::string tmp = path + ".tmp" + std::to_string(getpid());
    f = fopen(tmp.c_str(), "wb");
    if (f) {
        uint32_t n = (uint32_t)h.keys.size();
        bool ok = fwrite(&n, 4, 1, f) == 1 && fwrite(h.keys.data(), 4, n, f) == n &&
                  fwrite(h.vals.data(), 4, n, f) == n && fwrite(h.bucket.data(), 4, 65537, f) == 65537;
        fclose(f);
        if (ok) rename(tmp.c_str(), path.c_str());
        else unlink(tmp.c_str());
    }
    return h;
}

// ---------------------------------------------------------------------------
// binning

struct Binning {
    int kind = 0;
    TriParams tri{};
    ThreeParams three{};
    PairParams pair{};
    int len = 0;
    double lmax = INFINITY;   // no counted triangle/pair has a side >= lmax
    bool tri_prune = false;   // triangle: test the s and q ranges on tile-triple side bounds
    double s_lo = 0, s_hi = 0, q_hi = 0;
    double lmin_pair = 0;     // pairs: no counted pair has d < lmin_pair
};

// Whether a job of this spec runs in the guarded FP32 kernels.  The fast
// triangle kernel keeps side words of 16 bits (s-bin below 255): binnings with
// more s bins are counted by the plain FP64 kernel, with the same histograms.
bool guarded_fp32(const tpcf_spec& sp, const Binning& bin) {
    if (sp.precision != TPCF_GUARDED_FP32) return false;
    if (sp.kind == TPCF_TRIANGLE || sp.kind == TPCF_TRIANGLE_JBJ) return bin.tri.S <= MAX_FAST_S;
    return true;
}

float ref_bw(float lo, float hi, int n) {
    // (hist_max - hist_min)/nbins in float, as distance_to_bin computes it
    volatile float d = hi - lo;
    volatile float r = d / (float)n;
    return r;
}

// The three-side bin of a side whose squared length (as the reference sums
// it) is d2: distance_to_bin of src/3pcf_C_version.cc:23-51 on sqrtf(d2),
// nbins + 1 standing for d >= hist_max.  IEEE single operations, as on the
// device.
static int three_side_bin_of_d2(float d2, float lo, float hi, float bw, int n) {
    volatile float d = sqrtf(d2);
    if (d < lo) return 0;
    if (d >= hi) return n + 1;
    volatile float x = d - lo;
    volatile float q = x / bw;
    return (int)q;
}

// The pair code of a squared separation d2 (ref_bin_tp of the pair program,
// src/2pcf_C_version.cc:57-86, on sqrtf(d2)): 0 below lo, bin + 1 inside,
// nbins + 2 at or above hi.  IEEE single operations, as on the device.
static int pair_code_of_d2(float d2, float lo, float hi, float bw, int n) {
    volatile float d = sqrtf(d2);
    if (d < lo) return 0;
    if (d >= hi) return n + 2;
    volatile float x = d - lo;
    volatile float q = x / bw;
    return (int)q + 1;
}

// Smallest non-negative float d2 whose code (a non-decreasing function of
// d2) is >= v, by bisection over the ordered bit patterns of floats.
template <class Code>
static float smallest_d2_with_code(int v, Code code) {
    uint32_t lo = 0, hi = 0x7F800000u;  // +0 .. +inf (the largest code)
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        float x;
        memcpy(&x, &mid, 4);
        if (code(x) >= v) hi = mid;
        else lo = mid + 1;
    }
    float r;
    memcpy(&r, &lo, 4);
    return r;
}

static bool pair_thresholds(PairParams& p) {
    if (p.n + 4 > PR_UMAX) return false;
    if (std::max(fabs((double)p.lo), fabs((double)p.hi)) / (double)p.bw > 16384.0) return false;
    p.inv_bw = 1.0f / p.bw;
    p.u[0] = -INFINITY;
    for (int v = 1; v <= p.n + 2; v++)
        p.u[v] = smallest_d2_with_code(v, [&](float x) { return pair_code_of_d2(x, p.lo, p.hi, p.bw, p.n); });
    for (int v = p.n + 3; v < PR_UMAX; v++) p.u[v] = NAN;
    return true;
}

// Thresholds u[v] (smallest float d2 >= 0 with bin >= v) by bisection over
// the ordered bit patterns of non-negative floats; the bin is a
// non-decreasing function of d2 (sqrt, subtraction, division and truncation
// all are).  Returns false where the first guess inv_bw * (sqrt(d2) - lo)
// might be off by more than one bin (very fine binnings).
static bool three_side_thresholds(ThreeParams& p) {
    if (p.n + 3 > TS_UMAX) return false;
    if (std::max(fabs((double)p.lo), fabs((double)p.hi)) / (double)p.bw > 16384.0) return false;
    p.inv_bw = 1.0f / p.bw;
    p.u[0] = -INFINITY;
    for (int v = 1; v <= p.n + 1; v++) {
        uint32_t lo = 0, hi = 0x7F800000u;  // +0 .. +inf (bin nbins + 1)
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            float x;
            memcpy(&x, &mid, 4);
            if (three_side_bin_of_d2(x, p.lo, p.hi, p.bw, p.n) >= v) hi = mid;
            else lo = mid + 1;
        }
        memcpy(&p.u[v], &lo, 4);
    }
    p.u[p.n + 2] = NAN;
    for (int v = p.n + 3; v < TS_UMAX; v++) p.u[v] = NAN;
    return true;
}

Binning make_binning(const tpcf_spec& sp) {
    Binning b;
    b.kind = sp.kind;
    auto check_axis = [](const tpcf_axis& a, const char* what) {
        if (a.nbins <= 0 || a.nbins > 100000) throw InvalidArg{std::string("bad nbins for ") + what};
        if (!(a.hi > a.lo)) throw InvalidArg{std::string("need hi > lo for ") + what};
    };
    if (sp.kind == TPCF_THREE_SIDE) {
        check_axis(sp.axis[0], "three-side axis");
        ThreeParams& p = b.three;
        p.n = sp.axis[0].nbins;
        if ((int64_t)p.n * p.n * p.n > (1 << 29)) throw InvalidArg{"three-side nbins too large"};
        p.lo = sp.axis[0].lo;
        p.hi = sp.axis[0].hi;
        p.bw = ref_bw(p.lo, p.hi, p.n);
        p.clean = sp.overflow == TPCF_OVERFLOW_CLEAN;
        p.len = p.n * p.n * p.n;
        b.len = p.len;
        if (p.clean) b.lmax = (double)p.hi * (1 + 1e-6);
        // (compat mode counts every triple: the side codes are a small part of its work)
        p.fast = p.clean && three_side_thresholds(p) ? 1 : 0;
        p.zcode = three_side_bin_of_d2(0.0f, p.lo, p.hi, p.bw, p.n);
    } else if (sp.kind == TPCF_TRIANGLE) {
        for (int a = 0; a < 3; a++) check_axis(sp.axis[a], "triangle axis");
        TriParams& p = b.tri;
        p.S = sp.axis[0].nbins;
        p.Q = sp.axis[1].nbins;
        p.T = sp.axis[2].nbins;
        if ((int64_t)p.S * p.Q * p.T > MAX_TRI_BINS) throw InvalidArg{"triangle binning too large"};
        p.len = p.S * p.Q * p.T;
        p.s_lo = sp.axis[0].lo;
        p.s_hi = sp.axis[0].hi;
        p.s_bw = ref_bw(p.s_lo, p.s_hi, p.S);
        p.q_lo = sp.axis[1].lo;
        p.q_hi = sp.axis[1].hi;
        p.q_bw = ref_bw(p.q_lo, p.q_hi, p.Q);
        p.t_lo = sp.axis[2].lo;
        p.t_hi = sp.axis[2].hi;
        p.t_bw = ref_bw(p.t_lo, p.t_hi, p.T);
        p.nan_zero = sp.nan_policy == TPCF_NAN_ZERO;
        // q coordinate: (q - q_lo)/q_bw; guard covers |fast - reference| <= ~9 ulp(q)/q_bw
        double qs = 1.0 / (double)p.q_bw;
        p.q_scale = (float)qs;
        p.q_off = (float)(-(double)p.q_lo * qs - 0.5);
        double qmax = std::max(fabs((double)p.q_lo), fabs((double)p.q_hi));
        p.q_thr = (float)(0.5 - (8e-7 * qmax * qs + 2e-6));
        // theta coordinate: acos(c)/(pi' t_bw) - t_lo/t_bw with pi' = 3.14159
        const double pi_ref = 3.14159, pi = 3.14159265358979323846;
        double K = 1.0 / (pi_ref * (double)p.t_bw);
        // acos(x) ~ sqrt(1 - x) * P(x) on [0, 1], P of degree 5: a minimax (Remez)
        // fit in absolute error, which equioscillates at 7 points with
        // |sqrt(1 - x) P(x) - acos(x)| <= 6.37e-7 rad (largest at x = 0; pinned
        // by tests/test_thresholds.py on a grid of 2e6 points).  The guard band
        // below budgets 6.4e-7 rad for it.
        static const double coef[6] = {1.5707956894727488, -0.2145428141209928, 0.08817102789580339,
                                       -0.0459271445289548, 0.020619951348088413, -0.004911124693855812};
        for (int i = 0; i < 6; i++) p.t_coef[i] = (float)(coef[i] * K);
        p.t_half = (float)(K * pi / 2);
        p.t_off0 = (float)(K * pi / 2 - (double)p.t_lo / (double)p.t_bw - 0.5);
        // fixed part: polynomial (6.4e-7 rad) + float evaluation + reference
        // acosf (<= 1.5 ulp) and roundings, bounded by 4e-6 rad; plus relative
        // rounding of the coordinate itself
        double tmax = std::max(fabs((double)p.t_lo), fabs((double)p.t_hi)) / (double)p.t_bw + K * pi;
        double A = 4e-6 * K + 1e-6 * tmax + 2e-6;
        p.t_thrA = (float)(0.5 - A);
        // c-dependent part: |dc| <= 5e-7 |c| amplified by 1/sqrt(1-c^2) <= 1/sqrt(1-|c|)
        p.t_thrB = (float)(5e-7 * K);
        p.t2_off = (float)((1.0 - 3.0 * (double)p.t_lo) / (double)p.t_bw - 1.5);
        p.theta_full = (p.t_lo <= 0.f && p.t_hi >= 1.f);
        b.len = p.len;
        // every counted permutation needs shortest or middle side < s_hi and a
        // ratio < q_hi; all sides are then below s_hi (1 + q_hi)
        if (p.s_hi > 0 && p.q_hi > 0) b.lmax = (double)p.s_hi * (1.0 + (double)p.q_hi) * (1 + 1e-5) + 1e-6;
        b.tri_prune = true;
        b.s_lo = p.s_lo;
        b.s_hi = p.s_hi;
        b.q_hi = (double)p.q_hi * (1 + 1e-5);
    } else if (sp.kind == TPCF_TRIANGLE_JBJ) {
        for (int a = 0; a < 3; a++) check_axis(sp.axis[a], "JBJ axis");
        TriParams& p = b.tri;
        p.S = sp.axis[0].nbins;
        p.Q = sp.axis[1].nbins;
        p.T = sp.axis[2].nbins;
        if ((int64_t)p.S * p.Q * p.T > MAX_TRI_BINS) throw InvalidArg{"JBJ binning too large"};
        p.len = p.S * p.Q * p.T;
        p.s_lo = sp.axis[0].lo;
        p.s_hi = sp.axis[0].hi;
        p.s_bw = ref_bw(p.s_lo, p.s_hi, p.S);
        p.q_lo = sp.axis[1].lo;
        p.q_hi = sp.axis[1].hi;
        p.q_bw = ref_bw(p.q_lo, p.q_hi, p.Q);
        p.t_lo = sp.axis[2].lo;
        p.t_hi = sp.axis[2].hi;
        p.t_bw = ref_bw(p.t_lo, p.t_hi, p.T);
        p.nan_zero = 0;  // no NaN reaches a counted JBJ bin (zero sides are dropped)
        b.len = p.len;
        // counted: s < s_hi, s/m >= q_lo, (l - m)/s < t_hi, so
        // l < s_hi/q_lo + max(t_hi, 0) s_hi (margins cover the float roundings)
        if (p.q_lo > 0 && p.s_hi > 0)
            b.lmax = ((double)p.s_hi / (double)p.q_lo + std::max(0.0, (double)p.t_hi) * (double)p.s_hi) * (1 + 1e-5) +
                     1e-6;
    } else if (sp.kind == TPCF_PAIR) {
        check_axis(sp.axis[0], "pair axis");
        PairParams& p = b.pair;
        p.n = sp.axis[0].nbins;
        p.lo = sp.axis[0].lo;
        p.hi = sp.axis[0].hi;
        p.bw = ref_bw(p.lo, p.hi, p.n);
        p.fast = pair_thresholds(p) ? 1 : 0;
        b.len = p.n;
        b.lmax = (double)p.hi * (1 + 1e-6) + 1e-6;
    } else {
        throw InvalidArg{"unknown kind"};
    }
    if (!sp.prune) {
        b.lmax = INFINITY;
        b.tri_prune = false;
    }
    // device copy of the bound, rounded up so that a float side >= it is >= lmax
    if (sp.kind == TPCF_TRIANGLE_JBJ) b.tri.lmax = b.lmax < 3e38 ? nextafterf((float)b.lmax, INFINITY) : INFINITY;
    if (sp.kind == TPCF_TRIANGLE) {
        b.tri.lmax = b.lmax < 3e38 ? nextafterf((float)b.lmax, INFINITY) : INFINITY;
        double mid = (double)b.tri.s_hi * (double)b.tri.q_hi * (1 + 1e-5) + 1e-6;
        b.tri.mid_hi = sp.prune && b.tri.q_hi > 0 ? nextafterf((float)mid, INFINITY) : INFINITY;
        // a permutation whose side ratio is at least q_rej (computed as a float
        // product with the shorter side) lies past q_hi by more than 1e-4 of
        // the q range, which no rounding of the reference's q = l/s and
        // (q - q_lo)/q_bw brings back into the last bin
        const double qr = (double)b.tri.q_hi + 1e-4 * ((double)b.tri.q_hi - (double)b.tri.q_lo) +
                          1e-5 * fabs((double)b.tri.q_hi);
        b.tri.q_rej = sp.prune ? nextafterf((float)qr, INFINITY) : INFINITY;
    }
    return b;
}

bool same_binning(const tpcf_spec& a, const tpcf_spec& b) {
    if (a.kind != b.kind || a.precision != b.precision) return false;
    if (a.kind == TPCF_TRIANGLE && a.nan_policy != b.nan_policy) return false;
    if ((a.kind == TPCF_THREE_SIDE || a.kind == TPCF_TRIANGLE_JBJ) && a.overflow != b.overflow) return false;
    int na = (a.kind == TPCF_TRIANGLE || a.kind == TPCF_TRIANGLE_JBJ) ? 3 : 1;
    for (int i = 0; i < na; i++)
        if (a.axis[i].lo != b.axis[i].lo || a.axis[i].hi != b.axis[i].hi || a.axis[i].nbins != b.axis[i].nbins)
            return false;
    return true;
}

// ---------------------------------------------------------------------------
// loop units (the reference's numcalc / fake_tot)

uint64_t loop_units(int kind, int loop, const int64_t n[3]) {
    if (kind == TPCF_THREE_SIDE) return (uint64_t)n[0] * n[1] * n[2];
    if (kind == TPCF_PAIR) {
        if (loop == TPCF_LOOP_SAME) {
            uint64_t u = 0;
            for (int64_t i = 0; i < n[0]; i++) u += i < n[1] ? (uint64_t)(n[1] - i) : 0;
            return u;
        }
        return (uint64_t)n[0] * n[1];
    }
    if (loop == TPCF_LOOP_ALL) return (uint64_t)n[0] * n[1] * n[2];
    uint64_t u = 0;
    for (int64_t j = 0; j < n[1]; j++) {
        uint64_t ks = j < n[2] ? (uint64_t)(n[2] - j) : 0;
        uint64_t is = loop == TPCF_LOOP_SAME ? (uint64_t)std::min<int64_t>(n[0], j + 1) : (uint64_t)n[0];
        u += is * ks;
    }
    return u;
}

// ---------------------------------------------------------------------------
// context

// tile triples (pairs) with their unit estimates, in enumeration order
typedef std::vector<std::pair<uint64_t, uint4>> TaskList;

// one window's task groups of the fast triangle kernel: sizes, boxes (lo, hi)
// of their A tiles and summed unit estimates; keys: radix-sort scratch
struct GroupedPart {
    std::vector<uint32_t> sizes;
    std::vector<float> boxes;
    std::vector<uint64_t> units;
    std::vector<uint64_t> keys[2];
};

// host buffers of the planner, kept from batch to batch so that they are not
// allocated (and paged in) again for every batch
struct PlanScratch {
    std::vector<TaskList> part;
    std::vector<GroupedPart> gpart;
    std::vector<uint4> tasks;
    std::vector<uint32_t> groups;
    std::vector<float> gbox;
    std::vector<uint4> tasks2;  // the second part of a pipelined plan
    std::vector<uint32_t> groups2;
    std::vector<float> gbox2;
    std::vector<uint4> tasks3;  // both parts in one (the merged plan)
    std::vector<uint32_t> groups3;
    std::vector<float> gbox3;
};

// One lane = one stream with its own scratch buffers.  The synchronous API uses
// lane 0; every serving worker owns one further lane, so batches of different
// workers run concurrently on the device.
struct Lane {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_mid = nullptr;
    uint64_t h2d = 0, d2h = 0;  // bytes copied since the last stats read
    DevBuf<DevJob> d_jobs;
    DevBuf<uint4> d_tasks;
    DevBuf<uint32_t> d_groups;  // fast triangle kernel: first task of each group (+ end)
    DevBuf<float> d_gbox;       // ... and the box of each group's A tiles
    // second part of a pipelined plan (the jobs after the first, planned while
    // the first job counts): its tasks, groups and boxes
    DevBuf<uint4> d_tasks2;
    DevBuf<uint32_t> d_groups2;
    DevBuf<float> d_gbox2;
    // the whole plan in one part, uploaded while the parts count, for the
    // repeats of the batch
    DevBuf<uint4> d_tasks3;
    DevBuf<uint32_t> d_groups3;
    DevBuf<float> d_gbox3;
    cudaStream_t side = nullptr;   // the second part: its upload and its launch
    cudaStream_t side2 = nullptr;  // the upload of the merged plan
    cudaEvent_t ev_side = nullptr;
    DevBuf<unsigned int> d_counters;  // [0] task counter, [1] recheck count, [2..5] evaluated/binned
    DevBuf<uint4> d_queue;
    DevBuf<unsigned long long> d_hist;
    PinnedBuf<unsigned long long> h_hist;
    PinnedBuf<unsigned int> h_counters;
    // last planned batch (see run_group)
    std::vector<uint64_t> plan_sig;
    size_t plan_ntasks = 0;
    size_t plan_ngroups = 0;  // task groups of the fast triangle kernel
    size_t plan_ntasks2 = 0, plan_ngroups2 = 0;  // second part of a pipelined plan (0: none)
    uint64_t plan_evaluated = 0;
    // the launch sequence of the last batch, captured as a CUDA graph and
    // replayed while the batch and every buffer it touches stay the same
    cudaGraphExec_t graph = nullptr;
    std::vector<uint64_t> graph_sig;
    bool graphs_ok = true;
    // SMs a launch of this lane may fill with its persistent CTAs (0: all);
    // the serving lane that runs heavy jobs leaves some to the light lanes
    int sm_cap = 0;
    // count in slices of the task list (heavy serving batches)
    bool slice_batches = false;
    PlanScratch scratch;
    tpcf_stats stats{};
    void drop_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        graph_sig.clear();
    }
    void release() {
        drop_graph();
        h_hist.release();
        h_counters.release();
        d_jobs.release();
        d_tasks.release();
        d_groups.release();
        d_gbox.release();
        d_tasks2.release();
        d_groups2.release();
        d_gbox2.release();
        d_tasks3.release();
        d_groups3.release();
        d_gbox3.release();
        if (ev_side) cudaEventDestroy(ev_side);
        if (side) cudaStreamDestroy(side);
        if (side2) cudaStreamDestroy(side2);
        ev_side = nullptr;
        side = side2 = nullptr;
        d_counters.release();
        d_queue.release();
        d_hist.release();
        scratch = PlanScratch();
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (ev_mid) cudaEventDestroy(ev_mid);
        if (stream) cudaStreamDestroy(stream);
        ev0 = ev1 = ev_mid = nullptr;
        stream = nullptr;
    }
};

struct Pending {
    uint64_t ticket;
    double t_submit = 0, t_start = 0, t_done = 0;  // steady-clock ms
    double cost = 0;                                // job_cost at submission
    tpcf_spec spec;
    tpcf_job job;
    std::vector<uint64_t> result;
    tpcf_status status = 1;  // 1 = pending
    bool cancelled = false;
};

struct GroupJob {
    const tpcf_spec* spec;
    const tpcf_job* job;
    uint64_t* out;
    bool accumulate = false;  // add into out (jobs sharing out share one device histogram)
};

}  // namespace

// Launch shape of a persistent kernel: warp-private histogram copies in
// shared memory (0: count straight into the 64-bit global histogram),
// resident CTAs per SM (the grid is that many per SM) and, for the
// three-side kernel, task pipelines per CTA (0: plain 8-warp CTAs; g > 0:
// one CTA per SM of g 8-warp pipelines around one large histogram).
struct Shape {
    int copies = 1;
    int per_sm = 1;
    int groups = 0;
    size_t smem = 0;
};

struct tpcf_ctx {
    int device = 0;
    int num_sms = 0;
    std::recursive_mutex mu;      // serialises the synchronous API (lane 0)
    std::recursive_mutex view_mu; // catalogs and spatial views
    std::mutex acos_mu;
    std::string last_error;
    uint64_t next_handle = 1;
    std::map<uint64_t, std::shared_ptr<Catalog>> catalogs;
    // (catalog, begin, end, tile points, global loop indices) -> view
    std::map<std::tuple<uint64_t, int64_t, int64_t, int, bool>, std::shared_ptr<View>> views;
    // full views of new catalogs being built in the background
    struct PendingView {
        std::shared_future<std::shared_ptr<View>> fut;
        uint64_t id;
        int64_t n;
    };
    std::map<std::tuple<uint64_t, int64_t, int64_t, int, bool>, PendingView> pending_views;
    int tile_points = TILE;  // points per spatial tile (<= TILE)
    uint64_t next_view_id = 0;
    // acos table
    bool acos_ready = false;
    DevBuf<uint32_t> acos_keys, acos_vals, acos_bucket;
    uint32_t acos_n = 0;
    std::vector<std::unique_ptr<Lane>> lanes;
    // serving
    std::mutex qmu;
    std::condition_variable qcv;
    std::deque<std::shared_ptr<Pending>> queue;
    std::map<uint64_t, std::shared_ptr<Pending>> tickets;
    uint64_t next_ticket = 1;
    std::vector<std::thread> workers;
    bool stop = false;
    // serving trace (TPCF_SERVING_TRACE=file): one line per batch, written by
    // tpcf_destroy: lane, jobs, first ticket, oldest submit, start, planned, done (ms)
    std::string trace_path;
    std::vector<std::string> trace;
    int64_t admit_bytes = (int64_t)8 << 30;
    double heavy_cost = 4e11;  // job_cost above which a job runs alone on the first serving lane (~50 ms)
    double light_batch_cost = 1e11;  // summed job_cost at which a batch of light jobs closes
    std::map<std::tuple<uint64_t, int64_t, int64_t, uint64_t, int64_t, int64_t, double>, double> density;
    int reserve_sms = 0;       // SMs a heavy serving batch leaves free for light jobs
    bool slice_heavy = true;   // heavy serving batches count in slices (light lanes run between them)
    int slice_tasks = 0;       // tasks per slice (0: at least 8 per CTA and at most 64 slices)
    int group_tasks = 0;       // fast triangle kernel: most tasks sharing one j-k table (0: by the batch)
    int64_t inflight_bytes = 0;  // device bytes of batches running on serving lanes
    // autotuner: launch shape per batch signature
    std::mutex tune_mu;
    std::map<uint64_t, Shape> tuned;
};

namespace {

tpcf_status fail(tpcf_ctx* ctx, tpcf_status s, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    g_tls_error = msg;
    return s;
}

// TPCF_PLAN_TRACE=1: wall times of view building and batch planning on stderr
bool plan_trace() {
    static const bool on = [] {
        const char* e = getenv("TPCF_PLAN_TRACE");
        return e && e[0] == '1';
    }();
    return on;
}

// Builds the spatial view of points [begin, end) of a catalog: k-d order,
// tiles, their boxes, and the device copy (on stream st, synchronized).
std::shared_ptr<View> build_view(const Catalog& c, int64_t begin, int64_t end, int tile, bool global, uint64_t id,
                                 cudaStream_t st) {
    const auto tv0 = std::chrono::steady_clock::now();
    auto v = std::make_shared<View>();
    v->id = id;
    int64_t n = end - begin;
    v->n = n;
    std::vector<float> xyz(3 * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        xyz[3 * i] = c.x[begin + i];
        xyz[3 * i + 1] = c.y[begin + i];
        xyz[3 * i + 2] = c.z[begin + i];
    }
    std::vector<int32_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    const auto tv1 = std::chrono::steady_clock::now();
    kd_order(xyz.data(), order, n, tile);
    const auto tv2 = std::chrono::steady_clock::now();
    v->ntiles = (int)((n + tile - 1) / tile);
    std::vector<float4> pts(std::max<int64_t>(n, 1));
    for (int64_t i = 0; i < n; i++) {
        int32_t o = order[i];
        float4 p;
        p.x = xyz[3 * (size_t)o];
        p.y = xyz[3 * (size_t)o + 1];
        p.z = xyz[3 * (size_t)o + 2];
        // loop index inside the range, or inside the whole catalog
        int32_t key_i = global ? (int32_t)(o + begin) : o;
        memcpy(&p.w, &key_i, 4);
        pts[i] = p;
    }
    v->h_tile_start.resize(v->ntiles + 1);
    v->boxes.resize(v->ntiles);
    for (int t = 0; t <= v->ntiles; t++) v->h_tile_start[t] = (int32_t)std::min<int64_t>((int64_t)t * tile, n);
    for (int t = 0; t < v->ntiles; t++) {
        Box b;
        for (int a = 0; a < 3; a++) {
            b.lo[a] = INFINITY;
            b.hi[a] = -INFINITY;
        }
        for (int i = v->h_tile_start[t]; i < v->h_tile_start[t + 1]; i++) {
            const float* q = &pts[i].x;
            for (int a = 0; a < 3; a++) {
                b.lo[a] = std::min(b.lo[a], q[a]);
                b.hi[a] = std::max(b.hi[a], q[a]);
            }
        }
        v->boxes[t] = b;
    }
    const auto tv3 = std::chrono::steady_clock::now();
    v->pts.reserve(pts.size());
    CK(cudaMemcpyAsync(v->pts.p, pts.data(), pts.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
    v->tile_start.reserve(v->ntiles + 1);
    CK(cudaMemcpyAsync(v->tile_start.p, v->h_tile_start.data(), (v->ntiles + 1) * sizeof(int32_t),
                       cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    v->upload_bytes = pts.size() * sizeof(float4) + (v->ntiles + 1) * sizeof(int32_t);
    if (plan_trace()) {
        auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
            return std::chrono::duration<double, std::milli>(b - a).count();
        };
        const auto tv4 = std::chrono::steady_clock::now();
        fprintf(stderr, "tpcf view: points %lld copy %.4f order %.4f pack %.4f upload %.4f\n", (long long)n,
                ms(tv0, tv1), ms(tv1, tv2), ms(tv2, tv3), ms(tv3, tv4));
    }
    return v;
}

// Id and point count of the view of catalog `handle` over [begin, end): a
// view being built in the background is not waited for (its id was assigned
// when it was started); any other is made now.
struct ViewRef {
    uint64_t id;
    int64_t n;
};

// The view of catalog `handle` over [begin, end) for the context's tile size:
// cached, being built in the background (a new catalog's full view), or built
// now on the lane's stream.  With ref != nullptr and the view still being
// built, returns nullptr at once and fills ref.
std::shared_ptr<View> get_view(tpcf_ctx* ctx, Lane& L, uint64_t handle, int64_t begin, int64_t end,
                               bool global = false, ViewRef* ref = nullptr) {
    std::unique_lock<std::recursive_mutex> vlk(ctx->view_mu);
    auto it = ctx->catalogs.find(handle);
    if (it == ctx->catalogs.end()) throw InvalidArg{"unknown catalog handle"};
    const std::shared_ptr<Catalog> cat = it->second;
    if (end < 0) end = cat->n;
    if (begin < 0 || begin > end || end > cat->n) throw InvalidArg{"catalog range out of bounds"};
    const int tile = ctx->tile_points;
    if (begin == 0) global = false;  // the same loop indices
    auto key = std::make_tuple(handle, begin, end, tile, global);
    auto vi = ctx->views.find(key);
    if (vi != ctx->views.end()) {
        if (ref) *ref = {vi->second->id, vi->second->n};
        return vi->second;
    }
    auto pi = ctx->pending_views.find(key);
    if (pi != ctx->pending_views.end()) {
        if (ref) {
            *ref = {pi->second.id, pi->second.n};
            return nullptr;
        }
        std::shared_future<std::shared_ptr<View>> fut = pi->second.fut;
        vlk.unlock();
        std::shared_ptr<View> v;
        try {
            v = fut.get();
        } catch (...) {
            vlk.lock();
            ctx->pending_views.erase(key);
            throw;
        }
        vlk.lock();
        ctx->pending_views.erase(key);
        if (!ctx->catalogs.count(handle)) throw InvalidArg{"unknown catalog handle"};
        auto ins = ctx->views.emplace(key, v);
        if (ins.second) L.h2d += v->upload_bytes;
        return ins.first->second;
    }
    auto v = build_view(*cat, begin, end, tile, global, ++ctx->next_view_id, L.stream);
    L.h2d += v->upload_bytes;
    ctx->views[key] = v;
    if (ref) *ref = {v->id, v->n};
    return v;
}

void ensure_acos(tpcf_ctx* ctx) {
    std::lock_guard<std::mutex> alk(ctx->acos_mu);
    if (ctx->acos_ready) return;
    AcosHost h = load_or_build_acos_table();
    ctx->acos_n = (uint32_t)h.keys.size();
    ctx->acos_keys.reserve(std::max<size_t>(h.keys.size(), 1));
    ctx->acos_vals.reserve(std::max<size_t>(h.vals.size(), 1));
    ctx->acos_bucket.reserve(65537);
    if (!h.keys.empty()) {
        CK(cudaMemcpy(ctx->acos_keys.p, h.keys.data(), h.keys.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->acos_vals.p, h.vals.data(), h.vals.size() * 4, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(ctx->acos_bucket.p, h.bucket.data(), 65537 * 4, cudaMemcpyHostToDevice));
    ctx->acos_ready = true;
}

AcosTable acos_table(tpcf_ctx* ctx) {
    AcosTable t;
    t.keys = ctx->acos_keys.p;
    t.vals = ctx->acos_vals.p;
    t.bucket = ctx->acos_bucket.p;
    t.n = ctx->acos_n;
    return t;
}

struct PlannedJob {
    std::shared_ptr<View> v[3];
    uint64_t loop_units = 0;
    // Loop ONE jobs of two arrays are counted with the point of the array that
    // appears once in role B or C and the pair array first, so that points
    // out of reach of a tile are skipped whole (guarded kernel only):
    //   swap 1, the D-D-R nest (A == B): roles (C, A, A), weight PRED_RDD;
    //   swap 2, the D-R-R nest (B == C): roles (B, B, A), unordered pairs of B first.
    int swap = 0;
    const View* role(int r) const {
        if (swap == 1) return r == 0 ? v[2].get() : v[0].get();
        if (swap == 2) return r == 2 ? v[0].get() : v[1].get();
        return v[r].get();
    }
};

inline bool close_enough(const View& a, int ta, const View& b, int tb, double lmax) {
    if (!(lmax < INFINITY)) return true;
    return box_lower_bound(a.boxes[ta], b.boxes[tb]) < lmax;
}

uint64_t task_units3(const View& A, int a, const View& B, int b, const View& C, int c, uint32_t flags) {
    uint64_t na = A.h_tile_start[a + 1] - A.h_tile_start[a];
    uint64_t nb = B.h_tile_start[b + 1] - B.h_tile_start[b];
    uint64_t nc = C.h_tile_start[c + 1] - C.h_tile_start[c];
    bool dij = flags & TASK_DIAG_IJ, djk = flags & TASK_DIAG_JK;
    if (dij && djk) return na * (na - 1) * (na - 2) / 6;
    if (dij) return na * (na - 1) / 2 * nc;
    if (djk) return na * (nb * (nb - 1) / 2);
    return na * nb * nc;
}

// Tile tasks of one triangle/three-side job.
// Lower/upper side bounds of every tile pair of two views, held densely when
// small enough (else computed on demand).
struct PairBounds {
    const View* a = nullptr;
    const View* b = nullptr;
    bool dense = false;
    std::vector<float> lb, ub;
    // sizes the table; fill_rows(i0, i1) then fills rows independently (threads)
    void alloc(const View& A, const View& B) {
        a = &A;
        b = &B;
        dense = (int64_t)A.ntiles * B.ntiles <= ((int64_t)1 << 24);
        if (!dense) return;
        lb.resize((size_t)A.ntiles * B.ntiles);
        ub.resize(lb.size());
    }
    void fill_rows(int i0, int i1) {
        if (!dense) return;
        for (int i = i0; i < i1; i++)
            for (int j = 0; j < b->ntiles; j++) {
                // float copies rounded outwards so they stay conservative
                lb[(size_t)i * b->ntiles + j] = nextafterf((float)box_lower_bound(a->boxes[i], b->boxes[j]), 0.f);
                ub[(size_t)i * b->ntiles + j] = nextafterf((float)box_upper_bound(a->boxes[i], b->boxes[j]), INFINITY);
            }
    }
    double L(int i, int j) const {
        return dense ? (double)lb[(size_t)i * b->ntiles + j] : box_lower_bound(a->boxes[i], b->boxes[j]);
    }
    double U(int i, int j) const {
        return dense ? (double)ub[(size_t)i * b->ntiles + j] : box_upper_bound(a->boxes[i], b->boxes[j]);
    }
};

// Whether a tile triple can hold a counted triangle-parametrization triangle:
// with the three pair bounds sorted (L1<=L2<=L3 lower, U1<=U2<=U3 upper) the
// shortest side lies in [L1,U1], the middle in [L2,U2], the longest in [L3,U3];
// permutations 0/2 need s_lo <= shortest < s_hi and middle < q_hi*shortest,
// permutation 1 needs s_lo <= middle < s_hi and longest < q_hi*middle.
bool tri_triple_possible(const Binning& bin, double l0, double l1, double l2, double u0, double u1, double u2) {
    double L[3] = {l0, l1, l2}, U[3] = {u0, u1, u2};
    if (L[0] > L[1]) std::swap(L[0], L[1]);
    if (L[1] > L[2]) std::swap(L[1], L[2]);
    if (L[0] > L[1]) std::swap(L[0], L[1]);
    if (U[0] > U[1]) std::swap(U[0], U[1]);
    if (U[1] > U[2]) std::swap(U[1], U[2]);
    if (U[0] > U[1]) std::swap(U[0], U[1]);
    bool p0 = L[0] < bin.s_hi && U[0] >= bin.s_lo && L[1] < bin.q_hi * U[0];
    bool p1 = L[1] < bin.s_hi && U[1] >= bin.s_lo && L[2] < bin.q_hi * U[1];
    return p0 || p1;
}


// Lower/upper side bounds and neighbour lists (tile pairs whose lower bound is
// below lmax) of one pair of views, shared by every job of a launch that
// pairs those views; rows() fills a range of rows (parallel planning).
struct PairTable {
    const View* x = nullptr;
    const View* y = nullptr;
    bool prune = false, need_nb = false;
    int listed = -1;  // the planning pass whose row list holds it
    double lmax = INFINITY;
    PairBounds pb;
    std::vector<std::vector<int>> nb;
    void init(const View& X, const View& Y, double lmax_) {
        x = &X;
        y = &Y;
        lmax = lmax_;
        prune = lmax < INFINITY;
        if (prune) pb.alloc(X, Y);
    }
    void rows(int r0, int r1) {
        if (prune) pb.fill_rows(r0, r1);
        if (!need_nb) return;
        for (int i = r0; i < r1; i++) {
            nb[i].clear();
            for (int j = 0; j < y->ntiles; j++)
                if (!prune || pb.L(i, j) < lmax) nb[i].push_back(j);
        }
    }
};

// Tile tasks of one triangle/three-side job: enumerate() lists the tile
// triples of a range of A tiles from the pair tables of (A,B), (A,C), (B,C).
struct TripletPlan {
    const tpcf_spec* sp = nullptr;
    const PlannedJob* pj = nullptr;
    const Binning* bin = nullptr;
    uint32_t slot = 0;
    bool empty = true, prune = false, tri = false, sameAB = false, sameBC = false;
    bool sym_three = true;  // TPCF_SYM3=0: ordered three-side tasks
    const PairTable *AB = nullptr, *AC = nullptr, *BC = nullptr;

    void init(const tpcf_spec& s, const PlannedJob& p, uint32_t sl, const Binning& b, const PairTable* ab,
              const PairTable* ac, const PairTable* bc) {
        sp = &s;
        pj = &p;
        bin = &b;
        slot = sl;
        const View &A = *p.role(0), &B = *p.role(1), &C = *p.role(2);
        empty = A.ntiles == 0 || B.ntiles == 0 || C.ntiles == 0;
        prune = b.lmax < INFINITY;
        tri = s.kind == TPCF_TRIANGLE || s.kind == TPCF_TRIANGLE_JBJ;
        sameAB = p.role(0) == p.role(1);
        sameBC = p.role(1) == p.role(2);
        const char* e3 = getenv("TPCF_SYM3");
        sym_three = !(e3 && e3[0] == '0');
        AB = ab;
        AC = ac;
        BC = bc;
    }
    // Tile triples of A tiles [a0, a1); with one A tile, only its neighbour-list
    // entries [blo, bhi) as tile B (a heavy tile's triples in several parts).
    void enumerate(int a0, int a1, TaskList& tasks, uint64_t& evaluated, size_t blo = 0,
                   size_t bhi = SIZE_MAX) const {
        if (empty) return;  // a role without tiles: no triple (and no neighbour lists)
        const View &A = *pj->role(0), &B = *pj->role(1), &C = *pj->role(2);
        const double lmax = bin->lmax;
        // bounds of the pair (a, b), looked up once for all its c
        struct AB_ {
            double l = 0, u = 0;
        };
        auto ab_bounds = [&](int a, int b) {
            AB_ r;
            if (prune) {
                r.l = AB->pb.L(a, b);
                r.u = AB->pb.U(a, b);
            }
            return r;
        };
        auto add = [&](int a, int b, int c, const AB_& ab, uint32_t pred, uint32_t flags) {
            if (prune) {
                const double lbc = BC->pb.L(b, c);
                if (!(lbc < lmax)) return;
                const double lac = AC->pb.L(a, c), uac = AC->pb.U(a, c);
                if (bin->tri_prune && !tri_triple_possible(*bin, ab.l, lac, lbc, ab.u, uac, BC->pb.U(b, c))) return;
                if (ab.u >= lmax) flags |= TASK_CHECK_B;
                if (uac >= lmax) flags |= TASK_CHECK_C;
            }
            uint64_t u = task_units3(A, a, B, b, C, c, flags);
            if (u == 0) return;
            evaluated += u;
            tasks.push_back({u, make_uint4(slot | (pred << TASK_PRED_SHIFT) | flags, (uint32_t)a, (uint32_t)b,
                                           (uint32_t)c)});
        };
        // the entries >= from of an ascending neighbour list
        auto from = [](const std::vector<int>& l, int v) { return std::lower_bound(l.begin(), l.end(), v); };
        // tile B's entries of the list: positions [blo, bhi), at least v
        struct Span {
            std::vector<int>::const_iterator b, e;
            std::vector<int>::const_iterator begin() const { return b; }
            std::vector<int>::const_iterator end() const { return e; }
        };
        auto bspan = [&](const std::vector<int>& l, int v) {
            auto lo = l.begin() + (ptrdiff_t)std::min(blo, l.size());
            auto hi = l.begin() + (ptrdiff_t)std::min(bhi, l.size());
            auto f = from(l, v);
            if (f > lo) lo = f;
            return Span{lo, std::max(lo, hi)};
        };
        const tpcf_spec& s = *sp;
        // three-side histogram of one catalog in all roles: the kernel counts
        // each multiset {i, j, k} once for all its orderings
        const bool sym3 = s.kind == TPCF_THREE_SIDE && s.loop == TPCF_LOOP_ALL && sym_three && sameAB && sameBC;
        if (pj->swap == 1) {
            // roles (C, A, A) of a D-D-R job: each point of C with every
            // unordered pair of the single array, weight [k_c >= j] + [k_c >= k]
            for (int a = a0; a < a1; a++)
                for (int b : bspan(AB->nb[a], INT_MIN)) {
                    const AB_ ab = ab_bounds(a, b);
                    for (auto c = from(AC->nb[a], b); c != AC->nb[a].end(); ++c)
                        add(a, b, *c, ab, PRED_RDD, b == *c ? TASK_DIAG_JK : 0);
                }
        } else if (pj->swap == 2) {
            // roles (B, B, A) of a D-R-R job: every unordered pair of the pair
            // array with each point of the other
            for (int a = a0; a < a1; a++)
                for (int b : bspan(AB->nb[a], a)) {
                    const AB_ ab = ab_bounds(a, b);
                    for (int c : AC->nb[a]) add(a, b, c, ab, PRED_NONE, a == b ? TASK_DIAG_IJ : 0);
                }
        } else if ((tri && s.loop == TPCF_LOOP_SAME || sym3) && sameAB && sameBC) {
            // i <= j <= k over one array: unordered distinct triples (triangle
            // programs), or every multiset of three points counted for each of
            // its orderings (three-side: PRED_SAME marks the task)
            for (int a = a0; a < a1; a++)
                for (int b : bspan(AB->nb[a], a)) {
                    const AB_ ab = ab_bounds(a, b);
                    for (auto c = from(AC->nb[a], b); c != AC->nb[a].end(); ++c) {
                        uint32_t f = (a == b ? TASK_DIAG_IJ : 0) | (b == *c ? TASK_DIAG_JK : 0);
                        add(a, b, *c, ab, sym3 ? PRED_SAME : PRED_NONE, f);
                    }
                }
        } else if (tri && s.loop == TPCF_LOOP_ONE && sameBC) {
            // j <= k over one array (j == k has a zero side): unordered pairs
            for (int a = a0; a < a1; a++)
                for (int b : bspan(AB->nb[a], INT_MIN)) {
                    const AB_ ab = ab_bounds(a, b);
                    for (auto c = from(AC->nb[a], b); c != AC->nb[a].end(); ++c)
                        add(a, b, *c, ab, PRED_NONE, b == *c ? TASK_DIAG_JK : 0);
                }
        } else if (tri && s.loop == TPCF_LOOP_ONE && sameAB) {
            // every ordered (i, j) of one array, k >= j: unordered {i, j} with
            // weight [k >= i] + [k >= j]
            for (int a = a0; a < a1; a++)
                for (int b : bspan(AB->nb[a], a)) {
                    const AB_ ab = ab_bounds(a, b);
                    for (int c : AC->nb[a]) add(a, b, c, ab, PRED_DDR, a == b ? TASK_DIAG_IJ : 0);
                }
        } else {
            uint32_t pred = PRED_NONE;
            if (tri) pred = s.loop == TPCF_LOOP_SAME ? PRED_SAME : s.loop == TPCF_LOOP_ONE ? PRED_ONE : PRED_NONE;
            for (int a = a0; a < a1; a++)
                for (int b : bspan(AB->nb[a], INT_MIN)) {
                    const AB_ ab = ab_bounds(a, b);
                    for (int c : AC->nb[a]) add(a, b, c, ab, pred, 0);
                }
        }
    }
};

// Pair tasks of A tiles [a0, a1).
void plan_pairs(const tpcf_spec& sp, const PlannedJob& pj, uint32_t slot, double lmax, int a0, int a1,
                TaskList& tasks, uint64_t& evaluated) {
    const View &A = *pj.v[0], &B = *pj.v[1];
    if (A.ntiles == 0 || B.ntiles == 0) return;
    const bool same = pj.v[0] == pj.v[1] && sp.loop == TPCF_LOOP_SAME;
    for (int a = a0; a < a1; a++)
        for (int b = same ? a : 0; b < B.ntiles; b++) {
            if (!close_enough(A, a, B, b, lmax)) continue;
            uint64_t na = A.h_tile_start[a + 1] - A.h_tile_start[a], nb = B.h_tile_start[b + 1] - B.h_tile_start[b];
            uint32_t flags = 0, pred = PRED_NONE;
            uint64_t u = na * nb;
            if (same && a == b) {
                flags = TASK_DIAG_IJ;
                u = na * (na + 1) / 2;
            } else if (!same && sp.loop == TPCF_LOOP_SAME) {
                pred = PRED_SAME;
            }
            evaluated += u;
            tasks.push_back({u, make_uint4(slot | (pred << TASK_PRED_SHIFT) | flags, (uint32_t)a, (uint32_t)b, 0)});
        }
}

// Host worker threads for planning, started once per process (thread
// creation would cost more than the planning work of a small batch).  run()
// calls fn(i) for i in [0, n) on the workers and the calling thread; a run
// that finds the pool busy (another lane planning) does its items inline.
class HostPool {
  public:
    static HostPool& get() {
        static HostPool pool;
        return pool;
    }
    // Runs fn(0..n) on this thread and the pool's threads.  Several callers
    // (a count's planning, background view builds, serving lanes) share the
    // pool: idle threads help whichever jobs have items left.
    void run(size_t n, const std::function<void(size_t)>& fn) {
        if (n == 0) return;
        if (workers_.empty() || n == 1) {
            for (size_t i = 0; i < n; i++) fn(i);
            return;
        }
        Job job;
        job.fn = &fn;
        job.n = n;
        {
            std::lock_guard<std::mutex> lk(mu_);
            jobs_.push_back(&job);
            posted_.fetch_add(1);
        }
        cv_.notify_all();
        try {
            work(job);
        } catch (...) {
            // no further items; wait for the helpers to leave the job (it lives
            // on this frame) before the exception leaves it
            job.next.store(n);
            std::unique_lock<std::mutex> lk(mu_);
            jobs_.erase(std::find(jobs_.begin(), jobs_.end(), &job));
            done_cv_.wait(lk, [&] { return job.users == 0; });
            throw;
        }
        std::unique_lock<std::mutex> lk(mu_);
        jobs_.erase(std::find(jobs_.begin(), jobs_.end(), &job));  // no new helpers
        done_cv_.wait(lk, [&] { return job.users == 0 && job.done.load() == n; });
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
            stop_flag_.store(true);
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }

  private:
    struct Job {
        const std::function<void(size_t)>* fn = nullptr;
        size_t n = 0;
        std::atomic<size_t> next{0}, done{0};
        size_t users = 0;  // pool threads working on it (under mu_)
    };
    HostPool() {
        const unsigned n = std::max(1u, std::thread::hardware_concurrency()) - 1;
        for (unsigned t = 0; t < n; t++) workers_.emplace_back([this] { loop(); });
    }
    void work(Job& j) {
        for (;;) {
            size_t i = j.next.fetch_add(1);
            if (i >= j.n) break;
            (*j.fn)(i);
            j.done.fetch_add(1);
        }
    }
    Job* open_job() {  // under mu_
        for (Job* j : jobs_)
            if (j->next.load() < j->n) return j;
        return nullptr;
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            // the phases of a planning pass follow one another within
            // microseconds: watch for the next job for a while before sleeping
            // (a wake-up from the condition variable costs tens of microseconds)
            const auto spin_end = std::chrono::steady_clock::now() + std::chrono::microseconds(300);
            while (posted_.load() == seen && !stop_flag_.load() && std::chrono::steady_clock::now() < spin_end)
                std::this_thread::yield();
            Job* j = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || (j = open_job()) != nullptr || posted_.load() != seen; });
                if (stop_) return;
                seen = posted_.load();
                if (!j) j = open_job();
                if (!j) continue;
                j->users++;
            }
            work(*j);
            {
                std::lock_guard<std::mutex> lk(mu_);
                j->users--;
            }
            done_cv_.notify_all();
        }
    }
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::vector<std::thread> workers_;
    std::vector<Job*> jobs_;
    std::atomic<uint64_t> posted_{0};  // jobs posted so far
    std::atomic<bool> stop_flag_{false};
    bool stop_ = false;
};

void parallel_items(size_t n, const std::function<void(size_t)>& fn) { HostPool::get().run(n, fn); }

size_t shape_smem(const tpcf_spec& sp, const Binning& bin, int copies, int groups) {
    if (sp.kind == TPCF_TRIANGLE || sp.kind == TPCF_TRIANGLE_JBJ) return triangle_smem_bytes(bin.len, copies);
    if (sp.kind == TPCF_THREE_SIDE) return three_side_smem_bytes(bin.three, copies, groups);
    return pair_smem_bytes(bin.len, copies);
}

// Launch shapes worth trying for a group, the default first.  The guarded
// triangle kernel is compiled for four CTAs per SM (its register budget);
// the others take as many CTAs as shared memory allows, up to 8.
std::vector<Shape> shape_candidates(tpcf_ctx* ctx, const tpcf_spec& sp, const Binning& bin, bool fp64) {
    int max_smem_sm = 0, max_smem_block = 0;
    cudaDeviceGetAttribute(&max_smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device);
    cudaDeviceGetAttribute(&max_smem_block, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    auto fit = [&](int copies, int cap_per_sm, int groups = 0) {
        Shape sh;
        sh.copies = copies;
        sh.groups = groups;
        sh.smem = shape_smem(sp, bin, copies, groups);
        sh.per_sm = 0;
        if (sh.smem + 1024 > (size_t)max_smem_block) return sh;  // leaves room for the kernels' static shared memory
        sh.per_sm = std::min(cap_per_sm, (int)(max_smem_sm / (sh.smem + 1024)));
        return sh;
    };
    std::vector<Shape> out;
    auto add = [&](Shape sh) {
        if (sh.per_sm < 1) return;
        for (const Shape& o : out)
            if (o.copies == sh.copies && o.per_sm == sh.per_sm && o.groups == sh.groups) return;
        out.push_back(sh);
    };
    if (sp.kind == TPCF_TRIANGLE || sp.kind == TPCF_TRIANGLE_JBJ) {
        const char* bps = getenv("TPCF_TRI_BLOCKS_PER_SM");
        const int tri_per_sm = fp64 ? 2 : (bps ? std::max(1, atoi(bps)) : 4);
        // default: as many copies as keep four CTAs on an SM (the kernel
        // needs the warps to hide the latency of its shared-memory tables);
        // the autotuner also tries three CTAs with more copies
        int c = 8;
        while (c > 1 && fit(c, tri_per_sm).per_sm < tri_per_sm) c /= 2;
        add(fit(c, tri_per_sm));
        if (!fp64) {
            for (int cc : {4, 2, 1}) add(fit(cc, tri_per_sm));
            if (!bps)
                for (int cc : {4, 2, 1}) add(fit(cc, 3));
        }
        if (out.empty()) throw InvalidArg{"triangle histogram too large for shared memory"};
    } else if (sp.kind == TPCF_THREE_SIDE) {
        // default: the most copies that still leave four 8-warp CTAs per SM,
        // else one CTA per SM of as many pipelines (up to four) as fit
        // around one shared histogram, else the global histogram
        Shape def;
        def.copies = -1;
        for (int cc : {4, 2, 1}) {
            Shape sh = fit(cc, 8);
            if (sh.per_sm >= 4) {
                def = sh;
                break;
            }
        }
        int groups = 4;
        while (groups > 1 && fit(1, 1, groups).per_sm < 1) groups--;
        if (def.copies < 0) def = fit(1, 1, groups);
        if (def.per_sm < 1) def = fit(0, 8);
        add(def);
        for (int cc : {8, 4, 2, 1, 0}) add(fit(cc, 8));
        add(fit(1, 1, groups));
    } else {
        Shape def;
        def.copies = -1;
        for (int cc : {8, 4, 2, 1}) {
            Shape sh = fit(cc, 8);
            if (sh.per_sm >= 2) {
                def = sh;
                break;
            }
        }
        if (def.copies < 0) def = fit(1, 8);
        if (def.per_sm < 1) throw InvalidArg{"pair histogram too large"};
        add(def);
        for (int cc : {8, 4, 2, 1}) add(fit(cc, 8));
    }
    return out;
}

int grid_for(tpcf_ctx* ctx, const Shape& sh, uint64_t ntasks, int sm_cap) {
    const int sms = sm_cap > 0 ? std::min(sm_cap, ctx->num_sms) : ctx->num_sms;
    uint64_t g = (uint64_t)sms * sh.per_sm;
    if (g > ntasks) g = std::max<uint64_t>(ntasks, 1);
    return (int)g;
}

// Task groups of the fast triangle kernel: tasks of one job with the same
// tiles B and C run one after another in one CTA, which builds their j-k
// table once.  Each window of planning parts (one job, a run of consecutive A
// tiles) groups its own tasks, in parallel with the others: a sort on (b, c)
// that keeps the order of A tiles, runs of equal (b, c) cut into groups of at
// most max_group tasks (a group is the unit a CTA takes, so large ones would
// leave a long tail at the end of the launch).  boxes: lo/hi of the union of each
// group's A tiles, for the j-k rows that no point of the group can reach;
// units: the group's summed task estimates.

void group_parts(const TaskList* parts, size_t nparts, const PlannedJob& J, size_t max_group, uint4* dst,
                 GroupedPart& out) {
    const uint64_t nc = (uint64_t)J.role(2)->ntiles;
    size_t n = 0;
    for (size_t i = 0; i < nparts; i++) n += parts[i].size();
    // (b, c) key above the task's index in the window, sorted by an LSD
    // radix sort on the key (stable: ties stay in the order of A tiles)
    std::vector<uint64_t>&ka = out.keys[0], &kb = out.keys[1];
    ka.resize(n);
    kb.resize(n);
    uint64_t kmax = 0;
    for (size_t i = 0, t = 0; i < nparts; i++)
        for (const auto& pr : parts[i]) {
            const uint64_t k = (uint64_t)pr.second.z * nc + pr.second.w;
            kmax = std::max(kmax, k);
            ka[t] = k << 32 | t;
            t++;
        }
    for (int shift = 32; shift < 64 && (kmax >> (shift - 32)) != 0; shift += 8) {
        uint32_t cnt[257] = {0};
        for (size_t t = 0; t < n; t++) cnt[((ka[t] >> shift) & 255) + 1]++;
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (size_t t = 0; t < n; t++) kb[cnt[(ka[t] >> shift) & 255]++] = ka[t];
        ka.swap(kb);
    }
    // the window's tasks by index
    std::vector<const std::pair<uint64_t, uint4>*> src(n);
    for (size_t i = 0, t = 0; i < nparts; i++)
        for (const auto& pr : parts[i]) src[t++] = &pr;
    const View& A = *J.role(0);
    out.sizes.resize(n);
    out.boxes.resize(6 * n);
    out.units.resize(n);
    size_t ng = 0;
    for (size_t t = 0; t < n;) {
        const uint64_t k = ka[t] >> 32;
        size_t e = t + 1;
        while (e < n && e - t < max_group && (ka[e] >> 32) == k) e++;
        float* bx = &out.boxes[6 * ng];
        bx[0] = bx[1] = bx[2] = INFINITY;
        bx[3] = bx[4] = bx[5] = -INFINITY;
        uint64_t u = 0;
        for (size_t q = t; q < e; q++) {
            const auto& pr = *src[(uint32_t)ka[q]];
            dst[q] = pr.second;
            u += pr.first;
            const Box& b = A.boxes[pr.second.y];
            for (int d = 0; d < 3; d++) {
                bx[d] = std::min(bx[d], b.lo[d]);
                bx[3 + d] = std::max(bx[3 + d], b.hi[d]);
            }
        }
        out.sizes[ng] = (uint32_t)(e - t);
        out.units[ng++] = u;
        t = e;
    }
    out.sizes.resize(ng);
    out.boxes.resize(6 * ng);
    out.units.resize(ng);
}

// Group starts (ngroups + 1 entries) and boxes of the grouped windows, whose
// tasks are in place in `tasks` (window w from toff[w]).  With few tasks per
// CTA the groups go largest first (summed estimates), so that the dynamic
// fetch balances the tail; else in window order (job order).
void assemble_groups(const std::vector<GroupedPart>& gp, size_t nw, const std::vector<size_t>& toff,
                     bool largest_first, std::vector<uint4>& tasks, std::vector<uint32_t>& starts,
                     std::vector<float>& boxes) {
    std::vector<size_t> goff(nw + 1, 0);
    for (size_t i = 0; i < nw; i++) goff[i + 1] = goff[i] + gp[i].sizes.size();
    const size_t total = toff[nw], ng = goff[nw];
    starts.resize(ng + 1);
    boxes.resize(6 * ng);
    starts[ng] = (uint32_t)total;
    if (largest_first) {
        std::vector<std::array<uint32_t, 2>> ref;  // window, group in window
        std::vector<uint32_t> first;                // its first task
        std::vector<uint64_t> units;
        for (size_t i = 0; i < nw; i++)
            for (uint32_t g = 0, t = (uint32_t)toff[i]; g < gp[i].sizes.size(); t += gp[i].sizes[g], g++) {
                ref.push_back({(uint32_t)i, g});
                first.push_back(t);
                units.push_back(gp[i].units[g]);
            }
        std::vector<uint32_t> order(ng);
        for (size_t g = 0; g < ng; g++) order[g] = (uint32_t)g;
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return units[a] > units[b]; });
        const std::vector<uint4> in(tasks.begin(), tasks.begin() + total);
        size_t w = 0;
        for (size_t o = 0; o < ng; o++) {
            const auto& r = ref[order[o]];
            const GroupedPart& P = gp[r[0]];
            starts[o] = (uint32_t)w;
            for (uint32_t t = 0; t < P.sizes[r[1]]; t++) tasks[w++] = in[first[order[o]] + t];
            std::copy(&P.boxes[6 * r[1]], &P.boxes[6 * r[1]] + 6, &boxes[6 * o]);
        }
        return;
    }
    parallel_items(nw, [&](size_t i) {
        const GroupedPart& P = gp[i];
        std::copy(P.boxes.begin(), P.boxes.end(), boxes.begin() + 6 * goff[i]);
        uint32_t s = (uint32_t)toff[i];
        for (size_t g = 0; g < P.sizes.size(); g++) {
            starts[goff[i] + g] = s;
            s += P.sizes[g];
        }
    });
}

// Runs one group of jobs that share kind, binning and precision in a single
// persistent launch.  outs[i] receives hist_len counts.
void run_group(tpcf_ctx* ctx, Lane& L, const std::vector<GroupJob>& group) {
    auto t_wall0 = std::chrono::steady_clock::now();
    const tpcf_spec& sp = *group[0].spec;
    Binning bin = make_binning(sp);
    const int ncat = sp.kind == TPCF_PAIR ? 2 : 3;
    if (group.size() > MAX_BATCH_JOBS) throw InvalidArg{"too many jobs in one batch"};
    std::vector<PlannedJob> pj(group.size());
    std::vector<DevJob> dj(group.size());
    uint64_t evaluated = 0, units = 0;
    // device histogram slots: one per job, or one per distinct output for
    // accumulating jobs
    std::vector<size_t> slot_of(group.size());
    std::vector<size_t> slot_job;  // first job of each slot
    {
        std::map<uint64_t*, size_t> by_out;
        for (size_t g = 0; g < group.size(); g++) {
            if (group[g].accumulate) {
                auto it = by_out.find(group[g].out);
                if (it != by_out.end()) {
                    slot_of[g] = it->second;
                    continue;
                }
                by_out[group[g].out] = slot_job.size();
            }
            slot_of[g] = slot_job.size();
            slot_job.push_back(g);
        }
    }
    const size_t nslots = slot_job.size();
    size_t hist_total = (size_t)bin.len * nslots;
    L.d_hist.reserve(hist_total);
    // signature of the batch: a repeated batch over the same resident views
    // reuses its task list and device upload
    std::vector<uint64_t> sig;
    sig.push_back((uint64_t)(uintptr_t)L.d_hist.p);
    const char* rdd_env = getenv("TPCF_RDD");
    const bool rdd = !(rdd_env && rdd_env[0] == '0');
    // The batch signature takes the jobs' view ids; views still being built
    // (new catalogs) are waited for only when a job's planning needs them.
    // (A batch of many jobs names few distinct catalog ranges: each is looked
    // up once.)
    struct RangeKey {
        uint64_t h;
        int64_t b, e;
        bool gl;
        bool operator==(const RangeKey& o) const { return h == o.h && b == o.b && e == o.e && gl == o.gl; }
    };
    struct RangeHash {
        size_t operator()(const RangeKey& k) const {
            uint64_t x = k.h * 0x9E3779B97F4A7C15ull ^ (uint64_t)k.b * 0xC2B2AE3D27D4EB4Full ^
                         (uint64_t)k.e * 0x165667B19E3779F9ull ^ (uint64_t)k.gl;
            return (size_t)(x ^ (x >> 29));
        }
    };
    std::unordered_map<RangeKey, ViewRef, RangeHash> refs;
    sig.reserve(1 + group.size() * 22);
    for (size_t g = 0; g < group.size(); g++) {
        const tpcf_job& job = *group[g].job;
        const tpcf_spec& jsp = *group[g].spec;  // same binning as sp; the loop nest may differ
        int64_t n[3] = {0, 0, 0};
        uint64_t vid[3] = {0, 0, 0};
        for (int r = 0; r < ncat; r++) {
            const RangeKey k{job.catalog[r], job.begin[r], job.end[r], (job.flags & TPCF_JOB_GLOBAL_INDEX) != 0};
            auto it = refs.find(k);
            if (it == refs.end()) {
                ViewRef ref{};
                get_view(ctx, L, k.h, k.b, k.e, k.gl, &ref);
                it = refs.emplace(k, ref).first;
            }
            vid[r] = it->second.id;
            n[r] = it->second.n;
        }
        if (ncat == 2) vid[2] = vid[1];
        pj[g].loop_units = loop_units(jsp.kind, jsp.loop, n);
        units += pj[g].loop_units;
        pj[g].swap = 0;
        if (rdd && (jsp.kind == TPCF_TRIANGLE || jsp.kind == TPCF_TRIANGLE_JBJ) &&
            guarded_fp32(jsp, bin) && jsp.loop == TPCF_LOOP_ONE) {
            if (vid[0] == vid[1] && vid[1] != vid[2]) pj[g].swap = 1;
            else if (vid[1] == vid[2] && vid[0] != vid[1]) pj[g].swap = 2;
        }
        for (int r = 0; r < 3; r++) {  // role r's view (PlannedJob::role)
            const int v = pj[g].swap == 1 ? (r == 0 ? 2 : 0) : pj[g].swap == 2 ? (r == 2 ? 0 : 1) : r;
            sig.push_back(vid[v]);
        }
        sig.push_back(pj[g].swap);
        sig.push_back(slot_of[g]);
        uint64_t f[6] = {(uint64_t)jsp.kind, (uint64_t)jsp.loop, (uint64_t)jsp.prune, (uint64_t)jsp.precision,
                         (uint64_t)jsp.nan_policy, (uint64_t)jsp.overflow};
        sig.insert(sig.end(), f, f + 6);
        for (int a = 0; a < 3; a++) {
            sig.push_back((uint64_t)fbits(jsp.axis[a].lo) << 32 | fbits(jsp.axis[a].hi));
            sig.push_back((uint64_t)(uint32_t)jsp.axis[a].nbins);
        }
    }
    // the views of job g (waiting for any still being built) and its device job
    auto attach = [&](size_t g) {
        const tpcf_job& job = *group[g].job;
        for (int r = 0; r < ncat; r++)
            pj[g].v[r] = get_view(ctx, L, job.catalog[r], job.begin[r], job.end[r],
                                  (job.flags & TPCF_JOB_GLOBAL_INDEX) != 0);
        if (ncat == 2) pj[g].v[2] = pj[g].v[1];
        for (int r = 0; r < 3; r++) {
            const View* rv = pj[g].role(r);
            dj[g].pts[r] = rv->pts.p;
            dj[g].tile_start[r] = rv->tile_start.p;
        }
        dj[g].hist = L.d_hist.p + (size_t)bin.len * slot_of[g];
    };
    cudaStream_t st = L.stream;
    L.d_counters.reserve(8);
    size_t ntasks = 0, ngroups = 0;
    const bool plan_hit = sig == L.plan_sig;
    std::vector<std::pair<const char*, double>> phases;
    auto phase = [&](const char* name) {
        if (plan_trace())
            phases.push_back({name, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() -
                                                                              t_wall0).count()});
    };
    const bool pairs = sp.kind == TPCF_PAIR;
    const bool fast_tri = (sp.kind == TPCF_TRIANGLE || sp.kind == TPCF_TRIANGLE_JBJ) && guarded_fp32(sp, bin);
    // A newly planned batch of two to eight fast-kernel jobs (an estimator's
    // DDD/DDR/DRR/RRR set) is pipelined: the first job is planned, uploaded and
    // launched, and the others are planned while it counts (a second launch
    // follows on the same stream).  Larger batches -- voxel and jackknife sets
    // of many similar jobs, whose first job is a small share -- keep one launch.
    const char* pl_env = getenv("TPCF_PIPELINE");
    const bool pipeline = !plan_hit && fast_tri && group.size() >= 2 && group.size() <= 8 && !L.slice_batches &&
                          !(pl_env && pl_env[0] == '0');
    // a pipelined batch waits here for the first job's views only (a planned
    // batch needs none: its device jobs are in place)
    if (!plan_hit)
        for (size_t g = 0; g < (pipeline ? 1 : group.size()); g++) attach(g);
    phase("views");
    size_t ntasks2 = 0, ngroups2 = 0;
    uint64_t evaluated2 = 0;
    // planning state shared by the parts of a plan: bound tables by view pair
    std::vector<TripletPlan> tp(pairs ? 0 : group.size());
    struct ViewPairHash {
        size_t operator()(const std::pair<const View*, const View*>& k) const {
            const uint64_t x = (uint64_t)(uintptr_t)k.first * 0x9E3779B97F4A7C15ull ^ (uint64_t)(uintptr_t)k.second;
            return (size_t)(x ^ (x >> 31));
        }
    };
    std::unordered_map<std::pair<const View*, const View*>, std::unique_ptr<PairTable>, ViewPairHash> tables;
    std::vector<PairTable*> table_list;
    int plan_pass = 0;
    // Plans jobs [g0, g1) into task list, group starts and group boxes (the
    // last two for the fast triangle kernel); returns the evaluated units.
    auto plan_jobs = [&](size_t g0, size_t g1, std::vector<uint4>& h_tasks, std::vector<uint32_t>& h_groups,
                         std::vector<float>& h_gbox) -> uint64_t {
        // plan in parallel: bound tables and neighbour lists by rows, then
        // tile triples (pairs) by ranges of A tiles
        uint64_t ev = 0;
        if (!pairs) {
            const size_t t_first = table_list.size();
            const int pass = plan_pass++;
            auto table = [&](const View* x, const View* y, bool nb) {
                auto& t = tables[std::make_pair(x, y)];
                if (!t) {
                    t.reset(new PairTable());
                    t->init(*x, *y, bin.lmax);
                    t->listed = pass;
                    table_list.push_back(t.get());
                }
                if (nb && !t->need_nb) {
                    if (t->listed != pass) {  // filled by an earlier pass without neighbour lists: fill again
                        t->listed = pass;
                        table_list.push_back(t.get());
                    }
                    t->need_nb = true;
                    t->nb.assign(x->ntiles, {});
                }
                return t.get();
            };
            for (size_t g = g0; g < g1; g++) {
                const View *A = pj[g].role(0), *B = pj[g].role(1), *C = pj[g].role(2);
                const bool empty = A->ntiles == 0 || B->ntiles == 0 || C->ntiles == 0;
                tp[g].init(*group[g].spec, pj[g], (uint32_t)g, bin, empty ? nullptr : table(A, B, true),
                           empty ? nullptr : table(A, C, true), empty ? nullptr : table(B, C, false));
            }
            std::vector<std::array<int, 3>> items;  // table, row begin, row end
            for (size_t t = t_first; t < table_list.size(); t++)
                for (int r = 0; r < table_list[t]->x->ntiles; r += 16)
                    items.push_back({(int)t, r, std::min(r + 16, table_list[t]->x->ntiles)});
            parallel_items(items.size(), [&](size_t i) {
                const auto& it = items[i];
                table_list[it[0]]->rows(it[1], it[2]);
            });
        }
        phase("tables");
        // items: job, A-tile begin, end, and for a heavy single tile the
        // part [lo, hi) of its neighbour list taken as tile B (the work of a
        // tile grows with the square of its neighbour count: the densest
        // tiles of a clustered catalog would otherwise each be one long item)
        std::vector<std::array<int, 5>> items;
        for (size_t g = g0; g < g1; g++) {
            const int na = pj[g].role(0)->ntiles, step = pairs ? 16 : 2;
            const PairTable* ab = pairs || tp[g].empty ? nullptr : tp[g].AB;
            for (int a0 = 0; a0 < na;) {
                const int nb = ab && ab->need_nb ? (int)ab->nb[a0].size() : 0;
                if (nb > 48) {
                    for (int lo = 0; lo < nb; lo += 24) items.push_back({(int)g, a0, a0 + 1, lo, lo + 24});
                    a0++;
                } else {
                    const int a1 = std::min(a0 + step, na);
                    items.push_back({(int)g, a0, a1, 0, INT_MAX});
                    a0 = a1;
                }
            }
        }
        // one task list per item, so that the concatenation keeps job order
        // (a CTA flushes its shared histogram whenever the job changes)
        PlanScratch& S = L.scratch;
        std::vector<TaskList>& part = S.part;
        if (part.size() < items.size()) part.resize(items.size());
        std::vector<uint64_t> part_eval(items.size(), 0);
        parallel_items(items.size(), [&](size_t i) {
            const auto& it = items[i];
            part[i].clear();
            if (pairs)
                plan_pairs(*group[it[0]].spec, pj[it[0]], (uint32_t)it[0], bin.lmax, it[1], it[2], part[i],
                           part_eval[i]);
            else
                tp[it[0]].enumerate(it[1], it[2], part[i], part_eval[i], (size_t)it[3], (size_t)it[4]);
        });
        phase("enumerate");
        std::vector<size_t> off(items.size() + 1, 0);  // each item's first task
        for (size_t i = 0; i < items.size(); i++) {
            ev += part_eval[i];
            off[i + 1] = off[i] + part[i].size();
        }
        const size_t total = off[items.size()];
        // tasks per group of the fast triangle kernel: 4, or 64 for sets of
        // many jobs with thousands of tasks per CTA (voxel and jackknife sets
        // of light tasks: the j-k tables are the larger share there, and the
        // tail of a few large groups a small one; tp10k 12.91 ms with 4, 13.00
        // with 8; voxel100k 267 ms with 4, 236 with 16, 230 with 32, 226 with
        // 64; a heavy serving batch of a few dense jobs keeps 4)
        const size_t group_max =
            ctx->group_tasks > 0 ? (size_t)ctx->group_tasks
                                 : (g1 - g0 > 64 && total >= (size_t)ctx->num_sms * 4 * 4096 ? MAX_GROUP_TASKS : 4);
        // fast triangle kernel: groups form in windows of consecutive items of
        // one job whose first A tiles lie in one aligned span of twice the
        // group size
        std::vector<std::array<size_t, 2>> windows;  // first item, item count
        if (fast_tri) {
            const int span = 2 * (int)group_max;
            for (size_t i = 0; i < items.size();) {
                size_t e = i + 1;
                while (e < items.size() && items[e][0] == items[i][0] && items[e][1] / span == items[i][1] / span) e++;
                windows.push_back({i, e - i});
                i = e;
            }
        }
        h_tasks.resize(total);
        h_groups.clear();
        h_gbox.clear();
        if (fast_tri) {
            if (S.gpart.size() < windows.size()) S.gpart.resize(windows.size());
            std::vector<size_t> toff(windows.size() + 1);
            for (size_t w = 0; w < windows.size(); w++) toff[w] = off[windows[w][0]];
            toff[windows.size()] = total;
            parallel_items(windows.size(), [&](size_t w) {
                group_parts(&part[windows[w][0]], windows[w][1], pj[items[windows[w][0]][0]],
                            group_max, h_tasks.data() + toff[w], S.gpart[w]);
            });
            assemble_groups(S.gpart, windows.size(), toff, total <= (size_t)ctx->num_sms * 3 * 64, h_tasks, h_groups,
                            h_gbox);
        } else if (total <= (size_t)ctx->num_sms * 3 * 64 && !(sp.kind == TPCF_THREE_SIDE && bin.len > 8192)) {
            // (three-side histograms above 8192 bins keep job order: their CTAs
            // flush, and the task pipelines of one CTA meet, at every job change)
            // few tasks per CTA: largest first, so that the dynamic fetch
            // balances the tail (a stable counting pass over 64 size classes)
            auto cls = [](uint64_t u) { return 63 - (u ? 63 - __builtin_clzll(u) : 0); };
            std::vector<size_t> start(65, 0);
            for (size_t i = 0; i < items.size(); i++)
                for (auto& e : part[i]) start[cls(e.first) + 1]++;
            for (int c = 0; c < 64; c++) start[c + 1] += start[c];
            for (size_t i = 0; i < items.size(); i++)
                for (auto& e : part[i]) h_tasks[start[cls(e.first)]++] = e.second;
        } else {
            // many tasks per CTA: the tail is a small share; job order
            parallel_items(items.size(), [&](size_t i) {
                for (size_t e = 0; e < part[i].size(); e++) h_tasks[off[i] + e] = part[i][e].second;
            });
        }
        phase("order");
        return ev;
    };
    // Uploads a planned part on stream s into the given buffers; returns the
    // group count.
    auto upload_part = [&](const std::vector<uint4>& h_tasks, const std::vector<uint32_t>& h_groups,
                           const std::vector<float>& h_gbox, DevBuf<uint4>& d_tasks, DevBuf<uint32_t>& d_groups,
                           DevBuf<float>& d_gbox, cudaStream_t s) -> size_t {
        const size_t ng = h_groups.empty() ? 0 : h_groups.size() - 1;
        if (ng) {
            d_groups.reserve(h_groups.size());
            d_gbox.reserve(h_gbox.size());
            CK(cudaMemcpyAsync(d_groups.p, h_groups.data(), h_groups.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(d_gbox.p, h_gbox.data(), h_gbox.size() * sizeof(float), cudaMemcpyHostToDevice, s));
            L.h2d += h_groups.size() * sizeof(uint32_t) + h_gbox.size() * sizeof(float);
        }
        d_tasks.reserve(std::max<size_t>(h_tasks.size(), 1));
        L.h2d += h_tasks.size() * sizeof(uint4);
        if (!h_tasks.empty())
            CK(cudaMemcpyAsync(d_tasks.p, h_tasks.data(), h_tasks.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
        return ng;
    };
    if (plan_hit) {
        ntasks = L.plan_ntasks;
        ngroups = L.plan_ngroups;
        ntasks2 = L.plan_ntasks2;
        ngroups2 = L.plan_ngroups2;
        evaluated = L.plan_evaluated;
    } else {
        L.plan_sig.clear();  // (set again once the whole plan is on the device)
        PlanScratch& S = L.scratch;
        const size_t g_first = pipeline ? 1 : group.size();
        evaluated = plan_jobs(0, g_first, S.tasks, S.groups, S.gbox);
        L.d_jobs.reserve(dj.size());
        CK(cudaMemcpyAsync(L.d_jobs.p, dj.data(), g_first * sizeof(DevJob), cudaMemcpyHostToDevice, st));
        L.h2d += g_first * sizeof(DevJob);
        ngroups = upload_part(S.tasks, S.groups, S.gbox, L.d_tasks, L.d_groups, L.d_gbox, st);
        ntasks = S.tasks.size();
        CK(cudaStreamSynchronize(st));
        if (!pipeline) {
            L.plan_sig = sig;
            L.plan_ntasks = ntasks;
            L.plan_ngroups = ngroups;
            L.plan_ntasks2 = L.plan_ngroups2 = 0;
            L.plan_evaluated = evaluated;
        }
        phase("upload");
    }
    // the second part of a pipelined plan, planned and uploaded (on the side
    // stream) while the first part counts; the counting stream waits for it
    bool second_pending = pipeline;
    auto plan_second = [&]() {
        PlanScratch& S = L.scratch;
        for (size_t g = 1; g < group.size(); g++) attach(g);
        evaluated2 = plan_jobs(1, group.size(), S.tasks2, S.groups2, S.gbox2);
        if (!L.side) {
            // (the lane's priority: a light serving lane's second part must
            // not queue behind a heavy batch's CTAs)
            int prio = 0;
            CK(cudaStreamGetPriority(st, &prio));
            CK(cudaStreamCreateWithPriority(&L.side, cudaStreamNonBlocking, prio));
            CK(cudaEventCreateWithFlags(&L.ev_side, cudaEventDisableTiming));
        }
        CK(cudaMemcpyAsync(L.d_jobs.p + 1, dj.data() + 1, (group.size() - 1) * sizeof(DevJob),
                           cudaMemcpyHostToDevice, L.side));
        L.h2d += (group.size() - 1) * sizeof(DevJob);
        ngroups2 = upload_part(S.tasks2, S.groups2, S.gbox2, L.d_tasks2, L.d_groups2, L.d_gbox2, L.side);
        ntasks2 = S.tasks2.size();
        evaluated += evaluated2;
        second_pending = false;
        phase("second part");
    };
    // The merged plan (the first part's groups, then the second's, its task
    // indices shifted), uploaded on a stream of its own while the parts count;
    // it replaces the two parts once they are done.
    bool merge_pending = pipeline;
    auto merge_plan = [&]() {
        PlanScratch& S = L.scratch;
        S.tasks3.resize(ntasks + ntasks2);
        std::copy(S.tasks.begin(), S.tasks.end(), S.tasks3.begin());
        std::copy(S.tasks2.begin(), S.tasks2.end(), S.tasks3.begin() + ntasks);
        S.groups3.resize(ngroups + ngroups2 + 1);
        for (size_t g = 0; g < ngroups; g++) S.groups3[g] = S.groups[g];
        for (size_t g = 0; g <= ngroups2; g++)
            S.groups3[ngroups + g] = (uint32_t)ntasks + (ngroups2 ? S.groups2[g] : 0u);
        S.gbox3.resize(6 * (ngroups + ngroups2));
        std::copy(S.gbox.begin(), S.gbox.begin() + 6 * ngroups, S.gbox3.begin());
        std::copy(S.gbox2.begin(), S.gbox2.begin() + 6 * ngroups2, S.gbox3.begin() + 6 * ngroups);
        if (!L.side2) CK(cudaStreamCreateWithFlags(&L.side2, cudaStreamNonBlocking));
        const uint64_t h2d0 = L.h2d;
        upload_part(S.tasks3, S.groups3, S.gbox3, L.d_tasks3, L.d_groups3, L.d_gbox3, L.side2);
        L.h2d = h2d0;  // (a copy for later calls: not this count's input)
        merge_pending = false;
    };
    L.stats.plan_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_wall0).count();
    const bool fp64 = !guarded_fp32(sp, bin);
    const bool fast_jbj = sp.kind == TPCF_TRIANGLE_JBJ && !fp64;  // the fast kernel's JBJ binning
    if (sp.kind == TPCF_TRIANGLE) ensure_acos(ctx);
    const AcosTable acos_t = sp.kind == TPCF_TRIANGLE ? acos_table(ctx) : AcosTable{};
    const unsigned int nt = (unsigned int)ntasks;
    uint64_t launches = (sp.kind == TPCF_TRIANGLE && !fp64) ? 2 : 1;  // counting (+ recheck)
    const char* genv = getenv("TPCF_GRAPHS");
    const bool graphs = L.graphs_ok && !(genv && genv[0] == '0');
    L.h_hist.reserve(hist_total);
    L.h_counters.reserve(8);
    // recheck queue: at least 4M entries; TPCF_RECHECK_CAP lowers the floor
    // (tests use it to run the overflow path: grow the queue, count again)
    size_t queue_floor = (size_t)1 << 22;
    if (const char* qc = getenv("TPCF_RECHECK_CAP")) queue_floor = (size_t)std::max(1L, std::atol(qc));
    unsigned int queue_cap = (unsigned int)std::max<size_t>(L.d_queue.n, queue_floor);
    uint64_t dev_evaluated = 0, dev_binned = 0, replays = 0, regrows = 0;

    // One complete count of the group with launch shape sh: zero, count,
    // recheck, copy back (replayed from a captured graph when allowed and
    // the batch repeats).  Returns the device time in ms.
    auto count_with = [&](const Shape& sh, bool allow_graph) -> float {
        const int copies = sh.copies;
        // units the persistent CTAs pull: task groups (fast triangle kernel) or tasks
        const unsigned int nwork = fast_tri ? (unsigned int)ngroups : nt;
        const int grid = grid_for(ctx, sh, nwork, L.sm_cap);
        // slices of at least 8 units per CTA, at most 64 of them
        unsigned int slice = L.slice_batches ? std::max<unsigned int>((unsigned int)grid * 8u, (nwork + 63u) / 64u)
                                             : std::max(nwork, 1u);
        if (L.slice_batches && ctx->slice_tasks > 0) slice = (unsigned int)ctx->slice_tasks;
        // a pipelined plan: two launches, one per part
        const bool two_part = fast_tri && (ngroups2 > 0 || second_pending);
        launches = (two_part ? 2 : (nwork > slice ? (nwork + slice - 1) / slice : 1)) +
                   ((sp.kind == TPCF_TRIANGLE && !fp64) ? 1 : 0);
        for (int attempt = 0; attempt < 3; attempt++) {
            RecheckQueue q{};
            if (sp.kind == TPCF_TRIANGLE && !fp64) {
                if (L.d_queue.n < queue_cap) L.drop_graph();
                L.d_queue.reserve(queue_cap);
                q.items = L.d_queue.p;
                q.count = L.d_counters.p + 1;
                q.cap = queue_cap;
                q.evaluated = reinterpret_cast<unsigned long long*>(L.d_counters.p + 2);
            } else if (fast_jbj) {
                q.count = L.d_counters.p + 1;  // no item is ever queued (cap 0)
                q.evaluated = reinterpret_cast<unsigned long long*>(L.d_counters.p + 2);
            }
            auto enqueue = [&](bool capturing) -> cudaError_t {
                const unsigned int ev_flags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
                cudaError_t e;
#define EQ(x)                                   \
    do {                                        \
        if ((e = (x)) != cudaSuccess) return e; \
    } while (0)
                EQ(cudaMemsetAsync(L.d_hist.p, 0, hist_total * sizeof(unsigned long long), st));
                EQ(cudaMemsetAsync(L.d_counters.p, 0, 8 * sizeof(unsigned int), st));
                EQ(cudaEventRecordWithFlags(L.ev0, st, ev_flags));
                // the counting kernel over tasks [t0, t0 + n) (groups [t0, t0 + n)
                // for the fast triangle kernel)
                auto launch_main = [&](unsigned int t0, unsigned int n) -> cudaError_t {
                    const uint4* tk = L.d_tasks.p + t0;
                    if (sp.kind == TPCF_TRIANGLE && fp64)
                        return launch_triangle_fp64(L.d_jobs.p, tk, n, L.d_counters.p, bin.tri, acos_t, grid, copies,
                                                    sp.precision == TPCF_GEOMETRY_FP64 ? 1 : 0, st);
                    if (sp.kind == TPCF_TRIANGLE || fast_jbj)  // JBJ in FP32: exact without a recheck
                        return launch_triangle_fast(L.d_jobs.p, L.d_tasks.p, L.d_groups.p + t0, L.d_gbox.p + 6 * (size_t)t0,
                                                    n, L.d_counters.p, bin.tri, q, grid, copies, fast_jbj ? 1 : 0, st);
                    if (sp.kind == TPCF_TRIANGLE_JBJ)
                        return launch_triangle_fp64(L.d_jobs.p, tk, n, L.d_counters.p, bin.tri, acos_t, grid, copies, 2,
                                                    st);
                    if (sp.kind == TPCF_THREE_SIDE)
                        return launch_three_side(L.d_jobs.p, tk, n, L.d_counters.p, bin.three, fp64, grid, copies,
                                                 sh.groups, st);
                    return launch_pairs(L.d_jobs.p, tk, n, L.d_counters.p, bin.pair, fp64, grid, copies, st);
                };
                if (two_part) {
                    // the first job's groups, then the others' (their own group
                    // counter, d_counters[6]); on the first count of a pipelined
                    // plan the second part is planned between the two launches
                    EQ(launch_main(0, (unsigned int)ngroups));
                    if (second_pending) plan_second();
                    if (ngroups2) {
                        // on the side stream, behind its upload and the zeroing of
                        // the histograms and counters: its CTAs take the SMs the
                        // first part's CTAs leave at its end
                        EQ(cudaStreamWaitEvent(L.side, L.ev0, 0));
                        EQ(launch_triangle_fast(L.d_jobs.p, L.d_tasks2.p, L.d_groups2.p, L.d_gbox2.p,
                                                (unsigned int)ngroups2, L.d_counters.p + 6, bin.tri, q,
                                                grid_for(ctx, sh, ngroups2, L.sm_cap), copies, fast_jbj ? 1 : 0,
                                                L.side));
                        EQ(cudaEventRecord(L.ev_side, L.side));
                        EQ(cudaStreamWaitEvent(st, L.ev_side, 0));
                    }
                    if (merge_pending) merge_plan();
                } else {
                    // one launch over all tasks, or (a heavy serving batch) slices of
                    // them, between which the device can start the kernels that
                    // higher-priority streams (the light serving lanes) have queued
                    EQ(launch_main(0, std::min(nwork, slice)));
                    for (unsigned int t0 = slice; t0 < nwork; t0 += slice) {
                        EQ(cudaMemsetAsync(L.d_counters.p, 0, sizeof(unsigned int), st));  // the slice's task counter
                        EQ(launch_main(t0, std::min(slice, nwork - t0)));
                    }
                }
                EQ(cudaEventRecordWithFlags(L.ev_mid, st, ev_flags));
                if (sp.kind == TPCF_TRIANGLE && !fp64)
                    EQ(launch_triangle_recheck(L.d_jobs.p, q, bin.tri, acos_t, ctx->num_sms * 8, st));
                EQ(cudaEventRecordWithFlags(L.ev1, st, ev_flags));
                EQ(cudaMemcpyAsync(L.h_counters.p, L.d_counters.p, 8 * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                   st));
                EQ(cudaMemcpyAsync(L.h_hist.p, L.d_hist.p, hist_total * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, st));
#undef EQ
                return cudaSuccess;
            };
            bool replayed = false;
            if (allow_graph) {
                // everything the captured launches read: the batch, its buffers, the shape
                std::vector<uint64_t> gsig = sig;
                const uint64_t extra[] = {(uint64_t)(uintptr_t)L.d_jobs.p, (uint64_t)(uintptr_t)L.d_tasks.p,
                                          (uint64_t)(uintptr_t)L.d_counters.p, (uint64_t)(uintptr_t)L.d_queue.p,
                                          (uint64_t)(uintptr_t)L.h_hist.p, (uint64_t)(uintptr_t)L.h_counters.p,
                                          (uint64_t)(uintptr_t)acos_t.keys, (uint64_t)(uintptr_t)acos_t.vals,
                                          (uint64_t)(uintptr_t)acos_t.bucket, (uint64_t)acos_t.n, queue_cap,
                                          (uint64_t)grid, (uint64_t)copies, (uint64_t)sh.groups, hist_total, ntasks,
                                          (uint64_t)slice, (uint64_t)(uintptr_t)L.d_groups.p,
                                          (uint64_t)(uintptr_t)L.d_gbox.p, (uint64_t)ngroups,
                                          (uint64_t)(uintptr_t)L.d_tasks2.p, (uint64_t)(uintptr_t)L.d_groups2.p,
                                          (uint64_t)(uintptr_t)L.d_gbox2.p, (uint64_t)ngroups2};
                gsig.insert(gsig.end(), extra, extra + sizeof(extra) / sizeof(extra[0]));
                if (!L.graph || gsig != L.graph_sig) {
                    L.drop_graph();
                    cudaGraph_t g = nullptr;
                    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
                    if (e == cudaSuccess) {
                        cudaError_t e1 = enqueue(true);
                        cudaError_t e2 = cudaStreamEndCapture(st, &g);
                        e = e1 != cudaSuccess ? e1 : e2;
                    }
                    if (e == cudaSuccess) e = cudaGraphInstantiate(&L.graph, g, 0);
                    if (g) cudaGraphDestroy(g);
                    if (e == cudaSuccess) {
                        L.graph_sig = gsig;
                    } else {
                        // capture unavailable here: issue the launches one by one from now on
                        (void)cudaGetLastError();
                        L.graph = nullptr;
                        L.graphs_ok = false;
                    }
                }
                if (L.graph) {
                    CK(cudaGraphLaunch(L.graph, st));
                    replayed = true;
                }
            }
            if (!replayed) CK(enqueue(false));
            CK(cudaStreamSynchronize(st));
            replays = replayed ? 1 : 0;
            const unsigned int* counters = L.h_counters.p;
            L.d2h += 8 * sizeof(unsigned int) + hist_total * sizeof(unsigned long long);
            L.stats.recheck_units = counters[1];
            memcpy(&dev_evaluated, &counters[2], sizeof(dev_evaluated));
            memcpy(&dev_binned, &counters[4], sizeof(dev_binned));
            if (sp.kind == TPCF_TRIANGLE && !fp64 && counters[1] > queue_cap) {
                // the recheck queue overflowed: grow it and count again
                queue_cap =
                    (unsigned int)std::min<uint64_t>((uint64_t)counters[1] + (counters[1] >> 2) + 1024, 0xF0000000ull);
                regrows++;
                continue;
            }
            break;
        }
        float t = 0;
        CK(cudaEventElapsedTime(&t, L.ev0, L.ev1));
        return t;
    };

    // Launch shape: the tuned one for this batch if the autotuner has seen it,
    // else the default.  A batch that repeats (its plan was cached) and has no
    // tuned shape yet is counted once with every candidate shape -- each count
    // is exact -- and the fastest is kept for the next calls.
    const std::vector<Shape> cands = shape_candidates(ctx, sp, bin, fp64);
    uint64_t key = 1469598103934665603ull;
    for (uint64_t v : sig) key = (key ^ v) * 1099511628211ull;
    const char* tenv = getenv("TPCF_AUTOTUNE");
    const bool autotune = !(tenv && tenv[0] == '0');
    Shape shape = cands[0];
    uint64_t tuned_runs = 0;
    {
        std::lock_guard<std::mutex> tlk(ctx->tune_mu);
        auto it = ctx->tuned.find(key);
        if (it != ctx->tuned.end()) shape = it->second;
    }
    bool tuned_known = false;
    {
        std::lock_guard<std::mutex> tlk(ctx->tune_mu);
        tuned_known = ctx->tuned.count(key) > 0;
    }
    if (autotune && plan_hit && !tuned_known && cands.size() > 1) {
        float best = INFINITY;
        for (const Shape& c : cands) {
            float t = count_with(c, false);
            tuned_runs++;
            if (t < best) {
                best = t;
                shape = c;
            }
        }
        std::lock_guard<std::mutex> tlk(ctx->tune_mu);
        ctx->tuned[key] = shape;
    } else {
        count_with(shape, graphs && !pipeline);  // (the first count of a pipelined plan is not captured)
    }
    if (pipeline) {
        // the parts are done: later counts of the batch use the merged plan
        CK(cudaStreamSynchronize(L.side2));
        L.d_tasks.swap(L.d_tasks3);
        L.d_groups.swap(L.d_groups3);
        L.d_gbox.swap(L.d_gbox3);
        L.plan_sig = sig;
        L.plan_ntasks = ntasks + ntasks2;
        L.plan_ngroups = ngroups + ngroups2;
        L.plan_ntasks2 = L.plan_ngroups2 = 0;
        L.plan_evaluated = evaluated;
    }
    L.stats.tuned_shapes = tuned_runs;
    L.stats.hist_copies = (uint64_t)shape.copies;
    L.stats.ctas_per_sm = (uint64_t)shape.per_sm;
    float ms = 0, ms_main = 0;
    CK(cudaEventElapsedTime(&ms, L.ev0, L.ev1));
    CK(cudaEventElapsedTime(&ms_main, L.ev0, L.ev_mid));
    L.stats.main_kernel_ms = ms_main;
    // JBJ compat: the reference's two extra counts in bin 0 per visited triangle
    if (sp.kind == TPCF_TRIANGLE_JBJ && sp.overflow == TPCF_OVERFLOW_COMPAT && bin.len > 0)
        for (size_t g = 0; g < group.size(); g++) L.h_hist.p[(size_t)bin.len * slot_of[g]] += 2 * pj[g].loop_units;
    for (size_t k = 0; k < nslots; k++) {
        const GroupJob& gj = group[slot_job[k]];
        const unsigned long long* src = L.h_hist.p + (size_t)bin.len * k;
        if (gj.accumulate) {
            for (int64_t b = 0; b < bin.len; b++) gj.out[b] += src[b];
        } else {
            memcpy(gj.out, src, (size_t)bin.len * sizeof(uint64_t));
        }
    }
    L.stats.graph_replays = replays;
    L.stats.kernel_ms = ms;
    L.stats.loop_units = units;
    // the fast triangle kernel skips (i,j) pairs that no counted triangle can
    // contain and counts the triangles it walks; other kernels walk every
    // triangle of their tasks
    const bool fast_kernel = (sp.kind == TPCF_TRIANGLE || sp.kind == TPCF_TRIANGLE_JBJ) && !fp64;
    L.stats.evaluated_units = fast_kernel ? dev_evaluated : evaluated;
    L.stats.binned_units = fast_kernel ? dev_binned : evaluated;
    L.stats.tasks = ntasks + ntasks2;
    L.stats.kernel_launches = launches * std::max<uint64_t>(1, tuned_runs);
    L.stats.recheck_regrows = regrows;
    L.stats.total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_wall0).count();
    if (plan_trace()) {
        std::string line = "tpcf plan: tasks " + std::to_string(ntasks + ntasks2) + " groups " +
                           std::to_string(ngroups + ngroups2) + (pipeline ? " (two parts)" : "");
        double prev = 0;
        for (auto& ph : phases) {
            line += std::string(" ") + ph.first + " " + std::to_string(ph.second - prev);
            prev = ph.second;
        }
        line += " total " + std::to_string(L.stats.total_ms);
        fprintf(stderr, "%s\n", line.c_str());
    }
}

void validate(const tpcf_spec* sp, const tpcf_job* job) {
    if (!sp || !job) throw InvalidArg{"null spec or job"};
    if (sp->kind != TPCF_THREE_SIDE && sp->kind != TPCF_TRIANGLE && sp->kind != TPCF_PAIR &&
        sp->kind != TPCF_TRIANGLE_JBJ)
        throw InvalidArg{"bad kind"};
    if (sp->loop < TPCF_LOOP_ALL || sp->loop > TPCF_LOOP_ONE) throw InvalidArg{"bad loop"};
    if (sp->precision != TPCF_GUARDED_FP32 && sp->precision != TPCF_PLAIN_FP64 && sp->precision != TPCF_GEOMETRY_FP64)
        throw InvalidArg{"bad precision"};
    if (sp->precision == TPCF_GEOMETRY_FP64 && sp->kind != TPCF_TRIANGLE)
        throw InvalidArg{"TPCF_GEOMETRY_FP64 is implemented for the triangle parametrization only"};
    if ((job->flags & ~(uint32_t)TPCF_JOB_GLOBAL_INDEX) != 0 || job->reserved != 0) throw InvalidArg{"bad job flags"};
    (void)make_binning(*sp);
}

template <typename F>
tpcf_status guarded(tpcf_ctx* ctx, F&& f) {
    try {
        f();
        return TPCF_OK;
    } catch (const InvalidArg& e) {
        return fail(ctx, TPCF_ERR_INVALID, e.msg);
    } catch (const CudaError& e) {
        cudaGetLastError();
        if (e.e == cudaErrorMemoryAllocation) return fail(ctx, TPCF_ERR_OOM, cudaGetErrorString(e.e));
        return fail(ctx, TPCF_ERR_CUDA, cudaGetErrorString(e.e));
    } catch (const std::bad_alloc&) {
        return fail(ctx, TPCF_ERR_OOM, "host allocation failed");
    } catch (...) {
        return fail(ctx, TPCF_ERR_INTERNAL, "unexpected exception");
    }
}

// footprint estimate of a job for admission (views are shared and cached)
int64_t job_bytes(tpcf_ctx* ctx, const tpcf_spec& sp, const tpcf_job& job) {
    int64_t b = 0;
    int nc = sp.kind == TPCF_PAIR ? 2 : 3;
    for (int r = 0; r < nc; r++) {
        auto it = ctx->catalogs.find(job.catalog[r]);
        if (it == ctx->catalogs.end()) continue;
        int64_t e = job.end[r] < 0 ? it->second->n : job.end[r];
        b += (e - job.begin[r]) * (int64_t)sizeof(float4);
    }
    int64_t len = 0;
    tpcf_hist_len(&sp, &len);
    return b + len * 8;
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Serving worker on lane 'lane'.  It takes the oldest pending job plus every
// pending job of the same binning that fits the admission budget (device
// bytes of all batches in flight on the serving lanes), counts them in one
// persistent launch on its own stream and completes their tickets.  Jobs that
// arrive meanwhile are taken by the next free worker, so batches overlap on
// the device.
// Work estimate of a job for scheduling: the product of its catalog range
// sizes (the loop size up to a constant).
// Mean number of points of catalog range b within 'reach' of a point of range
// a, from 64 points spread over range a (cached per ranges and reach).
// Called with ctx->mu held.
double neighbour_density(tpcf_ctx* ctx, uint64_t ha, int64_t a0, int64_t a1, uint64_t hb, int64_t b0, int64_t b1,
                         double reach) {
    auto key = std::make_tuple(ha, a0, a1, hb, b0, b1, reach);
    auto hit = ctx->density.find(key);
    if (hit != ctx->density.end()) return hit->second;
    const Catalog& A = *ctx->catalogs.at(ha);
    const Catalog& B = *ctx->catalogs.at(hb);
    const int64_t na = a1 - a0;
    const double r2 = reach * reach;
    const int samples = (int)std::min<int64_t>(64, na);
    uint64_t near = 0;
    for (int t = 0; t < samples; t++) {
        const int64_t i = a0 + (int64_t)t * na / samples;
        for (int64_t j = b0; j < b1; j++) {
            const double dx = (double)A.x[i] - B.x[j], dy = (double)A.y[i] - B.y[j], dz = (double)A.z[i] - B.z[j];
            near += dx * dx + dy * dy + dz * dz < r2;
        }
    }
    const double rho = samples ? (double)near / samples : 0.0;
    ctx->density[key] = rho;
    return rho;
}

// Work estimate of a job for serving (which lane, how many per batch): the
// number of index pairs (pairs) or of i-j, i-k pairs of sides (triangles)
// within the largest side that can be counted, from the neighbour densities;
// the product of the range sizes where every triple counts.  Called with
// ctx->mu held, at submission.
double job_cost(tpcf_ctx* ctx, const tpcf_spec& sp, const tpcf_job& job) {
    int nc = sp.kind == TPCF_PAIR ? 2 : 3;
    int64_t b[3] = {0, 0, 0}, e[3] = {0, 0, 0};
    double prod = 1;
    for (int r = 0; r < nc; r++) {
        auto it = ctx->catalogs.find(job.catalog[r]);
        if (it == ctx->catalogs.end()) return 0;
        b[r] = job.begin[r];
        e[r] = job.end[r] < 0 ? it->second->n : job.end[r];
        prod *= (double)std::max<int64_t>(e[r] - b[r], 0);
    }
    const double reach = make_binning(sp).lmax;
    if (!(reach < 1e30) || (sp.kind == TPCF_THREE_SIDE && sp.overflow != TPCF_OVERFLOW_CLEAN)) return prod;
    const double na = (double)(e[0] - b[0]);
    double c = na * neighbour_density(ctx, job.catalog[0], b[0], e[0], job.catalog[1], b[1], e[1], reach);
    if (nc == 3) c *= neighbour_density(ctx, job.catalog[0], b[0], e[0], job.catalog[2], b[2], e[2], reach);
    return c;
}

void worker_loop(tpcf_ctx* ctx, int lane) {
    Lane& L = *ctx->lanes[lane];
    cudaSetDevice(ctx->device);
    // the first serving lane takes any job; the others only light ones, so
    // that light jobs keep flowing while heavy ones run
    const bool light_only = lane >= 2;
    auto heavy = [&](const Pending& p) { return p.cost > ctx->heavy_cost; };
    for (;;) {
        std::vector<std::shared_ptr<Pending>> batch;
        int64_t used = 0;
        {
            std::unique_lock<std::mutex> lk(ctx->qmu);
            for (;;) {
                ctx->qcv.wait(lk, [&] { return ctx->stop || !ctx->queue.empty(); });
                if (ctx->stop && ctx->queue.empty()) return;
                // drop cancelled jobs
                for (auto it = ctx->queue.begin(); it != ctx->queue.end();) {
                    if ((*it)->cancelled) {
                        (*it)->status = TPCF_ERR_CANCELLED;
                        (*it)->t_done = now_ms();
                        it = ctx->queue.erase(it);
                    } else {
                        ++it;
                    }
                }
                if (ctx->queue.empty()) continue;
                // the oldest job this lane takes
                std::shared_ptr<Pending> first;
                for (auto& p : ctx->queue)
                    if (!light_only || !heavy(*p)) {
                        first = p;
                        break;
                    }
                if (!first) {
                    ctx->qcv.wait(lk);
                    continue;
                }
                int64_t room = ctx->admit_bytes - ctx->inflight_bytes;
                int64_t fb = job_bytes(ctx, first->spec, first->job);
                // the oldest job waits for memory unless nothing else is in flight
                if (fb > room && ctx->inflight_bytes > 0) {
                    ctx->qcv.wait(lk);
                    continue;
                }
                // a heavy job runs alone; light jobs of the same binning share a
                // launch, up to a summed work estimate, so that a light batch
                // stays short and the jobs behind it start soon
                const bool first_heavy = heavy(*first);
                double batch_cost = 0;
                for (auto it = ctx->queue.begin(); it != ctx->queue.end();) {
                    auto& p = *it;
                    if (!same_binning(p->spec, first->spec) || p->spec.prune != first->spec.prune ||
                        (p != first && (first_heavy || heavy(*p)))) {
                        ++it;
                        continue;
                    }
                    const double c = p->cost;
                    if (!batch.empty() && batch_cost + c > ctx->light_batch_cost) break;
                    int64_t jb = job_bytes(ctx, p->spec, p->job);
                    if (!batch.empty() && used + jb > room) break;
                    used += jb;
                    batch_cost += c;
                    batch.push_back(p);
                    it = ctx->queue.erase(it);
                    if (batch.size() >= 4096) break;
                }
                // a heavy batch leaves SMs to the light lanes (its CTAs are persistent)
                L.sm_cap = first_heavy && ctx->reserve_sms > 0 ? ctx->num_sms - ctx->reserve_sms : 0;
                L.slice_batches = first_heavy && ctx->slice_heavy;
                ctx->inflight_bytes += used;
                break;
            }
        }
        ctx->qcv.notify_all();
        std::vector<GroupJob> group;
        int64_t len = 0;
        tpcf_hist_len(&batch[0]->spec, &len);
        double t_start = now_ms();
        for (auto& p : batch) {
            p->result.assign((size_t)len, 0);
            p->t_start = t_start;
            group.push_back({&p->spec, &p->job, p->result.data(), false});
        }
        tpcf_status st = guarded(ctx, [&] { run_group(ctx, L, group); });
        double t_done = now_ms();
        if (!ctx->trace_path.empty()) {
            double oldest = t_start;
            for (auto& p : batch) oldest = std::min(oldest, p->t_submit);
            char line[256];
            snprintf(line, sizeof(line), "%d %zu %llu %.3f %.3f %.3f %.3f\n", lane, batch.size(),
                     (unsigned long long)batch[0]->ticket, oldest, t_start, t_start + L.stats.plan_ms, t_done);
            std::lock_guard<std::mutex> lk(ctx->qmu);
            ctx->trace.push_back(line);
        }
        {
            std::lock_guard<std::mutex> lk(ctx->qmu);
            ctx->inflight_bytes -= used;
            for (auto& p : batch) {
                p->status = st;
                p->t_done = t_done;
            }
        }
        ctx->qcv.notify_all();
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

int32_t tpcf_abi_version(void) { return TPCF_ABI_VERSION; }

const char* tpcf_status_string(tpcf_status s) {
    switch (s) {
        case TPCF_OK: return "ok";
        case TPCF_ERR_INVALID: return "invalid argument";
        case TPCF_ERR_CUDA: return "CUDA error";
        case TPCF_ERR_NO_DEVICE: return "no CUDA device";
        case TPCF_ERR_OOM: return "out of memory";
        case TPCF_ERR_TIMEOUT: return "timeout";
        case TPCF_ERR_NOT_FOUND: return "not found";
        case TPCF_ERR_CANCELLED: return "cancelled";
        case TPCF_ERR_INTERNAL: return "internal error";
        case TPCF_ERR_IO: return "I/O error";
        default: return "unknown status";
    }
}

const char* tpcf_last_error(tpcf_ctx* ctx) { return ctx ? ctx->last_error.c_str() : g_tls_error.c_str(); }

tpcf_status tpcf_create(tpcf_ctx** out, int32_t device) {
    if (!out) return fail(nullptr, TPCF_ERR_INVALID, "null output pointer");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return fail(nullptr, TPCF_ERR_NO_DEVICE, "no CUDA device visible");
    }
    if (device < 0 || device >= count) return fail(nullptr, TPCF_ERR_INVALID, "device index out of range");
    tpcf_ctx* ctx = new tpcf_ctx();
    tpcf_status s = guarded(ctx, [&] {
        ctx->device = device;
        CK(cudaSetDevice(device));
        CK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
        CK(prepare_kernels(device));
        const char* tp = getenv("TPCF_TILE_POINTS");
        if (tp) ctx->tile_points = std::max(8, std::min(TILE, atoi(tp)));
        const char* adm = getenv("TPCF_ADMIT_BYTES");
        if (adm) ctx->admit_bytes = atoll(adm);
        const char* hc = getenv("TPCF_HEAVY_COST");
        if (hc) ctx->heavy_cost = atof(hc);
        if (const char* tr = getenv("TPCF_SERVING_TRACE")) ctx->trace_path = tr;
        if (const char* gt = getenv("TPCF_GROUP_TASKS")) ctx->group_tasks = std::min(MAX_GROUP_TASKS, std::max(1, atoi(gt)));
        const char* shv = getenv("TPCF_SLICE_HEAVY");
        if (shv) ctx->slice_heavy = shv[0] != '0';
        const char* stk = getenv("TPCF_SLICE_TASKS");
        if (stk) ctx->slice_tasks = std::max(0, atoi(stk));
        const char* lbc = getenv("TPCF_LIGHT_BATCH_COST");
        if (lbc) ctx->light_batch_cost = atof(lbc);
        // SMs a heavy serving batch leaves to the light lanes: none by default
        // (a quarter measured a higher p99 on the serving workload: the
        // heavy jobs themselves, slower, are the tail)
        const char* rs = getenv("TPCF_SERVING_RESERVE_SMS");
        if (rs) ctx->reserve_sms = std::max(0, std::min(ctx->num_sms - 1, atoi(rs)));
        const char* nw = getenv("TPCF_SERVING_LANES");
        int workers = nw ? std::max(1, std::min(8, atoi(nw))) : 3;
        for (int i = 0; i <= workers; i++) {
            auto L = std::make_unique<Lane>();
            // the light serving lanes (2 and up) get the highest stream
            // priority: their kernels start at the next slice boundary of a
            // heavy batch
            int prio_least = 0, prio_greatest = 0;
            CK(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
            CK(cudaStreamCreateWithPriority(&L->stream, cudaStreamNonBlocking, i >= 2 ? prio_greatest : prio_least));
            CK(cudaEventCreate(&L->ev0));
            CK(cudaEventCreate(&L->ev1));
            CK(cudaEventCreate(&L->ev_mid));
            if (i >= 1) {
                // serving lanes: buffers sized up front.  A device or
                // page-locked allocation issued while another lane's kernel
                // runs keeps this lane's next kernel from running beside it
                // (implicit synchronisation), so light batches must not allocate.
                L->h_hist.reserve((size_t)1 << 20);
                L->h_counters.reserve(8);
                L->d_hist.reserve((size_t)1 << 22);
                L->d_counters.reserve(8);
                L->d_jobs.reserve((size_t)1 << 16);
                L->d_tasks.reserve((size_t)1 << 21);
                L->d_queue.reserve((size_t)1 << 22);
            }
            ctx->lanes.push_back(std::move(L));
        }
    });
    if (s != TPCF_OK) {
        g_tls_error = ctx->last_error;
        for (auto& L : ctx->lanes) L->release();
        delete ctx;
        return s;
    }
    for (size_t i = 1; i < ctx->lanes.size(); i++) ctx->workers.emplace_back(worker_loop, ctx, (int)i);
    *out = ctx;
    return TPCF_OK;
}

tpcf_status tpcf_destroy(tpcf_ctx* ctx) {
    if (!ctx) return TPCF_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(ctx->qmu);
        ctx->stop = true;
    }
    ctx->qcv.notify_all();
    for (auto& t : ctx->workers)
        if (t.joinable()) t.join();
    if (!ctx->trace_path.empty()) {
        if (FILE* f = fopen(ctx->trace_path.c_str(), "w")) {
            for (auto& l : ctx->trace) fputs(l.c_str(), f);
            fclose(f);
        }
    }
    {
        std::lock_guard<std::recursive_mutex> lk(ctx->mu);
        std::lock_guard<std::recursive_mutex> vlk(ctx->view_mu);
        cudaSetDevice(ctx->device);
        for (auto& kv : ctx->pending_views) kv.second.fut.wait();
        ctx->pending_views.clear();
        ctx->views.clear();
        for (auto& L : ctx->lanes) L->release();
        ctx->acos_keys.release();
        ctx->acos_vals.release();
        ctx->acos_bucket.release();
    }
    delete ctx;
    return TPCF_OK;
}

tpcf_status tpcf_catalog_create(tpcf_ctx* ctx, const float* x, const float* y, const float* z, int64_t n,
                                uint64_t* handle) {
    if (!ctx || !handle || n < 0 || (n > 0 && (!x || !y || !z))) return fail(ctx, TPCF_ERR_INVALID, "bad catalog arguments");
    if (n > (int64_t)1 << 30) return fail(ctx, TPCF_ERR_INVALID, "catalog too large");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    return guarded(ctx, [&] {
        CK(cudaSetDevice(ctx->device));
        auto c = std::make_shared<Catalog>();
        c->n = n;
        c->x.assign(x, x + n);
        c->y.assign(y, y + n);
        c->z.assign(z, z + n);
        std::lock_guard<std::recursive_mutex> vlk(ctx->view_mu);
        uint64_t h = ctx->next_handle++;
        ctx->catalogs[h] = c;
        // the resident form of a catalog is its spatial view (sorted points,
        // tiles, device copy), built on a thread of its own so that the
        // caller's next catalog (or anything else) proceeds meanwhile; the
        // first use waits for it.  Sub-range views are made on demand from the
        // host copy.
        const int dev = ctx->device, tile = ctx->tile_points;
        const uint64_t id = ++ctx->next_view_id;
        ctx->pending_views[std::make_tuple(h, (int64_t)0, n, tile, false)].id = id;
        ctx->pending_views[std::make_tuple(h, (int64_t)0, n, tile, false)].n = n;
        ctx->pending_views[std::make_tuple(h, (int64_t)0, n, tile, false)].fut =
            std::async(std::launch::async, [c, n, tile, dev, id] {
                CK(cudaSetDevice(dev));
                cudaStream_t st = nullptr;
                CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
                try {
                    auto v = build_view(*c, 0, n, tile, false, id, st);
                    cudaStreamDestroy(st);
                    return v;
                } catch (...) {
                    cudaStreamDestroy(st);
                    throw;
                }
            }).share();
        *handle = h;
    });
}

tpcf_status tpcf_catalog_release(tpcf_ctx* ctx, uint64_t handle) {
    if (!ctx) return TPCF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> vlk(ctx->view_mu);
    if (!ctx->catalogs.count(handle)) return fail(ctx, TPCF_ERR_NOT_FOUND, "unknown catalog handle");
    ctx->catalogs.erase(handle);
    for (auto it = ctx->views.begin(); it != ctx->views.end();) {
        if (std::get<0>(it->first) == handle) it = ctx->views.erase(it);
        else ++it;
    }
    // a view still being built: wait for it (its device buffers are freed
    // with the last reference), whatever its outcome
    for (auto it = ctx->pending_views.begin(); it != ctx->pending_views.end();) {
        if (std::get<0>(it->first) == handle) {
            it->second.fut.wait();
            it = ctx->pending_views.erase(it);
        } else {
            ++it;
        }
    }
    return TPCF_OK;
}

tpcf_status tpcf_resident_bytes(tpcf_ctx* ctx, int64_t* bytes) {
    if (!ctx || !bytes) return TPCF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(ctx->view_mu);
    int64_t b = 0;
    for (auto& kv : ctx->views) b += (int64_t)kv.second->bytes();
    for (auto& kv : ctx->pending_views) {  // (a failed build holds nothing)
        try {
            b += (int64_t)kv.second.fut.get()->bytes();
        } catch (...) {
        }
    }
    *bytes = b;
    return TPCF_OK;
}

tpcf_status tpcf_hist_len(const tpcf_spec* sp, int64_t* len) {
    if (!sp || !len) return TPCF_ERR_INVALID;
    if (sp->kind == TPCF_THREE_SIDE) *len = (int64_t)sp->axis[0].nbins * sp->axis[0].nbins * sp->axis[0].nbins;
    else if (sp->kind == TPCF_TRIANGLE || sp->kind == TPCF_TRIANGLE_JBJ)
        *len = (int64_t)sp->axis[0].nbins * sp->axis[1].nbins * sp->axis[2].nbins;
    else if (sp->kind == TPCF_PAIR) *len = sp->axis[0].nbins;
    else return TPCF_ERR_INVALID;
    return TPCF_OK;
}

tpcf_status tpcf_loop_units(tpcf_ctx* ctx, const tpcf_spec* sp, const tpcf_job* job, uint64_t* units) {
    if (!ctx || !sp || !job || !units) return TPCF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(ctx->view_mu);
    int64_t n[3] = {0, 0, 0};
    int nc = sp->kind == TPCF_PAIR ? 2 : 3;
    for (int r = 0; r < nc; r++) {
        auto it = ctx->catalogs.find(job->catalog[r]);
        if (it == ctx->catalogs.end()) return fail(ctx, TPCF_ERR_NOT_FOUND, "unknown catalog handle");
        int64_t e = job->end[r] < 0 ? it->second->n : job->end[r];
        n[r] = e - job->begin[r];
    }
    *units = loop_units(sp->kind, sp->loop, n);
    return TPCF_OK;
}

namespace {

// Jobs grouped by binning (and pruning); each group is one persistent launch.
// out_index == nullptr: job i writes hists[i]; else job i adds into
// hists[out_index[i]] (zeroed first).
tpcf_status count_jobs(tpcf_ctx* ctx, const tpcf_spec* specs, const tpcf_job* jobs, int32_t n,
                       const int32_t* out_index, int32_t n_out, uint64_t* const* hists) {
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    return guarded(ctx, [&] {
        CK(cudaSetDevice(ctx->device));
        std::vector<int64_t> out_len(out_index ? n_out : 0, -1);
        for (int i = 0; i < n; i++) {
            validate(&specs[i], &jobs[i]);
            if (out_index) {
                const int32_t o = out_index[i];
                if (o < 0 || o >= n_out) throw InvalidArg{"out_index out of range"};
                if (!hists[o]) throw InvalidArg{"null histogram pointer"};
                int64_t len = 0;
                tpcf_hist_len(&specs[i], &len);
                if (out_len[o] >= 0 && out_len[o] != len) throw InvalidArg{"jobs of one output differ in histogram length"};
                out_len[o] = len;
            } else if (!hists[i]) {
                throw InvalidArg{"null histogram pointer"};
            }
        }
        if (out_index)
            for (int32_t o = 0; o < n_out; o++)
                if (out_len[o] > 0) memset(hists[o], 0, (size_t)out_len[o] * sizeof(uint64_t));
        std::vector<char> done(n, 0);
        tpcf_stats acc{};
        for (int i = 0; i < n; i++) {
            if (done[i]) continue;
            std::vector<GroupJob> g;
            for (int k = i; k < n; k++)
                if (!done[k] && same_binning(specs[k], specs[i]) && specs[k].prune == specs[i].prune) {
                    if (out_index) g.push_back({&specs[k], &jobs[k], hists[out_index[k]], true});
                    else g.push_back({&specs[k], &jobs[k], hists[k], false});
                    done[k] = 1;
                }
            Lane& L = *ctx->lanes[0];
            run_group(ctx, L, g);
            acc.kernel_ms += L.stats.kernel_ms;
            acc.main_kernel_ms += L.stats.main_kernel_ms;
            acc.binned_units += L.stats.binned_units;
            acc.total_ms += L.stats.total_ms;
            acc.loop_units += L.stats.loop_units;
            acc.evaluated_units += L.stats.evaluated_units;
            acc.recheck_units += L.stats.recheck_units;
            acc.recheck_regrows += L.stats.recheck_regrows;
            acc.tasks += L.stats.tasks;
            acc.kernel_launches += L.stats.kernel_launches;
            acc.graph_replays += L.stats.graph_replays;
            acc.plan_ms += L.stats.plan_ms;
            acc.tuned_shapes += L.stats.tuned_shapes;
            acc.hist_copies = L.stats.hist_copies;
            acc.ctas_per_sm = L.stats.ctas_per_sm;
        }
        ctx->lanes[0]->stats = acc;
    });
}

}  // namespace

tpcf_status tpcf_count_batch(tpcf_ctx* ctx, const tpcf_spec* specs, const tpcf_job* jobs, int32_t n,
                             uint64_t* const* hists) {
    if (!ctx || !specs || !jobs || !hists || n < 0) return fail(ctx, TPCF_ERR_INVALID, "bad batch arguments");
    return count_jobs(ctx, specs, jobs, n, nullptr, 0, hists);
}

tpcf_status tpcf_count_batch_into(tpcf_ctx* ctx, const tpcf_spec* specs, const tpcf_job* jobs, int32_t n,
                                  const int32_t* out_index, int32_t n_out, uint64_t* const* hists) {
    if (!ctx || !specs || !jobs || !out_index || !hists || n < 0 || n_out < 0)
        return fail(ctx, TPCF_ERR_INVALID, "bad batch arguments");
    return count_jobs(ctx, specs, jobs, n, out_index, n_out, hists);
}

tpcf_status tpcf_convert_radecz(tpcf_ctx* ctx, const double* ra, const double* dec, const double* redshift,
                                int64_t n, const double* poly, float* x, float* y, float* z) {
    if (!ctx || n < 0 || (n > 0 && (!ra || !dec || !redshift || !x || !y || !z)))
        return fail(ctx, TPCF_ERR_INVALID, "bad conversion arguments");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    return guarded(ctx, [&] {
        if (n == 0) return;
        CK(cudaSetDevice(ctx->device));
        const double mice[3] = {-1.07199554e+00, 3.01313296e+03, -6.38827998e+02};  // the script's fit
        const double* pc = poly ? poly : mice;
        Lane& L = *ctx->lanes[0];
        DevBuf<double> d_in;
        DevBuf<float> d_out;
        d_in.reserve(3 * (size_t)n);
        d_out.reserve(3 * (size_t)n);
        const size_t b = (size_t)n * sizeof(double);
        CK(cudaMemcpyAsync(d_in.p, ra, b, cudaMemcpyHostToDevice, L.stream));
        CK(cudaMemcpyAsync(d_in.p + n, dec, b, cudaMemcpyHostToDevice, L.stream));
        CK(cudaMemcpyAsync(d_in.p + 2 * n, redshift, b, cudaMemcpyHostToDevice, L.stream));
        CK(launch_radecz_to_xyz(d_in.p, d_in.p + n, d_in.p + 2 * n, n, pc, d_out.p, d_out.p + n, d_out.p + 2 * n,
                                L.stream));
        const size_t fb = (size_t)n * sizeof(float);
        CK(cudaMemcpyAsync(x, d_out.p, fb, cudaMemcpyDeviceToHost, L.stream));
        CK(cudaMemcpyAsync(y, d_out.p + n, fb, cudaMemcpyDeviceToHost, L.stream));
        CK(cudaMemcpyAsync(z, d_out.p + 2 * n, fb, cudaMemcpyDeviceToHost, L.stream));
        CK(cudaStreamSynchronize(L.stream));
        L.h2d += 3 * b;
        L.d2h += 3 * fb;
    });
}

tpcf_status tpcf_count(tpcf_ctx* ctx, const tpcf_spec* spec, const tpcf_job* job, uint64_t* hist, int64_t hist_len) {
    if (!ctx || !spec || !job || !hist) return fail(ctx, TPCF_ERR_INVALID, "null argument");
    int64_t len = 0;
    if (tpcf_hist_len(spec, &len) != TPCF_OK || len != hist_len) return fail(ctx, TPCF_ERR_INVALID, "hist_len mismatch");
    uint64_t* hp[1] = {hist};
    return tpcf_count_batch(ctx, spec, job, 1, hp);
}

tpcf_status tpcf_submit(tpcf_ctx* ctx, const tpcf_spec* spec, const tpcf_job* job, uint64_t* ticket) {
    if (!ctx || !spec || !job || !ticket) return fail(ctx, TPCF_ERR_INVALID, "null argument");
    double cost = 0;
    tpcf_status s = guarded(ctx, [&] {
        std::lock_guard<std::recursive_mutex> lk(ctx->mu);
        validate(spec, job);
        int nc = spec->kind == TPCF_PAIR ? 2 : 3;
        for (int r = 0; r < nc; r++) {
            auto it = ctx->catalogs.find(job->catalog[r]);
            if (it == ctx->catalogs.end()) throw InvalidArg{"unknown catalog handle"};
            const int64_t e = job->end[r] < 0 ? it->second->n : job->end[r];
            if (job->begin[r] < 0 || job->begin[r] > e || e > it->second->n) throw InvalidArg{"catalog range out of bounds"};
        }
        cost = job_cost(ctx, *spec, *job);
    });
    if (s != TPCF_OK) return s;
    auto p = std::make_shared<Pending>();
    p->cost = cost;
    p->spec = *spec;
    p->job = *job;
    p->t_submit = now_ms();
    {
        std::lock_guard<std::mutex> lk(ctx->qmu);
        p->ticket = ctx->next_ticket++;
        ctx->queue.push_back(p);
        ctx->tickets[p->ticket] = p;
        *ticket = p->ticket;
    }
    ctx->qcv.notify_all();
    return TPCF_OK;
}

tpcf_status tpcf_wait_timed(tpcf_ctx* ctx, uint64_t ticket, uint64_t* hist, int64_t hist_len, int64_t timeout_ms,
                            double* latency_ms, double* run_ms) {
    if (!ctx) return TPCF_ERR_INVALID;
    std::unique_lock<std::mutex> lk(ctx->qmu);
    auto it = ctx->tickets.find(ticket);
    if (it == ctx->tickets.end()) return fail(ctx, TPCF_ERR_NOT_FOUND, "unknown ticket");
    auto p = it->second;
    auto ready = [&] { return p->status != 1; };
    if (timeout_ms < 0) ctx->qcv.wait(lk, ready);
    else if (!ctx->qcv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return TPCF_ERR_TIMEOUT;
    ctx->tickets.erase(ticket);
    if (latency_ms) *latency_ms = p->t_done - p->t_submit;
    if (run_ms) *run_ms = p->t_start > 0 ? p->t_done - p->t_start : 0.0;
    if (p->status != TPCF_OK) return p->status;
    if (hist) {
        if ((int64_t)p->result.size() != hist_len) return fail(ctx, TPCF_ERR_INVALID, "hist_len mismatch");
        memcpy(hist, p->result.data(), p->result.size() * sizeof(uint64_t));
    }
    return TPCF_OK;
}

tpcf_status tpcf_wait(tpcf_ctx* ctx, uint64_t ticket, uint64_t* hist, int64_t hist_len, int64_t timeout_ms) {
    return tpcf_wait_timed(ctx, ticket, hist, hist_len, timeout_ms, nullptr, nullptr);
}

tpcf_status tpcf_cancel(tpcf_ctx* ctx, uint64_t ticket) {
    if (!ctx) return TPCF_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->qmu);
    auto it = ctx->tickets.find(ticket);
    if (it == ctx->tickets.end()) return TPCF_ERR_NOT_FOUND;
    if (it->second->status != 1) return TPCF_ERR_INVALID;  // already ran
    it->second->cancelled = true;
    for (auto q = ctx->queue.begin(); q != ctx->queue.end(); ++q)
        if ((*q)->ticket == ticket) {
            (*q)->status = TPCF_ERR_CANCELLED;
            ctx->queue.erase(q);
            break;
        }
    ctx->qcv.notify_all();
    return TPCF_OK;
}

tpcf_status tpcf_last_stats(tpcf_ctx* ctx, tpcf_stats* stats) {
    if (!ctx || !stats) return TPCF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    Lane& L = *ctx->lanes[0];
    *stats = L.stats;
    // byte counters cover everything copied since the previous stats read
    stats->h2d_bytes = L.h2d;
    stats->d2h_bytes = L.d2h;
    L.h2d = L.d2h = 0;
    return TPCF_OK;
}

// test hook (not in the public header): checks the device exception table
// against its own entries; returns the mismatch count or -1.
int64_t tpcf_debug_acos_selfcheck(tpcf_ctx* ctx, int64_t* table_size) {
    if (!ctx) return -1;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    int64_t r = -1;
    guarded(ctx, [&] {
        CK(cudaSetDevice(ctx->device));
        ensure_acos(ctx);
        DevBuf<unsigned int> mm;
        mm.reserve(1);
        CK(cudaMemset(mm.p, 0, 4));
        cudaStream_t st = ctx->lanes[0]->stream;
        CK(launch_acos_check(acos_table(ctx), 0, ctx->acos_n, mm.p, st));
        unsigned int h = 0;
        CK(cudaMemcpyAsync(&h, mm.p, 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        r = h;
        if (table_size) *table_size = ctx->acos_n;
    });
    return r;
}

}  // extern "C"

// test hook (not in the public header): size and FNV-1a hash of this host's
// exact-acosf exception table (built or loaded from the cache; no GPU needed)
extern "C" int32_t tpcf_debug_acos_table_hash(uint64_t* n, uint64_t* hash) {
    AcosHost h = load_or_build_acos_table();
    uint64_t x = 1469598103934665603ull;
    for (size_t i = 0; i < h.keys.size(); i++) {
        x = (x ^ h.keys[i]) * 1099511628211ull;
        x = (x ^ h.vals[i]) * 1099511628211ull;
    }
    if (n) *n = h.keys.size();
    if (hash) *hash = x;
    return TPCF_OK;
}

// test hook (not in the public header): this host's exact-acosf exceptions as
// keys (float bits of c, sorted) and the direction (+1/-1 ulp) of glibc's value
// relative to (float)tpcf_acos_d(c).  Call with keys == NULL for the count.
extern "C" int32_t tpcf_debug_acos_exceptions(uint32_t* keys, int8_t* dir, uint64_t cap, uint64_t* n) {
    AcosHost h = load_or_build_acos_table();
    if (n) *n = h.keys.size();
    if (!keys || !dir) return TPCF_OK;
    for (size_t i = 0; i < h.keys.size() && i < cap; i++) {
        keys[i] = h.keys[i];
        int64_t d = (int64_t)h.vals[i] - (int64_t)fbits((float)tpcf_acos_d((double)ffrom(h.keys[i])));
        dir[i] = (int8_t)(d > 0 ? 1 : (d < 0 ? -1 : 0));
    }
    return TPCF_OK;
}

// test hook (not in the public header): replaces the context's exception table
// by the given one (e.g. another machine's glibc, to compare with files that
// machine produced).  dir: +1/-1 ulp relative to (float)tpcf_acos_d(c).
extern "C" int32_t tpcf_debug_set_acos_exceptions(tpcf_ctx* ctx, const uint32_t* keys, const int8_t* dir, uint64_t n) {
    if (!ctx || (n && (!keys || !dir))) return TPCF_ERR_INVALID;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    return guarded(ctx, [&] {
        CK(cudaSetDevice(ctx->device));
        AcosHost h;
        h.keys.assign(keys, keys + n);
        h.vals.resize(n);
        for (uint64_t i = 0; i < n; i++) {
            if (i && keys[i] <= keys[i - 1]) throw InvalidArg{"exception keys must be strictly increasing"};
            h.vals[i] = fbits((float)tpcf_acos_d((double)ffrom(keys[i]))) + (uint32_t)(int32_t)dir[i];
        }
        h.bucket.assign(65537, 0);
        size_t j = 0;
        for (uint32_t b = 0; b <= 65536; b++) {
            while (j < h.keys.size() && (h.keys[j] >> 16) < b) j++;
            h.bucket[b] = (uint32_t)j;
        }
        ctx->acos_n = (uint32_t)n;
        ctx->acos_keys.reserve(std::max<size_t>(n, 1));
        ctx->acos_vals.reserve(std::max<size_t>(n, 1));
        ctx->acos_bucket.reserve(65537);
        if (n) {
            CK(cudaMemcpy(ctx->acos_keys.p, h.keys.data(), n * 4, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(ctx->acos_vals.p, h.vals.data(), n * 4, cudaMemcpyHostToDevice));
        }
        CK(cudaMemcpy(ctx->acos_bucket.p, h.bucket.data(), 65537 * 4, cudaMemcpyHostToDevice));
        ctx->acos_ready = true;
    });
}
