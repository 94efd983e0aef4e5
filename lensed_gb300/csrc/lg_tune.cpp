// Launch-shape autotuner: candidate shapes, parallel NVRTC compilation and
// the cache of tuned shapes.
//
// The reference sizes its work groups from device queries
// (src/lensed.c:866-1047: render work-group size from
// CL_KERNEL_WORK_GROUP_SIZE, convolution tiles halved until they fit local
// memory).  Here the shape of every kernel is a compile-time constant of the
// composed program, so the tuner compiles a few candidates side by side and
// the owner of the program (a context or a batch of systems) times them on
// candidate parameters drawn from the priors:
//
//   render       threads per block (rt), pixels per thread group (rppt) and
//                the quadrature split (qs: threads of a group sharing its
//                pixels, each taking every qs-th quadrature point; fast mode
//                only, since it reorders the quadrature sum);
//   convolution  output tile (ctx x cty) and outputs per thread (cr).
//
// The two stages are separate kernels, so render candidates are timed with
// the default convolution and convolution candidates with the default
// render; the best of each are then combined.  Results are cached per
// (program, device, batch, flags): in memory for the process, and in the
// text file named by LG_TUNE_CACHE when that variable is set.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "lg_internal.h"

namespace lg {

std::string Shape::str() const
{
    std::ostringstream o;
    o << "render " << rt << "x" << rppt << " qs " << qs << ", conv " << ctx << "x" << cty << "/" << cr
      << (pair_rows ? " paired" : "");
    return o.str();
}

Fp fp_mode(int flags)
{
    if (flags & LG_FLAG_STRICT_FP) return Fp::STRICT;
    if (flags & LG_FLAG_FAST_MATH) return Fp::FAST;
    return Fp::EXACT;
}

bool fp_ieee(int flags) { return fp_mode(flags) != Fp::FAST || (flags & LG_FLAG_IEEE_DIV); }

std::vector<Shape> render_candidates(const Shape& base, Fp mode)
{
    // (threads, pixels per group, quadrature split); the strict mode keeps
    // one quadrature point per step (split 1); the exact mode splits with an
    // ordered sum
    static const int fast[][3] = {{128, 2, 1}, {256, 2, 1}, {64, 2, 1}, {128, 4, 1}, {128, 2, 2}, {256, 2, 2},
                                  {128, 2, 4}, {128, 2, 8}};
    static const int exact[][3] = {{128, 2, 1}, {256, 2, 1}, {64, 2, 1}, {128, 4, 1}, {128, 2, 2}, {128, 2, 4},
                                   {128, 2, 8}};
    static const int scalar[][3] = {{128, 2, 1}, {256, 2, 1}, {64, 2, 1}, {128, 1, 1}, {128, 4, 1}};
    const int(*tab)[3] = mode == Fp::FAST ? fast : (mode == Fp::EXACT ? exact : scalar);
    const int n = mode == Fp::FAST ? (int)(sizeof fast / sizeof fast[0])
                                   : (mode == Fp::EXACT ? (int)(sizeof exact / sizeof exact[0])
                                                        : (int)(sizeof scalar / sizeof scalar[0]));
    std::vector<Shape> out;
    for (int i = 0; i < n; ++i) {
        const int* c = tab[i];
        Shape s = base;
        s.rt = c[0];
        s.rppt = c[1];
        s.qs = c[2];
        out.push_back(s);
    }
    return out;
}

std::vector<Shape> conv_candidates(const Shape& base, bool multi)
{
    // (tile width, tile height, outputs per thread); paired tiles hold two
    // row halves, so their height is even and their outputs a multiple of 8.
    // The multi-system kernels count thread rows (a paired unit covers two
    // of them per thread) and need outputs in multiples of 8.
    // (the smallest tiles keep small batches spread over the SMs)
    static const int paired[][3] = {{32, 64, 8}, {32, 32, 8}, {64, 64, 8}, {64, 32, 8}, {32, 64, 16}, {32, 16, 8}};
    static const int single[][3] = {{32, 32, 8}, {32, 16, 8}, {64, 32, 8}, {32, 32, 16}, {32, 64, 8}, {32, 8, 8}};
    static const int units[][3] = {{32, 32, 8}, {32, 16, 8}, {64, 32, 8}, {64, 16, 8}, {32, 32, 16}, {32, 8, 8}};
    std::vector<Shape> out;
    const int n = 6;
    for (int i = 0; i < n; ++i) {
        const int* c = multi ? units[i] : base.pair_rows ? paired[i] : single[i];
        Shape s = base;
        s.ctx = c[0];
        s.cty = c[1];
        s.cr = c[2];
        out.push_back(s);
    }
    if (!multi && base.pair_rows) {
        // single-row tiles of two or four outputs per thread: the most
        // threads for a batch of one or a few candidates (same per-pixel
        // arithmetic)
        static const int small[][3] = {{32, 16, 4}, {16, 16, 4}, {32, 8, 2}, {16, 16, 2}};
        for (const auto& c : small) {
            Shape s = base;
            s.ctx = c[0];
            s.cty = c[1];
            s.cr = c[2];
            s.pair_rows = false;
            out.push_back(s);
        }
    }
    return out;
}

std::string check_shape(const Shape& s, Fp mode, bool psf, int psfw)
{
    const bool strict = mode == Fp::STRICT;
    if (s.rt < 32 || s.rt > 1024 || s.rt % 32) return "render threads must be a multiple of 32 in [32, 1024]";
    if (s.rppt < 1 || s.rppt > 8) return "pixels per thread group must be in [1, 8]";
    if (s.qs != 1 && s.qs != 2 && s.qs != 4 && s.qs != 8) return "quadrature split must be 1, 2, 4 or 8";
    if (strict && s.qs != 1) return "strict mode keeps the quadrature sum in order (split 1)";
    if (mode == Fp::EXACT && s.qs != 1 && s.rppt % 2)
        return "the exact mode splits the quadrature of pixel pairs only (even pixels per group)";
    if (!psf) return "";
    if (s.cr != 2 && s.cr != 4 && s.cr != 8 && s.cr != 16) return "convolution outputs per thread must be 2, 4, 8 or 16";
    if (s.ctx < s.cr || s.ctx % s.cr || s.ctx > 256) return "convolution tile width must be a multiple of cr";
    if (s.pair_rows && (strict || psfw > 49)) return "paired rows need the fast or exact mode and a PSF up to 49 wide";
    if (s.pair_rows && (s.cr % 8 || s.cty % 2)) return "paired rows need cr % 8 == 0 and an even tile height";
    if (s.cty < 1 || s.cty > 256) return "convolution tile height must be in [1, 256]";
    const int threads = (s.ctx / s.cr) * s.conv_block_y();
    if (threads < 32 || threads > 1024 || threads % 32) return "convolution block must be whole warps, <= 1024";
    return "";
}

void compile_parallel(const std::vector<std::string>& srcs, bool fmad, bool ieee,
                      std::vector<std::vector<char>>& cubins, std::vector<int>& rcs, std::vector<std::string>& logs)
{
    const size_t n = srcs.size();
    cubins.assign(n, {});
    rcs.assign(n, LG_ERR_COMPILE);
    logs.assign(n, "");
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t i; (i = next++) < n;) rcs[i] = compile_program(srcs[i], fmad, cubins[i], logs[i], ieee);
    };
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::min(n, std::min<size_t>(hw, 16));
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nt; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
}

namespace {

std::mutex g_cache_mu;
std::map<std::string, Shape> g_cache;
bool g_cache_loaded = false;

const char* cache_path() { return std::getenv("LG_TUNE_CACHE"); }

void load_cache_file()
{
    if (g_cache_loaded) return;
    g_cache_loaded = true;
    const char* p = cache_path();
    if (!p) return;
    std::ifstream f(p);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string key;
        Shape s;
        int pr = 0;
        if (is >> key >> s.rt >> s.rppt >> s.qs >> s.ctx >> s.cty >> s.cr >> pr) {
            s.pair_rows = pr != 0;
            g_cache[key] = s;
        }
    }
}

}  // namespace

std::string device_signature(int device)
{
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return "unknown";
    return std::string(p.name) + "/" + std::to_string(p.multiProcessorCount) + "sm/cc" +
           std::to_string(p.major * 10 + p.minor);
}

std::string tune_key(const std::string& program, int device, int batch, int flags)
{
    // FNV-1a over the program text (composed with the default shape) and
    // the device, batch and flags the timings belong to
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const std::string& s) {
        for (unsigned char ch : s) {
            h ^= ch;
            h *= 1099511628211ull;
        }
    };
    mix(program);
    mix(device_signature(device));
    mix(std::to_string(batch) + "/" + std::to_string(flags));
    char buf[24];
    std::snprintf(buf, sizeof buf, "%016llx", (unsigned long long)h);
    return buf;
}

bool tune_cache_get(const std::string& key, Shape& s)
{
    std::lock_guard<std::mutex> lk(g_cache_mu);
    load_cache_file();
    auto it = g_cache.find(key);
    if (it == g_cache.end()) return false;
    s = it->second;
    return true;
}

void tune_cache_put(const std::string& key, const Shape& s)
{
    std::lock_guard<std::mutex> lk(g_cache_mu);
    load_cache_file();
    g_cache[key] = s;
    if (const char* p = cache_path()) {
        if (FILE* f = std::fopen(p, "a")) {
            std::fprintf(f, "%s %d %d %d %d %d %d %d\n", key.c_str(), s.rt, s.rppt, s.qs, s.ctx, s.cty, s.cr,
                         s.pair_rows ? 1 : 0);
            std::fclose(f);
        }
    }
}

void tune_cache_clear()
{
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache.clear();
    g_cache_loaded = true;  // the file is not re-read after a clear
}

}  // namespace lg
