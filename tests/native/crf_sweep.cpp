// Host harness for the correctly rounded single-precision functions of the
// exact evaluation modules (lensed_gb300/device/lg_crfloat.cuh, compiled for
// the host with LG_CRF_HOST): compares fn(x) with the function evaluated in
// double and rounded once, over float bit patterns start, start + step, ...
// below stop, and counts the inputs whose double-word result could not be
// rounded with certainty (the lanes that take the double path).
//   crf_sweep <fn: 0 exp, 1 log, 2 atan, 3 atanh> <start> <stop> <step>
// prints: inputs mismatches in_range slow
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static thread_local long g_slow = 0;
#define LG_CRF_SLOW_COUNT() (++g_slow)
#define LG_CRF_HOST 1
#include "../../lensed_gb300/device/lg_crfloat.cuh"

static float crf(int fn, float x)
{
    return fn == 0 ? lg_crf_exp(x) : fn == 1 ? lg_crf_log(x) : fn == 2 ? lg_crf_atan(x) : lg_crf_atanh(x);
}
static float dbl(int fn, float x)
{
    return fn == 0   ? (float)std::exp((double)x)
           : fn == 1 ? (float)std::log((double)x)
           : fn == 2 ? (float)std::atan((double)x)
                     : (float)std::atanh((double)x);
}
// inputs handled by the single-precision path (the rest go to double by design)
static bool in_range(int fn, float x)
{
    return fn == 0 ? (x <= 88.0f && x > LG_CRF_EXP_ZERO)
           : fn == 1 ? (x >= 0x1p-126f && x <= 0x1.fffffep127f)
           : fn == 2 ? std::fabs(x) <= 0x1.fffffep127f
                     : std::fabs(x) < 1.0f;
}

int main(int argc, char** argv)
{
    if (argc != 5) return 2;
    const int fn = std::atoi(argv[1]);
    const long long start = std::atoll(argv[2]), stop = std::atoll(argv[3]), step = std::atoll(argv[4]);
    long long n = 0, bad = 0, nin = 0, slow = 0;
#pragma omp parallel reduction(+ : n, bad, nin, slow)
    {
#pragma omp for schedule(dynamic, 4096)
        for (long long u = start; u < stop; u += step) {
            const unsigned b = (unsigned)u;
            float x;
            std::memcpy(&x, &b, 4);
            const long s0 = g_slow;
            const float got = crf(fn, x), want = dbl(fn, x);
            unsigned gb, wb;
            std::memcpy(&gb, &got, 4);
            std::memcpy(&wb, &want, 4);
            if (gb != wb && !(got != got && want != want)) {
                ++bad;
                if (bad <= 5) std::fprintf(stderr, "fn %d x = %a: %a, double gives %a\n", fn, x, got, want);
            }
            ++n;
            if (in_range(fn, x)) {
                ++nin;
                slow += g_slow - s0;
            }
        }
    }
    std::printf("%lld %lld %lld %lld\n", n, bad, nin, slow);
    return 0;
}
