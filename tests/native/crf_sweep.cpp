// Host harness for the correctly rounded single-precision functions of the
// exact evaluation modules (lensed_gb300/device/lg_crfloat.cuh, compiled for
// the host with LG_CRF_HOST): compares fn(x) with the function evaluated in
// double and rounded once, over float bit patterns start, start + step, ...
// below stop, and counts the inputs whose double-word result could not be
// rounded with certainty (the lanes that take the double path).
//   crf_sweep <fn> <start> <stop> <step>
//   fn: 0 exp, 1 log, 2 atan, 3 atanh, 4 sin, 5 cos, 6 pow(x, Y[u % 16]) with
//   the exponents of the EPL lens and others, 7 atan2(x, p(u)), 8 pow(|x|,
//   p(u)) with p(u) the float of bit pattern u * 0x9E3779B1 (a partner that
//   sweeps the second argument too)
// prints: inputs mismatches in_range slow
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static thread_local long g_slow = 0;
#define LG_CRF_SLOW_COUNT() (++g_slow)
#define LG_CRF_HOST 1
#include "../../lensed_gb300/device/lg_crfloat.cuh"

static const float Y[16] = {-1.2f, -1.0f, -0.8f, -0.5f, 0.5f, -0.25f, 0.2f, 1.0f / 3,
                            2.5f, -2.2f, 0.999f, 1.5f, -0.1f, 3.7f, 0.05f, -7.5f};
static float partner(unsigned u)
{
    const unsigned b = u * 0x9E3779B1u;
    float p;
    std::memcpy(&p, &b, 4);
    return p;
}
static float crf(int fn, float x, unsigned u)
{
    float s, c;
    switch (fn) {
    case 0: return lg_crf_exp(x);
    case 1: return lg_crf_log(x);
    case 2: return lg_crf_atan(x);
    case 3: return lg_crf_atanh(x);
    case 4: lg_crf_sincos(x, &s, &c); return s;
    case 5: lg_crf_sincos(x, &s, &c); return c;
    case 6: return lg_crf_pow(x, Y[u % 16]);
    case 7: return lg_crf_atan2(x, partner(u));
    default: return lg_crf_pow(std::fabs(x), partner(u));
    }
}
static float dbl(int fn, float x, unsigned u)
{
    switch (fn) {
    case 0: return (float)std::exp((double)x);
    case 1: return (float)std::log((double)x);
    case 2: return (float)std::atan((double)x);
    case 3: return (float)std::atanh((double)x);
    case 4: return (float)std::sin((double)x);
    case 5: return (float)std::cos((double)x);
    case 6: return (float)std::pow((double)x, (double)Y[u % 16]);
    case 7: return (float)std::atan2((double)x, (double)partner(u));
    default: return (float)std::pow((double)std::fabs(x), (double)partner(u));
    }
}
// inputs handled by the single-precision path (the rest go to double by design)
static bool in_range(int fn, float x, unsigned u)
{
    switch (fn) {
    case 0: return x <= 88.0f && x > LG_CRF_EXP_ZERO;
    case 1: return x >= 0x1p-126f && x <= 0x1.fffffep127f;
    case 2: return std::fabs(x) <= 0x1.fffffep127f;
    case 3: return std::fabs(x) < 1.0f;
    case 4:
    case 5: return std::fabs(x) <= 128.0f;
    case 6: {
        const double t = Y[u % 16] * std::log((double)x);
        return x >= 0x1p-126f && x <= 0x1.fffffep127f && t >= -86.9 && t <= 87.9;
    }
    case 7: {
        const double a = std::fabs((double)x), b = std::fabs((double)partner(u));
        const double lo = a < b ? a : b, hi = a < b ? b : a;
        return lo >= 0x1p-100 && hi < 0x1p126 && lo >= hi * 0x1p-99;
    }
    default: {
        const double t = (double)partner(u) * std::log(std::fabs((double)x));
        return std::fabs(x) >= 0x1p-126f && std::fabs(x) <= 0x1.fffffep127f && t >= -86.9 && t <= 87.9;
    }
    }
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
            const float got = crf(fn, x, b), want = dbl(fn, x, b);
            unsigned gb, wb;
            std::memcpy(&gb, &got, 4);
            std::memcpy(&wb, &want, 4);
            if (gb != wb && !(got != got && want != want)) {
                ++bad;
                if (bad <= 5)
                    std::fprintf(stderr, "fn %d x = %a (u %u): %a, double gives %a\n", fn, x, b, got, want);
            }
            ++n;
            if (in_range(fn, x, b)) {
                ++nin;
                slow += g_slow - s0;
            }
        }
    }
    std::printf("%lld %lld %lld %lld\n", n, bad, nin, slow);
    return 0;
}
