// Diagnostic entry points: the paired-ray elementary functions of the
// device prelude (exp, log, square root, reciprocal, arctangent and inverse
// hyperbolic tangent used by the fast evaluation modules) and the correctly
// rounded functions of the exact modules (lg_crfloat.cuh), evaluated on a
// vector of inputs, so their accuracy can be checked against
// double-precision references on the host; and a sweep that compares the
// correctly rounded functions with the double evaluation on the device over
// a range of float bit patterns.

#include <cuda_runtime.h>

#include "lg_internal.h"
#include "../device/lg_prelude.cuh"
#include "../device/lg_crfloat.cuh"

namespace {

// correctly rounded function fn (0 exp, 1 log, 2 atan, 3 atanh) of a pair
__device__ float2 crf_pair(int fn, float2 a)
{
    return fn == 0 ? lg_crf_exp(a) : fn == 1 ? lg_crf_log(a) : fn == 2 ? lg_crf_atan(a) : lg_crf_atanh(a);
}
__device__ float crf_scalar(int fn, float x)
{
    return fn == 0 ? lg_crf_exp(x) : fn == 1 ? lg_crf_log(x) : fn == 2 ? lg_crf_atan(x) : lg_crf_atanh(x);
}
__device__ float crf_double(int fn, float x)
{
    return fn == 0   ? (float)exp((double)x)
           : fn == 1 ? (float)log((double)x)
           : fn == 2 ? (float)atan((double)x)
                     : (float)atanh((double)x);
}

// the EPL lens's functions, one value: fn 4 sin, 5 cos, 6 pow(x, Y[u % 16])
// with the lens's exponents and others, 7 atan2(x, p), 8 pow(|x|, p), p the
// float of bit pattern u * 0x9E3779B1 (the second argument swept too)
__constant__ float lg_probe_y[16] = {-1.2f, -1.0f, -0.8f, -0.5f, 0.5f, -0.25f, 0.2f, 1.0f / 3,
                                     2.5f, -2.2f, 0.999f, 1.5f, -0.1f, 3.7f, 0.05f, -7.5f};
__device__ float crf_two(int fn, float x, unsigned u)
{
    const float p = __uint_as_float(u * 0x9E3779B1u);
    float s, c;
    switch (fn) {
    case 4: lg_crf_sincos(x, &s, &c); return s;
    case 5: lg_crf_sincos(x, &s, &c); return c;
    case 6: return lg_crf_pow(x, lg_probe_y[u % 16]);
    case 7: return lg_crf_atan2(x, p);
    default: return lg_crf_pow(fabsf(x), p);
    }
}
__device__ float crf_two_double(int fn, float x, unsigned u)
{
    const float p = __uint_as_float(u * 0x9E3779B1u);
    switch (fn) {
    case 4: return (float)sin((double)x);
    case 5: return (float)cos((double)x);
    case 6: return (float)pow((double)x, (double)lg_probe_y[u % 16]);
    case 7: return (float)atan2((double)x, (double)p);
    default: return (float)pow((double)fabsf(x), (double)p);
    }
}

// every bit pattern u in [lo, hi) as lane 0 of a pair whose lane 1 is an
// unrelated input (u times an odd constant, a bijection of the 32-bit
// patterns), so that the lanes of a pair take different paths and table
// entries, and through the one-lane version; counts inputs whose bits
// differ from the double evaluation in either (NaN equal to NaN), and
// keeps the first few
__global__ void lg_crf_sweep_kernel(int fn, unsigned long long lo, unsigned long long hi,
                                    unsigned long long* __restrict__ bad, unsigned* __restrict__ first, int nfirst)
{
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    unsigned long long nbad = 0;
    for (unsigned long long u = lo + blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < hi; u += stride) {
        const float x0 = __uint_as_float((unsigned)u);
        if (fn >= 4) {
            const float r0 = crf_two(fn, x0, (unsigned)u), w0 = crf_two_double(fn, x0, (unsigned)u);
            if (!(__float_as_uint(r0) == __float_as_uint(w0) || (r0 != r0 && w0 != w0))) {
                ++nbad;
                const unsigned long long k = atomicAdd(bad + 1, 1ull);
                if (k < (unsigned long long)nfirst) first[k] = (unsigned)u;
            }
            continue;
        }
        const float x1 = __uint_as_float((unsigned)u * 0x9E3779B1u);
        const float2 r = crf_pair(fn, make_float2(x0, x1));
        const float w0 = crf_double(fn, x0), w1 = crf_double(fn, x1);
        // the one-lane version (what the exact render calls) on x0 too
        const float r0 = crf_scalar(fn, x0);
        const bool ok0 = (__float_as_uint(r.x) == __float_as_uint(w0) || (r.x != r.x && w0 != w0)) &&
                         (__float_as_uint(r0) == __float_as_uint(w0) || (r0 != r0 && w0 != w0));
        const bool ok1 = __float_as_uint(r.y) == __float_as_uint(w1) || (r.y != r.y && w1 != w1);
        if (!ok0 || !ok1) {
            nbad += (!ok0) + (!ok1);
            const unsigned long long k = atomicAdd(bad + 1, 1ull);
            if (k < (unsigned long long)nfirst) first[k] = ok0 ? __float_as_uint(x1) : (unsigned)u;
        }
    }
    if (nbad) atomicAdd(bad, nbad);
}

__global__ void lg_pair_math_kernel(int fn, const float* __restrict__ x, int n, float* __restrict__ out)
{
    const int i = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    const lg_pair a = lg_pair_of(x[i], i + 1 < n ? x[i + 1] : 1.0f);
    const lg_pair r = fn == 0   ? expf(a)
                      : fn == 1 ? logf(a)
                      : fn == 2 ? sqrtf(a)
                      : fn == 3 ? 1.0f / a
                      : fn == 4 ? atanf(a)
                      : fn == 5 ? atanhf(a)
                                : lg_pair{crf_pair(fn - 6, a.v)};
    out[i] = r.v.x;
    if (i + 1 < n) out[i + 1] = r.v.y;
}

}  // namespace

extern "C" int lg_probe_pair_math(int device, int fn, const float* x, int n, float* out)
{
    if (!x || !out || n < 0 || fn < 0 || fn > 9) return LG_ERR_INPUT;
    if (n == 0) return LG_OK;
    auto fail = [](cudaError_t e) {
        lg::set_global_error(cudaGetErrorString(e));
        return LG_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(e);
    float *dx = nullptr, *dy = nullptr;
    const size_t bytes = (size_t)n * 4;
    if ((e = cudaMalloc((void**)&dx, bytes)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&dy, bytes)) != cudaSuccess) {
        cudaFree(dx);
        return fail(e);
    }
    e = cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int pairs = (n + 1) / 2;
        lg_pair_math_kernel<<<(pairs + 255) / 256, 256>>>(fn, dx, n, dy);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dy, bytes, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    return e == cudaSuccess ? LG_OK : fail(e);
}

extern "C" int lg_probe_crf_sweep(int device, int fn, unsigned long long lo, unsigned long long hi,
                                  unsigned long long* mismatches, unsigned* first, int nfirst)
{
    if (fn < 0 || fn > 8 || lo > hi || hi > (1ull << 32) || !mismatches || nfirst < 0 || (nfirst && !first))
        return LG_ERR_INPUT;
    auto fail = [](cudaError_t e) {
        lg::set_global_error(cudaGetErrorString(e));
        return LG_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(e);
    unsigned long long* d_bad = nullptr;
    unsigned* d_first = nullptr;
    if ((e = cudaMalloc((void**)&d_bad, 2 * sizeof(unsigned long long))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&d_first, (nfirst ? nfirst : 1) * sizeof(unsigned))) != cudaSuccess) {
        cudaFree(d_bad);
        return fail(e);
    }
    e = cudaMemset(d_bad, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess && hi > lo) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        lg_crf_sweep_kernel<<<sms * 8, 256>>>(fn, lo, hi, d_bad, d_first, nfirst);
        e = cudaGetLastError();
    }
    unsigned long long h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d_bad, sizeof h, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nfirst)
        e = cudaMemcpy(first, d_first, (size_t)(h[1] < (unsigned long long)nfirst ? h[1] : nfirst) * sizeof(unsigned),
                       cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    cudaFree(d_first);
    if (e != cudaSuccess) return fail(e);
    *mismatches = h[0];
    return LG_OK;
}
