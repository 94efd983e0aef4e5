// Diagnostic entry point: the paired-ray elementary functions of the device
// prelude (exp, log, square root, reciprocal, arctangent and inverse
// hyperbolic tangent used by the fast evaluation modules),
// evaluated on a vector of inputs, so their accuracy can be checked against
// double-precision references on the host.

#include <cuda_runtime.h>

#include "lg_internal.h"
#include "../device/lg_prelude.cuh"

namespace {

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
                                : atanhf(a);
    out[i] = r.v.x;
    if (i + 1 < n) out[i + 1] = r.v.y;
}

}  // namespace

extern "C" int lg_probe_pair_math(int device, int fn, const float* x, int n, float* out)
{
    if (!x || !out || n < 0 || fn < 0 || fn > 5) return LG_ERR_INPUT;
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
