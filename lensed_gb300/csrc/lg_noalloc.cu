// Log-likelihood of model images the caller already holds on the GPU,
// computed without allocating any memory.
//
// Some callers cannot allocate device memory at the point where they need a
// likelihood: a host framework that owns every byte of the GPU through its
// own pool and forbids cudaMalloc from plug-ins, or code that runs while the
// caller is recording a memory-frozen execution (for instance inside a
// sampler step whose allocations were all made up front).  For them this file
// provides lg_loglike_images_noalloc(), the chi^2 reduction of the likelihood
// path (per-pixel w*(m-d)^2 in FP32, FP64 sums in a fixed order, logL =
// -chi^2/2) with its scratch -- the per-tile partial sums -- in a file-scope
// device array instead of a context's allocation.
//
// The array holds LG_NOALLOC_MAX_PARTIALS doubles (512 KiB) on every GPU that
// loads this library, for as long as the process runs.  All calls share it
// and it keeps the last call's contents; calls that overlap on the GPU (two
// streams, or two host threads) race on it and must be serialised by the
// caller.  Nothing in it needs clearing: every partial a call reads was
// written earlier in the same call.
//
// Set-up: the first call in a CUDA context (per device, and again after
// cudaDeviceReset) looks up the array's device address.  With CUDA's lazy
// module loading that lookup is also what loads this file's kernels and
// places the array on the device -- a one-time allocation made by the
// driver.  A caller that may not allocate at all makes one call at its own
// set-up time, before any stream capture; later calls allocate nothing.

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "lensed_gb300.h"

namespace lg {
void set_global_error(const char* msg);
}

static __device__ __align__(256) double lg_noalloc_scratch[LG_NOALLOC_MAX_PARTIALS];

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;
constexpr long kPixelsPerTile = 2048;

std::mutex g_mu;

// The scratch address, valid in the CUDA context it was looked up in.
// Contexts are told apart by their driver-assigned unique id (never reused
// within a process), so a context re-created after cudaDeviceReset gets a
// fresh lookup instead of a stale address.
struct Scratch {
    unsigned long long ctx_id = 0;
    double* ptr = nullptr;
};
Scratch g_scratch[kMaxDevices];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

template <class F>
bool resolve(const char* name, F& f)
{
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
        return false;
    f = reinterpret_cast<F>(p);
    return true;
}

// Unique id of the current context; 0 if the driver cannot say (the address
// is then looked up on every call).
unsigned long long current_context_id()
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        resolved = true;
        if (!resolve("cuCtxGetCurrent", get_current) || !resolve("cuCtxGetId", get_id)) get_current = nullptr;
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array in the current context of `device`
// (the array's name in host code is only a host-side stand-in).
int scratch_for(int device, double** out)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Scratch& sc = g_scratch[device];
    const unsigned long long id = current_context_id();
    if (!sc.ptr || id == 0 || sc.ctx_id != id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, lg_noalloc_scratch);
        if (e != cudaSuccess) {
            char msg[256];
            std::snprintf(msg, sizeof msg, "lg_loglike_images_noalloc: cudaGetSymbolAddress: %s",
                          cudaGetErrorString(e));
            lg::set_global_error(msg);
            return LG_ERR_CUDA;
        }
        sc.ptr = static_cast<double*>(p);
        // cudaGetSymbolAddress made the context current if it was not
        sc.ctx_id = id ? id : current_context_id();
    }
    *out = sc.ptr;
    return LG_OK;
}

__device__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order block sum, valid in thread 0.
__device__ double block_sum(double v)
{
    __shared__ double red[kThreads / 32];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kThreads / 32; ++i) s += red[i];
    return s;
}

// Block (tile, candidate): the chi^2 of one tile of pixels of one model.
__global__ void __launch_bounds__(kThreads)
    chi2_partials(const float* __restrict__ image, const float* __restrict__ weight,
                  const float* __restrict__ models, long n, long tile, double* __restrict__ partials)
{
    const int b = blockIdx.y;
    const long k0 = (long)blockIdx.x * tile;
    const long k1 = k0 + tile < n ? k0 + tile : n;
    const float* m = models + (size_t)b * n;
    double s = 0.0;
    for (long k = k0 + threadIdx.x; k < k1; k += kThreads) {
        const float d = m[k] - image[k];
        s += (double)(weight[k] * d * d);
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partials[(size_t)b * gridDim.x + blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads)
    chi2_finish(const double* __restrict__ partials, int tiles, double* __restrict__ logL)
{
    const int b = blockIdx.x;
    double s = 0.0;
    for (int t = threadIdx.x; t < tiles; t += kThreads) s += partials[(size_t)b * tiles + t];
    s = block_sum(s);
    if (threadIdx.x == 0) logL[b] = -0.5 * s;
}

}  // namespace

extern "C" int lg_loglike_images_noalloc(const float* d_image, const float* d_weight, const float* d_models,
                                         long n_pixels, int B, double* d_logL, void* stream)
{
    char msg[256];
    if (!d_image || !d_weight || !d_models || !d_logL || n_pixels <= 0 || B <= 0) {
        lg::set_global_error("lg_loglike_images_noalloc: null pointer or non-positive size");
        return LG_ERR_INPUT;
    }
    if (B > LG_NOALLOC_MAX_PARTIALS || B > 65535) {
        std::snprintf(msg, sizeof msg,
                      "lg_loglike_images_noalloc: %d models exceed the maximum of 65535 per call "
                      "(static scratch of %d partial sums)",
                      B, LG_NOALLOC_MAX_PARTIALS);
        lg::set_global_error(msg);
        return LG_ERR_INPUT;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
        lg::set_global_error("lg_loglike_images_noalloc: no current CUDA device");
        return LG_ERR_CUDA;
    }
    double* partials = nullptr;
    int rc = scratch_for(device, &partials);
    if (rc) return rc;
    // tiles per model: about kPixelsPerTile pixels each, and B * tiles within
    // the scratch array
    long tiles = (n_pixels + kPixelsPerTile - 1) / kPixelsPerTile;
    const long cap = LG_NOALLOC_MAX_PARTIALS / B;
    if (tiles > cap) tiles = cap;
    if (tiles < 1) tiles = 1;
    const long tile = (n_pixels + tiles - 1) / tiles;
    tiles = (n_pixels + tile - 1) / tile;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    chi2_partials<<<dim3((unsigned)tiles, (unsigned)B), kThreads, 0, s>>>(d_image, d_weight, d_models, n_pixels,
                                                                          tile, partials);
    chi2_finish<<<B, kThreads, 0, s>>>(partials, (int)tiles, d_logL);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::snprintf(msg, sizeof msg, "lg_loglike_images_noalloc: launch: %s", cudaGetErrorString(e));
        lg::set_global_error(msg);
        return LG_ERR_CUDA;
    }
    return LG_OK;
}
