// Ellipsoidal proposals of the nested sampler drawn on the GPU.
//
// The sampler bounds its live points by one or several ellipsoids (fitted on
// the host, lg_nested.cpp) and needs a batch of points uniform in their
// union and in the unit cube for every batched likelihood call.  Drawing
// them on the host costs about as much as the likelihood calls themselves
// (a normal vector, a triangular mat-vec and a radius per draw); here a
// kernel draws many candidates at once from a counter-based RNG, keeps each
// with probability 1 / (number of ellipsoids holding it), wraps periodic
// dimensions into [0, 1), drops points outside the cube, and an
// order-preserving compaction hands the first B kept points to the host.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "lg_internal.h"
#include "lg_nested.h"

namespace lg {
namespace {

constexpr int kMaxDim = 64;

// uniform in (0, 1) from (key, counter): splitmix64 finaliser, the top 23
// bits as an odd multiple of 2^-24 (exact in FP32)
__device__ __forceinline__ float lg_prop_u01(unsigned long long key, unsigned long long ctr)
{
    unsigned long long z = key + 0x9E3779B97F4A7C15ull * (ctr + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((((unsigned)(z >> 41)) << 1) | 1u) * 0x1p-24f;
}

// Per ellipsoid in the FP32 table F (stride 2 d^2 + 2): its lower Cholesky
// factor L and L^-1 (d x d each, row-major), sqrt(scale) and scale (the
// bound is |L^-1 (x - mu)|^2 <= scale).  Centres stay in FP64 (mu, d per
// ellipsoid); dmu[k][j] = mu_k - mu_j in FP32.
struct EllTable {
    int d, nell;
    const double* mu;
    const float* F;
    const float* dmu;
    const float* cum;  // cumulative volume fractions
    __device__ int stride() const { return 2 * d * d + 2; }
};

// M candidates: ellipsoid k chosen by volume, a uniform point in it
// (offset from its centre in FP32, the centre added in FP64), the
// multiple-cover rejection, wrapping and the cube test.  GB300 runs FP64
// at a small fraction of the FP32 rate, so only the final additions and
// the cube test are FP64.  flag[i] = 1 when draw i is kept.
__global__ void __launch_bounds__(128)
    lg_ell_draw(unsigned long long key, int M, EllTable T, const float* __restrict__ wrap, double* __restrict__ X,
                int* __restrict__ flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const int d = T.d, nell = T.nell;
    const unsigned long long c0 = (unsigned long long)i * (kMaxDim + 4);
    const float t = lg_prop_u01(key, c0) * T.cum[nell - 1];
    int k = 0;
    while (k + 1 < nell && T.cum[k] < t) ++k;
    const float* Fk = T.F + (size_t)k * T.stride();
    float z[kMaxDim], off[kMaxDim];
    float n2 = 0.0f;
    for (int a = 0; a < d; a += 2) {
        const float u1 = lg_prop_u01(key, c0 + 1 + a), u2 = lg_prop_u01(key, c0 + 2 + a);
        const float r = sqrtf(-2.0f * logf(u1));
        float sn, cs;
        sincospif(2.0f * u2, &sn, &cs);
        z[a] = r * cs;
        n2 += z[a] * z[a];
        if (a + 1 < d) {
            z[a + 1] = r * sn;
            n2 += z[a + 1] * z[a + 1];
        }
    }
    const float rad = Fk[2 * d * d] * exp2f(log2f(lg_prop_u01(key, c0 + kMaxDim + 1)) / d) * rsqrtf(n2);
    for (int a = 0; a < d; ++a) {
        float s = 0.0f;
        for (int b = 0; b <= a; ++b) s += Fk[a * d + b] * z[b];
        off[a] = rad * s;
    }
    int keep = 1;
    if (nell > 1) {
        // uniform in the union: keep with probability 1 / (ellipsoids holding x)
        int inside = 0;
        for (int j = 0; j < nell; ++j) {
            const float* Fj = T.F + (size_t)j * T.stride();
            const float* dm = T.dmu + ((size_t)k * nell + j) * d;
            float m = 0.0f;
            for (int a = 0; a < d; ++a) {  // L_j^-1 (x - mu_j), x - mu_j = off + mu_k - mu_j
                float s = 0.0f;
                for (int b = 0; b <= a; ++b) s += Fj[d * d + a * d + b] * (off[b] + dm[b]);
                m += s * s;
            }
            inside += m <= Fj[2 * d * d + 1];
        }
        if (inside > 1 && lg_prop_u01(key, c0 + kMaxDim + 2) * inside >= 1.0f) keep = 0;
    }
    const double* mu = T.mu + (size_t)k * d;
    for (int a = 0; a < d; ++a) {
        double x = mu[a] + (double)off[a];
        if (wrap && wrap[a] != 0.0f) x -= floor(x);
        if (!(x >= 0.0 && x <= 1.0)) keep = 0;
        X[(size_t)i * d + a] = x;
    }
    flag[i] = keep;
}

// The first `room` kept draws, in draw order, to out; cnt[0] = how many,
// cnt[1] = how many draws were kept in all (the acceptance estimate).
__global__ void __launch_bounds__(1024)
    lg_ell_compact(const int* __restrict__ flag, int M, const double* __restrict__ X, int d, int room,
                   double* __restrict__ out, int* __restrict__ cnt)
{
    __shared__ int part[1024];
    const int T = blockDim.x, t = threadIdx.x;
    const int per = (M + T - 1) / T, lo = t * per, hi = min(M, lo + per);
    int c = 0;
    for (int i = lo; i < hi; ++i) c += flag[i];
    part[t] = c;
    __syncthreads();
    if (t == 0) {
        int s = 0;
        for (int j = 0; j < T; ++j) {
            const int v = part[j];
            part[j] = s;
            s += v;
        }
        cnt[0] = min(s, room);
        cnt[1] = s;
    }
    __syncthreads();
    int pos = part[t];
    for (int i = lo; i < hi && pos < room; ++i)
        if (flag[i]) {
            for (int a = 0; a < d; ++a) out[(size_t)pos * d + a] = X[(size_t)i * d + a];
            ++pos;
        }
}

template <typename T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
    bool host = false;
    ~Buf() { host ? cudaFreeHost(p) : cudaFree(p); }
    bool ensure(size_t count, bool pinned = false)
    {
        if (count <= n) return true;
        host ? cudaFreeHost(p) : cudaFree(p);
        p = nullptr;
        n = 0;
        host = pinned;
        const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
        if ((pinned ? cudaMallocHost((void**)&p, bytes) : cudaMalloc((void**)&p, bytes)) != cudaSuccess) return false;
        n = count;
        return true;
    }
};

class GpuEllipsoidDrawer : public EllipsoidDrawer {
public:
    int device = 0;
    cudaStream_t s = nullptr;
    Buf<double> dmu, dX, dout, hmu, hout;
    Buf<float> dF, hF;
    Buf<int> dflag, dcnt, hcnt;
    double accept = 0.5;  // running estimate of the kept fraction

    ~GpuEllipsoidDrawer()
    {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }

    int draw(int d, int nell, const double* packed, const double* logv, const int* wrap, double* out, int B,
             uint64_t seed) override
    {
        if (d < 1 || d > kMaxDim || nell < 1 || B < 1) return -1;
        cudaSetDevice(device);
        if (!s && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return -1;
        const size_t stride = (size_t)d + (size_t)d * d + 1;  // packed: mu, L, scale per ellipsoid
        const size_t fs = 2 * (size_t)d * d + 2, nf = nell * fs + (size_t)nell * nell * d + nell;
        if (!hmu.ensure((size_t)nell * d, true) || !dmu.ensure((size_t)nell * d) || !hF.ensure(nf + d, true) ||
            !dF.ensure(nf + d) || !dcnt.ensure(2) || !hcnt.ensure(2, true) ||
            !dout.ensure((size_t)B * d) || !hout.ensure((size_t)B * d, true))
            return -1;
        // FP32 table: L, L^-1, sqrt(scale), scale per ellipsoid; centre
        // differences; cumulative volume fractions; then the wrap flags
        float* F = hF.p;
        float* dm = F + nell * fs;
        float* cum = dm + (size_t)nell * nell * d;
        std::vector<double> Li((size_t)d * d);
        for (int k = 0; k < nell; ++k) {
            const double* e = packed + k * stride;
            const double* L = e + d;
            std::memcpy(hmu.p + (size_t)k * d, e, d * sizeof(double));
            // L^-1 by forward substitution on the unit vectors
            std::fill(Li.begin(), Li.end(), 0.0);
            for (int c = 0; c < d; ++c)
                for (int a = c; a < d; ++a) {
                    double v = a == c ? 1.0 : 0.0;
                    for (int b = c; b < a; ++b) v -= L[(size_t)a * d + b] * Li[(size_t)b * d + c];
                    Li[(size_t)a * d + c] = v / L[(size_t)a * d + a];
                }
            float* Fk = F + k * fs;
            for (size_t q = 0; q < (size_t)d * d; ++q) {
                Fk[q] = (float)L[q];
                Fk[(size_t)d * d + q] = (float)Li[q];
            }
            Fk[2 * d * d] = (float)std::sqrt(e[stride - 1]);
            Fk[2 * d * d + 1] = (float)e[stride - 1];
        }
        for (int k = 0; k < nell; ++k)
            for (int j = 0; j < nell; ++j)
                for (int a = 0; a < d; ++a)
                    dm[((size_t)k * nell + j) * d + a] = (float)(packed[k * stride + a] - packed[j * stride + a]);
        double mx = -HUGE_VAL;
        for (int k = 0; k < nell; ++k) mx = std::max(mx, logv[k]);
        double c = 0;
        for (int k = 0; k < nell; ++k) cum[k] = (float)(c += std::exp(logv[k] - mx));
        float* hw = hF.p + nf;  // wrap flags as 0 / 1
        for (int a = 0; a < d; ++a) hw[a] = wrap && wrap[a] ? 1.0f : 0.0f;
        if (cudaMemcpyAsync(dmu.p, hmu.p, (size_t)nell * d * sizeof(double), cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(dF.p, hF.p, (nf + d) * sizeof(float), cudaMemcpyHostToDevice, s))
            return -1;
        EllTable T{d, nell, dmu.p, dF.p, dF.p + nell * fs, dF.p + nell * fs + (size_t)nell * nell * d};
        const float* dw = dF.p + nf;
        int got = 0;
        for (int round = 0; round < 16 && got < B; ++round) {
            const int need = B - got;
            const int M = (int)std::min<double>(1 << 20, std::max(2.0 * need, 1.3 * need / std::max(accept, 1e-4)));
            if (!dX.ensure((size_t)M * d) || !dflag.ensure(M)) return -1;
            lg_ell_draw<<<(M + 127) / 128, 128, 0, s>>>(seed + 0x632BE59BD9B4E019ull * (uint64_t)round, M, T, dw, dX.p,
                                                         dflag.p);
            lg_ell_compact<<<1, 1024, 0, s>>>(dflag.p, M, dX.p, d, need, dout.p + (size_t)got * d, dcnt.p);
            // the counts and the room for this pass's points in one wait
            if (cudaMemcpyAsync(hcnt.p, dcnt.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s) ||
                cudaMemcpyAsync(hout.p + (size_t)got * d, dout.p + (size_t)got * d, (size_t)need * d * sizeof(double),
                                cudaMemcpyDeviceToHost, s) ||
                cudaStreamSynchronize(s))
                return -1;
            // kept fraction of all draws of this pass
            accept = 0.5 * accept + 0.5 * std::max((double)hcnt.p[1] / M, 1e-6);
            got += hcnt.p[0];
        }
        if (got > 0) std::memcpy(out, hout.p, (size_t)got * d * sizeof(double));
        return got;
    }
};

}  // namespace

EllipsoidDrawer* make_gpu_ellipsoid_drawer(int device, std::string& err)
{
    auto* g = new (std::nothrow) GpuEllipsoidDrawer();
    if (!g) {
        err = "ellipsoid drawer: out of memory";
        return nullptr;
    }
    g->device = device;
    return g;
}

}  // namespace lg

extern "C" int lg_ellipsoid_draw_check(int device, int d, int nell, const double* packed, const double* logv,
                                       const int* wrap, double* out, int B, unsigned long long seed)
{
    if (!packed || !logv || !out || B <= 0 || d < 1 || nell < 1) return LG_ERR_INPUT;
    std::string err;
    std::unique_ptr<lg::EllipsoidDrawer> g(lg::make_gpu_ellipsoid_drawer(device, err));
    if (!g) return LG_ERR_ALLOC;
    const int n = g->draw(d, nell, packed, logv, wrap, out, B, seed);
    return n < 0 ? LG_ERR_CUDA : n;
}
