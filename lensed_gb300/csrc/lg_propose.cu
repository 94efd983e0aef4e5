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

// uniform in (0, 1) from (key, counter): splitmix64 finaliser
__device__ __forceinline__ double lg_prop_u01(unsigned long long key, unsigned long long ctr)
{
    unsigned long long z = key + 0x9E3779B97F4A7C15ull * (ctr + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// M candidates: ellipsoid k chosen by volume (cum: cumulative volume
// fractions), a uniform point in it, the multiple-cover rejection, wrapping
// and the cube test.  E holds per ellipsoid its centre (d), lower Cholesky
// factor (d x d, row-major) and scale (the bound is (x-mu)^T C^-1 (x-mu) <=
// scale).  flag[i] = 1 when draw i is kept.
__global__ void __launch_bounds__(128)
    lg_ell_draw(unsigned long long key, int M, int d, int nell, const double* __restrict__ E,
                const double* __restrict__ cum, const int* __restrict__ wrap, double* __restrict__ X,
                int* __restrict__ flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const size_t stride = (size_t)d + (size_t)d * d + 1;
    const unsigned long long c0 = (unsigned long long)i * (kMaxDim + 4);
    const double t = lg_prop_u01(key, c0) * cum[nell - 1];
    int k = 0;
    while (k + 1 < nell && cum[k] < t) ++k;
    const double* mu = E + k * stride;
    const double* L = mu + d;
    const double scale = L[(size_t)d * d];
    double z[kMaxDim], x[kMaxDim];
    double n2 = 0.0;
    for (int a = 0; a < d; a += 2) {
        const double u1 = lg_prop_u01(key, c0 + 1 + a), u2 = lg_prop_u01(key, c0 + 2 + a);
        const double r = sqrt(-2.0 * log(u1));
        double s, c;
        sincospi(2.0 * u2, &s, &c);
        z[a] = r * c;
        n2 += z[a] * z[a];
        if (a + 1 < d) {
            z[a + 1] = r * s;
            n2 += z[a + 1] * z[a + 1];
        }
    }
    const double rad = sqrt(scale) * pow(lg_prop_u01(key, c0 + kMaxDim + 1), 1.0 / d) / sqrt(n2);
    for (int a = 0; a < d; ++a) {
        double s = 0.0;
        for (int b = 0; b <= a; ++b) s += L[(size_t)a * d + b] * z[b];
        x[a] = mu[a] + rad * s;
    }
    int keep = 1;
    if (nell > 1) {
        // uniform in the union: keep with probability 1 / (ellipsoids holding x)
        int inside = 0;
        for (int j = 0; j < nell; ++j) {
            const double* mj = E + j * stride;
            const double* Lj = mj + d;
            double m = 0.0;
            for (int a = 0; a < d; ++a) {  // forward substitution L y = x - mu
                double s = x[a] - mj[a];
                for (int b = 0; b < a; ++b) s -= Lj[(size_t)a * d + b] * z[b];
                z[a] = s / Lj[(size_t)a * d + a];
                m += z[a] * z[a];
            }
            inside += m <= Lj[(size_t)d * d];
        }
        if (inside > 1 && lg_prop_u01(key, c0 + kMaxDim + 2) * inside >= 1.0) keep = 0;
    }
    for (int a = 0; a < d; ++a) {
        if (wrap && wrap[a]) x[a] -= floor(x[a]);
        if (!(x[a] >= 0.0 && x[a] <= 1.0)) keep = 0;
        X[(size_t)i * d + a] = x[a];
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
    Buf<double> dE, dcum, dX, dout, hE, hout;
    Buf<int> dwrap, dflag, dcnt, hcnt;
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
        const size_t stride = (size_t)d + (size_t)d * d + 1;
        if (!hE.ensure(nell * stride + nell + d, true) || !dE.ensure(nell * stride) || !dcum.ensure(nell) ||
            !dwrap.ensure(d) || !dcnt.ensure(2) || !hcnt.ensure(2, true) || !dout.ensure((size_t)B * d) ||
            !hout.ensure((size_t)B * d, true))
            return -1;
        // ellipsoids, cumulative volume fractions and wrap flags: one upload
        std::memcpy(hE.p, packed, nell * stride * sizeof(double));
        double mx = -HUGE_VAL;
        for (int k = 0; k < nell; ++k) mx = std::max(mx, logv[k]);
        double c = 0;
        for (int k = 0; k < nell; ++k) hE.p[nell * stride + k] = c += std::exp(logv[k] - mx);
        double* hw = hE.p + nell * stride + nell;
        for (int a = 0; a < d; ++a) hw[a] = wrap && wrap[a] ? 1.0 : 0.0;
        std::vector<int> iw(d);
        for (int a = 0; a < d; ++a) iw[a] = hw[a] != 0.0;
        if (cudaMemcpyAsync(dE.p, hE.p, nell * stride * sizeof(double), cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(dcum.p, hE.p + nell * stride, nell * sizeof(double), cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(dwrap.p, iw.data(), d * sizeof(int), cudaMemcpyHostToDevice, s))
            return -1;
        int got = 0;
        for (int round = 0; round < 16 && got < B; ++round) {
            const int need = B - got;
            const int M = (int)std::min<double>(1 << 20, std::max(2.0 * need, 1.3 * need / std::max(accept, 1e-4)));
            if (!dX.ensure((size_t)M * d) || !dflag.ensure(M)) return -1;
            lg_ell_draw<<<(M + 127) / 128, 128, 0, s>>>(seed + 0x632BE59BD9B4E019ull * (uint64_t)round, M, d, nell,
                                                         dE.p, dcum.p, dwrap.p, dX.p, dflag.p);
            lg_ell_compact<<<1, 1024, 0, s>>>(dflag.p, M, dX.p, d, need, dout.p + (size_t)got * d, dcnt.p);
            // the counts and the room for this round's points in one wait
            if (cudaMemcpyAsync(hcnt.p, dcnt.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s) ||
                cudaMemcpyAsync(hout.p + (size_t)got * d, dout.p + (size_t)got * d, (size_t)need * d * sizeof(double),
                                cudaMemcpyDeviceToHost, s) ||
                cudaStreamSynchronize(s))
                return -1;
            // kept fraction of all draws of this round
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
