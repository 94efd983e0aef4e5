// Learned proposal for the nested sampler: an affine-coupling normalising
// flow (Dinh, Sohl-Dickstein & Bengio 2017) trained by maximum likelihood on
// the live points, with hand-written CUDA kernels for training and inference.
//
// Space: the unit-cube live points are standardised per dimension (mean and
// standard deviation of the live set), u = (x - m) / s.  Layer l splits the
// dimensions at h = d/2 into a conditioning half A and a transformed half B
// (A = [0, h) on even layers, [h, d) on odd ones):
//     z_B = u_B * exp(s(u_A)) + t(u_A),   z_A = u_A,
// with s = c * tanh(s_raw / c) (c = LG_FLOW_CLAMP) and (s_raw, t) from an MLP
// conditioner (width W, `hidden` ReLU layers, zero-initialised output layer so
// training starts from the identity).  log p(x) = log N(z; 0, I) + sum s
// - sum log s_std.  Weights and gradients are FP32; hidden activations are
// stored in BF16 for the backward pass (the BF16 variant can be switched off
// to check gradients against the CPU restatement).
//
// Proposals (as nessai, Williams et al. 2021): z uniform in a ball of radius
// `expand` x the largest latent radius of the live points, mapped back to the
// cube; a draw is kept with probability |det dx/dz| / W, W a bound calibrated
// on a large latent sample at each training, which makes the kept draws
// uniform in the image of the ball; draws outside the cube are dropped.  The
// flow is trained with a held-out split and early stopping so that it stays
// smooth; a flow whose calibrated kept fraction is below 1% is not used.
// Every kept draw is then judged by the exact likelihood in the sampler.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "lg_internal.h"
#include "lg_nested.h"

#define LG_FLOW_CLAMP 5.0f

namespace lg {
namespace {

constexpr int TS = 32;  // GEMM tile

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ void from_f(float& d, float v) { d = v; }
__device__ __forceinline__ void from_f(__nv_bfloat16& d, float v) { d = __float2bfloat16_rn(v); }

// C = act(op(A) op(B) + bias) [* (mask > 0)] [+ C]
// op(A)(m, k) = ta ? A[k * lda + m] : A[m * lda + k]; op(B)(k, n) likewise.
// 16 x 16 threads, 2 x 2 outputs each, 32 x 32 tiles staged in shared memory.
template <typename TA, typename TB, typename TC, typename TM>
__global__ void __launch_bounds__(256) gemm(const TA* __restrict__ A, int lda, int ta, const TB* __restrict__ B,
                                            int ldb, int tb, TC* __restrict__ C, int ldc, int M, int N, int K,
                                            const float* __restrict__ bias, int relu, const TM* __restrict__ mask,
                                            int accumulate)
{
    __shared__ float As[TS][TS + 1], Bs[TS][TS + 1];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 16 + tx;
    const int row0 = blockIdx.y * TS, col0 = blockIdx.x * TS;
    float acc[2][2] = {{0, 0}, {0, 0}};
    for (int k0 = 0; k0 < K; k0 += TS) {
        for (int e = tid; e < TS * TS; e += 256) {
            const int i = e / TS, j = e % TS;
            const int m = row0 + i, k = k0 + j;
            As[i][j] = (m < M && k < K) ? to_f(ta ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]) : 0.0f;
            const int kb = k0 + i, n = col0 + j;
            Bs[i][j] = (kb < K && n < N) ? to_f(tb ? B[(size_t)n * ldb + kb] : B[(size_t)kb * ldb + n]) : 0.0f;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < TS; ++kk) {
            const float a0 = As[ty * 2][kk], a1 = As[ty * 2 + 1][kk];
            const float b0 = Bs[kk][tx * 2], b1 = Bs[kk][tx * 2 + 1];
            acc[0][0] += a0 * b0;
            acc[0][1] += a0 * b1;
            acc[1][0] += a1 * b0;
            acc[1][1] += a1 * b1;
        }
        __syncthreads();
    }
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) {
            const int m = row0 + ty * 2 + i, n = col0 + tx * 2 + j;
            if (m >= M || n >= N) continue;
            float v = acc[i][j] + (bias ? bias[n] : 0.0f);
            if (relu) v = v > 0 ? v : 0;
            if (mask && !(to_f(mask[(size_t)m * N + n]) > 0)) v = 0;
            TC* c = &C[(size_t)m * ldc + n];
            if (accumulate) v += to_f(*c);
            from_f(*c, v);
        }
}

// column sums: out[n] (+)= sum_m X[m][n]
__global__ void colsum(const float* __restrict__ X, int M, int N, float* __restrict__ out, int accumulate)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0;
    for (int m = 0; m < M; ++m) s += X[(size_t)m * N + n];
    out[n] = accumulate ? out[n] + s : s;
}

// gather the conditioning half: in[m][j] = u[m][a0 + j]
__global__ void gather_half(const float* __restrict__ u, int d, int a0, int da, int M, float* __restrict__ in)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M * da) return;
    const int m = e / da, j = e % da;
    in[e] = u[(size_t)m * d + a0 + j];
}

// forward coupling: v = u with v_B = u_B exp(s) + t; logdet += sum s
__global__ void coupling_fwd(const float* __restrict__ u, const float* __restrict__ o, int d, int b0, int db,
                             int M, float* __restrict__ v, float* __restrict__ logdet)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    float ld = 0;
    for (int j = 0; j < d; ++j) v[(size_t)m * d + j] = u[(size_t)m * d + j];
    for (int j = 0; j < db; ++j) {
        const float sr = o[(size_t)m * 2 * db + j], t = o[(size_t)m * 2 * db + db + j];
        const float s = LG_FLOW_CLAMP * tanhf(sr / LG_FLOW_CLAMP);
        v[(size_t)m * d + b0 + j] = u[(size_t)m * d + b0 + j] * expf(s) + t;
        ld += s;
    }
    logdet[m] += ld;
}

// inverse coupling: u_B = (v_B - t) exp(-s); logdet -= sum s
__global__ void coupling_inv(const float* __restrict__ v, const float* __restrict__ o, int d, int b0, int db, int M,
                             float* __restrict__ u, float* __restrict__ logdet)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    float ld = 0;
    for (int j = 0; j < d; ++j) u[(size_t)m * d + j] = v[(size_t)m * d + j];
    for (int j = 0; j < db; ++j) {
        const float sr = o[(size_t)m * 2 * db + j], t = o[(size_t)m * 2 * db + db + j];
        const float s = LG_FLOW_CLAMP * tanhf(sr / LG_FLOW_CLAMP);
        u[(size_t)m * d + b0 + j] = (v[(size_t)m * d + b0 + j] - t) * expf(-s);
        ld -= s;
    }
    logdet[m] += ld;
}

// backward of a coupling layer.  dv: gradient w.r.t. the layer output;
// writes do (gradient w.r.t. the conditioner output) and du (w.r.t. the
// input, conditioning half still missing the conditioner's contribution).
// dlogdet is the gradient of the loss w.r.t. every s (the loss is
// -mean(logdet), so -1/M).
__global__ void coupling_bwd(const float* __restrict__ u, const float* __restrict__ o, const float* __restrict__ dv,
                             int d, int b0, int db, int M, float dlogdet, float* __restrict__ dout,
                             float* __restrict__ du)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    for (int j = 0; j < d; ++j) du[(size_t)m * d + j] = dv[(size_t)m * d + j];
    for (int j = 0; j < db; ++j) {
        const float sr = o[(size_t)m * 2 * db + j];
        const float th = tanhf(sr / LG_FLOW_CLAMP);
        const float s = LG_FLOW_CLAMP * th, es = expf(s);
        const float g = dv[(size_t)m * d + b0 + j];
        const float ub = u[(size_t)m * d + b0 + j];
        const float ds = g * ub * es + dlogdet;
        dout[(size_t)m * 2 * db + j] = ds * (1.0f - th * th);
        dout[(size_t)m * 2 * db + db + j] = g;
        du[(size_t)m * d + b0 + j] = g * es;
    }
}

// scatter-add the conditioner's input gradient into du's conditioning half
__global__ void add_half(float* __restrict__ du, int d, int a0, int da, int M, const float* __restrict__ din)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= M * da) return;
    const int m = e / da, j = e % da;
    du[(size_t)m * d + a0 + j] += din[e];
}

// loss terms: per sample 0.5|z|^2 - logdet; dz = z / M
__global__ void nll(const float* __restrict__ z, const float* __restrict__ logdet, int d, int M,
                    float* __restrict__ per, float* __restrict__ dz)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    float q = 0;
    for (int j = 0; j < d; ++j) {
        const float v = z[(size_t)m * d + j];
        q += v * v;
        if (dz) dz[(size_t)m * d + j] = v / M;
    }
    per[m] = 0.5f * q - logdet[m];
}

__global__ void adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                     float* __restrict__ m2, long n, float lr, float b1, float b2, float c1, float c2)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    m1[i] = b1 * m1[i] + (1 - b1) * gi;
    m2[i] = b2 * m2[i] + (1 - b2) * gi * gi;
    p[i] -= lr * (m1[i] / c1) / (sqrtf(m2[i] / c2) + 1e-8f);
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DevBuf() { cudaFree(p); }
    bool ensure(size_t count)
    {
        if (count <= n) return true;
        cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return false;
        n = count;
        return true;
    }
};

}  // namespace

// The flow: parameters, optimiser state and work buffers on one device.
class Flow {
public:
    int d = 0, L = 8, W = 128, NH = 2, h = 0;
    bool bf16 = true;
    std::vector<size_t> off;  // per layer, per dense layer: weight offset, bias offset
    std::vector<int> din, dout;
    size_t nparams = 0;
    DevBuf<float> P, G, M1, M2;
    std::vector<float> mean, sdev;
    long step = 0;
    bool want_loss = true;  // read the loss back (off inside training loops)

    int da(int l) const { return (l % 2 == 0) ? h : d - h; }
    int a0(int l) const { return (l % 2 == 0) ? 0 : h; }
    int db(int l) const { return d - da(l); }
    int b0(int l) const { return (l % 2 == 0) ? h : 0; }
    int ndense() const { return NH + 1; }
    size_t woff(int l, int k) const { return off[(size_t)(l * ndense() + k) * 2]; }
    size_t boff(int l, int k) const { return off[(size_t)(l * ndense() + k) * 2 + 1]; }
    int kin(int l, int k) const { return k == 0 ? da(l) : W; }
    int kout(int l, int k) const { return k == ndense() - 1 ? 2 * db(l) : W; }

    bool init(int dim, int layers, int width, int hidden, uint64_t seed)
    {
        d = dim;
        L = layers;
        W = width;
        NH = hidden;
        h = d / 2;
        if (d < 2) return false;
        off.clear();
        nparams = 0;
        for (int l = 0; l < L; ++l)
            for (int k = 0; k < ndense(); ++k) {
                off.push_back(nparams);
                nparams += (size_t)kin(l, k) * kout(l, k);
                off.push_back(nparams);
                nparams += kout(l, k);
            }
        if (!P.ensure(nparams) || !G.ensure(nparams) || !M1.ensure(nparams) || !M2.ensure(nparams)) return false;
        // He-uniform hidden weights, zero output layer and biases: the flow
        // starts as the identity map
        std::vector<float> host(nparams, 0.0f);
        uint64_t s = seed * 6364136223846793005ull + 1442695040888963407ull;
        auto unif = [&]() {
            s = s * 6364136223846793005ull + 1442695040888963407ull;
            return ((s >> 11) * (1.0 / 9007199254740992.0)) * 2 - 1;
        };
        for (int l = 0; l < L; ++l)
            for (int k = 0; k + 1 < ndense(); ++k) {
                const double lim = std::sqrt(6.0 / kin(l, k));
                for (size_t i = 0; i < (size_t)kin(l, k) * kout(l, k); ++i) host[woff(l, k) + i] = (float)(lim * unif());
            }
        cudaMemcpy(P.p, host.data(), nparams * 4, cudaMemcpyHostToDevice);
        cudaMemset(M1.p, 0, nparams * 4);
        cudaMemset(M2.p, 0, nparams * 4);
        step = 0;
        return cudaGetLastError() == cudaSuccess;
    }

    // work buffers for a batch of M samples
    DevBuf<float> u, in, o, ld, per, dz, du, dv, dob, din_b, tmp;
    DevBuf<__nv_bfloat16> hb;
    DevBuf<float> hf;

    bool reserve(int M)
    {
        const size_t hs = (size_t)L * NH * M * W;
        return u.ensure((size_t)(L + 1) * M * d) && in.ensure((size_t)L * M * std::max(h, d - h) + 1) &&
               o.ensure((size_t)L * M * 2 * std::max(h, d - h) + 1) && ld.ensure(M) && per.ensure(M) &&
               dz.ensure((size_t)M * d) && du.ensure((size_t)M * d) && dv.ensure((size_t)M * d) &&
               dob.ensure((size_t)M * 2 * std::max(h, d - h) + 1) && din_b.ensure((size_t)M * std::max(W, d) + 1) &&
               tmp.ensure((size_t)M * std::max(W, d) + 1) &&
               (bf16 ? hb.ensure(hs) : hf.ensure(hs));
    }

    template <typename TA, typename TB, typename TC, typename TM>
    static void mm(const TA* A, int lda, int ta, const TB* B, int ldb, int tb, TC* C, int ldc, int M, int N, int K,
                   const float* bias, int relu, const TM* mask, int acc)
    {
        dim3 g((N + TS - 1) / TS, (M + TS - 1) / TS);
        gemm<TA, TB, TC, TM><<<g, dim3(16, 16)>>>(A, lda, ta, B, ldb, tb, C, ldc, M, N, K, bias, relu, mask, acc);
    }

    template <typename TH>
    TH* hid(TH* base, int l, int k, int M) const
    {
        return base + ((size_t)l * NH + k) * M * W;
    }

    // conditioner of layer l on in (M x da) -> o (M x 2db), hidden
    // activations stored for the backward pass
    template <typename TH>
    void conditioner(int l, const float* x, int M, float* out, TH* hbase)
    {
        const float* p = P.p;
        // first hidden layer from the float input
        mm<float, float, TH, float>(x, da(l), 0, p + woff(l, 0), W, 0, hid(hbase, l, 0, M), W, M, W, da(l),
                                    p + boff(l, 0), 1, nullptr, 0);
        for (int k = 1; k < NH; ++k)
            mm<TH, float, TH, float>(hid(hbase, l, k - 1, M), W, 0, p + woff(l, k), W, 0, hid(hbase, l, k, M), W, M,
                                     W, W, p + boff(l, k), 1, nullptr, 0);
        mm<TH, float, float, float>(hid(hbase, l, NH - 1, M), W, 0, p + woff(l, NH), 2 * db(l), 0, out, 2 * db(l),
                                    M, 2 * db(l), W, p + boff(l, NH), 0, nullptr, 0);
    }

    template <typename TH>
    float forward_backward(const float* x, int M, bool grad, TH* hbase)
    {
        const int T = 128;
        cudaMemcpy(u.p, x, (size_t)M * d * 4, cudaMemcpyDeviceToDevice);
        cudaMemset(ld.p, 0, (size_t)M * 4);
        for (int l = 0; l < L; ++l) {
            float* ul = u.p + (size_t)l * M * d;
            float* il = in.p + (size_t)l * M * std::max(h, d - h);
            float* ol = o.p + (size_t)l * M * 2 * std::max(h, d - h);
            gather_half<<<(M * da(l) + T - 1) / T, T>>>(ul, d, a0(l), da(l), M, il);
            conditioner(l, il, M, ol, hbase);
            coupling_fwd<<<(M + T - 1) / T, T>>>(ul, ol, d, b0(l), db(l), M, ul + (size_t)M * d, ld.p);
        }
        nll<<<(M + T - 1) / T, T>>>(u.p + (size_t)L * M * d, ld.p, d, M, per.p, grad ? dz.p : nullptr);
        double loss = 0;
        if (want_loss) {
            std::vector<float> hp(M);
            cudaMemcpy(hp.data(), per.p, (size_t)M * 4, cudaMemcpyDeviceToHost);
            for (float v : hp) loss += v;
            loss /= M;
        }
        if (!grad) return (float)loss;
        cudaMemset(G.p, 0, nparams * 4);
        cudaMemcpy(dv.p, dz.p, (size_t)M * d * 4, cudaMemcpyDeviceToDevice);
        for (int l = L - 1; l >= 0; --l) {
            float* ul = u.p + (size_t)l * M * d;
            float* il = in.p + (size_t)l * M * std::max(h, d - h);
            float* ol = o.p + (size_t)l * M * 2 * std::max(h, d - h);
            coupling_bwd<<<(M + T - 1) / T, T>>>(ul, ol, dv.p, d, b0(l), db(l), M, -1.0f / M, dob.p, du.p);
            float* g = G.p;
            const float* p = P.p;
            // output dense layer
            TH* hl = hid(hbase, l, NH - 1, M);
            mm<TH, float, float, float>(hl, W, 1, dob.p, 2 * db(l), 0, g + woff(l, NH), 2 * db(l), W, 2 * db(l), M,
                                        nullptr, 0, nullptr, 0);
            colsum<<<(2 * db(l) + T - 1) / T, T>>>(dob.p, M, 2 * db(l), g + boff(l, NH), 0);
            // gradient w.r.t. the last hidden activation, masked by ReLU
            // (kept in din_b as float)
            mm<float, float, float, TH>(dob.p, 2 * db(l), 0, p + woff(l, NH), 2 * db(l), 1, din_b.p, W, M, W,
                                        2 * db(l), nullptr, 0, hl, 0);
            for (int k = NH - 1; k >= 1; --k) {
                TH* hprev = hid(hbase, l, k - 1, M);
                mm<TH, float, float, float>(hprev, W, 1, din_b.p, W, 0, g + woff(l, k), W, W, W, M, nullptr, 0,
                                            nullptr, 0);
                colsum<<<(W + T - 1) / T, T>>>(din_b.p, M, W, g + boff(l, k), 0);
                mm<float, float, float, TH>(din_b.p, W, 0, p + woff(l, k), W, 1, tmp.p, W, M, W, W, nullptr, 0,
                                            hprev, 0);
                std::swap(din_b.p, tmp.p);
            }
            // first dense layer
            mm<float, float, float, float>(il, da(l), 1, din_b.p, W, 0, g + woff(l, 0), W, da(l), W, M, nullptr, 0,
                                           nullptr, 0);
            colsum<<<(W + T - 1) / T, T>>>(din_b.p, M, W, g + boff(l, 0), 0);
            // gradient w.r.t. the conditioning input, added to du
            mm<float, float, float, float>(din_b.p, W, 0, p + woff(l, 0), W, 1, tmp.p, da(l), M, da(l), W, nullptr,
                                           0, nullptr, 0);
            add_half<<<(M * da(l) + T - 1) / T, T>>>(du.p, d, a0(l), da(l), M, tmp.p);
            std::swap(dv.p, du.p);
        }
        return (float)loss;
    }

    float loss_and_grad(const float* x, int M, bool grad)
    {
        return bf16 ? forward_backward<__nv_bfloat16>(x, M, grad, hb.p) : forward_backward<float>(x, M, grad, hf.p);
    }

    void adam_step(float lr)
    {
        ++step;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1 - std::pow(b1, (float)step), c2 = 1 - std::pow(b2, (float)step);
        adam<<<(unsigned)((nparams + 255) / 256), 256>>>(P.p, G.p, M1.p, M2.p, (long)nparams, lr, b1, b2, c1, c2);
    }

    // inverse map of M latent points (device) -> standardised u (device),
    // log|det du/dz| per point (device)
    template <typename TH>
    void inverse(const float* z, int M, float* uout, TH* hbase)
    {
        const int T = 128;
        float* cur = u.p;
        cudaMemcpy(cur, z, (size_t)M * d * 4, cudaMemcpyDeviceToDevice);
        cudaMemset(ld.p, 0, (size_t)M * 4);
        for (int l = L - 1; l >= 0; --l) {
            float* nxt = (l % 2 == 0) ? dv.p : du.p;
            if (l == 0) nxt = uout;
            gather_half<<<(M * da(l) + T - 1) / T, T>>>(cur, d, a0(l), da(l), M, in.p);
            conditioner(l, in.p, M, o.p, hbase);
            coupling_inv<<<(M + T - 1) / T, T>>>(cur, o.p, d, b0(l), db(l), M, nxt, ld.p);
            cur = nxt;
        }
    }
};

// The proposal used by the sampler.
class FlowProposal : public Proposal {
public:
    Flow flow;
    lg_flow_options opt;
    int device = 0;
    uint64_t seed = 1;
    bool trained = false;
    double radius = 0, last_loss = 0;
    long ntrain = 0;
    std::vector<float> hx;
    DevBuf<float> dx, dzlat, dulat, dval, best;

    int train(const double* live, int n, int d) override
    {
        cudaSetDevice(device);
        if (flow.d != d) {
            flow.bf16 = true;
            if (!flow.init(d, opt.layers, opt.width, opt.hidden, seed)) return LG_ERR_CUDA;
        }
        // standardise by the live set
        flow.mean.assign(d, 0);
        flow.sdev.assign(d, 0);
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < d; ++a) flow.mean[a] += (float)live[(size_t)i * d + a];
        for (auto& m : flow.mean) m /= n;
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < d; ++a) {
                const double v = live[(size_t)i * d + a] - flow.mean[a];
                flow.sdev[a] += (float)(v * v);
            }
        for (auto& s : flow.sdev) s = std::sqrt(std::max(s / n, 1e-24f));
        hx.resize((size_t)n * d);
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < d; ++a)
                hx[(size_t)i * d + a] = (float)((live[(size_t)i * d + a] - flow.mean[a]) / flow.sdev[a]);
        // hold out 20% of the live points for early stopping: the best
        // weights on the held-out set are kept (the flow has far more
        // parameters than there are live points)
        std::vector<int> idx(n);
        std::iota(idx.begin(), idx.end(), 0);
        uint64_t s = seed ^ 0x5bd1e995u ^ ((uint64_t)ntrain << 32);
        for (int i = n - 1; i > 0; --i) {
            s = s * 6364136223846793005ull + 1442695040888963407ull;
            std::swap(idx[i], idx[(s >> 33) % (uint64_t)(i + 1)]);
        }
        const int nval = std::max(1, n / 5), ntr = n - nval;
        std::vector<float> vx((size_t)nval * d);
        for (int i = 0; i < nval; ++i) std::memcpy(&vx[(size_t)i * d], &hx[(size_t)idx[ntr + i] * d], d * 4);
        idx.resize(ntr);
        const int Mb = std::min(opt.batch, ntr);
        if (!dx.ensure((size_t)n * d) || !dval.ensure((size_t)nval * d) || !best.ensure(flow.nparams) ||
            !flow.reserve(std::max(Mb, n)))
            return LG_ERR_ALLOC;
        cudaMemcpy(dval.p, vx.data(), vx.size() * 4, cudaMemcpyHostToDevice);
        auto val_loss = [&]() {
            flow.want_loss = true;
            const float l = flow.loss_and_grad(dval.p, nval, false);
            flow.want_loss = false;
            return l;
        };
        float best_loss = val_loss();
        cudaMemcpy(best.p, flow.P.p, flow.nparams * 4, cudaMemcpyDeviceToDevice);
        int since_best = 0;
        const int patience = 20;
        std::vector<float> bx((size_t)Mb * d);
        // warm start: later retrainings continue from the previous weights
        // with a quarter of the epochs
        const int epochs = ntrain == 0 ? opt.epochs : std::max(1, opt.epochs / 4);
        ++ntrain;
        flow.want_loss = false;
        const bool dbg = std::getenv("LG_FLOW_DEBUG") != nullptr;
        for (int ep = 0; ep < epochs; ++ep) {
            if (dbg && ntrain == 1 && (ep % 25 == 0)) {
                flow.want_loss = true;
                cudaMemcpy(dx.p, hx.data(), (size_t)n * d * 4, cudaMemcpyHostToDevice);
                std::fprintf(stderr, "flow: epoch %d loss %.4f\n", ep, flow.loss_and_grad(dx.p, n, false));
                flow.want_loss = false;
            }
            for (int i = ntr - 1; i > 0; --i) {
                s = s * 6364136223846793005ull + 1442695040888963407ull;
                std::swap(idx[i], idx[(s >> 33) % (uint64_t)(i + 1)]);
            }
            for (int b0 = 0; b0 + Mb <= ntr; b0 += Mb) {
                for (int i = 0; i < Mb; ++i)
                    std::memcpy(&bx[(size_t)i * d], &hx[(size_t)idx[b0 + i] * d], d * 4);
                cudaMemcpy(dx.p, bx.data(), (size_t)Mb * d * 4, cudaMemcpyHostToDevice);
                flow.loss_and_grad(dx.p, Mb, true);
                flow.adam_step((float)opt.lr);
            }
            const float vl = val_loss();
            if (std::isfinite(vl) && vl < best_loss) {
                best_loss = vl;
                since_best = 0;
                cudaMemcpy(best.p, flow.P.p, flow.nparams * 4, cudaMemcpyDeviceToDevice);
            } else if (++since_best >= patience) {
                break;
            }
        }
        cudaMemcpy(flow.P.p, best.p, flow.nparams * 4, cudaMemcpyDeviceToDevice);
        if (dbg) std::fprintf(stderr, "flow: best held-out loss %.4f\n", best_loss);
        // latent radius of the live points
        flow.want_loss = true;
        cudaMemcpy(dx.p, hx.data(), (size_t)n * d * 4, cudaMemcpyHostToDevice);
        last_loss = flow.loss_and_grad(dx.p, n, false);
        std::vector<float> z((size_t)n * d);
        cudaMemcpy(z.data(), flow.u.p + (size_t)flow.L * n * d, z.size() * 4, cudaMemcpyDeviceToHost);
        double r = 0;
        for (int i = 0; i < n; ++i) {
            double q = 0;
            for (int a = 0; a < d; ++a) q += (double)z[(size_t)i * d + a] * z[(size_t)i * d + a];
            r = std::max(r, std::sqrt(q));
        }
        radius = r * opt.expand;
        trained = std::isfinite(radius) && radius > 0 && cudaGetLastError() == cudaSuccess;
        if (trained) trained = calibrate(d);
        if (std::getenv("LG_FLOW_DEBUG"))
            std::fprintf(stderr, "flow: train %ld epochs %d loss %.4f latent radius %.3f ok %d\n", ntrain, epochs,
                         last_loss, radius, (int)trained);
        return trained ? LG_OK : LG_ERR_CUDA;
    }

    double wnorm = 0;       // log weight normaliser (calibrated at training)
    double efficiency = 0;  // mean kept fraction of latent draws

    // M latent draws uniform in the ball, mapped to the standardised space
    // (uu), with their log weights log|det dx/dz|
    bool latent_batch(Rng& r, int M, int d, std::vector<float>& z, std::vector<float>& uu, std::vector<float>& lw)
    {
        if (!dzlat.ensure((size_t)M * d) || !dulat.ensure((size_t)M * d) || !flow.reserve(M)) return false;
        z.resize((size_t)M * d);
        uu.resize((size_t)M * d);
        lw.resize(M);
        // uniform in the latent ball
        for (int i = 0; i < M; ++i) {
            double n2 = 0;
            for (int a = 0; a < d; ++a) {
                const double v = r.normal();
                z[(size_t)i * d + a] = (float)v;
                n2 += v * v;
            }
            const double rad = radius * std::pow(r.uniform(), 1.0 / d) / std::sqrt(n2);
            for (int a = 0; a < d; ++a) z[(size_t)i * d + a] = (float)(z[(size_t)i * d + a] * rad);
        }
        cudaMemcpy(dzlat.p, z.data(), z.size() * 4, cudaMemcpyHostToDevice);
        if (flow.bf16) flow.inverse(dzlat.p, M, dulat.p, flow.hb.p);
        else flow.inverse(dzlat.p, M, dulat.p, flow.hf.p);
        cudaMemcpy(uu.data(), dulat.p, uu.size() * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(lw.data(), flow.ld.p, (size_t)M * 4, cudaMemcpyDeviceToHost);
        return cudaGetLastError() == cudaSuccess;
    }

    // Calibrate the normaliser on a large latent sample (its maximum plus a
    // margin, so that the rejection step is exact unless a weight exceeds it)
    // and estimate the efficiency; a flow whose kept fraction is below 1% is
    // not used (the sampler stays on the ellipsoid).
    bool calibrate(int d)
    {
        Rng r(seed * 7919 + (uint64_t)ntrain);
        std::vector<float> z, uu, lw;
        const int M = 16384;
        if (!latent_batch(r, M, d, z, uu, lw)) return false;
        double mx = -INFINITY;
        for (float v : lw)
            if (std::isfinite(v)) mx = std::max(mx, (double)v);
        if (!std::isfinite(mx)) return false;
        wnorm = mx + 1.0;
        double acc = 0;
        for (float v : lw)
            if (std::isfinite(v)) acc += std::exp(v - wnorm);
        efficiency = acc / M;
        if (std::getenv("LG_FLOW_DEBUG"))
            std::fprintf(stderr, "flow: calibrated efficiency %.4f\n", efficiency);
        return efficiency >= 0.01;
    }

    // volume of the image of the latent ball: V_ball(R) E[|det dx/dz|]
    double log_volume() const override
    {
        if (!trained || efficiency <= 0) return HUGE_VAL;
        const int d = flow.d;
        double lv = 0.5 * d * std::log(M_PI) - std::lgamma(0.5 * d + 1) + d * std::log(radius);
        lv += std::log(efficiency) + wnorm;
        for (float sd : flow.sdev) lv += std::log((double)sd);
        return lv;
    }

    int propose(const double*, int, int d, double* out, int B, uint64_t sd) override
    {
        if (!trained) return 0;
        cudaSetDevice(device);
        Rng r(sd);
        const int M = std::max(4 * B, (int)std::min(65536.0, 2.0 * B / std::max(efficiency, 1e-3)));
        std::vector<float> z, uu, ldet;
        int got = 0;
        for (int round = 0; round < 4 && got < B; ++round) {
            // keep x with probability proportional to 1 / q_x(x) = |det dx/dz|
            // (z uniform in the ball), normalised by the calibrated bound (a
            // weight above it raises the bound for the rest of the round)
            if (!latent_batch(r, M, d, z, uu, ldet)) return 0;
            double lmax = wnorm;
            for (int i = 0; i < M; ++i)
                if (std::isfinite(ldet[i]) && ldet[i] > lmax) lmax = ldet[i];
            wnorm = lmax;
            int kept = 0;
            for (int i = 0; i < M && got < B; ++i) {
                if (!std::isfinite(ldet[i]) || r.uniform() > std::exp((double)ldet[i] - lmax)) continue;
                ++kept;
                bool in = true;
                double* x = out + (size_t)got * d;
                for (int a = 0; a < d && in; ++a) {
                    x[a] = flow.mean[a] + (double)flow.sdev[a] * uu[(size_t)i * d + a];
                    in = x[a] >= 0 && x[a] <= 1;
                }
                if (in) ++got;
            }
            if (std::getenv("LG_FLOW_DEBUG") && round == 0) {
                std::vector<float> w(ldet);
                std::sort(w.begin(), w.end());
                const float lmaxf = (float)lmax;
                std::fprintf(stderr,
                             "flow: propose %d latent, %d kept by the weight test, %d in the cube; log weight "
                             "quantiles 1%% %.2f 50%% %.2f 99%% %.2f max %.2f\n",
                             M, kept, got, w[M / 100] - lmaxf, w[M / 2] - lmaxf, w[M - 1 - M / 100] - lmaxf,
                             w[M - 1] - lmaxf);
            }
        }
        return got;
    }
};

}  // namespace lg

lg::Proposal* lg::make_flow_proposal(int device, int d, const lg_flow_options* opts, std::string& err)
{
    (void)d;
    auto* p = new (std::nothrow) FlowProposal();
    if (!p) {
        err = "flow proposal: out of memory";
        return nullptr;
    }
    p->device = device;
    p->opt = opts ? *opts : lg_flow_defaults();
    return p;
}

extern "C" {

lg_flow_options lg_flow_defaults(void)
{
    lg_flow_options o;
    o.layers = 8;
    o.width = 128;
    o.hidden = 2;
    o.epochs = 200;
    o.batch = 256;
    o.lr = 1e-3;
    o.expand = 1.1;
    return o;
}

// Loss and gradient of the flow on n points (standardised space, host
// arrays), for gradient checks against the CPU restatement: params in/out
// (lg_flow_nparams values), grad out.  bf16 = 0 keeps activations in FP32.
long lg_flow_nparams(int d, int layers, int width, int hidden)
{
    lg::Flow f;
    f.d = d;
    f.L = layers;
    f.W = width;
    f.NH = hidden;
    f.h = d / 2;
    long n = 0;
    for (int l = 0; l < f.L; ++l)
        for (int k = 0; k < f.ndense(); ++k) n += (long)f.kin(l, k) * f.kout(l, k) + f.kout(l, k);
    return n;
}

int lg_flow_loss_grad(int device, int d, int layers, int width, int hidden, int bf16, const float* params,
                      const float* x, int n, float* loss, float* grad)
{
    if (cudaSetDevice(device) != cudaSuccess) return LG_ERR_CUDA;
    lg::Flow f;
    f.bf16 = bf16 != 0;
    if (!f.init(d, layers, width, hidden, 1) || !f.reserve(n)) return LG_ERR_ALLOC;
    cudaMemcpy(f.P.p, params, f.nparams * 4, cudaMemcpyHostToDevice);
    lg::DevBuf<float> dx;
    if (!dx.ensure((size_t)n * d)) return LG_ERR_ALLOC;
    cudaMemcpy(dx.p, x, (size_t)n * d * 4, cudaMemcpyHostToDevice);
    *loss = f.loss_and_grad(dx.p, n, true);
    cudaMemcpy(grad, f.G.p, f.nparams * 4, cudaMemcpyDeviceToHost);
    return cudaDeviceSynchronize() == cudaSuccess ? LG_OK : LG_ERR_CUDA;
}

}  // extern "C"
