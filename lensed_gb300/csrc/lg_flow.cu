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
// - sum log s_std.  Weights, gradients and optimiser state are FP32; hidden
// activations are rounded to BF16 as they are produced (the next layer and
// the backward pass use the rounded values; the BF16 variant can be switched
// off to check gradients against the CPU restatement).
//
// Kernels (all the flow's work for one step is one launch):
//   lg_flow_step   a block takes FR (FP32: FR32) rows of a minibatch through every
//                  coupling layer and back: forward, loss, backward, and the
//                  block's partial weight gradients (its rows' sums) into
//                  its own slice of a partial-gradient buffer;
//   lg_flow_adam   sums the blocks' slices in a fixed order (deterministic)
//                  and takes an Adam step;
//   lg_flow_check  held-out loss in a fixed order; keeps the best weights
//                  and stops training after `patience` epochs without
//                  improvement -- on the device, so a whole retraining is
//                  issued without a host synchronisation (later launches of
//                  a stopped training return at once);
//   lg_flow_inverse  latent points back to the cube through every layer;
//   lg_flow_latent / _max_part / _accept / _scan / _scatter  proposals:
//                  uniform draws in the latent ball (counter-based RNG,
//                  Box-Muller), the weight bound, the rejection test
//                  against it, the unit-cube test and an order-preserving
//                  compaction, all in FP32 (GB300's FP64 rate is a small
//                  fraction of its FP32 rate).
//
// Proposals (as nessai, Williams et al. 2021): z uniform in the ball through
// the farthest live point in latent space, its volume enlarged by `expand`
// (as the plain sampler enlarges its ellipsoid), mapped back to the cube; a draw is kept with probability |det dx/dz| / W, W a bound calibrated
// on a large latent sample at each training, which makes the kept draws
// uniform in the image of the ball; draws outside the cube are dropped.  The
// flow is trained with a held-out split and early stopping so that it stays
// smooth; a flow whose calibrated kept fraction is below 0.2% is not used.
// Every kept draw is then evaluated by the exact likelihood in the sampler.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
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
#define LG_FLOW_HISTORY 256

namespace lg {
namespace {

constexpr int FT = 256;        // threads per block of the fused kernels
constexpr int FR = 16;         // minibatch rows per training block (BF16 activations)
constexpr int FR32 = 8;        // the same with FP32 activations (twice the shared memory per row)
constexpr int FRI = 32;        // rows per inverse block
constexpr int MAX_W = 128;     // conditioner width limit (shared-memory tiles)
constexpr int MAX_D = 64;      // dimension limit
constexpr int MAX_DENSE = 64;  // coupling layers x dense layers limit
// smallest calibrated kept fraction of latent draws for which a flow is used
// (its draws cost little on the tensor cores; below, the ellipsoid is used)
constexpr double kMinKept = 0.002;

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ void from_f(float& d, float v) { d = v; }
__device__ __forceinline__ void from_f(__nv_bfloat16& d, float v) { d = __float2bfloat16_rn(v); }

// Shape of a flow, passed by value to the kernels.
struct FlowDims {
    int d, h, L, W, NH;
    __host__ __device__ int da(int l) const { return (l % 2 == 0) ? h : d - h; }
    __host__ __device__ int a0(int l) const { return (l % 2 == 0) ? 0 : h; }
    __host__ __device__ int db(int l) const { return d - da(l); }
    __host__ __device__ int b0(int l) const { return (l % 2 == 0) ? h : 0; }
    __host__ __device__ int kin(int l, int k) const { return k == 0 ? da(l) : W; }
    __host__ __device__ int kout(int l, int k) const { return k == NH ? 2 * db(l) : W; }
    __host__ __device__ int dbmax() const { return d - h; }
};

// Parameter offsets of every dense layer: weights [kin][kout] row-major, then
// the bias [kout], layer by layer (the layout of the CPU restatement).
__device__ void fill_offsets(const FlowDims& f, int* offs)
{
    if (threadIdx.x == 0) {
        int n = 0;
        for (int l = 0; l < f.L; ++l)
            for (int k = 0; k <= f.NH; ++k) {
                offs[2 * (l * (f.NH + 1) + k)] = n;
                n += f.kin(l, k) * f.kout(l, k);
                offs[2 * (l * (f.NH + 1) + k) + 1] = n;
                n += f.kout(l, k);
            }
    }
    __syncthreads();
}

// Asynchronous 4-byte global -> shared copies (no registers held while in
// flight, so a thread's whole share of a weight matrix is requested at once).
__device__ __forceinline__ void cp_async4(float* dst, const float* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Stage a K x N row-major weight matrix into shared memory: Ws[k][n] (pitch
// N) or, transposed, Ws[n][k] (pitch K + 1, conflict-free both ways).
__device__ void stage_weights(float* Ws, const float* __restrict__ Wg, int K, int N, bool transpose)
{
    const int pk = K + 1;
    for (int e = threadIdx.x; e < K * N; e += FT) {
        const int k = e / N, n = e - k * N;
        cp_async4(transpose ? Ws + n * pk + k : Ws + e, Wg + e);
    }
    cp_async_wait_all();
    __syncthreads();
}

// Y[r][n] = act(sum_k X[r][k] W[k][n] + b[n]) for R rows (X, Y in shared
// memory, W staged into Ws).  Micro-tile per thread: CPT adjacent columns
// (LANES column slots) x R / (FT / LANES) rows, all compile-time so that the
// accumulators stay in registers; the k loop runs in order with FP32
// accumulation (rows read four k at a time when their pitch allows), then
// the bias and the ReLU.  With Hs, the result is also rounded to TH (stored
// there and written back to Y as the rounded value).
template <int R, int LANES, int CPT, typename TH>
__device__ void dense_fwd_tile(const float* X, int ldx, int K, const float* Ws, const float* __restrict__ bg, int N,
                               bool relu, float* Y, int ldy, TH* Hs)
{
    constexpr int GROUPS = FT / LANES, RPT = R / GROUPS;
    static_assert(R % GROUPS == 0, "rows per block must split over the thread groups");
    const int lane = threadIdx.x % LANES, g = threadIdx.x / LANES;
    const float* x0 = X + g * RPT * ldx;
    const bool vec = (ldx % 4) == 0;
    for (int c = lane * CPT; c < N; c += LANES * CPT) {
        float acc[RPT][CPT];
#pragma unroll
        for (int i = 0; i < RPT; ++i)
#pragma unroll
            for (int j = 0; j < CPT; ++j) acc[i][j] = 0.0f;
        int k = 0;
        if (vec)
            for (; k + 3 < K; k += 4) {
                float w[4][CPT];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (CPT == 2) {
                        const float2 t = *reinterpret_cast<const float2*>(Ws + (k + q) * N + c);
                        w[q][0] = t.x;
                        w[q][CPT - 1] = t.y;
                    } else {
                        w[q][0] = Ws[(k + q) * N + c];
                    }
                }
#pragma unroll
                for (int i = 0; i < RPT; ++i) {
                    const float4 xv = *reinterpret_cast<const float4*>(x0 + i * ldx + k);
#pragma unroll
                    for (int j = 0; j < CPT; ++j) {
                        float a = acc[i][j];
                        a += xv.x * w[0][j];
                        a += xv.y * w[1][j];
                        a += xv.z * w[2][j];
                        a += xv.w * w[3][j];
                        acc[i][j] = a;
                    }
                }
            }
        for (; k < K; ++k) {
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                const float w = Ws[k * N + c + j];
#pragma unroll
                for (int i = 0; i < RPT; ++i) acc[i][j] += x0[i * ldx + k] * w;
            }
        }
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            const float b = __ldg(bg + c + j);
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int r = g * RPT + i;
                float v = acc[i][j] + b;
                if (relu) v = v > 0.0f ? v : 0.0f;
                if (Hs) {
                    from_f(Hs[r * N + c + j], v);
                    v = to_f(Hs[r * N + c + j]);
                }
                Y[r * ldy + c + j] = v;
            }
        }
    }
}

template <int R, typename TH>
__device__ void dense_fwd(const float* X, int ldx, int K, const float* __restrict__ Wg, const float* __restrict__ bg,
                          int N, bool relu, float* Y, int ldy, TH* Hs, float* Ws)
{
    stage_weights(Ws, Wg, K, N, false);
    if (N >= 128 && N % 2 == 0)
        dense_fwd_tile<R, 64, 2, TH>(X, ldx, K, Ws, bg, N, relu, Y, ldy, Hs);
    else if (N >= 64 && N % 2 == 0)
        dense_fwd_tile<R, 32, 2, TH>(X, ldx, K, Ws, bg, N, relu, Y, ldy, Hs);
    else
        dense_fwd_tile<R, 32, 1, TH>(X, ldx, K, Ws, bg, N, relu, Y, ldy, Hs);
    __syncthreads();
}

// dX[r][k] = sum_n dY[r][n] W[k][n] from the transposed weights WT[n][k]
// (pitch K + 1), masked by X > 0 when mask_relu; thread column k, R /
// (FT / LANES) rows per thread (compile-time).
template <int R, int LANES, typename TX>
__device__ void dense_dx(const TX* X, int ldx, int K, const float* dY, int ldy, int N, const float* WT, float* dX,
                         int lddx, bool mask_relu)
{
    constexpr int GROUPS = FT / LANES, RPT = R / GROUPS;
    static_assert(R % GROUPS == 0, "rows per block must split over the thread groups");
    const int pk = K + 1, g = threadIdx.x / LANES;
    const float* y0 = dY + g * RPT * ldy;
    for (int k = threadIdx.x % LANES; k < K; k += LANES) {
        float acc[RPT];
#pragma unroll
        for (int i = 0; i < RPT; ++i) acc[i] = 0.0f;
        for (int n = 0; n < N; ++n) {
            const float w = WT[n * pk + k];
#pragma unroll
            for (int i = 0; i < RPT; ++i) acc[i] += y0[i * ldy + n] * w;
        }
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            const int r = g * RPT + i;
            float v = acc[i];
            if (mask_relu && !(to_f(X[r * ldx + k]) > 0.0f)) v = 0.0f;
            dX[r * lddx + k] = v;
        }
    }
}

// Backward of a dense layer for R rows: partial weight and bias gradients
// of this block's rows (written to gW, gb: the block's slice), and
// dX[r][k] = sum_n dY[r][n] W[k][n], masked by X > 0 when mask_relu (the
// input was a ReLU output).  X is read as TH (stored activations) or float.
template <int R, typename TX>
__device__ void dense_bwd(const TX* X, int ldx, int K, const float* dY, int ldy, int N, const float* __restrict__ Wg,
                          float* __restrict__ gW, float* __restrict__ gb, float* dX, int lddx, bool mask_relu,
                          float* WT)
{
    // W transposed, WT[n][k] (requested now, waited for before dX)
    const int pk = K + 1;
    if (dX)
        for (int e = threadIdx.x; e < K * N; e += FT) {
            const int k = e / N, n = e - k * N;
            cp_async4(WT + n * pk + k, Wg + e);
        }
    // weight gradient: thread column n, all R rows of dY in registers
    int lanes = 32;
    while (lanes < N && lanes < FT) lanes <<= 1;
    int groups = FT / lanes;
    for (int n = threadIdx.x % lanes; n < N; n += lanes) {
        float dy[R];
#pragma unroll
        for (int r = 0; r < R; ++r) dy[r] = dY[r * ldy + n];
        for (int k = threadIdx.x / lanes; k < K; k += groups) {
            float acc = 0.0f;
#pragma unroll
            for (int r = 0; r < R; ++r) acc += to_f(X[r * ldx + k]) * dy[r];
            gW[(size_t)k * N + n] = acc;
        }
        if (threadIdx.x / lanes == 0) {
            float acc = 0.0f;
#pragma unroll
            for (int r = 0; r < R; ++r) acc += dy[r];
            gb[n] = acc;
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // input gradient: thread column k, rows split over the groups
    if (dX) {
        if (K >= 64)
            dense_dx<R, 64>(X, ldx, K, dY, ldy, N, WT, dX, lddx, mask_relu);
        else
            dense_dx<R, 32>(X, ldx, K, dY, ldy, N, WT, dX, lddx, mask_relu);
    }
    __syncthreads();
}

// Shared-memory layout of lg_flow_step for R rows (floats unless noted).
struct StepSmem {
    int us, os, ld, xa, a, b, da, db, wt, dv, du, hs, offs, total;
    __host__ __device__ StepSmem(const FlowDims& f, int R, int hbytes)
    {
        int o = 0;
        auto take = [&](int n) {
            const int at = o;
            o += (n + 3) / 4 * 4;
            return at;
        };
        us = take((f.L + 1) * R * f.d);
        os = take(f.L * R * 2 * f.dbmax());
        ld = take(R);
        // work rows: hidden activations (W wide), conditioner outputs and
        // their gradients (2 dbmax wide)
        const int wr = f.W > 2 * f.dbmax() ? f.W : 2 * f.dbmax();
        xa = take(R * f.dbmax());
        a = take(R * wr);
        b = take(R * wr);
        da = take(R * wr);
        db = take(R * wr);
        wt = take(f.W * (f.W + 1) > 2 * f.dbmax() * (f.W + 1) ? f.W * (f.W + 1) : 2 * f.dbmax() * (f.W + 1));
        dv = take(R * f.d);
        du = take(R * f.d);
        offs = take(2 * (f.L * (f.NH + 1)));
        hs = o;  // TH activations: L x NH x R x W
        total = o * 4 + ((f.L * f.NH * R * f.W * hbytes + 15) / 16) * 16;
    }
};

// One training step (or a forward evaluation, grad = 0) of the flow on rows
// idx[row0 + r] (or row0 + r when idx is NULL) of X (n x d, standardised),
// R rows per block, M rows in the minibatch.  Writes per-row losses
// 0.5 |z|^2 - logdet (loss), optionally |z|^2 (znorm2), and with grad the
// block's partial gradient slice gpart[blockIdx.x][nparams].
template <int R, typename TH>
__global__ void __launch_bounds__(FT)
    lg_flow_step(FlowDims f, const float* __restrict__ P, const float* __restrict__ X,
                 const int* __restrict__ idx, int row0, int M, int grad, float* __restrict__ loss,
                 float* __restrict__ znorm2, float* __restrict__ gpart, long nparams, const int* __restrict__ stop)
{
    if (stop && *stop) return;
    extern __shared__ float4 smem4[];
    float* sm = reinterpret_cast<float*>(smem4);
    const StepSmem L(f, R, (int)sizeof(TH));
    float* Us = sm + L.us;
    float* Os = sm + L.os;
    float* ld = sm + L.ld;
    float* xa = sm + L.xa;
    float* A = sm + L.a;
    float* B = sm + L.b;
    float* dA = sm + L.da;
    float* dB = sm + L.db;
    float* WT = sm + L.wt;
    float* dv = sm + L.dv;
    float* du = sm + L.du;
    int* offs = reinterpret_cast<int*>(sm + L.offs);
    TH* Hs = reinterpret_cast<TH*>(sm + L.hs);
    const int d = f.d, W = f.W, NH = f.NH, nd = NH + 1, dbm = f.dbmax();
    fill_offsets(f, offs);
    const int base = blockIdx.x * R;
    // rows beyond M are zero inputs; their loss and gradient are dropped
    for (int e = threadIdx.x; e < R * d; e += FT) {
        const int r = e / d, j = e - r * d;
        const int m = base + r;
        Us[e] = m < M ? X[(size_t)(idx ? idx[row0 + m] : row0 + m) * d + j] : 0.0f;
    }
    if (threadIdx.x < R) ld[threadIdx.x] = 0.0f;
    __syncthreads();
    // ---- forward
    for (int l = 0; l < f.L; ++l) {
        const int da = f.da(l), db = f.db(l), a0 = f.a0(l), b0 = f.b0(l);
        const float* u = Us + l * R * d;
        for (int e = threadIdx.x; e < R * da; e += FT) {
            const int r = e / da, j = e - r * da;
            xa[r * dbm + j] = u[r * d + a0 + j];
        }
        __syncthreads();
        const int* of = offs + 2 * l * nd;
        TH* hl = Hs + (size_t)l * NH * R * W;
        dense_fwd<R, TH>(xa, dbm, da, P + of[0], P + of[1], W, true, A, W, hl, WT);
        for (int k = 1; k < NH; ++k) {
            dense_fwd<R, TH>(A, W, W, P + of[2 * k], P + of[2 * k + 1], W, true, B, W, hl + (size_t)k * R * W, WT);
            float* t = A;
            A = B;
            B = t;
        }
        float* o = Os + l * R * 2 * dbm;
        dense_fwd<R, TH>(A, W, W, P + of[2 * NH], P + of[2 * NH + 1], 2 * db, false, o, 2 * dbm, (TH*)nullptr, WT);
        // coupling: v = u, v_B = u_B exp(s) + t; logdet += sum s
        float* v = Us + (l + 1) * R * d;
        for (int e = threadIdx.x; e < R * d; e += FT) v[e] = u[e];
        __syncthreads();
        if (threadIdx.x < R) {
            const int r = threadIdx.x;
            float acc = 0.0f;
            for (int j = 0; j < db; ++j) {
                const float s = LG_FLOW_CLAMP * tanhf(o[r * 2 * dbm + j] / LG_FLOW_CLAMP);
                v[r * d + b0 + j] = u[r * d + b0 + j] * expf(s) + o[r * 2 * dbm + db + j];
                acc += s;
            }
            ld[r] += acc;
        }
        __syncthreads();
    }
    // ---- loss: 0.5 |z|^2 - logdet per row
    const float* z = Us + f.L * R * d;
    if (threadIdx.x < R) {
        const int r = threadIdx.x;
        float q = 0.0f;
        for (int j = 0; j < d; ++j) q += z[r * d + j] * z[r * d + j];
        if (base + r < M) {
            loss[base + r] = 0.5f * q - ld[r];
            if (znorm2) znorm2[base + r] = q;
        }
    }
    if (!grad) return;
    // ---- backward: dz = z / M, dlogdet = -1 / M (mean loss); rows beyond M
    // carry no gradient
    for (int e = threadIdx.x; e < R * d; e += FT) dv[e] = (base + e / d < M) ? z[e] / M : 0.0f;
    __syncthreads();
    float* gp = gpart + (size_t)blockIdx.x * nparams;
    for (int l = f.L - 1; l >= 0; --l) {
        const int da = f.da(l), db = f.db(l), a0 = f.a0(l), b0 = f.b0(l);
        const float* u = Us + l * R * d;
        const float* o = Os + l * R * 2 * dbm;
        // coupling backward: dO = (ds (1 - th^2), g), du = dv with du_B = g e^s
        float* dO = dB;  // R x 2db, pitch 2 dbm
        for (int e = threadIdx.x; e < R * d; e += FT) du[e] = dv[e];
        __syncthreads();
        for (int e = threadIdx.x; e < R * db; e += FT) {
            const int r = e / db, j = e - r * db;
            const float th = tanhf(o[r * 2 * dbm + j] / LG_FLOW_CLAMP);
            const float s = LG_FLOW_CLAMP * th, es = expf(s);
            const float g = dv[r * d + b0 + j];
            const float dlog = base + r < M ? -1.0f / M : 0.0f;
            const float ds = g * u[r * d + b0 + j] * es + dlog;
            dO[r * 2 * dbm + j] = ds * (1.0f - th * th);
            dO[r * 2 * dbm + db + j] = g;
            du[r * d + b0 + j] = g * es;
        }
        __syncthreads();
        const int* of = offs + 2 * l * nd;
        const TH* hl = Hs + (size_t)l * NH * R * W;
        // output dense: input the last hidden activation
        dense_bwd<R, TH>(hl + (size_t)(NH - 1) * R * W, W, W, dO, 2 * dbm, 2 * db, P + of[2 * NH], gp + of[2 * NH],
                         gp + of[2 * NH + 1], dA, W, true, WT);
        for (int k = NH - 1; k >= 1; --k) {
            dense_bwd<R, TH>(hl + (size_t)(k - 1) * R * W, W, W, dA, W, W, P + of[2 * k], gp + of[2 * k],
                             gp + of[2 * k + 1], dB, W, true, WT);
            float* t = dA;
            dA = dB;
            dB = t;
        }
        // first dense: input the conditioning half of u
        for (int e = threadIdx.x; e < R * da; e += FT) {
            const int r = e / da, j = e - r * da;
            xa[r * dbm + j] = u[r * d + a0 + j];
        }
        __syncthreads();
        dense_bwd<R, float>(xa, dbm, da, dA, W, W, P + of[0], gp + of[0], gp + of[1], dB, dbm, false, WT);
        for (int e = threadIdx.x; e < R * da; e += FT) {
            const int r = e / da, j = e - r * da;
            du[r * d + a0 + j] += dB[r * dbm + j];
        }
        __syncthreads();
        for (int e = threadIdx.x; e < R * d; e += FT) dv[e] = du[e];
        __syncthreads();
    }
}

// Early stopping on the device.  state: [0] best held-out loss, [1] epochs
// since the best (as float), [2] last held-out loss, [3] training epochs
// completed (counted when epoch = 1), [4] 1 if the last check improved,
// [8 + e] the held-out loss after epoch e; stop: set once `patience` epochs
// pass without improvement.  The held-out loss is the mean of the per-row
// losses (lane j sums rows j, j + 32, ... in order, then a fixed tree).
__global__ void __launch_bounds__(32)
    lg_flow_check(const float* __restrict__ loss, int n, float* __restrict__ state, int patience, int* stop,
                  int epoch)
{
    if (*stop) return;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) s += loss[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) {
        const float v = (float)(s / n);
        state[2] = v;
        state[3] += (float)epoch;
        const int e = (int)state[3];
        if (e < LG_FLOW_HISTORY) state[8 + e] = v;
        const bool improved = isfinite(v) && v < state[0];
        state[4] = improved ? 1.0f : 0.0f;
        if (improved) {
            state[0] = v;
            state[1] = 0.0f;
        } else {
            state[1] += 1.0f;
            if (state[1] >= (float)patience) *stop = 1;
        }
    }
}

// best = P after a check that improved (state[4]); skipped once stopped.
__global__ void __launch_bounds__(256)
    lg_flow_keep(const float* __restrict__ state, const int* __restrict__ stop, const float* __restrict__ P,
                 float* __restrict__ best, long n)
{
    if (state[4] == 0.0f) return;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) best[i] = P[i];
    (void)stop;
}

// Shared-memory layout of lg_flow_inverse for R rows (floats unless noted).
struct InvSmem {
    int cur, xa, a, b, o, ld, offs, ws, hb, total;
    __host__ __device__ InvSmem(const FlowDims& f, int R, int hbytes)
    {
        int q = 0;
        auto take = [&](int n) {
            const int at = q;
            q += (n + 3) / 4 * 4;
            return at;
        };
        const int wr = f.W > 2 * f.dbmax() ? f.W : 2 * f.dbmax();
        cur = take(R * f.d);
        xa = take(R * f.dbmax());
        a = take(R * wr);
        b = take(R * wr);
        o = take(R * 2 * f.dbmax());
        ld = take(R);
        offs = take(2 * (f.L * (f.NH + 1)));
        ws = take(f.W * (f.W > 2 * f.dbmax() ? f.W : 2 * f.dbmax()));
        hb = q;
        total = q * 4 + ((R * f.W * hbytes + 15) / 16) * 16;
    }
};

// Inverse flow of M latent points (R rows per block): z -> u (standardised
// cube coordinates), ldet = log |det du/dz| = -sum s.
template <int R, typename TH>
__global__ void __launch_bounds__(FT)
    lg_flow_inverse(FlowDims f, const float* __restrict__ P, const float* __restrict__ Z, int M,
                    float* __restrict__ Uout, float* __restrict__ ldet)
{
    extern __shared__ float4 smem4[];
    float* sm = reinterpret_cast<float*>(smem4);
    const InvSmem L(f, R, (int)sizeof(TH));
    const int d = f.d, W = f.W, NH = f.NH, nd = NH + 1, dbm = f.dbmax();
    float* cur = sm + L.cur;
    float* xa = sm + L.xa;
    float* A = sm + L.a;
    float* B = sm + L.b;
    float* o = sm + L.o;
    float* ld = sm + L.ld;
    int* offs = reinterpret_cast<int*>(sm + L.offs);
    float* Ws = sm + L.ws;
    TH* hbuf = reinterpret_cast<TH*>(sm + L.hb);  // rounding buffer of a hidden layer
    fill_offsets(f, offs);
    const int base = blockIdx.x * R;
    for (int e = threadIdx.x; e < R * d; e += FT) cur[e] = base + e / d < M ? Z[(size_t)base * d + e] : 0.0f;
    if (threadIdx.x < R) ld[threadIdx.x] = 0.0f;
    __syncthreads();
    for (int l = f.L - 1; l >= 0; --l) {
        const int da = f.da(l), db = f.db(l), a0 = f.a0(l), b0 = f.b0(l);
        for (int e = threadIdx.x; e < R * da; e += FT) {
            const int r = e / da, j = e - r * da;
            xa[r * dbm + j] = cur[r * d + a0 + j];
        }
        __syncthreads();
        const int* of = offs + 2 * l * nd;
        dense_fwd<R, TH>(xa, dbm, da, P + of[0], P + of[1], W, true, A, W, hbuf, Ws);
        for (int k = 1; k < NH; ++k) {
            dense_fwd<R, TH>(A, W, W, P + of[2 * k], P + of[2 * k + 1], W, true, B, W, hbuf, Ws);
            float* t = A;
            A = B;
            B = t;
        }
        dense_fwd<R, TH>(A, W, W, P + of[2 * NH], P + of[2 * NH + 1], 2 * db, false, o, 2 * dbm, (TH*)nullptr, Ws);
        // u_B = (v_B - t) exp(-s); logdet -= sum s
        for (int r = threadIdx.x; r < R; r += FT) {
            float acc = 0.0f;
            for (int j = 0; j < db; ++j) {
                const float s = LG_FLOW_CLAMP * tanhf(o[r * 2 * dbm + j] / LG_FLOW_CLAMP);
                cur[r * d + b0 + j] = (cur[r * d + b0 + j] - o[r * 2 * dbm + db + j]) * expf(-s);
                acc -= s;
            }
            ld[r] += acc;
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < R * d; e += FT)
        if (base + e / d < M) Uout[(size_t)base * d + e] = cur[e];
    for (int r = threadIdx.x; r < R; r += FT)
        if (base + r < M) ldet[base + r] = ld[r];
}

// ------------------------------------------------ tensor-core inverse --
// The proposal's inverse flow on the 5th-generation tensor cores: a block
// takes 128 latent points (the MMA's M) through every coupling layer.  Each
// dense layer is one chain of tcgen05.mma (kind::f16: BF16 operands, FP32
// accumulators in tensor memory) issued by one thread: activations (A,
// 128 x K) and weights (B, N x K) in shared memory, both K-major without
// swizzle in 8 x 16-byte core matrices.  A layer's weights, packed once per
// retraining into that layout (lg_flow_pack), arrive by one bulk TMA copy
// into one of two buffers, the next layer's copy in flight while this one
// computes.  Epilogues read the accumulators back with tcgen05.ld (thread =
// row), add the bias, apply the ReLU and store BF16 activations as the next
// layer's A; the coupling (exp, tanh) runs in FP32 per row.  The map differs
// from the FP32-weight flow by the BF16 rounding of weights and of the
// conditioner's input; the log-determinant is that of the map applied, so
// the calibrated rejection step stays exact for it.

__device__ __forceinline__ uint32_t lg_saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: K-major, no swizzle; lbo = bytes between
// core matrices along K, sbo = bytes between 8-row groups.
__device__ __forceinline__ uint64_t lg_umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor: BF16 A and B (K-major), FP32 D, M x N.
__device__ __forceinline__ uint32_t lg_umma_idesc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void lg_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                     tmem),
                 "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void lg_mma_commit(void* mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(lg_saddr(mbar))
                 : "memory");
}

// Polls of an mbarrier phase before a bounded wait gives up.
constexpr long kMbarTries = 1L << 20;

// Bounded wait on an mbarrier phase (one thread): at most `tries` polls
// (none for tries <= 0); false when it ran out.
__device__ __forceinline__ bool lg_mbar_wait(void* mbar, uint32_t parity, long tries = kMbarTries)
{
    uint32_t done = 0;
    for (long it = 0; it < tries && !done; ++it)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done)
                     : "r"(lg_saddr(mbar)), "r"(parity)
                     : "memory");
    return done != 0;
}

// 16 FP32 accumulator columns of this thread's tensor-memory lane.
__device__ __forceinline__ void lg_tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Sizes of the packed weights of one coupling layer (BF16 elements): the
// input dense (W x Kp0), the hidden denses (W x W each) and the output dense
// (Np x W), every block N x K in core-matrix order; Kp0 = dbmax rounded up
// to 16, Np = 2 dbmax rounded up to 16.
struct TcDims {
    int kp0, np, s0, sh, so, sl;
    __host__ __device__ explicit TcDims(const FlowDims& f)
    {
        kp0 = (f.dbmax() + 15) / 16 * 16;
        np = (2 * f.dbmax() + 15) / 16 * 16;
        s0 = f.W * kp0;
        sh = f.W * f.W;
        so = np * f.W;
        sl = s0 + (f.NH - 1) * sh + so;
    }
};

// Element offset of (row n, column k) in an N x K block of core matrices.
__host__ __device__ __forceinline__ int lg_core_off(int n, int k, int K)
{
    return (n / 8) * (K / 8) * 64 + (k / 8) * 64 + (n % 8) * 8 + (k % 8);
}

// Pack FP32 weights P (library layout, W[k][n] per dense) into BF16 B
// operands: element (n, k) of each dense = W[k][n], zero in the padding.
__global__ void __launch_bounds__(256)
    lg_flow_pack(FlowDims f, const float* __restrict__ P, __nv_bfloat16* __restrict__ out)
{
    const TcDims t(f);
    const long total = (long)f.L * t.sl;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const int l = (int)(e / t.sl);
        int o = (int)(e - (long)l * t.sl);
        int dn, K, N, Kp;
        if (o < t.s0) {
            dn = 0, K = f.da(l), N = f.W, Kp = t.kp0;
        } else if (o < t.s0 + (f.NH - 1) * t.sh) {
            o -= t.s0;
            dn = 1 + o / t.sh;
            o -= (dn - 1) * t.sh;
            K = f.W, N = f.W, Kp = f.W;
        } else {
            o -= t.s0 + (f.NH - 1) * t.sh;
            dn = f.NH, K = f.W, N = 2 * f.db(l), Kp = f.W;
        }
        // invert lg_core_off
        const int g = o / ((Kp / 8) * 64), rem = o - g * (Kp / 8) * 64;
        const int j = rem / 64, rem2 = rem - j * 64;
        const int n = g * 8 + rem2 / 8, k = j * 8 + rem2 % 8;
        // weight offset of dense (l, dn) in the library layout
        long w = 0;
        for (int ll = 0; ll < l; ++ll)
            for (int kk = 0; kk <= f.NH; ++kk) w += (long)f.kin(ll, kk) * f.kout(ll, kk) + f.kout(ll, kk);
        for (int kk = 0; kk < dn; ++kk) w += (long)f.kin(l, kk) * f.kout(l, kk) + f.kout(l, kk);
        const float v = (k < K && n < N) ? P[w + (long)k * N + n] : 0.0f;
        out[e] = __float2bfloat16_rn(v);
    }
}

// Library index i of a weight -> its position in the packed BF16 operands
// (lg_flow_pack's layout); -1 for a bias.
__device__ long lg_packed_index(const FlowDims& f, const TcDims& t, long i)
{
    for (int l = 0; l < f.L; ++l)
        for (int k = 0; k <= f.NH; ++k) {
            const int K = f.kin(l, k), N = f.kout(l, k);
            const long nw = (long)K * N;
            if (i < nw) {
                const int kk = (int)(i / N), n = (int)(i - (long)kk * N);
                const long at = (long)l * t.sl + (k == 0 ? 0 : t.s0 + (long)(k - 1) * t.sh);
                return at + lg_core_off(n, kk, k == 0 ? t.kp0 : f.W);
            }
            i -= nw;
            if (i < N) return -1;
            i -= N;
        }
    return -1;
}

// Gradient = sum of the blocks' slices in block order; then (adam) an Adam
// step with bias corrections c1, c2 of this step, and (packed) the updated
// weight's BF16 copy in the tensor-core operands.
__global__ void __launch_bounds__(256)
    lg_flow_adam(float* __restrict__ P, const float* __restrict__ gpart, int nparts, long n, float* __restrict__ G,
                 float* __restrict__ m1, float* __restrict__ m2, int adam, float lr, float b1, float b2, float c1,
                 float c2, const int* __restrict__ stop, FlowDims f, __nv_bfloat16* __restrict__ packed)
{
    if (stop && *stop) return;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = 0.0f;
    for (int c = 0; c < nparts; ++c) g += gpart[(size_t)c * n + i];
    if (G) G[i] = g;
    if (!adam) return;
    const float a = b1 * m1[i] + (1 - b1) * g, b = b2 * m2[i] + (1 - b2) * g * g;
    m1[i] = a;
    m2[i] = b;
    const float p = P[i] - lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
    P[i] = p;
    if (packed) {
        const long q = lg_packed_index(f, TcDims(f), i);
        if (q >= 0) packed[q] = __float2bfloat16_rn(p);
    }
}

// Two floats as BF16 (round to nearest even), the first in the low half.
__device__ __forceinline__ uint32_t lg_pack_bf16(float lo, float hi)
{
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

// Shared-memory layout of lg_flow_inverse_tc (bytes): one layer's weights,
// the conditioner input and one hidden activation tile (each epilogue
// overwrites the tile its MMA chain has finished reading), so that two
// blocks fit on an SM and one block's epilogues overlap the other's MMAs
// and weight copies.
struct TcSmem {
    int wbuf, a0, a1, cur, obuf, ld, bias, bar, total;
    __host__ __device__ explicit TcSmem(const FlowDims& f)
    {
        const TcDims t(f);
        int q = 0;
        auto take = [&](int bytes) {
            const int at = q;
            q += (bytes + 127) / 128 * 128;
            return at;
        };
        wbuf = take(2 * t.sl);
        a0 = take(128 * t.kp0 * 2);
        a1 = take(128 * f.W * 2);
        cur = take(128 * f.d * 4);
        obuf = take(128 * t.np * 4);
        ld = take(128 * 4);
        bias = take((f.NH * f.W + t.np) * 4);
        bar = take(64);
        total = q;
    }
};

__global__ void __launch_bounds__(256, 2)
    lg_flow_inverse_tc(FlowDims f, const float* __restrict__ P, const __nv_bfloat16* __restrict__ packed,
                       const float* __restrict__ Z, int M, float* __restrict__ Uout, float* __restrict__ ldet,
                       int* __restrict__ err, long tries)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const TcDims td(f);
    const TcSmem L(f);
    const int t = threadIdx.x, w = t / 32, lane = t % 32;
    const int d = f.d, W = f.W, NH = f.NH;
    unsigned char* wb = smem + L.wbuf;
    __nv_bfloat16* A0 = reinterpret_cast<__nv_bfloat16*>(smem + L.a0);
    __nv_bfloat16* A1 = reinterpret_cast<__nv_bfloat16*>(smem + L.a1);
    float* cur = reinterpret_cast<float*>(smem + L.cur);
    float* ob = reinterpret_cast<float*>(smem + L.obuf);
    float* ld = reinterpret_cast<float*>(smem + L.ld);
    float* bsm = reinterpret_cast<float*>(smem + L.bias);  // the layer's biases: hidden denses, output
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L.bar);  // [0] MMA, [1] weights
    uint32_t* misc = reinterpret_cast<uint32_t*>(smem + L.bar + 32);  // [0] TMEM base, [1] abort flag
    const uint32_t lbytes = 2u * td.sl;
    // one accumulator of max(W, np) columns
    uint32_t tcols = 32;
    while (tcols < (uint32_t)max(W, td.np)) tcols <<= 1;

    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(lg_saddr(misc)),
                     "r"(tcols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (t == 0) {
        for (int i = 0; i < 2; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(lg_saddr(bars + i)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;");
        misc[1] = 0;
    }
    // latent rows
    const int base = blockIdx.x * 128;
    for (int e = t; e < 128 * d; e += 256) cur[e] = base + e / d < M ? Z[(size_t)base * d + e] : 0.0f;
    if (t < 128) ld[t] = 0.0f;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = misc[0];
    auto issue_weights = [&](int l) {
        void* bar = bars + 1;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(lg_saddr(bar)), "r"(lbytes)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         lg_saddr(wb)),
                     "l"(packed + (size_t)l * td.sl), "r"(lbytes), "r"(lg_saddr(bar))
                     : "memory");
    };
    // weight copies issued and waited for (thread 0's view; every thread
    // keeps the same counts); the inverse runs from layer L-1 down
    int issued = 1, waited = 0;
    if (t == 0) issue_weights(f.L - 1);
    uint32_t mma_phase = 0;
    bool ok = true;
    // a chain whose completion wait ran out (thread 0): drained before the
    // tensor memory is freed
    bool mma_pending = false;
    uint32_t pending_parity = 0;
    // one MMA chain: D (tmem) = A (128 x K) . B (N x K)^T
    auto gemm = [&](const void* A, const void* B, int K, int N) {
        if (t == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t sb = (uint32_t)(K / 8) * 128, idesc = lg_umma_idesc(128, N);
            for (int ks = 0; ks < K / 16; ++ks)
                lg_mma(tmem, lg_umma_desc(lg_saddr(A) + ks * 256, 128, sb),
                       lg_umma_desc(lg_saddr(B) + ks * 256, 128, sb), idesc, ks > 0);
            lg_mma_commit(bars);
            if (!lg_mbar_wait(bars, mma_phase, tries)) {
                misc[1] = 1;
                mma_pending = true;
                pending_parity = mma_phase;
            }
        }
        mma_phase ^= 1u;
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        return misc[1] == 0;
    };
    // epilogue of a hidden dense: tmem columns [0, W) + bias, ReLU, BF16
    // into A1 (128 x W core matrices; the chain that read A1 has completed);
    // warp w reads lanes of w % 4, warps 0-3 the first half of the columns,
    // 4-7 the second
    auto hidden_epilogue = [&](const float* bias) {
        const int m = 32 * (w % 4) + lane, half = w / 4;
        const uint32_t taddr = tmem + ((uint32_t)(32 * (w % 4)) << 16);
        for (int n0 = half * (W / 2); n0 < (half + 1) * (W / 2); n0 += 16) {
            float v[16];
            lg_tmem_ld16(taddr + n0, v);
            uint32_t h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float x0 = v[2 * j] + bias[n0 + 2 * j], x1 = v[2 * j + 1] + bias[n0 + 2 * j + 1];
                h[j] = lg_pack_bf16(x0 > 0.0f ? x0 : 0.0f, x1 > 0.0f ? x1 : 0.0f);
            }
            uint4* dst = reinterpret_cast<uint4*>(A1 + lg_core_off(m, n0, W));
            dst[0] = make_uint4(h[0], h[1], h[2], h[3]);
            dst[8] = make_uint4(h[4], h[5], h[6], h[7]);  // next core matrix along K: +64 elements
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
    };
    for (int l = f.L - 1; l >= 0 && ok; --l) {
        const int da = f.da(l), db = f.db(l), a0 = f.a0(l), b0 = f.b0(l);
        // parameter offsets of this layer's biases (library layout)
        long woff = 0;
        for (int ll = 0; ll < l; ++ll)
            for (int kk = 0; kk <= NH; ++kk) woff += (long)f.kin(ll, kk) * f.kout(ll, kk) + f.kout(ll, kk);
        // the layer's biases into shared memory (read by every epilogue)
        for (int e = t; e < NH * W + td.np; e += 256) {
            long o = woff;
            const int kk = e < NH * W ? e / W : NH, n = e < NH * W ? e - kk * W : e - NH * W;
            for (int j = 0; j < kk; ++j) o += (long)f.kin(l, j) * f.kout(l, j) + f.kout(l, j);
            o += (long)f.kin(l, kk) * f.kout(l, kk);
            bsm[e] = n < f.kout(l, kk) ? P[o + n] : 0.0f;
        }
        // the conditioning half as BF16 A0 (zero padding to kp0)
        for (int e = t; e < 128 * td.kp0; e += 256) {
            const int m = e / td.kp0, k = e - m * td.kp0;
            A0[lg_core_off(m, k, td.kp0)] = __float2bfloat16_rn(k < da ? cur[m * d + a0 + k] : 0.0f);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (t == 0 && !lg_mbar_wait(bars + 1, (uint32_t)waited & 1u, tries)) misc[1] = 1;
        __syncthreads();
        if (!misc[1]) ++waited;
        if (misc[1]) {
            ok = false;
            break;
        }
        // input dense
        long bo = woff + (long)f.kin(l, 0) * f.kout(l, 0);
        if (!(ok = gemm(A0, wb, td.kp0, W))) break;
        hidden_epilogue(bsm);
        long wo = bo + f.kout(l, 0);
        // hidden denses, in place in A1
        for (int k = 1; k < NH && ok; ++k) {
            ok = gemm(A1, wb + 2 * (td.s0 + (size_t)(k - 1) * td.sh), W, W);
            if (!ok) break;
            bo = wo + (long)f.kin(l, k) * f.kout(l, k);
            hidden_epilogue(bsm + k * W);
            wo = bo + f.kout(l, k);
        }
        if (!ok) break;
        // output dense
        if (!(ok = gemm(A1, wb + 2 * (td.s0 + (size_t)(NH - 1) * td.sh), W, td.np))) break;
        // this layer's weights are consumed: the next layer's copy runs
        // under the output epilogue and the coupling
        if (l - 1 >= 0) {
            if (t == 0) issue_weights(l - 1);
            ++issued;
        }
        // output accumulators -> obuf (rows 0..127), then the coupling
        if (w < 4) {
            const uint32_t taddr = tmem + ((uint32_t)(32 * w) << 16);
            const int m = 32 * w + lane;
            for (int n0 = 0; n0 < td.np; n0 += 16) {
                float v[16];
                lg_tmem_ld16(taddr + n0, v);
#pragma unroll
                for (int j = 0; j < 16; ++j) ob[m * td.np + n0 + j] = v[j];
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        if (t < 128) {
            float acc = 0.0f;
            for (int j = 0; j < db; ++j) {
                const float sr = ob[t * td.np + j] + bsm[NH * W + j];
                const float tt = ob[t * td.np + db + j] + bsm[NH * W + db + j];
                const float s = LG_FLOW_CLAMP * tanhf(sr / LG_FLOW_CLAMP);
                cur[t * d + b0 + j] = (cur[t * d + b0 + j] - tt) * expf(-s);
                acc -= s;
            }
            ld[t] += acc;
        }
        __syncthreads();
    }
    if (ok) {
        for (int e = t; e < 128 * d; e += 256)
            if (base + e / d < M) Uout[(size_t)base * d + e] = cur[e];
        if (t < 128 && base + t < M) ldet[base + t] = ld[t];
    } else if (t == 0) {
        atomicExch(err, 1);
        // what is still in flight completes before the tensor memory is
        // freed and the block exits: the MMA chain whose wait gave up, and
        // the weight copies issued (waits with the full budget)
        if (mma_pending) lg_mbar_wait(bars, pending_parity);
        for (; waited < issued; ++waited) lg_mbar_wait(bars + 1, (uint32_t)waited & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols));
}

// ------------------------------------------------- tensor-core training --
// A training step (or a forward pass) of the flow on the tensor cores, for
// the conditioner shape the proposal uses (width 128, two hidden layers): a
// block takes 128 minibatch rows (the MMA's M) forward through every
// coupling layer and back.  The forward denses are the inverse's (BF16
// weights and conditioner input, BF16 hidden activations, FP32 accumulators
// in tensor memory), so training and proposals run the same network.  The
// backward products read the same shared-memory tiles transposed: a K-major
// tile of X (rows r, columns k) is, described MN-major, the tile of X^T, so
//   dW_out = H1^T dO,   dH1 = dO W_out      (dO: 128 x 16, BF16)
//   dW1    = H0^T dY1,  dH0 = dY1 W1        (dY1 = dH1 [H1 > 0], in place of H1)
//   dW0^T  = dY0^T A0,  dA0 = dY0 W0        (dY0 = dH0 [H0 > 0], in place of H0)
// each a chain of tcgen05.mma with both operands in shared memory and no
// transposed copies (the packed weights serve the forward products as
// K-major and the backward ones as MN-major operands).  Weight gradients go
// from tensor memory into the block's slice of the partial-gradient buffer
// (summed in block order by lg_flow_adam, which also refreshes the packed
// BF16 weights); bias gradients are column sums in a fixed order.  A
// layer's hidden activations are recomputed in the backward pass (all
// layers' would need 512 KB); the layer inputs u_l stay in shared memory
// (FP32).  Every mbarrier wait is bounded as in the inverse; a wait that
// runs out sets *err and the early-stop flag, lets the block's copies and
// MMA chains in flight complete, frees the tensor memory and returns.

// Shared-memory layout of lg_flow_step_tc (bytes).
struct TcStepSmem {
    int wbuf, a0, h0, h1, dob, us, ob, dv, du, ld, cs, bias, stg, bar, total;
    __host__ __device__ explicit TcStepSmem(const FlowDims& f)
    {
        const TcDims t(f);
        int q = 0;
        auto take = [&](int bytes) {
            const int at = q;
            q += (bytes + 127) / 128 * 128;
            return at;
        };
        wbuf = take(2 * t.sl);
        a0 = take(128 * t.kp0 * 2);
        h0 = take(128 * f.W * 2);
        h1 = take(128 * f.W * 2);
        dob = take(128 * t.np * 2);
        us = take((f.L + 1) * 128 * f.d * 4);
        ob = take(128 * t.np * 4);
        dv = take(128 * f.d * 4);
        du = take(128 * f.d * 4);
        ld = take(128 * 4);
        cs = take(2 * f.W * 4);
        bias = take((2 * f.W + t.np) * 4);
        stg = take(128 * 16 * 4);
        bar = take(64);
        total = q;
    }
};

// Instruction descriptor with operand majors: amaj / bmaj = 1 for an
// MN-major (transposed) A / B.
__device__ __forceinline__ uint32_t lg_umma_idesc_t(int M, int N, int amaj, int bmaj)
{
    return lg_umma_idesc(M, N) | ((uint32_t)amaj << 15) | ((uint32_t)bmaj << 16);
}

__global__ void __launch_bounds__(256, 1)
    lg_flow_step_tc(FlowDims f, const float* __restrict__ P, const __nv_bfloat16* __restrict__ packed,
                    const float* __restrict__ X, const int* __restrict__ idx, int row0, int M, int grad,
                    float* __restrict__ loss, float* __restrict__ znorm2, float* __restrict__ gpart, long nparams,
                    int* __restrict__ stop, int* __restrict__ err, long tries)
{
    // (read once per block: another block of this launch may set it)
    __shared__ int stopped;
    if (threadIdx.x == 0) stopped = stop ? *(volatile int*)stop : 0;
    __syncthreads();
    if (stopped) return;
    extern __shared__ __align__(1024) unsigned char smem[];
    const TcDims td(f);
    const TcStepSmem L(f);
    const int t = threadIdx.x, w = t / 32, lane = t % 32;
    const int d = f.d, W = f.W, kp0 = td.kp0, np = td.np;
    unsigned char* wb = smem + L.wbuf;
    __nv_bfloat16* A0 = reinterpret_cast<__nv_bfloat16*>(smem + L.a0);
    __nv_bfloat16* H0 = reinterpret_cast<__nv_bfloat16*>(smem + L.h0);
    __nv_bfloat16* H1 = reinterpret_cast<__nv_bfloat16*>(smem + L.h1);
    __nv_bfloat16* DO = reinterpret_cast<__nv_bfloat16*>(smem + L.dob);
    float* Us = reinterpret_cast<float*>(smem + L.us);
    float* ob = reinterpret_cast<float*>(smem + L.ob);
    float* dv = reinterpret_cast<float*>(smem + L.dv);
    float* du = reinterpret_cast<float*>(smem + L.du);
    float* ld = reinterpret_cast<float*>(smem + L.ld);
    float* cs = reinterpret_cast<float*>(smem + L.cs);
    float* bs = reinterpret_cast<float*>(smem + L.bias);  // the layer's biases: dense 0, dense 1, output
    float* stg = reinterpret_cast<float*>(smem + L.stg);  // 128 x 16 weight-gradient columns on their way out
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L.bar);       // [0] MMA, [1] weights
    uint32_t* misc = reinterpret_cast<uint32_t*>(smem + L.bar + 32);  // [0] TMEM base, [1] abort flag
    const uint32_t lbytes = 2u * td.sl;
    // tensor-memory columns: the row-indexed accumulator (forward denses,
    // dH1, dH0), dW1, the output dense, dW_out, dW0^T, dA0
    constexpr uint32_t kCols = 512, cD = 0, cW1 = 128, cO = 256, cWo = 272, cW0 = 288, cX0 = 304;
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(lg_saddr(misc)),
                     "r"(kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (t == 0) {
        for (int i = 0; i < 2; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(lg_saddr(bars + i)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;");
        misc[1] = 0;
    }
    // rows beyond M are zero inputs; their loss and gradient are dropped
    const int base = blockIdx.x * 128;
    for (int e = t; e < 128 * d; e += 256) {
        const int r = e / d, j = e - r * d, m = base + r;
        Us[e] = m < M ? X[(size_t)(idx ? idx[row0 + m] : row0 + m) * d + j] : 0.0f;
    }
    if (t < 128) ld[t] = 0.0f;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = misc[0];
    const uint32_t sA0 = lg_saddr(A0), sH0 = lg_saddr(H0), sH1 = lg_saddr(H1), sDO = lg_saddr(DO);
    const uint32_t sW0 = lg_saddr(wb), sW1 = sW0 + 2u * td.s0, sWo = sW1 + 2u * td.sh;

    int issued = 0, waited = 0;
    auto issue_weights = [&](int l) {
        if (t == 0) {
            void* bar = bars + 1;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(lg_saddr(bar)), "r"(lbytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    lg_saddr(wb)),
                "l"(packed + (size_t)l * td.sl), "r"(lbytes), "r"(lg_saddr(bar))
                : "memory");
        }
        ++issued;
    };
    // wait for the last weight copy issued (every thread)
    auto wait_weights = [&]() {
        if (t == 0 && !lg_mbar_wait(bars + 1, (uint32_t)waited & 1u, tries)) misc[1] = 1;
        __syncthreads();
        if (misc[1]) return false;
        ++waited;
        return true;
    };
    uint32_t mma_phase = 0;
    bool mma_pending = false;
    uint32_t pending_parity = 0;
    // one MMA chain D[col] (+)= A . B^T over `steps` K-steps of 16, from
    // start addresses, leading / stride byte offsets and per-step advances
    auto chain = [&](uint32_t col, uint32_t a, uint32_t alb, uint32_t asb, uint32_t ast, uint32_t b, uint32_t blb,
                     uint32_t bsb, uint32_t bst, int steps, uint32_t id) {
        if (t == 0)
            for (int ks = 0; ks < steps; ++ks)
                lg_mma(tmem + col, lg_umma_desc(a + ks * ast, alb, asb), lg_umma_desc(b + ks * bst, blb, bsb), id,
                       ks > 0);
    };
    // descriptors of a tile with C columns stored K-major (rows r): as a
    // K-major operand (reduction over its columns) ...
    auto KM = [](int C, uint32_t& lbo, uint32_t& sbo, uint32_t& st) {
        lbo = 128;
        sbo = (uint32_t)C * 16;
        st = 256;
    };
    // ... and as an MN-major operand (reduction over its rows): the K
    // direction's core-matrix stride in the leading byte offset, the MN
    // direction's in the stride byte offset
    auto MN = [](int C, uint32_t& lbo, uint32_t& sbo, uint32_t& st) {
        lbo = (uint32_t)C * 16;
        sbo = 128;
        st = (uint32_t)C * 32;
    };
    auto begin_mma = [&]() {
        if (t == 0) asm volatile("tcgen05.fence::after_thread_sync;");
    };
    auto commit_wait = [&]() {
        if (t == 0) {
            lg_mma_commit(bars);
            if (!lg_mbar_wait(bars, mma_phase, tries)) {
                misc[1] = 1;
                mma_pending = true;
                pending_parity = mma_phase;
            }
        }
        mma_phase ^= 1u;
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        return misc[1] == 0;
    };
    auto publish = [&]() {  // shared-memory tiles written by threads -> visible to the MMAs
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
    };
    // tensor-memory lane group and column half of this warp
    const int m = 32 * (w % 4) + lane, half = w / 4;
    const uint32_t tlane = tmem + ((uint32_t)(32 * (w % 4)) << 16);
    // hidden epilogue: columns [0, W) + bias, ReLU, BF16 into dst
    auto hidden_epilogue = [&](const float* bias, __nv_bfloat16* dst) {
        for (int n0 = half * (W / 2); n0 < (half + 1) * (W / 2); n0 += 16) {
            float v[16];
            lg_tmem_ld16(tlane + cD + n0, v);
            uint32_t h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float x0 = v[2 * j] + bias[n0 + 2 * j], x1 = v[2 * j + 1] + bias[n0 + 2 * j + 1];
                h[j] = lg_pack_bf16(x0 > 0.0f ? x0 : 0.0f, x1 > 0.0f ? x1 : 0.0f);
            }
            uint4* q = reinterpret_cast<uint4*>(dst + lg_core_off(m, n0, W));
            q[0] = make_uint4(h[0], h[1], h[2], h[3]);
            q[8] = make_uint4(h[4], h[5], h[6], h[7]);
        }
        publish();
    };
    // backward epilogue: dst (holding the activations H) <- D [H > 0], BF16
    auto mask_epilogue = [&](__nv_bfloat16* dst) {
        for (int n0 = half * (W / 2); n0 < (half + 1) * (W / 2); n0 += 16) {
            float v[16];
            lg_tmem_ld16(tlane + cD + n0, v);
            uint4* q = reinterpret_cast<uint4*>(dst + lg_core_off(m, n0, W));
            const uint4 a = q[0], b = q[8];
            const uint32_t hin[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
            uint32_t h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)  // a BF16 activation is > 0 iff its sign bit is clear and it is not zero
                h[j] = lg_pack_bf16((hin[j] & 0x8000u) == 0 && (hin[j] & 0x7FFFu) != 0 ? v[2 * j] : 0.0f,
                                    (hin[j] >> 31) == 0 && (hin[j] & 0x7FFF0000u) != 0 ? v[2 * j + 1] : 0.0f);
            q[0] = make_uint4(h[0], h[1], h[2], h[3]);
            q[8] = make_uint4(h[4], h[5], h[6], h[7]);
        }
        publish();
    };
    // out[n] = sum over the 128 rows of the BF16 tile T (W columns), fixed order
    auto colsum = [&](const __nv_bfloat16* T, float* __restrict__ out) {
        const int n = t % 128, hh = t / 128;
        float s = 0.0f;
        for (int r = hh * 64; r < hh * 64 + 64; ++r) s += __bfloat162float(T[lg_core_off(r, n, W)]);
        cs[hh * 128 + n] = s;
        __syncthreads();
        if (t < 128) out[t] = cs[t] + cs[128 + t];
        __syncthreads();
    };
    // parameter offsets of layer l (library layout)
    auto layer_offset = [&](int l) {
        long o = 0;
        for (int ll = 0; ll < l; ++ll)
            for (int kk = 0; kk <= f.NH; ++kk) o += (long)f.kin(ll, kk) * f.kout(ll, kk) + f.kout(ll, kk);
        return o;
    };
    // forward of layer l up to the conditioner output o = D_out + b_out in
    // ob (FP32, 128 x np, zero past 2 db); the layer's weights resident
    auto conditioner = [&](int l, long woff, bool next_weights) {
        const int da = f.da(l), db = f.db(l), a0 = f.a0(l);
        const float* u = Us + (size_t)l * 128 * d;
        for (int e = t; e < 128 * kp0; e += 256) {
            const int r = e / kp0, k = e - r * kp0;
            A0[lg_core_off(r, k, kp0)] = __float2bfloat16_rn(k < da ? u[r * d + a0 + k] : 0.0f);
        }
        publish();
        uint32_t al, as, at;
        const long ob0 = woff + (long)da * W, ob1 = ob0 + W + (long)W * W,
                   obo = ob1 + W + (long)W * 2 * db;
        for (int e = t; e < 2 * W + np; e += 256)
            bs[e] = e < W ? P[ob0 + e] : (e < 2 * W ? P[ob1 + e - W] : (e - 2 * W < 2 * db ? P[obo + e - 2 * W] : 0.0f));
        begin_mma();
        KM(kp0, al, as, at);
        chain(cD, sA0, al, as, at, sW0, al, as, at, kp0 / 16, lg_umma_idesc(128, W));
        if (!commit_wait()) return false;
        hidden_epilogue(bs, H0);
        begin_mma();
        KM(W, al, as, at);
        chain(cD, sH0, al, as, at, sW1, al, as, at, W / 16, lg_umma_idesc(128, W));
        if (!commit_wait()) return false;
        hidden_epilogue(bs + W, H1);
        begin_mma();
        chain(cO, sH1, al, as, at, sWo, al, as, at, W / 16, lg_umma_idesc(128, np));
        if (!commit_wait()) return false;
        if (next_weights) issue_weights(l + 1);  // the buffer is free: the next layer's copy runs under the coupling
        if (w < 4) {
            for (int n0 = 0; n0 < np; n0 += 16) {
                float v[16];
                lg_tmem_ld16(tlane + cO + n0, v);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int n = n0 + j;
                    ob[m * np + n] = v[j] + bs[2 * W + n];
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        return true;
    };

    bool ok = true;
    issue_weights(0);
    // ---- forward
    for (int l = 0; l < f.L && ok; ++l) {
        if (!(ok = wait_weights())) break;
        if (!(ok = conditioner(l, layer_offset(l), l + 1 < f.L))) break;
        const int db = f.db(l), b0 = f.b0(l);
        const float* u = Us + (size_t)l * 128 * d;
        float* v = Us + (size_t)(l + 1) * 128 * d;
        if (t < 128) {
            for (int j = 0; j < d; ++j) v[t * d + j] = u[t * d + j];
            float acc = 0.0f;
            for (int j = 0; j < db; ++j) {
                const float s = LG_FLOW_CLAMP * tanhf(ob[t * np + j] / LG_FLOW_CLAMP);
                v[t * d + b0 + j] = u[t * d + b0 + j] * expf(s) + ob[t * np + db + j];
                acc += s;
            }
            ld[t] += acc;
        }
        __syncthreads();
    }
    // ---- loss: 0.5 |z|^2 - logdet per row
    const float* z = Us + (size_t)f.L * 128 * d;
    if (ok && t < 128) {
        float q = 0.0f;
        for (int j = 0; j < d; ++j) q += z[t * d + j] * z[t * d + j];
        if (base + t < M) {
            loss[base + t] = 0.5f * q - ld[t];
            if (znorm2) znorm2[base + t] = q;
        }
    }
    if (ok && grad) {
        // ---- backward: dz = z / M, dlogdet = -1 / M (mean loss)
        for (int e = t; e < 128 * d; e += 256) dv[e] = (base + e / d < M) ? z[e] / M : 0.0f;
        __syncthreads();
        float* gp = gpart + (size_t)blockIdx.x * nparams;
        for (int l = f.L - 1; l >= 0 && ok; --l) {
            const int da = f.da(l), db = f.db(l), a0 = f.a0(l), b0 = f.b0(l);
            const long woff = layer_offset(l), ob0 = woff + (long)da * W, ow1 = ob0 + W, ob1 = ow1 + (long)W * W,
                       owo = ob1 + W, obo = owo + (long)W * 2 * db;
            // the layer's conditioner again (the last layer's is still there)
            if (l < f.L - 1) {
                if (!(ok = wait_weights())) break;
                if (!(ok = conditioner(l, woff, false))) break;
            }
            // coupling backward: dO = (ds (1 - th^2), g) into ob (FP32) and DO
            // (BF16), du = dv with du_B = g e^s
            const float* u = Us + (size_t)l * 128 * d;
            if (t < 128) {
                for (int j = 0; j < d; ++j) du[t * d + j] = dv[t * d + j];
                const float dlog = base + t < M ? -1.0f / M : 0.0f;
                for (int j = 0; j < db; ++j) {
                    const float th = tanhf(ob[t * np + j] / LG_FLOW_CLAMP);
                    const float es = expf(LG_FLOW_CLAMP * th);
                    const float g = dv[t * d + b0 + j];
                    const float ds = g * u[t * d + b0 + j] * es + dlog;
                    ob[t * np + j] = ds * (1.0f - th * th);
                    ob[t * np + db + j] = g;
                    du[t * d + b0 + j] = g * es;
                }
                for (int n = 0; n < np; ++n) DO[lg_core_off(t, n, np)] = __float2bfloat16_rn(ob[t * np + n]);
            }
            publish();
            uint32_t al, as, at, bl, bs, bt;
            // dW_out = H1^T dO (lanes k, 16 columns n); dH1 = dO W_out (lanes r)
            begin_mma();
            MN(W, al, as, at);
            MN(np, bl, bs, bt);
            chain(cWo, sH1, al, as, at, sDO, bl, bs, bt, 128 / 16, lg_umma_idesc_t(128, np, 1, 1));
            KM(np, al, as, at);
            MN(W, bl, bs, bt);
            chain(cD, sDO, al, as, at, sWo, bl, bs, bt, np / 16, lg_umma_idesc_t(128, W, 0, 1));
            // output bias gradient (FP32 dO, rows in order) under the MMAs
            if (t < 2 * db) {
                float s = 0.0f;
                for (int r = 0; r < 128; ++r) s += ob[r * np + t];
                gp[obo + t] = s;
            }
            if (!(ok = commit_wait())) break;
            if (w < 4) {
                float v[16];
                lg_tmem_ld16(tlane + cWo, v);
#pragma unroll
                for (int n = 0; n < 16; ++n)
                    if (n < 2 * db) gp[owo + (long)m * 2 * db + n] = v[n];
            }
            mask_epilogue(H1);  // dY1 in place of H1
            // dW1 = H0^T dY1 (lanes k, columns n); dH0 = dY1 W1 (lanes r)
            begin_mma();
            MN(W, al, as, at);
            chain(cW1, sH0, al, as, at, sH1, al, as, at, 128 / 16, lg_umma_idesc_t(128, W, 1, 1));
            KM(W, al, as, at);
            MN(W, bl, bs, bt);
            chain(cD, sH1, al, as, at, sW1, bl, bs, bt, W / 16, lg_umma_idesc_t(128, W, 0, 1));
            colsum(H1, gp + ob1);  // dense 1 bias gradient, under the MMAs
            if (!(ok = commit_wait())) break;
            // 16 columns at a time through shared memory, so that
            // consecutive threads write consecutive gradient entries
            for (int n0 = 0; n0 < W; n0 += 16) {
                if (w < 4) {
                    float v[16];
                    lg_tmem_ld16(tlane + cW1 + n0, v);
                    float4* q = reinterpret_cast<float4*>(stg + m * 16);
#pragma unroll
                    for (int j = 0; j < 4; ++j) q[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int e = t + 256 * i, k = e / 16, j = e % 16;
                    gp[ow1 + (long)k * W + n0 + j] = stg[e];
                }
                __syncthreads();
            }
            mask_epilogue(H0);  // dY0 in place of H0
            // dW0^T = dY0^T A0 (lanes n, columns k); dA0 = dY0 W0 (lanes r)
            begin_mma();
            MN(W, al, as, at);
            MN(kp0, bl, bs, bt);
            chain(cW0, sH0, al, as, at, sA0, bl, bs, bt, 128 / 16, lg_umma_idesc_t(128, kp0, 1, 1));
            KM(W, al, as, at);
            MN(kp0, bl, bs, bt);
            chain(cX0, sH0, al, as, at, sW0, bl, bs, bt, W / 16, lg_umma_idesc_t(128, kp0, 0, 1));
            colsum(H0, gp + ob0);  // dense 0 bias gradient, under the MMAs
            if (!(ok = commit_wait())) break;
            if (l > 0) issue_weights(l - 1);  // the buffer is free
            {
                float v[16];
                if (w < 4) {
                    lg_tmem_ld16(tlane + cW0, v);  // lanes n: dW0[k][n]
#pragma unroll
                    for (int k = 0; k < 16; ++k)
                        if (k < da) gp[woff + (long)k * W + m] = v[k];
                } else {
                    lg_tmem_ld16(tlane + cX0, v);  // lanes r: dA0[r][k]
#pragma unroll
                    for (int k = 0; k < 16; ++k)
                        if (k < da) du[m * d + a0 + k] += v[k];
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncthreads();
            for (int e = t; e < 128 * d; e += 256) dv[e] = du[e];
            __syncthreads();
        }
    }
    if (!ok && t == 0) {
        atomicExch(err, 1);
        if (stop) atomicExch(stop, 1);
        // what is still in flight completes before the tensor memory is
        // freed and the block exits (waits with the full budget)
        if (mma_pending) lg_mbar_wait(bars, pending_parity);
        for (; waited < issued; ++waited) lg_mbar_wait(bars + 1, (uint32_t)waited & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
}

// Counter-based uniforms in (0, 1): splitmix64 finaliser of (key, counter),
// the top 23 bits as an odd multiple of 2^-24 (exact in FP32).  The
// proposal kernels stay in FP32: GB300 runs FP64 at a small fraction of
// the FP32 rate.
__device__ __forceinline__ float lg_u01(unsigned long long key, unsigned long long ctr)
{
    unsigned long long z = key + 0x9E3779B97F4A7C15ull * (ctr + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((((unsigned)(z >> 41)) << 1) | 1u) * 0x1p-24f;
}

// M points uniform in the d-ball of radius rad = scale sqrt(rad2[0]): normal
// direction (Box-Muller pairs, regenerated from the counter for the second
// pass instead of being held) scaled by rad u^(1/d).
__device__ __forceinline__ float2 lg_normal_pair(unsigned long long key, unsigned long long c)
{
    const float u1 = lg_u01(key, c), u2 = lg_u01(key, c + 1);
    const float r = sqrtf(-2.0f * logf(u1));
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    return make_float2(r * cs, r * sn);
}

__global__ void __launch_bounds__(256)
    lg_flow_latent(unsigned long long key, int M, int d, const double* __restrict__ rad2, float rscale,
                   float* __restrict__ Z)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    const float rad = rscale * sqrtf((float)rad2[0]);
    const unsigned long long c0 = (unsigned long long)i * (MAX_D + 2);
    float n2 = 0.0f;
    for (int a = 0; a < d; a += 2) {
        const float2 v = lg_normal_pair(key, c0 + a);
        n2 += v.x * v.x + (a + 1 < d ? v.y * v.y : 0.0f);
    }
    const float scale = rad * exp2f(log2f(lg_u01(key, c0 + MAX_D)) / d) * rsqrtf(n2);
    for (int a = 0; a < d; a += 2) {
        const float2 v = lg_normal_pair(key, c0 + a);
        Z[(size_t)i * d + a] = v.x * scale;
        if (a + 1 < d) Z[(size_t)i * d + a + 1] = v.y * scale;
    }
}

// FP32 maximum of a block's share of v (finite values only), by warp
// shuffles and one warp; -inf when there are none.
__device__ __forceinline__ float lg_block_max(const float* __restrict__ v, int lo, int hi, int step)
{
    __shared__ float red[32];
    float m = -INFINITY;
    for (int i = lo; i < hi; i += step)
        if (isfinite(v[i])) m = fmaxf(m, v[i]);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = -INFINITY;
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    return m;  // valid in thread 0
}

// Maximum of the finite log weights and of a floor (the calibrated bound),
// in one block: out[0].
__global__ void __launch_bounds__(1024) lg_flow_max(const float* __restrict__ v, int n, double floor_,
                                                     double* __restrict__ out)
{
    const float m = lg_block_max(v, threadIdx.x, n, blockDim.x);
    if (threadIdx.x == 0) out[0] = fmax(floor_, (double)m);
}

// The same over many blocks: part[b] = block b's maximum of its contiguous
// share, then lg_flow_max over the parts (the maximum does not depend on
// the grouping).
__global__ void __launch_bounds__(256) lg_flow_max_part(const float* __restrict__ v, int n, int per,
                                                         float* __restrict__ part)
{
    const int lo = blockIdx.x * per, hi = min(n, lo + per);
    const float m = lg_block_max(v, lo + threadIdx.x, hi, blockDim.x);
    if (threadIdx.x == 0) part[blockIdx.x] = m;
}

// Calibration sums: out[1] = sum exp(v - out[0]) over finite v (one block:
// FP32 terms summed per thread in a fixed order, then an FP64 tree).
__global__ void __launch_bounds__(1024) lg_flow_expsum(const float* __restrict__ v, int n, double* __restrict__ out)
{
    __shared__ double red[1024];
    const float m = (float)out[0];
    float s = 0.0f;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (isfinite(v[i])) s += expf(v[i] - m);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[1] = red[0];
}

// Rejection and cube tests of M proposals: keep draw i with probability
// exp(ldet_i - lmax) (lmax = bound[0]), then x = mean + sdev u, wrapped into
// [0, 1) on periodic dimensions, must lie in the unit cube (FP32; the row
// stores it in FP64 with |z|^2 last).  flag[i] = 2 kept and inside, 1 kept
// outside, 0 rejected; bcnt[2 b], bcnt[2 b + 1] = block b's counts of
// flag 2 and of flag > 0 (blocks of 256).
__global__ void __launch_bounds__(256)
    lg_flow_accept(unsigned long long key, int M, int d, const float* __restrict__ Z, const float* __restrict__ U,
                   const float* __restrict__ ldet, const double* __restrict__ bound, const float* __restrict__ mean,
                   const float* __restrict__ sdev, const int* __restrict__ wrap, double* __restrict__ X,
                   int* __restrict__ flag, int* __restrict__ bcnt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int f = 0;
    if (i < M) {
        const float l = ldet[i];
        if (isfinite(l) && !(lg_u01(key, (unsigned long long)i) > expf(l - (float)bound[0]))) {
            f = 2;
            float z2 = 0.0f;
            for (int a = 0; a < d; ++a) {
                float x = fmaf(sdev[a], U[(size_t)i * d + a], mean[a]);
                if (wrap[a]) x -= floorf(x);  // periodic dimension
                X[(size_t)i * (d + 1) + a] = x;
                if (!(x >= 0.0f && x <= 1.0f)) f = 1;
                const float zz = Z[(size_t)i * d + a];
                z2 = fmaf(zz, zz, z2);
            }
            X[(size_t)i * (d + 1) + d] = z2;  // latent radius^2, for later radius updates
        }
        flag[i] = f;
    }
    const int n2 = __syncthreads_count(f == 2), nk = __syncthreads_count(f > 0);
    if (threadIdx.x == 0) {
        bcnt[2 * blockIdx.x] = n2;
        bcnt[2 * blockIdx.x + 1] = nk;
    }
}

// Exclusive offsets of the blocks' kept-and-inside counts (one block, in
// block order): boff[b]; cnt[0] = min(total, room), cnt[1] = draws that
// passed the weight test.
__global__ void __launch_bounds__(1024)
    lg_flow_scan(const int* __restrict__ bcnt, int nb, int room, int* __restrict__ boff, int* __restrict__ cnt)
{
    __shared__ int part[1024], kept[1024];
    const int T = blockDim.x, t = threadIdx.x;
    const int per = (nb + T - 1) / T, lo = t * per, hi = min(nb, lo + per);
    int c = 0, k = 0;
    for (int b = lo; b < hi; ++b) {
        c += bcnt[2 * b];
        k += bcnt[2 * b + 1];
    }
    part[t] = c;
    kept[t] = k;
    __syncthreads();
    if (t == 0) {
        int s = 0, ks = 0;
        for (int j = 0; j < T; ++j) {
            const int v = part[j];
            part[j] = s;
            s += v;
            ks += kept[j];
        }
        cnt[0] = min(s, room);
        cnt[1] = ks;
    }
    __syncthreads();
    int pos = part[t];
    for (int b = lo; b < hi; ++b) {
        boff[b] = pos;
        pos += bcnt[2 * b];
    }
}

// Scatter of the kept-and-inside rows (w values each) to out in draw
// order: one block per accept block, ranks within the block by warp
// ballots; rows past `room` are dropped.
__global__ void __launch_bounds__(256)
    lg_flow_scatter(const int* __restrict__ flag, int M, const double* __restrict__ X, int w, int room,
                    const int* __restrict__ boff, double* __restrict__ out)
{
    __shared__ int wsum[8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const bool keep = i < M && flag[i] == 2;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wsum[wp] = __popc(bal);
    __syncthreads();
    int base = boff[blockIdx.x];
    for (int j = 0; j < wp; ++j) base += wsum[j];
    const int pos = base + __popc(bal & ((1u << lane) - 1u));
    if (keep && pos < room)
        for (int a = 0; a < w; ++a) out[(size_t)pos * w + a] = X[(size_t)i * w + a];
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
        if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return false;
        n = count;
        return true;
    }
};

template <typename T>
struct HostBuf {
    T* p = nullptr;
    size_t n = 0;
    ~HostBuf() { cudaFreeHost(p); }
    bool ensure(size_t count)
    {
        if (count <= n) return true;
        cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (cudaMallocHost((void**)&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return false;
        n = count;
        return true;
    }
};

}  // namespace

// The flow: parameters, optimiser state and work buffers on one device.
class Flow {
public:
    FlowDims f{};
    bool bf16 = true;
    bool tc = false;  // proposals' inverse on the tensor cores (BF16 activations, width % 32 == 0)
    // training steps on the tensor cores (lg_flow_step_tc): asked for by the
    // owner before init, on when the shape allows it
    bool want_tct = false, tct = false;
    size_t nparams = 0;
    DevBuf<float> P, G, M1, M2, gpart, loss, znorm;
    DevBuf<__nv_bfloat16> tpack;  // packed BF16 copy of P for lg_flow_step_tc (refreshed by the Adam steps)
    DevBuf<int> terr;             // set when a bounded wait of lg_flow_step_tc ran out
    std::vector<float> mean, sdev;
    long step = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    ~Flow()
    {
        if (stream) cudaStreamDestroy(stream);
    }

    static size_t count_params(const FlowDims& f)
    {
        size_t n = 0;
        for (int l = 0; l < f.L; ++l)
            for (int k = 0; k <= f.NH; ++k) n += (size_t)f.kin(l, k) * f.kout(l, k) + f.kout(l, k);
        return n;
    }

    // rows per block and shared memory of the FP32-weight step kernel (also
    // the forward passes that track the live points between trainings)
    int simt_rows() const { return bf16 ? FR : FR32; }
    int step_smem() const { return StepSmem(f, simt_rows(), bf16 ? 2 : 4).total; }
    int rows() const { return tct ? 128 : simt_rows(); }  // minibatch rows per training block
    int inverse_smem() const { return InvSmem(f, FRI, bf16 ? 2 : 4).total; }

    bool init(int dim, int layers, int width, int hidden, uint64_t seed)
    {
        f.d = dim;
        f.h = dim / 2;
        f.L = layers;
        f.W = width;
        f.NH = hidden;
        if (dim < 2 || dim > MAX_D || width < 1 || width > MAX_W || hidden < 1 || layers < 1 ||
            layers * (hidden + 1) > MAX_DENSE) {
            err = "flow: dimension 2-64, width 1-128, at least one layer and hidden layer, layers x (hidden + 1) <= 64";
            return false;
        }
        int optin = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (step_smem() > optin || inverse_smem() > optin) {
            err = "flow: layers x hidden x width too large for the training block's shared memory";
            return false;
        }
        int cc = 0;
        cudaDeviceGetAttribute(&cc, cudaDevAttrComputeCapabilityMajor, dev);
        tc = bf16 && cc >= 10 && width % 32 == 0 && width <= 256 && TcDims(f).np <= width &&
             TcSmem(f).total <= optin && !std::getenv("LG_FLOW_NO_TC");
        if (tc) cudaFuncSetAttribute(lg_flow_inverse_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TcSmem(f).total);
        // tensor-core training: width 128, two hidden layers, at most 8
        // transformed dimensions (one 16-wide K block for the input dense,
        // one 16-wide N block for the output dense)
        // (plus 1 KB of static shared memory: the block's stop flag, aligned)
        tct = want_tct && tc && width == 128 && hidden == 2 && TcDims(f).kp0 == 16 && TcDims(f).np == 16 &&
              TcStepSmem(f).total + 1024 <= optin;
        if (tct)
            cudaFuncSetAttribute(lg_flow_step_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TcStepSmem(f).total);
        // the highest stream priority: training launches are small and
        // run beside the likelihood's large grids, whose blocks they then
        // pass in the queue as SMs free up
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (!stream && cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, hi) != cudaSuccess) return false;
        const int sm_step = step_smem(), sm_inv = inverse_smem();
        if (bf16) {
            cudaFuncSetAttribute(lg_flow_step<FR, __nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_step);
            cudaFuncSetAttribute(lg_flow_inverse<FRI, __nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 sm_inv);
        } else {
            cudaFuncSetAttribute(lg_flow_step<FR32, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_step);
            cudaFuncSetAttribute(lg_flow_inverse<FRI, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_inv);
        }
        nparams = count_params(f);
        if (!P.ensure(nparams) || !G.ensure(nparams) || !M1.ensure(nparams) || !M2.ensure(nparams)) return false;
        // He-uniform hidden weights, zero output layer and biases: the flow
        // starts as the identity map
        std::vector<float> host(nparams, 0.0f);
        uint64_t s = seed * 6364136223846793005ull + 1442695040888963407ull;
        auto unif = [&]() {
            s = s * 6364136223846793005ull + 1442695040888963407ull;
            return ((s >> 11) * (1.0 / 9007199254740992.0)) * 2 - 1;
        };
        size_t o = 0;
        for (int l = 0; l < f.L; ++l)
            for (int k = 0; k <= f.NH; ++k) {
                const size_t nw = (size_t)f.kin(l, k) * f.kout(l, k);
                if (k < f.NH) {
                    const double lim = std::sqrt(6.0 / f.kin(l, k));
                    for (size_t i = 0; i < nw; ++i) host[o + i] = (float)(lim * unif());
                }
                o += nw + f.kout(l, k);
            }
        cudaMemcpy(P.p, host.data(), nparams * 4, cudaMemcpyHostToDevice);
        if (tct) {
            if (!tpack.ensure(packed_size()) || !terr.ensure(1)) return false;
            cudaMemset(terr.p, 0, sizeof(int));
            if (!repack(stream)) return false;
        }
        cudaMemset(M1.p, 0, nparams * 4);
        cudaMemset(M2.p, 0, nparams * 4);
        step = 0;
        return cudaGetLastError() == cudaSuccess;
    }

    // Work buffers for passes over up to n rows and gradient passes over up
    // to mb rows (reserved before a retraining is enqueued, so that no
    // buffer is reallocated under enqueued kernels).
    bool reserve(int n, int mb)
    {
        return loss.ensure(n) && znorm.ensure(n) && gpart.ensure((size_t)((mb + rows() - 1) / rows()) * nparams);
    }

    // Enqueue one forward (+ backward) pass over rows [row0, row0 + M) of
    // the index list (or of X when idx is NULL): per-row losses in loss,
    // |z|^2 in znorm (when asked), partial gradients in gpart.
    bool pass(const float* X, const int* idx, int row0, int M, bool grad, bool want_z, int* stop)
    {
        const int blocks = (M + rows() - 1) / rows();
        if (!loss.ensure(M) || (want_z && !znorm.ensure(M)) || (grad && !gpart.ensure((size_t)blocks * nparams)))
            return false;
        if (tct) {
            lg_flow_step_tc<<<blocks, 256, TcStepSmem(f).total, stream>>>(
                f, P.p, tpack.p, X, idx, row0, M, grad, loss.p, want_z ? znorm.p : nullptr, gpart.p, (long)nparams,
                stop, terr.p, wait_tries);
            return cudaGetLastError() == cudaSuccess;
        }
        const int sm = step_smem();
        if (bf16)
            lg_flow_step<FR, __nv_bfloat16><<<blocks, FT, sm, stream>>>(f, P.p, X, idx, row0, M, grad, loss.p,
                                                                        want_z ? znorm.p : nullptr, gpart.p,
                                                                        (long)nparams, stop);
        else
            lg_flow_step<FR32, float><<<blocks, FT, sm, stream>>>(f, P.p, X, idx, row0, M, grad, loss.p,
                                                                want_z ? znorm.p : nullptr, gpart.p, (long)nparams,
                                                                stop);
        return cudaGetLastError() == cudaSuccess;
    }

    // Sum of the partial gradients into G and (adam) an Adam step.
    bool update(int M, bool adam, float lr, const int* stop)
    {
        const int blocks = (M + rows() - 1) / rows();
        float c1 = 1, c2 = 1;
        if (adam) {
            ++step;
            c1 = 1 - std::pow(0.9f, (float)step);
            c2 = 1 - std::pow(0.999f, (float)step);
        }
        lg_flow_adam<<<(unsigned)((nparams + 255) / 256), 256, 0, stream>>>(
            P.p, gpart.p, blocks, (long)nparams, adam ? nullptr : G.p, M1.p, M2.p, adam ? 1 : 0, lr, 0.9f, 0.999f,
            c1, c2, stop, f, adam && tct ? tpack.p : nullptr);
        return cudaGetLastError() == cudaSuccess;
    }

    // the training kernel's packed weights from P (after P was set from
    // outside the Adam steps)
    bool repack(cudaStream_t st) { return !tct || pack(P.p, tpack.p, st); }

    size_t packed_size() const { return (size_t)f.L * TcDims(f).sl; }

    // polls per bounded wait of the tensor-core inverse
    long wait_tries = kMbarTries;

    // BF16 tensor-core operands of the weights W (for the tc inverse).
    bool pack(const float* W, __nv_bfloat16* out, cudaStream_t st)
    {
        lg_flow_pack<<<(unsigned)std::min<size_t>((packed_size() + 255) / 256, 4096), 256, 0, st>>>(f, W, out);
        return cudaGetLastError() == cudaSuccess;
    }

    // Inverse map of M latent points (device) through the weights W (and
    // their packed copy when the tensor-core path is on) -> standardised u
    // (device), log|det du/dz| per point (device); err is set by the
    // tensor-core kernel if one of its bounded waits ran out.
    bool inverse(const float* W, const __nv_bfloat16* packed, const float* z, int M, float* uout, float* ldet,
                 cudaStream_t st, int* err)
    {
        if (tc && packed) {
            lg_flow_inverse_tc<<<(M + 127) / 128, 256, TcSmem(f).total, st>>>(f, W, packed, z, M, uout, ldet, err,
                                                                              wait_tries);
            return cudaGetLastError() == cudaSuccess;
        }
        const int blocks = (M + FRI - 1) / FRI, sm = inverse_smem();
        if (bf16)
            lg_flow_inverse<FRI, __nv_bfloat16><<<blocks, FT, sm, st>>>(f, W, z, M, uout, ldet);
        else
            lg_flow_inverse<FRI, float><<<blocks, FT, sm, st>>>(f, W, z, M, uout, ldet);
        return cudaGetLastError() == cudaSuccess;
    }
};

// The proposal used by the sampler.  Retraining runs on the flow's own
// stream while the sampler goes on with the current proposal: train()
// enqueues the whole retraining -- epochs with device-side early stopping,
// the best weights copied into the idle one of two proposal slots, the
// latent radius of the live points and the calibration of the weight bound
// -- and returns; the new slot takes over when advance() reaches `lag`
// replacements (waiting for the retraining then if it is still running) or
// at the next train(), whichever comes first.  Proposals run on a second
// stream from the active slot.
class FlowProposal : public Proposal {
public:
    Flow flow;
    lg_flow_options opt;
    int device = 0;
    uint64_t seed = 1;
    long ntrain = 0;
    cudaStream_t ps = nullptr;  // proposals
    cudaEvent_t done = nullptr, started = nullptr;  // a retraining's end and start on its stream
    bool pending = false;
    int act = -1, pslot = 0;  // active slot (-1: none) and the slot being trained
    // per slot: weights, standardisation, latent radius^2 and calibration
    DevBuf<float> Puse[2], dmean[2], dsdev[2];
    DevBuf<__nv_bfloat16> dpack[2];  // tensor-core operands of Puse
    DevBuf<int> dtcerr;              // set by the tensor-core inverse on a timeout
    DevBuf<int> dwrap;               // periodic dimensions
    std::vector<int> wrap;
    DevBuf<double> dres[2];  // [0] max |z|^2 of the live points, [1] max log weight, [2] sum exp(w - max)
    std::vector<float> hmean[2], hsdev[2];
    double radius[2] = {0, 0}, wnorm[2] = {0, 0}, efficiency[2] = {0, 0};
    bool usable[2] = {false, false};
    // training inputs and results
    DevBuf<float> dx, best, state;
    DevBuf<int> didx, dstop;
    HostBuf<float> hx, hstate, hinit;
    HostBuf<int> hidx;
    HostBuf<double> hres;
    int steps_per_epoch = 0;
    long step0 = 0;
    // calibration and proposal work buffers (separate: they run on
    // different streams)
    DevBuf<float> cz, cu, cld, dz, du, dld, dpart;
    DevBuf<int> dflag, dcnt, dbcnt, dboff;
    DevBuf<double> dX, dout, dbound;
    // Proposals come from a pool of kept draws of the active flow, refilled
    // by one batch of latent draws at a time on the proposal stream; the
    // next refill is enqueued as soon as the pool holds less than two
    // batches, so that it runs under the likelihood calls of the next
    // two.  Kept draws do not depend on the likelihood threshold, only on
    // the flow and the weight bound, so they stay valid until the flow is
    // replaced (gen counts the weights a slot has held).
    HostBuf<double> hout;  // refill: kept draws
    HostBuf<double> hbound;
    HostBuf<int> hcnt;     // refill: [0] kept and in the cube, [1] kept, [2] inverse timeout
    std::vector<double> pool;
    size_t pool_pos = 0;
    int pool_slot = -1;
    long gen[2] = {0, 0}, pool_gen = -1;
    bool inflight = false;
    int refill_slot = -1;
    long refill_gen = -1;
    int refill_room = 0, refill_M = 0;
    double kept_frac[2] = {0, 0};  // kept draws in the cube per latent draw
    cudaEvent_t refill_done = nullptr;
    // Between trainings the latent ball follows the live points: every
    // refresh() runs the live points through the active flow (largest
    // latent radius) and recalibrates the weight bound for that ball on the
    // proposal stream; the result is applied at the next refresh(), a fixed
    // number of replacements later, so that runs repeat.  A smaller ball
    // keeps the pooled draws inside it (each carries its latent radius), a
    // larger one drops the pool.
    double r2live[2] = {0, 0};  // largest |z|^2 of the live points per slot
    HostBuf<float> hlive;
    HostBuf<double> htrack;
    DevBuf<float> dlive, dtl, dtz, tz, tu, tld;
    DevBuf<double> dtrack;  // [0] max |z|^2 of the live points, [1] max log weight, [2] sum exp(w - max)
    bool track_pending = false;
    int track_slot = -1;
    long track_gen = -1, ntrack = 0;
    cudaEvent_t track_done = nullptr;

    ~FlowProposal()
    {
        if (flow.stream) cudaStreamSynchronize(flow.stream);
        if (ps) cudaStreamSynchronize(ps);
        if (ps) cudaStreamDestroy(ps);
        if (done) cudaEventDestroy(done);
        if (started) cudaEventDestroy(started);
        if (refill_done) cudaEventDestroy(refill_done);
        if (track_done) cudaEventDestroy(track_done);
    }

    // latent radius factor: the ball through the farthest live point,
    // its volume enlarged by opt.expand
    double rexp(int d) const { return std::pow(std::max(opt.expand, 1.0), 1.0 / d); }

    static int fail_cuda()
    {
        cudaGetLastError();
        return LG_ERR_CUDA;
    }

    int train(const double* live, int n, int d) override
    {
        cudaSetDevice(device);
        if (pending) finish();
        if (flow.f.d != d) {
            flow.bf16 = true;
            flow.want_tct = opt.train_tc != 0;
            flow.wait_tries = opt.wait_tries == 0 ? kMbarTries : (opt.wait_tries < 0 ? 0 : opt.wait_tries);
            if (!flow.init(d, opt.layers, opt.width, opt.hidden, seed)) return LG_ERR_INPUT;
        }
        if (!ps && cudaStreamCreateWithFlags(&ps, cudaStreamNonBlocking) != cudaSuccess) return fail_cuda();
        if (!done && cudaEventCreate(&done) != cudaSuccess) return fail_cuda();
        if (!started && cudaEventCreate(&started) != cudaSuccess) return fail_cuda();
        if (!refill_done && cudaEventCreateWithFlags(&refill_done, cudaEventDisableTiming) != cudaSuccess)
            return fail_cuda();
        cudaStream_t s = flow.stream;
        pslot = act < 0 ? 0 : 1 - act;
        // a refill or a radius update still reading this slot's weights
        // runs first
        if (inflight && cudaStreamWaitEvent(s, refill_done, 0) != cudaSuccess) return fail_cuda();
        if (track_pending && cudaStreamWaitEvent(s, track_done, 0) != cudaSuccess) return fail_cuda();
        // standardise by the live set
        std::vector<float>& mean = hmean[pslot];
        std::vector<float>& sdev = hsdev[pslot];
        mean.assign(d, 0);
        sdev.assign(d, 0);
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < d; ++a) mean[a] += (float)live[(size_t)i * d + a];
        for (auto& m : mean) m /= n;
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < d; ++a) {
                const double v = live[(size_t)i * d + a] - mean[a];
                sdev[a] += (float)(v * v);
            }
        for (auto& sd : sdev) sd = std::sqrt(std::max(sd / n, 1e-24f));
        // hold out 20% of the live points for early stopping: the best
        // weights on the held-out set are kept (the flow has far more
        // parameters than there are live points)
        const int nval = std::max(1, n / 5), ntr = n - nval;
        // warm start: later retrainings continue from the previous weights
        // with an eighth of the epochs (early stopping ends most of them
        // after 6 to 11)
        const int epochs = ntrain == 0 ? opt.epochs : std::max(1, opt.epochs / 8);
        const int Mb = std::min(opt.batch, ntr);
        steps_per_epoch = ntr / Mb;
        const size_t nidx = (size_t)nval + (size_t)epochs * ntr, nst = 8 + LG_FLOW_HISTORY;
        if (!hx.ensure((size_t)n * d + 2 * (size_t)d) || !hidx.ensure(nidx) || !dx.ensure((size_t)n * d) ||
            !didx.ensure(nidx) || !best.ensure(flow.nparams) || !state.ensure(nst) || !dstop.ensure(1) ||
            !hstate.ensure(nst) || !hinit.ensure(nst) || !hres.ensure(5) || !Puse[pslot].ensure(flow.nparams) ||
            !dmean[pslot].ensure(d) || !dsdev[pslot].ensure(d) || !dres[pslot].ensure(3) || !flow.reserve(n, Mb) ||
            !cz.ensure((size_t)16384 * d) || !cu.ensure((size_t)16384 * d) || !cld.ensure(16384) ||
            !dtcerr.ensure(2) || (flow.tc && !dpack[pslot].ensure(flow.packed_size())))
            return LG_ERR_ALLOC;
        // rows: the standardised live set (then mean and sdev); index list:
        // the held-out rows, then one shuffle of the training rows per epoch
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < d; ++a)
                hx.p[(size_t)i * d + a] = (float)((live[(size_t)i * d + a] - mean[a]) / sdev[a]);
        std::memcpy(hx.p + (size_t)n * d, mean.data(), d * 4);
        std::memcpy(hx.p + (size_t)n * d + d, sdev.data(), d * 4);
        std::vector<int> idx(n);
        std::iota(idx.begin(), idx.end(), 0);
        uint64_t st = seed ^ 0x5bd1e995u ^ ((uint64_t)ntrain << 32);
        auto next = [&]() {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            return st >> 33;
        };
        for (int i = n - 1; i > 0; --i) std::swap(idx[i], idx[next() % (uint64_t)(i + 1)]);
        std::memcpy(hidx.p, idx.data() + ntr, (size_t)nval * sizeof(int));
        idx.resize(ntr);
        for (int ep = 0; ep < epochs; ++ep) {
            for (int i = ntr - 1; i > 0; --i) std::swap(idx[i], idx[next() % (uint64_t)(i + 1)]);
            std::memcpy(hidx.p + nval + (size_t)ep * ntr, idx.data(), (size_t)ntr * sizeof(int));
        }
        std::fill(hinit.p, hinit.p + nst, NAN);
        hinit.p[0] = INFINITY;
        hinit.p[1] = hinit.p[2] = hinit.p[3] = hinit.p[4] = 0.0f;
        const uint64_t cal_key = seed * 7919 + (uint64_t)ntrain;
        ++ntrain;
        step0 = flow.step;
        if (cudaMemcpyAsync(dx.p, hx.p, (size_t)n * d * 4, cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(dmean[pslot].p, hx.p + (size_t)n * d, d * 4, cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(dsdev[pslot].p, hx.p + (size_t)n * d + d, d * 4, cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(didx.p, hidx.p, nidx * sizeof(int), cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(state.p, hinit.p, nst * sizeof(float), cudaMemcpyHostToDevice, s) ||
            cudaMemsetAsync(dstop.p, 0, sizeof(int), s) ||
            // timeout flags: [0] this stream's calibration, [1] the proposal
            // stream's inverses (cleared there when a flow takes over)
            cudaMemsetAsync(dtcerr.p, 0, (ntrain == 1 ? 2 : 1) * sizeof(int), s) ||
            (flow.tct && cudaMemsetAsync(flow.terr.p, 0, sizeof(int), s)) || cudaEventRecord(started, s) ||
            // the training kernel's packed weights (P may have been set from
            // the best weights of the previous retraining)
            !flow.repack(s))
            return fail_cuda();
        // the whole retraining is enqueued at once: the held-out check stops
        // it on the device, keeping the best weights
        const int patience = std::max(1, opt.patience);
        const unsigned kb = (unsigned)((flow.nparams + 255) / 256);
        bool ok = flow.pass(dx.p, didx.p, 0, nval, false, false, dstop.p);
        lg_flow_check<<<1, 32, 0, s>>>(flow.loss.p, nval, state.p, patience, dstop.p, 0);
        lg_flow_keep<<<kb, 256, 0, s>>>(state.p, dstop.p, flow.P.p, best.p, (long)flow.nparams);
        for (int ep = 0; ok && ep < epochs; ++ep) {
            const int row0 = nval + ep * ntr;
            for (int b = 0; ok && b < steps_per_epoch; ++b)
                ok = flow.pass(dx.p, didx.p, row0 + b * Mb, Mb, true, false, dstop.p) &&
                     flow.update(Mb, true, (float)opt.lr, dstop.p);
            ok = ok && flow.pass(dx.p, didx.p, 0, nval, false, false, dstop.p);
            lg_flow_check<<<1, 32, 0, s>>>(flow.loss.p, nval, state.p, patience, dstop.p, 1);
            lg_flow_keep<<<kb, 256, 0, s>>>(state.p, dstop.p, flow.P.p, best.p, (long)flow.nparams);
        }
        // best weights: the training state and the proposal slot
        if (!ok || cudaMemcpyAsync(flow.P.p, best.p, flow.nparams * 4, cudaMemcpyDeviceToDevice, s) ||
            cudaMemcpyAsync(Puse[pslot].p, best.p, flow.nparams * 4, cudaMemcpyDeviceToDevice, s) ||
            (flow.tc && !flow.pack(Puse[pslot].p, dpack[pslot].p, s)) || !flow.repack(s))
            return fail_cuda();
        // latent radius of the live points: max |z|^2 over all of them
        if (!flow.pass(dx.p, nullptr, 0, n, false, true, nullptr)) return fail_cuda();
        double* r = dres[pslot].p;
        lg_flow_max<<<1, 1024, 0, s>>>(flow.znorm.p, n, -INFINITY, r);
        // calibration of the weight bound on 16384 latent draws: their
        // maximum log weight and sum of exp(weight - maximum)
        const int Mc = 16384;
        lg_flow_latent<<<(Mc + 255) / 256, 256, 0, s>>>(cal_key, Mc, d, r, rexp(d), cz.p);
        if (!flow.inverse(Puse[pslot].p, dpack[pslot].p, cz.p, Mc, cu.p, cld.p, s, dtcerr.p)) return fail_cuda();
        lg_flow_max<<<1, 1024, 0, s>>>(cld.p, Mc, -INFINITY, r + 1);
        lg_flow_expsum<<<1, 1024, 0, s>>>(cld.p, Mc, r + 1);
        hres.p[4] = 0;  // (no retraining is pending: nothing writes hres now)
        if (cudaMemcpyAsync(hres.p, r, 3 * sizeof(double), cudaMemcpyDeviceToHost, s) ||
            cudaMemcpyAsync(hres.p + 3, dtcerr.p, sizeof(int), cudaMemcpyDeviceToHost, s) ||
            (flow.tct && cudaMemcpyAsync(hres.p + 4, flow.terr.p, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
            cudaMemcpyAsync(hstate.p, state.p, nst * sizeof(float), cudaMemcpyDeviceToHost, s) ||
            cudaEventRecord(done, s))
            return fail_cuda();
        pending = true;
        return LG_OK;
    }

    // Wait for the pending retraining and make its slot the active one (or
    // leave no flow active when it is unusable: a kept fraction below 0.2%).
    void finish()
    {
        pending = false;
        const auto tw = std::chrono::steady_clock::now();
        if (cudaEventSynchronize(done) != cudaSuccess) {
            fail_cuda();
            act = -1;
            return;
        }
        const double waited_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tw).count();
        float train_ms = 0;
        cudaEventElapsedTime(&train_ms, started, done);
        const int k = pslot, d = flow.f.d;
        // Adam steps the device actually took (those after the stop returned
        // at once): the bias corrections of the next retraining continue
        // from there
        flow.step = step0 + (long)hstate.p[3] * steps_per_epoch;
        r2live[k] = hres.p[0];
        radius[k] = std::sqrt(hres.p[0]) * rexp(d);
        const double mx = hres.p[1];
        wnorm[k] = mx + 1.0;
        efficiency[k] = hres.p[2] * std::exp(-1.0) / 16384;  // mean exp(w - wnorm)
        int tcerr = 0, trerr = 0;
        std::memcpy(&tcerr, hres.p + 3, sizeof tcerr);
        std::memcpy(&trerr, hres.p + 4, sizeof trerr);
        usable[k] = std::isfinite(radius[k]) && radius[k] > 0 && std::isfinite(mx) && efficiency[k] >= kMinKept &&
                    tcerr == 0 && trerr == 0;
        if (tcerr) std::fprintf(stderr, "lensed_gb300: flow inverse: a bounded wait ran out; flow not used\n");
        if (trerr) std::fprintf(stderr, "lensed_gb300: flow training: a bounded wait ran out; flow not used\n");
        act = usable[k] ? k : -1;
        ++gen[k];
        kept_frac[k] = efficiency[k];
        // the proposal stream's timeout flag starts clear for the new flow
        // (after the work already queued there)
        if (ps) cudaMemsetAsync(dtcerr.p + 1, 0, sizeof(int), ps);
        if (std::getenv("LG_FLOW_DEBUG"))
            std::fprintf(stderr,
                         "flow: train %ld epochs %d, held-out loss %.4f, latent radius %.3f, calibrated efficiency "
                         "%.4f, usable %d (d %d), on the GPU %.2f ms, waited %.2f ms\n",
                         ntrain, (int)hstate.p[3], hstate.p[0], radius[k], efficiency[k], (int)usable[k], d, train_ms,
                         waited_ms);
    }

    void set_wrap(const int* w, int d) override
    {
        wrap.assign(d, 0);
        if (w)
            for (int a = 0; a < d; ++a) wrap[a] = w[a] != 0;
        if (dwrap.ensure(d)) cudaMemcpy(dwrap.p, wrap.data(), d * sizeof(int), cudaMemcpyHostToDevice);
    }

    void advance(long since_train) override
    {
        if (pending && since_train >= opt.lag) finish();
    }

    // cost factor of a proposal: 1 + draw_cost x latent draws per point kept
    // by the weight test
    double log_cost() const override
    {
        return act < 0 ? 0.0 : std::log1p(std::max(opt.draw_cost, 0.0) / std::max(efficiency[act], kMinKept));
    }

    // volume of the image of the latent ball: V_ball(R) E[|det dx/dz|]
    double log_volume() const override
    {
        if (act < 0) return HUGE_VAL;
        const int d = flow.f.d;
        double lv = 0.5 * d * std::log(M_PI) - std::lgamma(0.5 * d + 1) + d * std::log(radius[act]);
        lv += std::log(efficiency[act]) + wnorm[act];
        for (float sd : hsdev[act]) lv += std::log((double)sd);
        return lv;
    }

    // Enqueue one refill of the pool from slot k: latent draws enough for
    // about four batches of kept draws (at most 2^20), the inverse flow, the
    // weight test against the bound (a weight above it raises the bound),
    // the cube test and an order-preserving compaction (block counts, one
    // scan, a scatter), and the copies of the counts, the bound and the
    // kept draws back to the host.
    bool enqueue_refill(int k, int d, int B, uint64_t key)
    {
        const double kf = std::max(kept_frac[k], kMinKept);
        const int M = (int)std::max(4.0 * B, std::min((double)(1 << 20), 4.0 * B / kf));
        const int room = 8 * B, w = d + 1;  // rows: the point, then its latent radius^2
        const int nb = (M + 255) / 256, per = 4096, np = (M + per - 1) / per;
        if (!dz.ensure((size_t)M * d) || !du.ensure((size_t)M * d) || !dld.ensure(M) || !dX.ensure((size_t)M * w) ||
            !dflag.ensure(M) || !dout.ensure((size_t)room * w) || !dcnt.ensure(2) || !dbound.ensure(1) ||
            !hbound.ensure(1) || !hcnt.ensure(3) || !hout.ensure((size_t)room * w) || !dbcnt.ensure(2 * (size_t)nb) ||
            !dboff.ensure(nb) || !dpart.ensure(np))
            return false;
        if ((int)wrap.size() != d) set_wrap(nullptr, d);
        Rng r(key);
        const uint64_t k_lat = r.next(), k_acc = r.next();
        // keep x with probability proportional to 1 / q_x(x) = |det dx/dz|
        // (z uniform in the ball), normalised by the calibrated bound
        lg_flow_latent<<<(M + 255) / 256, 256, 0, ps>>>(k_lat, M, d, dres[k].p, rexp(d), dz.p);
        if (!flow.inverse(Puse[k].p, dpack[k].p, dz.p, M, du.p, dld.p, ps, dtcerr.p + 1)) return false;
        lg_flow_max_part<<<np, 256, 0, ps>>>(dld.p, M, per, dpart.p);
        lg_flow_max<<<1, 256, 0, ps>>>(dpart.p, np, wnorm[k], dbound.p);
        lg_flow_accept<<<nb, 256, 0, ps>>>(k_acc, M, d, dz.p, du.p, dld.p, dbound.p, dmean[k].p, dsdev[k].p, dwrap.p,
                                           dX.p, dflag.p, dbcnt.p);
        lg_flow_scan<<<1, 1024, 0, ps>>>(dbcnt.p, nb, room, dboff.p, dcnt.p);
        lg_flow_scatter<<<nb, 256, 0, ps>>>(dflag.p, M, dX.p, w, room, dboff.p, dout.p);
        if (cudaMemcpyAsync(hcnt.p, dcnt.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, ps) ||
            cudaMemcpyAsync(hcnt.p + 2, dtcerr.p + 1, sizeof(int), cudaMemcpyDeviceToHost, ps) ||
            cudaMemcpyAsync(hbound.p, dbound.p, sizeof(double), cudaMemcpyDeviceToHost, ps) ||
            cudaMemcpyAsync(hout.p, dout.p, (size_t)room * w * sizeof(double), cudaMemcpyDeviceToHost, ps) ||
            cudaEventRecord(refill_done, ps))
            return false;
        inflight = true;
        refill_slot = k;
        refill_gen = gen[k];
        refill_room = room;
        refill_M = M;
        return true;
    }

    // Wait for the refill in flight and append its draws to the pool when
    // they come from the active flow; false on a CUDA error or an inverse
    // timeout (the flow is then dropped).
    bool merge(int d)
    {
        inflight = false;
        if (cudaEventSynchronize(refill_done) != cudaSuccess) return false;
        if (hcnt.p[2]) {
            std::fprintf(stderr, "lensed_gb300: flow inverse: a bounded wait ran out; flow dropped\n");
            act = -1;
            return false;
        }
        const int k = refill_slot;
        if (k != act || refill_gen != gen[k]) return true;
        wnorm[k] = hbound.p[0];
        const int n = std::min(hcnt.p[0], refill_room);
        kept_frac[k] = 0.5 * kept_frac[k] + 0.5 * (double)hcnt.p[0] / refill_M;
        if (std::getenv("LG_FLOW_DEBUG"))
            std::fprintf(stderr, "flow: refill %d latent, %d kept by the weight test, %d in the cube\n", refill_M,
                         hcnt.p[1], hcnt.p[0]);
        pool.erase(pool.begin(), pool.begin() + (long)pool_pos * (d + 1));
        pool_pos = 0;
        // draws of a ball larger than the current one are kept when they
        // fall inside it
        const double b2 = ball2(k, d);
        for (int i = 0; i < n; ++i) {
            const double* row = hout.p + (size_t)i * (d + 1);
            if (row[d] <= b2) pool.insert(pool.end(), row, row + d + 1);
        }
        return true;
    }

    // squared latent radius of slot k's ball (a relative margin of 1e-5
    // for the FP32 rounding of the draws)
    double ball2(int k, int d) const { return r2live[k] * rexp(d) * rexp(d) * (1.0 + 1e-5); }

    void refresh(const double* live, int n, int d) override
    {
        if (act < 0 || !ps || n < 1) return;
        cudaSetDevice(device);
        if (track_pending) apply_track(d);
        if (act < 0) return;
        const int k = act, Mc = 16384;
        if (!track_done && cudaEventCreateWithFlags(&track_done, cudaEventDisableTiming) != cudaSuccess) return;
        if (!hlive.ensure((size_t)n * d) || !dlive.ensure((size_t)n * d) || !dtl.ensure(n) || !dtz.ensure(n) ||
            !dtrack.ensure(3) || !htrack.ensure(3) || !tz.ensure((size_t)Mc * d) || !tu.ensure((size_t)Mc * d) ||
            !tld.ensure(Mc))
            return;
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < d; ++a)
                hlive.p[(size_t)i * d + a] = (float)((live[(size_t)i * d + a] - hmean[k][a]) / hsdev[k][a]);
        if (cudaMemcpyAsync(dlive.p, hlive.p, (size_t)n * d * sizeof(float), cudaMemcpyHostToDevice, ps)) return;
        // the live points' latent radii through the active weights
        const int blocks = (n + flow.simt_rows() - 1) / flow.simt_rows(), sm = flow.step_smem();
        if (flow.bf16)
            lg_flow_step<FR, __nv_bfloat16><<<blocks, FT, sm, ps>>>(flow.f, Puse[k].p, dlive.p, nullptr, 0, n, 0,
                                                                    dtl.p, dtz.p, nullptr, (long)flow.nparams,
                                                                    nullptr);
        else
            lg_flow_step<FR32, float><<<blocks, FT, sm, ps>>>(flow.f, Puse[k].p, dlive.p, nullptr, 0, n, 0, dtl.p,
                                                            dtz.p, nullptr, (long)flow.nparams, nullptr);
        if (cudaGetLastError() != cudaSuccess) return;  // (no update of the ball then)
        lg_flow_max<<<1, 1024, 0, ps>>>(dtz.p, n, -INFINITY, dtrack.p);
        // the weight bound of that ball, calibrated as at training
        const uint64_t key = seed * 0x9E3779B97F4A7C15ull + 0xD1B54A32D192ED03ull * (uint64_t)(++ntrack);
        lg_flow_latent<<<(Mc + 255) / 256, 256, 0, ps>>>(key, Mc, d, dtrack.p, rexp(d), tz.p);
        if (!flow.inverse(Puse[k].p, dpack[k].p, tz.p, Mc, tu.p, tld.p, ps, dtcerr.p + 1)) return;
        lg_flow_max<<<1, 1024, 0, ps>>>(tld.p, Mc, -INFINITY, dtrack.p + 1);
        lg_flow_expsum<<<1, 1024, 0, ps>>>(tld.p, Mc, dtrack.p + 1);
        if (cudaMemcpyAsync(htrack.p, dtrack.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, ps) ||
            cudaEventRecord(track_done, ps))
            return;
        track_pending = true;
        track_slot = k;
        track_gen = gen[k];
    }

    // Take the radius update enqueued at the previous refresh(): the ball,
    // the weight bound and the kept fraction of the active slot.
    void apply_track(int d)
    {
        track_pending = false;
        if (cudaEventSynchronize(track_done) != cudaSuccess) return;
        const int k = track_slot;
        if (k != act || track_gen != gen[k]) return;
        const double r2 = htrack.p[0], mx = htrack.p[1], eff = htrack.p[2] * std::exp(-1.0) / 16384;
        if (!(std::isfinite(r2) && r2 > 0 && std::isfinite(mx) && eff >= kMinKept)) return;
        if (r2 > r2live[k]) {  // a larger ball: the pooled draws no longer cover it
            ++gen[k];
            pool.clear();
            pool_pos = 0;
            pool_gen = gen[k];
        }
        r2live[k] = r2;
        radius[k] = std::sqrt(r2) * rexp(d);
        wnorm[k] = mx + 1.0;
        efficiency[k] = eff;
        kept_frac[k] = eff;
        cudaMemcpyAsync(dres[k].p, dtrack.p, sizeof(double), cudaMemcpyDeviceToDevice, ps);
        // pooled draws outside the smaller ball are dropped
        const double b2 = ball2(k, d);
        size_t o = 0;
        for (size_t i = pool_pos; i < pool.size() / (d + 1); ++i) {
            const double* row = &pool[i * (d + 1)];
            if (row[d] <= b2) {
                std::memmove(&pool[o * (d + 1)], row, (d + 1) * sizeof(double));
                ++o;
            }
        }
        pool.resize(o * (d + 1));
        pool_pos = 0;
        if (std::getenv("LG_FLOW_DEBUG"))
            std::fprintf(stderr, "flow: radius update: latent radius %.3f, efficiency %.4f, pool %zu\n", radius[k],
                         eff, o);
    }

    int propose(const double*, int, int d, double* out, int B, uint64_t sd) override
    {
        if (act < 0) return 0;
        cudaSetDevice(device);
        const int k = act;
        if (pool_slot != k || pool_gen != gen[k]) {  // a new flow: its own pool
            pool.clear();
            pool_pos = 0;
            pool_slot = k;
            pool_gen = gen[k];
        }
        Rng r(sd);
        int got = 0, refills = 0;
        const size_t w = (size_t)d + 1;
        for (;;) {
            const size_t avail = pool.size() / w - pool_pos;
            const int take = (int)std::min<size_t>(avail, (size_t)(B - got));
            for (int i = 0; i < take; ++i)
                std::memcpy(out + (size_t)(got + i) * d, pool.data() + (pool_pos + i) * w, d * sizeof(double));
            pool_pos += take;
            got += take;
            if (got == B) break;
            if (!inflight) {
                if (refills++ == 8) break;
                if (!enqueue_refill(k, d, B, r.next())) return fail_cuda(), 0;
            }
            if (!merge(d)) return act < 0 ? 0 : (fail_cuda(), 0);
        }
        // the next refill runs under the likelihood calls of this batch
        // and the next
        if (!inflight && pool.size() / w - pool_pos < 2 * (size_t)B && !enqueue_refill(k, d, B, r.next()))
            return fail_cuda(), 0;
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
    o.expand = 1.25;
    o.patience = 4;
    o.lag = 800;
    o.draw_cost = 0.005;
    o.wait_tries = 0;
    // the FP32-weight training kernels; the tensor-core steps (train_tc = 1)
    // train flows that propose as well (16 seeds of the sampler workload:
    // 785 k likelihood calls against 788 k) in steps 28% faster, a few
    // hundredths of a second of a run
    o.train_tc = 0;
    return o;
}

long lg_flow_nparams(int d, int layers, int width, int hidden)
{
    lg::FlowDims f{d, d / 2, layers, width, hidden};
    return (long)lg::Flow::count_params(f);
}

// Train a flow proposal on n points (row-major n x d, any scale: they are
// standardised as the sampler's live points are) exactly as the sampler
// retrains it, for tests: history[0..] receives the held-out loss before
// training and after each epoch (up to max_history values, NaN past the
// epochs that ran); returns the number of epochs run (negative on error;
// LG_ERR_TIMEOUT when a bounded wait of the calibration's tensor-core
// inverse ran out); *efficiency the calibrated kept fraction of latent
// draws.
int lg_flow_fit(int device, int d, const lg_flow_options* opts, const double* pts, int n, float* history,
                int max_history, double* efficiency)
{
    if (!pts || n < 10 || d < 2) return LG_ERR_INPUT;
    std::string err;
    std::unique_ptr<lg::FlowProposal> p(static_cast<lg::FlowProposal*>(lg::make_flow_proposal(device, d, opts, err)));
    if (!p) return LG_ERR_ALLOC;
    const int rc = p->train(pts, n, d);
    if (rc) return rc;
    p->finish();
    for (int i = 0; i < max_history && history; ++i) history[i] = i < LG_FLOW_HISTORY ? p->hstate.p[8 + i] : NAN;
    if (efficiency) *efficiency = p->efficiency[p->pslot];
    int tcerr = 0, trerr = 0;
    std::memcpy(&tcerr, p->hres.p + 3, sizeof tcerr);
    std::memcpy(&trerr, p->hres.p + 4, sizeof trerr);
    if (trerr) {
        lg::set_global_error("flow fit: a bounded wait of the tensor-core training step ran out");
        return LG_ERR_TIMEOUT;
    }
    if (tcerr) {
        lg::set_global_error("flow fit: a bounded wait of the tensor-core inverse ran out (calibration)");
        return LG_ERR_TIMEOUT;
    }
    return (int)p->hstate.p[3];
}

// Inverse of a flow with the given parameters on M latent points (host
// arrays), for checks against the CPU restatement: tc = 1 runs the
// tensor-core kernel (BF16 weights and conditioner input), tc = 0 the FP32
// one; bf16 selects BF16 hidden activations for the latter.
int lg_flow_inverse_check(int device, int d, int layers, int width, int hidden, int bf16, int tc,
                          const float* params, const float* z, int M, float* u, float* ldet)
{
    if (!params || !z || !u || !ldet || M <= 0) return LG_ERR_INPUT;
    if (cudaSetDevice(device) != cudaSuccess) return LG_ERR_CUDA;
    lg::Flow f;
    f.bf16 = bf16 != 0 || tc != 0;
    if (!f.init(d, layers, width, hidden, 1)) {
        lg::set_global_error(f.err.c_str());
        return f.err.empty() ? LG_ERR_ALLOC : LG_ERR_INPUT;
    }
    if (tc && !f.tc) {
        lg::set_global_error("flow inverse check: the tensor-core path needs width % 32 == 0 (<= 256) on sm_100+");
        return LG_ERR_UNSUPPORTED;
    }
    f.tc = tc != 0;
    lg::DevBuf<float> dz, du, dl;
    lg::DevBuf<__nv_bfloat16> pk;
    lg::DevBuf<int> e;
    if (!dz.ensure((size_t)M * d) || !du.ensure((size_t)M * d) || !dl.ensure(M) || !e.ensure(1) ||
        (f.tc && !pk.ensure(f.packed_size())))
        return LG_ERR_ALLOC;
    cudaMemcpy(f.P.p, params, f.nparams * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dz.p, z, (size_t)M * d * 4, cudaMemcpyHostToDevice);
    cudaMemset(e.p, 0, sizeof(int));
    if ((f.tc && !f.pack(f.P.p, pk.p, f.stream)) ||
        !f.inverse(f.P.p, f.tc ? pk.p : nullptr, dz.p, M, du.p, dl.p, f.stream, e.p))
        return LG_ERR_CUDA;
    int herr = 0;
    if (cudaMemcpyAsync(u, du.p, (size_t)M * d * 4, cudaMemcpyDeviceToHost, f.stream) ||
        cudaMemcpyAsync(ldet, dl.p, (size_t)M * 4, cudaMemcpyDeviceToHost, f.stream) ||
        cudaMemcpyAsync(&herr, e.p, sizeof(int), cudaMemcpyDeviceToHost, f.stream) || cudaStreamSynchronize(f.stream))
        return LG_ERR_CUDA;
    return herr ? LG_ERR_TIMEOUT : LG_OK;
}

// Device time of the inverse flow on M latent points (uploaded once): reps
// launches after two warm-up launches, CUDA events on the launching stream;
// *ms = milliseconds per launch.
int lg_flow_inverse_time(int device, int d, int layers, int width, int hidden, int tc, const float* params,
                         const float* z, int M, int reps, float* ms)
{
    if (!params || !z || !ms || M <= 0 || reps <= 0) return LG_ERR_INPUT;
    if (cudaSetDevice(device) != cudaSuccess) return LG_ERR_CUDA;
    lg::Flow f;
    f.bf16 = true;
    if (!f.init(d, layers, width, hidden, 1)) {
        lg::set_global_error(f.err.c_str());
        return f.err.empty() ? LG_ERR_ALLOC : LG_ERR_INPUT;
    }
    if (tc && !f.tc) {
        lg::set_global_error("flow inverse timing: the tensor-core path needs width % 32 == 0 (<= 256) on sm_100+");
        return LG_ERR_UNSUPPORTED;
    }
    f.tc = tc != 0;
    lg::DevBuf<float> dz, du, dl;
    lg::DevBuf<__nv_bfloat16> pk;
    lg::DevBuf<int> e;
    if (!dz.ensure((size_t)M * d) || !du.ensure((size_t)M * d) || !dl.ensure(M) || !e.ensure(1) ||
        (f.tc && !pk.ensure(f.packed_size())))
        return LG_ERR_ALLOC;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaMemcpy(f.P.p, params, f.nparams * 4, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dz.p, z, (size_t)M * d * 4, cudaMemcpyHostToDevice) || cudaMemset(e.p, 0, sizeof(int)) ||
        (f.tc && !f.pack(f.P.p, pk.p, f.stream)) || cudaEventCreate(&e0) || cudaEventCreate(&e1))
        return LG_ERR_CUDA;
    bool ok = true;
    for (int i = 0; i < 2 && ok; ++i) ok = f.inverse(f.P.p, f.tc ? pk.p : nullptr, dz.p, M, du.p, dl.p, f.stream, e.p);
    ok = ok && cudaEventRecord(e0, f.stream) == cudaSuccess;
    for (int i = 0; i < reps && ok; ++i) ok = f.inverse(f.P.p, f.tc ? pk.p : nullptr, dz.p, M, du.p, dl.p, f.stream, e.p);
    int herr = 0;
    float t = 0;
    ok = ok && cudaEventRecord(e1, f.stream) == cudaSuccess &&
         cudaMemcpyAsync(&herr, e.p, sizeof(int), cudaMemcpyDeviceToHost, f.stream) == cudaSuccess &&
         cudaStreamSynchronize(f.stream) == cudaSuccess && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!ok) return LG_ERR_CUDA;
    *ms = t / reps;
    return herr ? LG_ERR_TIMEOUT : LG_OK;
}

// Device time of training steps (forward + backward of a minibatch of
// `batch` rows, then the Adam step) on n points uploaded once: tc = 1 the
// tensor-core step, 0 the FP32-weight step with BF16 activations; reps
// steps after two warm-up steps, CUDA events on the launching stream; *ms =
// milliseconds per step (both launches).
int lg_flow_train_time(int device, int d, int layers, int width, int hidden, int tc, const float* params,
                       const float* x, int n, int batch, int reps, float* ms)
{
    if (!params || !x || !ms || n <= 0 || batch <= 0 || batch > n || reps <= 0) return LG_ERR_INPUT;
    if (cudaSetDevice(device) != cudaSuccess) return LG_ERR_CUDA;
    lg::Flow f;
    f.bf16 = true;
    f.want_tct = tc != 0;
    if (!f.init(d, layers, width, hidden, 1)) {
        lg::set_global_error(f.err.c_str());
        return f.err.empty() ? LG_ERR_ALLOC : LG_ERR_INPUT;
    }
    if (tc && !f.tct) {
        lg::set_global_error("flow training timing: the tensor-core step needs width 128, two hidden layers, d <= 16 "
                             "and sm_100+");
        return LG_ERR_UNSUPPORTED;
    }
    lg::DevBuf<float> dx;
    if (!dx.ensure((size_t)n * d) || !f.reserve(n, batch)) return LG_ERR_ALLOC;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaMemcpy(f.P.p, params, f.nparams * 4, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dx.p, x, (size_t)n * d * 4, cudaMemcpyHostToDevice) || !f.repack(f.stream) ||
        cudaEventCreate(&e0) || cudaEventCreate(&e1))
        return LG_ERR_CUDA;
    const int nb = n / batch;
    auto step = [&](int i) {
        return f.pass(dx.p, nullptr, (i % nb) * batch, batch, true, false, nullptr) &&
               f.update(batch, true, 1e-4f, nullptr);
    };
    bool ok = step(0) && step(1);
    ok = ok && cudaEventRecord(e0, f.stream) == cudaSuccess;
    for (int i = 0; i < reps && ok; ++i) ok = step(i);
    int herr = 0;
    float t = 0;
    ok = ok && cudaEventRecord(e1, f.stream) == cudaSuccess &&
         (!f.tct || cudaMemcpyAsync(&herr, f.terr.p, sizeof(int), cudaMemcpyDeviceToHost, f.stream) == cudaSuccess) &&
         cudaStreamSynchronize(f.stream) == cudaSuccess && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!ok) return LG_ERR_CUDA;
    *ms = t / reps;
    return herr ? LG_ERR_TIMEOUT : LG_OK;
}

// Loss and gradient of the flow on n points (standardised space, host
// arrays), for gradient checks against the CPU restatement: params in,
// loss (mean over the points) and grad out.  bf16 = 0 keeps activations in
// FP32.  Runs the training kernels themselves (one step, no update).
int lg_flow_loss_grad(int device, int d, int layers, int width, int hidden, int bf16, const float* params,
                      const float* x, int n, float* loss, float* grad)
{
    if (!params || !x || !loss || !grad || n <= 0) return LG_ERR_INPUT;
    if (cudaSetDevice(device) != cudaSuccess) return LG_ERR_CUDA;
    lg::Flow f;
    f.bf16 = bf16 != 0;
    f.want_tct = bf16 == 2;
    if (!f.init(d, layers, width, hidden, 1)) {
        lg::set_global_error(f.err.c_str());
        return f.err.empty() ? LG_ERR_ALLOC : LG_ERR_INPUT;
    }
    if (bf16 == 2 && !f.tct) {
        lg::set_global_error("flow loss/grad: the tensor-core training step needs width 128, two hidden layers, "
                             "d <= 16 and sm_100+");
        return LG_ERR_UNSUPPORTED;
    }
    cudaMemcpy(f.P.p, params, f.nparams * 4, cudaMemcpyHostToDevice);
    lg::DevBuf<float> dx;
    if (!dx.ensure((size_t)n * d)) return LG_ERR_ALLOC;
    cudaMemcpy(dx.p, x, (size_t)n * d * 4, cudaMemcpyHostToDevice);
    if (!f.repack(f.stream) || !f.pass(dx.p, nullptr, 0, n, true, false, nullptr) ||
        !f.update(n, false, 0.0f, nullptr))
        return LG_ERR_CUDA;
    std::vector<float> per(n);
    int herr = 0;
    if (cudaMemcpyAsync(per.data(), f.loss.p, (size_t)n * 4, cudaMemcpyDeviceToHost, f.stream) ||
        cudaMemcpyAsync(grad, f.G.p, f.nparams * 4, cudaMemcpyDeviceToHost, f.stream) ||
        (f.tct && cudaMemcpyAsync(&herr, f.terr.p, sizeof(int), cudaMemcpyDeviceToHost, f.stream)) ||
        cudaStreamSynchronize(f.stream))
        return LG_ERR_CUDA;
    if (herr) {
        lg::set_global_error("flow loss/grad: a bounded wait of the tensor-core training step ran out");
        return LG_ERR_TIMEOUT;
    }
    double s = 0;
    for (float v : per) s += v;
    *loss = (float)(s / n);
    return LG_OK;
}

}  // extern "C"
