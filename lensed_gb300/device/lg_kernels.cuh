// Kernels of the composed likelihood program.  Compiled by NVRTC after the
// prelude, the plugins and the generated model section, which defines:
//   LG_W, LG_H, LG_N          image size (pixels)
//   LG_Q                      quadrature points; lg_qq[], lg_ww[] (constant)
//   LG_RX, LG_RY, LG_SX, LG_SY pixel coordinate system (after the even-PSF shift)
//   LG_HAS_PSF, LG_PSF_W, LG_PSF_H, lg_psf[] (normalised PSF, constant)
//   LG_NPARS, lg_model, lg_compute()
// and the launch-shape parameters LG_RT, LG_RPPT, LG_QS (render) and LG_CTX,
// LG_CTY, LG_CR (convolution).
//
// Data layout in HBM, per context:
//   models   lg_model[B]              object data of each candidate
//   raw      float[B][N]              unconvolved model (PSF path only)
//   partials double[B][ntiles]        per-tile chi^2 partial sums
//   counters unsigned[B]              tiles done per candidate (zero between launches)
//   logL     double[B]
//   image, weight float[N]            resident for the context's lifetime
//
// The chi^2 of a pixel is w*(m-d)^2 in FP32 as in kernel/lensed.cl:41-55;
// sums are FP64 (per thread, then a fixed-order block tree, then a
// fixed-order sum over tiles by the block that finishes a candidate's last
// tile), so results are deterministic run to run.

#ifndef LG_RT
#define LG_RT 128
#endif
#ifndef LG_RPPT
#define LG_RPPT 2
#endif
// quadrature split: LG_QS adjacent threads share a thread's pixels, each
// taking every LG_QS-th quadrature point (fast mode: partial sums combined
// by a butterfly, which reorders the quadrature sum; exact mode: the values
// gathered and summed in the rule's order)
#ifndef LG_QS
#define LG_QS 1
#endif
#define LG_RG (LG_RT / LG_QS)
#define LG_RTILE (LG_RG * LG_RPPT)
#define LG_RTILES ((LG_N + LG_RTILE - 1) / LG_RTILE)
static_assert(LG_QS == 1 || LG_QS == 2 || LG_QS == 4 || LG_QS == 8, "quadrature split of 1, 2, 4 or 8 threads");
static_assert(LG_RT % 32 == 0, "render block of whole warps");

// ------------------------------------------------------------ reductions --
LG_DEV double lg_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order block sum; the result is valid in thread 0.
template <int NT>
LG_DEV double lg_block_sum(double v, double* red)
{
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    v = lg_warp_sum(v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (tid == 0) {
#pragma unroll
        for (int i = 0; i < NT / 32; ++i) s += red[i];
    }
    return s;
}

// A tile's chi^2 partial sum (valid in thread 0) is written; the block that
// completes a candidate's last tile (counted with an atomic per candidate)
// then sums that candidate's partials in tile order -- the same order
// whichever block comes last, so results stay deterministic -- writes
// logL = -chi2/2 (src/nested.c:106-115) and resets the counter for the next
// launch.
template <int NT>
LG_DEV void lg_tile_done(double s, double* __restrict__ partials, int ntiles, int tile, int b,
                         unsigned* __restrict__ counters, double* __restrict__ logL, double* red)
{
    __shared__ int last;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (tid == 0) {
        partials[(size_t)b * ntiles + tile] = s;
        __threadfence();
        last = atomicAdd(counters + b, 1u) == (unsigned)(ntiles - 1);
    }
    __syncthreads();
    if (!last || tid >= 32) return;
    // one warp, lane l summing tiles l, l + 32, ... in order, then a fixed
    // shuffle tree: the grouping does not depend on the launch shape (the
    // multi-system finish sums the same way)
    __threadfence();
    double acc = 0.0;
    for (int t = tid; t < ntiles; t += 32) acc += __ldcg(partials + (size_t)b * ntiles + t);
    acc = lg_warp_sum(acc);
    if (tid == 0) {
        logL[b] = -0.5 * acc;
        counters[b] = 0u;
    }
    (void)red;
}

// ---------------------------------------------------------------- render --
// kernel/lensed.cl:9-39.  Block (tile, candidate); each group of LG_QS
// threads integrates LG_RPPT pixels over the quadrature rule: strided by the
// group count in the scalar kernel (so that loads and stores coalesce),
// adjacent in the paired kernel (a thread's two rays are neighbours, so they
// mostly take the same branches; stores are float2).  With LG_QS > 1 the
// threads of a group take quadrature points n = sub, sub + LG_QS, ... and
// their sums are combined by a butterfly of shuffles (every lane ends with
// the same, order-independent result).  MODE 0 stores the raw model, MODE 1
// reduces the chi^2 directly (no PSF), MODE 2 stores value and error for one
// candidate.
#if defined(LG_PAIRED) && LG_RPPT % 2 == 0
#define LG_PIX(t, j) (LG_RPPT * (t) + (j))
#else
#define LG_PIX(t, j) ((t) + (j) * LG_RG)
#endif

// sum of v over the LG_QS lanes of a quadrature group
LG_DEV float lg_qs_sum(float v)
{
#pragma unroll
    for (int o = 1; o < LG_QS; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <int MODE>
LG_DEV void lg_render_tile(const lg_model* __restrict__ models, float* __restrict__ out, float* __restrict__ err,
                           const float* __restrict__ image, const float* __restrict__ weight,
                           double* __restrict__ partials, unsigned* __restrict__ counters,
                           double* __restrict__ logL)
{
    const int b = blockIdx.y;
    const lg_model m = models[b];
    const int base = blockIdx.x * LG_RTILE;
    const int grp = threadIdx.x / LG_QS, sub = threadIdx.x % LG_QS;
    float2 xp[LG_RPPT];
    float v[LG_RPPT], e[LG_RPPT];
#pragma unroll
    for (int j = 0; j < LG_RPPT; ++j) {
        int k = base + LG_PIX(grp, j);
        k = k < LG_N ? k : LG_N - 1;
        xp[j] = make_float2(LG_RX + LG_SX * (float)(k % LG_W), LG_RY + LG_SY * (float)(k / LG_W));
        v[j] = 0.0f;
        e[j] = 0.0f;
    }
#if defined(LG_PAIRED) && LG_RPPT % 2 == 0
    // the fast mode traces the thread's pixels two at a time with paired
    // FP32 instructions; each lane computes what the scalar loop computes
    lg_pair px[LG_RPPT / 2], py[LG_RPPT / 2], pv[LG_RPPT / 2], pe[LG_RPPT / 2];
#pragma unroll
    for (int j = 0; j < LG_RPPT / 2; ++j) {
        px[j] = lg_pair_of(xp[2 * j].x, xp[2 * j + 1].x);
        py[j] = lg_pair_of(xp[2 * j].y, xp[2 * j + 1].y);
        pv[j] = lg_pair_of(0.0f);
        pe[j] = lg_pair_of(0.0f);
    }
#if defined(LG_EXACT) && LG_QS > 1
    // exact mode with a quadrature split: the threads of a group evaluate
    // every LG_QS-th point, the values meet in shared memory, and every
    // lane of the group sums all of them in the rule's order -- the sum the
    // unsplit kernel forms, bit for bit
    __shared__ float2 lg_fq[LG_RT][(LG_Q + LG_QS - 1) / LG_QS][LG_RPPT / 2];
#pragma unroll 1
    for (int n = sub, kq = 0; n < LG_Q; n += LG_QS, ++kq) {
        const float2 q = lg_qq[n];
#pragma unroll
        for (int j = 0; j < LG_RPPT / 2; ++j) lg_fq[threadIdx.x][kq][j] = lg_compute2(m, lg_pair2{px[j] + q.x, py[j] + q.y}).v;
    }
    __syncwarp();
#pragma unroll 1
    for (int n = 0; n < LG_Q; ++n) {
        const float2 w = lg_ww[n];
        const int src = grp * LG_QS + n % LG_QS;
#pragma unroll
        for (int j = 0; j < LG_RPPT / 2; ++j) {
            const lg_pair f = {lg_fq[src][n / LG_QS][j]};
            pv[j] += w.x * f;
            if (MODE == 2) pe[j] += w.y * f;
        }
    }
#else
#pragma unroll 1
    for (int n = sub; n < LG_Q; n += LG_QS) {
        const float2 q = lg_qq[n];
        const float2 w = lg_ww[n];
#pragma unroll
        for (int j = 0; j < LG_RPPT / 2; ++j) {
            const lg_pair f = lg_compute2(m, lg_pair2{px[j] + q.x, py[j] + q.y});
            pv[j] += w.x * f;
            if (MODE == 2) pe[j] += w.y * f;
        }
    }
#endif
#pragma unroll
    for (int j = 0; j < LG_RPPT / 2; ++j) {
        v[2 * j] = pv[j].v.x;
        v[2 * j + 1] = pv[j].v.y;
        e[2 * j] = pe[j].v.x;
        e[2 * j + 1] = pe[j].v.y;
    }
#else
#pragma unroll 1
    for (int n = sub; n < LG_Q; n += LG_QS) {
        const float2 q = lg_qq[n];
        const float2 w = lg_ww[n];
#pragma unroll
        for (int j = 0; j < LG_RPPT; ++j) {
            const float f = lg_compute(m, xp[j] + q);
            v[j] += w.x * f;
            if (MODE == 2) e[j] += w.y * f;
        }
    }
#endif
#ifndef LG_EXACT
    if (LG_QS > 1) {
#pragma unroll
        for (int j = 0; j < LG_RPPT; ++j) {
            v[j] = lg_qs_sum(v[j]);
            if (MODE == 2) e[j] = lg_qs_sum(e[j]);
        }
    }
#endif
    if (MODE == 1) {
        __shared__ double red[LG_RT / 32];
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < LG_RPPT; ++j) {
            const int k = base + LG_PIX(grp, j);
            if (sub == 0 && k < LG_N) {
                const float d = v[j] - image[k];
                s += (double)(weight[k] * d * d);
            }
        }
        s = lg_block_sum<LG_RT>(s, red);
        lg_tile_done<LG_RT>(s, partials, gridDim.x, blockIdx.x, b, counters, logL, red);
    } else {
#if defined(LG_PAIRED) && LG_RPPT % 2 == 0 && LG_N % 2 == 0
        // adjacent pixel pairs: one 8-byte store per pair (N even, so the
        // pair's address is 8-byte aligned)
#pragma unroll
        for (int j = 0; j < LG_RPPT; j += 2) {
            const int k = base + LG_PIX(grp, j);
            if (sub == 0 && k < LG_N) {
                *reinterpret_cast<float2*>(out + (size_t)b * LG_N + k) = make_float2(v[j], v[j + 1]);
                if (MODE == 2) *reinterpret_cast<float2*>(err + (size_t)b * LG_N + k) = make_float2(e[j], e[j + 1]);
            }
        }
#else
#pragma unroll
        for (int j = 0; j < LG_RPPT; ++j) {
            const int k = base + LG_PIX(grp, j);
            if (sub == 0 && k < LG_N) {
                out[(size_t)b * LG_N + k] = v[j];
                if (MODE == 2) err[(size_t)b * LG_N + k] = e[j];
            }
        }
#endif
    }
}

// exact modules: 1024 resident threads per SM (64 registers a thread) --
// the correctly rounded functions are issue-bound, and the extra warps hide
// their latencies better than the 80 registers the compiler would use
#if defined(LG_EXACT)
#define LG_RENDER_MINB (1024 / LG_RT)
#else
#define LG_RENDER_MINB 1
#endif
extern "C" __global__ void __launch_bounds__(LG_RT, LG_RENDER_MINB) lg_render_raw(const lg_model* __restrict__ models,
                                                                                  float* __restrict__ raw)
{
    lg_render_tile<0>(models, raw, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
}

extern "C" __global__ void __launch_bounds__(LG_RT, LG_RENDER_MINB)
    lg_render_chi2(const lg_model* __restrict__ models, const float* __restrict__ image,
                   const float* __restrict__ weight, double* __restrict__ partials, unsigned* __restrict__ counters,
                   double* __restrict__ logL)
{
    lg_render_tile<1>(models, nullptr, nullptr, image, weight, partials, counters, logL);
}

extern "C" __global__ void __launch_bounds__(LG_RT)
    lg_render_dump(const lg_model* __restrict__ models, float* __restrict__ value, float* __restrict__ error)
{
    lg_render_tile<2>(models, value, error, nullptr, nullptr, nullptr, nullptr, nullptr);
}

// -------------------------------------------------------------- convolve --
// kernel/lensed.cl:56-103: out(x, y) = sum_j sum_i psf[j][i] *
// in(clamp(y + OY - j), clamp(x + OX - i)) with OX = PW-1-PW/2,
// OY = PH-1-PH/2, rows j outer, columns i inner (the reference's order).
// A block computes an LG_CTX x LG_CTY output tile from a clamped halo tile in
// shared memory; each thread owns LG_CR consecutive outputs of one row and
// slides a register window of LG_CR + PW - 1 inputs along each PSF row.
#if LG_HAS_PSF
#ifndef LG_CTX
#define LG_CTX 32
#endif
#ifndef LG_CTY
#define LG_CTY 32
#endif
#ifndef LG_CR
#define LG_CR 8
#endif
#define LG_OX (LG_PSF_W - 1 - LG_PSF_W / 2)
#define LG_OY (LG_PSF_H - 1 - LG_PSF_H / 2)
#define LG_CTILES_X ((LG_W + LG_CTX - 1) / LG_CTX)
#define LG_CTILES_Y ((LG_H + LG_CTY - 1) / LG_CTY)
#define LG_CTILES (LG_CTILES_X * LG_CTILES_Y)

// chi^2 of a thread's outputs (MODE 1) or their store (MODE 0)
template <int MODE>
LG_DEV double lg_conv_out(int b, int gy, int gx0, const float* acc, float* __restrict__ out,
                          const float* __restrict__ image, const float* __restrict__ weight)
{
    double s = 0.0;
    if (gy < LG_H) {
#pragma unroll
        for (int o = 0; o < LG_CR; ++o) {
            const int gx = gx0 + o;
            if (gx < LG_W) {
                const int k = gy * LG_W + gx;
                if (MODE == 1) {
                    const float d = acc[o] - image[k];
                    s += (double)(weight[k] * d * d);
                } else {
                    out[(size_t)b * LG_N + k] = acc[o];
                }
            }
        }
    }
    return s;
}

#if defined(LG_PAIRED) && LG_PSF_W <= 49 && !defined(LG_CONV_SINGLE)
// Paired rows (fast and exact modes, PSFs up to 49 pixels wide, unless the
// launch shape asks for single rows -- small tiles for small batches): a
// thread computes LG_CR columns of two output rows, y and y + LG_CTY/2, with
// f32x2 instructions (fmas in the fast mode, a product then a sum in the
// exact mode), every lane in the scalar kernel's order.  The halo tile holds each input row together with the row
// LG_CTY/2 below it as float2 pairs; pair column c of a row sits at float
// offset 2c + 4 floor(c/8) and the row pitch is 16 (mod 32) words, so the
// float4 loads of a quarter warp (four column groups of two rows) fall in
// distinct banks.
#define LG_CD (LG_CTY / 2)
#define LG_CWIN ((LG_CR + LG_PSF_W - 1 + 1) / 2 * 2)
#define LG_CNC (LG_CTX - LG_CR + LG_CWIN)
#define LG_CCOL(c) (2 * (c) + 4 * ((c) / 8))
#define LG_CROWW (LG_CCOL(LG_CNC - 1) + 2)
#define LG_CP ((LG_CROWW - 16 + 31) / 32 * 32 + 16)
#define LG_CNR (LG_CD + LG_PSF_H - 1)
#define LG_CTHREADS ((LG_CTX / LG_CR) * LG_CD)
#define LG_CSMEM (LG_CNR * LG_CP * 4)
static_assert(LG_CR % 8 == 0 && LG_CTY % 2 == 0, "paired convolution layout");

template <int MODE>
LG_DEV void lg_conv_tile(const float* __restrict__ raw, float* __restrict__ out, const float* __restrict__ image,
                         const float* __restrict__ weight, double* __restrict__ partials,
                         unsigned* __restrict__ counters, double* __restrict__ logL)
{
    extern __shared__ float4 lg_smem4[];
    float* tile = reinterpret_cast<float*>(lg_smem4);
    const int b = blockIdx.z;
    const float* src = raw + (size_t)b * LG_N;
    const int X0 = blockIdx.x * LG_CTX, Y0 = blockIdx.y * LG_CTY;
    const int br = Y0 + LG_OY - (LG_PSF_H - 1), bc = X0 + LG_OX - (LG_PSF_W - 1);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int i = tid; i < LG_CNR * LG_CNC; i += LG_CTHREADS) {
        const int r = i / LG_CNC, c = i - r * LG_CNC;
        int gy0 = br + r, gy1 = br + r + LG_CD, gx = bc + c;
        gy0 = gy0 < 0 ? 0 : (gy0 > LG_H - 1 ? LG_H - 1 : gy0);
        gy1 = gy1 < 0 ? 0 : (gy1 > LG_H - 1 ? LG_H - 1 : gy1);
        gx = gx < 0 ? 0 : (gx > LG_W - 1 ? LG_W - 1 : gx);
        *reinterpret_cast<float2*>(tile + r * LG_CP + LG_CCOL(c)) = make_float2(src[gy0 * LG_W + gx], src[gy1 * LG_W + gx]);
    }
    __syncthreads();
    const int lx0 = threadIdx.x * LG_CR, ly = threadIdx.y;
    float2 acc[LG_CR];
#pragma unroll
    for (int o = 0; o < LG_CR; ++o) acc[o] = make_float2(0.0f, 0.0f);
#pragma unroll 1
    for (int j = 0; j < LG_PSF_H; ++j) {
        const float* row = tile + (ly + LG_PSF_H - 1 - j) * LG_CP + LG_CCOL(lx0);
        float2 win[LG_CWIN];
#pragma unroll
        for (int t = 0; t < LG_CWIN / 2; ++t) {
            const float4 q = *reinterpret_cast<const float4*>(row + 4 * t + 4 * (t / 4));
            win[2 * t] = make_float2(q.x, q.y);
            win[2 * t + 1] = make_float2(q.z, q.w);
        }
        const float* prow = lg_psf + j * LG_PSF_W;
#pragma unroll
        for (int i = 0; i < LG_PSF_W; ++i) {
            const float2 p = make_float2(prow[i], prow[i]);
#pragma unroll
            for (int o = 0; o < LG_CR; ++o) acc[o] = lg_pp_fma(p, win[o + LG_PSF_W - 1 - i], acc[o]);
        }
    }
    float a0[LG_CR], a1[LG_CR];
#pragma unroll
    for (int o = 0; o < LG_CR; ++o) {
        a0[o] = acc[o].x;
        a1[o] = acc[o].y;
    }
    double s = lg_conv_out<MODE>(b, Y0 + ly, X0 + lx0, a0, out, image, weight);
    s += lg_conv_out<MODE>(b, Y0 + ly + LG_CD, X0 + lx0, a1, out, image, weight);
    if (MODE == 1) {
        __shared__ double red[LG_CTHREADS / 32];
        s = lg_block_sum<LG_CTHREADS>(s, red);
        lg_tile_done<LG_CTHREADS>(s, partials, LG_CTILES, blockIdx.y * LG_CTILES_X + blockIdx.x, b, counters, logL,
                                  red);
    }
}
#else
// a thread's window of LG_CR + PW - 1 inputs is read as float4 (LG_CR a
// multiple of 4) or float2 (LG_CR = 2: a thread's first input sits at an
// even offset, 8-byte aligned)
#if LG_CR % 4 == 0
#define LG_WVEC 4
#else
#define LG_WVEC 2
#endif
#define LG_WIN4 ((LG_CR + LG_PSF_W - 1 + LG_WVEC - 1) / LG_WVEC * LG_WVEC)
#define LG_TW_NEED (LG_CTX - LG_CR + LG_WIN4)
// row pitch = 4 (mod 32) words: the float4 loads of a quarter warp (two
// rows of four threads) then fall in distinct banks
#define LG_TWP (((LG_TW_NEED + 27) / 32) * 32 + 4)
#define LG_TH (LG_CTY + LG_PSF_H - 1)
#define LG_CTHREADS ((LG_CTX / LG_CR) * LG_CTY)
#define LG_CSMEM (LG_TH * LG_TWP * 4)

template <int MODE>
LG_DEV void lg_conv_tile(const float* __restrict__ raw, float* __restrict__ out, const float* __restrict__ image,
                         const float* __restrict__ weight, double* __restrict__ partials,
                         unsigned* __restrict__ counters, double* __restrict__ logL)
{
    extern __shared__ float4 lg_smem4[];
    float* tile = reinterpret_cast<float*>(lg_smem4);
    const int b = blockIdx.z;
    const float* src = raw + (size_t)b * LG_N;
    const int X0 = blockIdx.x * LG_CTX, Y0 = blockIdx.y * LG_CTY;
    const int br = Y0 + LG_OY - (LG_PSF_H - 1), bc = X0 + LG_OX - (LG_PSF_W - 1);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int i = tid; i < LG_TH * LG_TWP; i += LG_CTHREADS) {
        const int r = i / LG_TWP, c = i - r * LG_TWP;
        int gy = br + r, gx = bc + c;
        gy = gy < 0 ? 0 : (gy > LG_H - 1 ? LG_H - 1 : gy);
        gx = gx < 0 ? 0 : (gx > LG_W - 1 ? LG_W - 1 : gx);
        tile[i] = src[gy * LG_W + gx];
    }
    __syncthreads();
    const int lx0 = threadIdx.x * LG_CR, ly = threadIdx.y;
    float acc[LG_CR];
#pragma unroll
    for (int o = 0; o < LG_CR; ++o) acc[o] = 0.0f;
#pragma unroll 1
    for (int j = 0; j < LG_PSF_H; ++j) {
        float win[LG_WIN4];
#if LG_WVEC == 4
        const float4* row = reinterpret_cast<const float4*>(tile + (ly + LG_PSF_H - 1 - j) * LG_TWP + lx0);
#pragma unroll
        for (int t = 0; t < LG_WIN4 / 4; ++t) {
            const float4 q = row[t];
            win[4 * t + 0] = q.x;
            win[4 * t + 1] = q.y;
            win[4 * t + 2] = q.z;
            win[4 * t + 3] = q.w;
        }
#else
        const float2* row = reinterpret_cast<const float2*>(tile + (ly + LG_PSF_H - 1 - j) * LG_TWP + lx0);
#pragma unroll
        for (int t = 0; t < LG_WIN4 / 2; ++t) {
            const float2 q = row[t];
            win[2 * t + 0] = q.x;
            win[2 * t + 1] = q.y;
        }
#endif
        const float* prow = lg_psf + j * LG_PSF_W;
#pragma unroll
        for (int i = 0; i < LG_PSF_W; ++i) {
            const float p = prow[i];
#pragma unroll
            for (int o = 0; o < LG_CR; ++o) acc[o] += p * win[o + LG_PSF_W - 1 - i];
        }
    }
    double s = lg_conv_out<MODE>(b, Y0 + ly, X0 + lx0, acc, out, image, weight);
    if (MODE == 1) {
        __shared__ double red[LG_CTHREADS / 32];
        s = lg_block_sum<LG_CTHREADS>(s, red);
        lg_tile_done<LG_CTHREADS>(s, partials, LG_CTILES, blockIdx.y * LG_CTILES_X + blockIdx.x, b, counters, logL,
                                  red);
    }
}
#endif

extern "C" __global__ void __launch_bounds__(LG_CTHREADS)
    lg_conv_chi2(const float* __restrict__ raw, const float* __restrict__ image, const float* __restrict__ weight,
                 double* __restrict__ partials, unsigned* __restrict__ counters, double* __restrict__ logL)
{
    lg_conv_tile<1>(raw, nullptr, image, weight, partials, counters, logL);
}

extern "C" __global__ void __launch_bounds__(LG_CTHREADS) lg_conv_dump(const float* __restrict__ raw,
                                                                       float* __restrict__ out)
{
    lg_conv_tile<0>(raw, out, nullptr, nullptr, nullptr, nullptr, nullptr);
}
#endif

// Sizes the host reads back after loading the module.
extern "C" __device__ const unsigned lg_model_bytes_eval = sizeof(lg_model);
extern "C" __device__ const int lg_render_tiles = LG_RTILES;
#if LG_HAS_PSF
extern "C" __device__ const int lg_conv_tiles = LG_CTILES;
extern "C" __device__ const int lg_conv_smem = LG_CSMEM;
extern "C" __device__ const int lg_conv_threads = LG_CTHREADS;
#endif
