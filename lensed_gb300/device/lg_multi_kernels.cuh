// Persistent kernels for a batch of lens systems of uneven sizes that share
// the object list and the quadrature rule.  Composed by NVRTC after the
// prelude, the plugins, the model struct, lg_compute and the quadrature
// table; the distinct PSF shapes of the batch are listed in LG_PSF_SHAPES
// (a sequence of LG_PSF_CASE(w, h) entries), and LG_MAX_PSF bounds them.
//
// Work is split into units -- (system, candidate, tile) -- enumerated
// system by system; a fixed grid of blocks strides over them, so one launch
// covers every image size and the launch shape does not depend on the
// per-call candidate counts (which live in device memory).  Per-pixel
// arithmetic and summation orders are those of the single-system kernels, so
// each system's logL is identical to its own context's.

#ifndef LG_RT
#define LG_RT 128
#endif
#ifndef LG_RPPT
#define LG_RPPT 2
#endif
// quadrature split (fast mode only), as in the single-system render kernel
#ifndef LG_QS
#define LG_QS 1
#endif
#define LG_RG (LG_RT / LG_QS)
#define LG_RTILE (LG_RG * LG_RPPT)
static_assert(LG_QS == 1 || LG_QS == 2 || LG_QS == 4 || LG_QS == 8, "quadrature split of 1, 2, 4 or 8 threads");
static_assert(LG_RT % 32 == 0, "render block of whole warps");
#ifndef LG_CTX
#define LG_CTX 32
#endif
#ifndef LG_CTY
#define LG_CTY 32
#endif
#ifndef LG_CR
#define LG_CR 8
#endif
#define LG_CTHREADS ((LG_CTX / LG_CR) * LG_CTY)

// static description of a system
struct lg_sysinfo {
    int W, H, N, pw, ph;
    int rtiles, ctiles_x, ctiles_y, ctiles;
    int psf_off;
    float rx, ry, sx, sy;
    long long img_off;
};

// per-call placement of a system's candidates
struct lg_sysplan {
    int count, cand0;
    long long r_unit0, c_unit0, raw0, part0;
};

// header: [0] render units, [1] convolution units, [2] candidates, [3] systems
LG_DEV int lg_find_system(const lg_sysplan* __restrict__ plan, int nsys, long long u, bool conv)
{
    int s = 0;
    while (s + 1 < nsys && (conv ? plan[s + 1].c_unit0 : plan[s + 1].r_unit0) <= u) ++s;
    return s;
}

LG_DEV double lg_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-order block sum, valid in thread 0; red must hold NT/32 doubles.
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
    __syncthreads();
    return s;
}

// ------------------------------------------------------------- render --
// WITH_PSF: store raw models; else reduce the chi^2 of each tile directly.
// Pixels of a thread group as in the single-system kernel: adjacent in the
// paired kernel, strided by the group count otherwise; LG_QS threads of a
// group split the quadrature points and combine their sums by shuffles.
#if defined(LG_PAIRED) && LG_RPPT % 2 == 0
#define LG_MPIX(t, j) (LG_RPPT * (t) + (j))
#else
#define LG_MPIX(t, j) ((t) + (j) * LG_RG)
#endif

LG_DEV float lg_qs_sum(float v)
{
#pragma unroll
    for (int o = 1; o < LG_QS; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <bool WITH_PSF>
LG_DEV void lg_multi_render_body(const lg_model* __restrict__ models, const lg_sysinfo* __restrict__ info,
                                 const lg_sysplan* __restrict__ plan, const long long* __restrict__ hdr,
                                 float* __restrict__ raw, const float* __restrict__ images,
                                 const float* __restrict__ weights, double* __restrict__ partials)
{
    __shared__ double red[LG_RT / 32];
    const long long U = hdr[0];
    const int nsys = (int)hdr[3];
    const int grp = threadIdx.x / LG_QS, sub = threadIdx.x % LG_QS;
    for (long long u = blockIdx.x; u < U; u += gridDim.x) {
        const int s = lg_find_system(plan, nsys, u, false);
        const lg_sysinfo I = info[s];
        const lg_sysplan P = plan[s];
        const long long local = u - P.r_unit0;
        const int b = (int)(local / I.rtiles), t = (int)(local - (long long)b * I.rtiles);
        const lg_model m = models[P.cand0 + b];
        const int base = t * LG_RTILE;
        float2 xp[LG_RPPT];
        float v[LG_RPPT];
#pragma unroll
        for (int j = 0; j < LG_RPPT; ++j) {
            int k = base + LG_MPIX(grp, j);
            k = k < I.N ? k : I.N - 1;
            xp[j] = make_float2(I.rx + I.sx * (float)(k % I.W), I.ry + I.sy * (float)(k / I.W));
            v[j] = 0.0f;
        }
#if defined(LG_PAIRED) && LG_RPPT % 2 == 0
        // paired FP32 ray tracing, as in the single-system render kernel
        lg_pair px[LG_RPPT / 2], py[LG_RPPT / 2], pv[LG_RPPT / 2];
#pragma unroll
        for (int j = 0; j < LG_RPPT / 2; ++j) {
            px[j] = lg_pair_of(xp[2 * j].x, xp[2 * j + 1].x);
            py[j] = lg_pair_of(xp[2 * j].y, xp[2 * j + 1].y);
            pv[j] = lg_pair_of(0.0f);
        }
#if defined(LG_EXACT) && LG_QS > 1
        // exact mode with a quadrature split: values gathered in shared
        // memory and summed in the rule's order (as the single-system kernel)
        __shared__ float2 lg_fq[LG_RT][(LG_Q + LG_QS - 1) / LG_QS][LG_RPPT / 2];
        __syncwarp();  // the previous unit's reads of lg_fq are done
#pragma unroll 1
        for (int n = sub, kq = 0; n < LG_Q; n += LG_QS, ++kq) {
            const float2 q = lg_qq[n];
#pragma unroll
            for (int j = 0; j < LG_RPPT / 2; ++j)
                lg_fq[threadIdx.x][kq][j] = lg_compute2(m, lg_pair2{px[j] + q.x, py[j] + q.y}).v;
        }
        __syncwarp();
#pragma unroll 1
        for (int n = 0; n < LG_Q; ++n) {
            const float2 w = lg_ww[n];
            const int src = grp * LG_QS + n % LG_QS;
#pragma unroll
            for (int j = 0; j < LG_RPPT / 2; ++j) pv[j] += w.x * lg_pair{lg_fq[src][n / LG_QS][j]};
        }
#else
#pragma unroll 1
        for (int n = sub; n < LG_Q; n += LG_QS) {
            const float2 q = lg_qq[n];
            const float2 w = lg_ww[n];
#pragma unroll
            for (int j = 0; j < LG_RPPT / 2; ++j) pv[j] += w.x * lg_compute2(m, lg_pair2{px[j] + q.x, py[j] + q.y});
        }
#endif
#pragma unroll
        for (int j = 0; j < LG_RPPT / 2; ++j) {
            v[2 * j] = pv[j].v.x;
            v[2 * j + 1] = pv[j].v.y;
        }
#else
#pragma unroll 1
        for (int n = sub; n < LG_Q; n += LG_QS) {
            const float2 q = lg_qq[n];
            const float2 w = lg_ww[n];
#pragma unroll
            for (int j = 0; j < LG_RPPT; ++j) v[j] += w.x * lg_compute(m, xp[j] + q);
        }
#endif
#ifndef LG_EXACT
        if (LG_QS > 1) {
#pragma unroll
            for (int j = 0; j < LG_RPPT; ++j) v[j] = lg_qs_sum(v[j]);
        }
#endif
        if (WITH_PSF) {
#pragma unroll
            for (int j = 0; j < LG_RPPT; ++j) {
                const int k = base + LG_MPIX(grp, j);
                if (sub == 0 && k < I.N) raw[P.raw0 + (long long)b * I.N + k] = v[j];
            }
        } else {
            double acc = 0.0;
#pragma unroll
            for (int j = 0; j < LG_RPPT; ++j) {
                const int k = base + LG_MPIX(grp, j);
                if (sub == 0 && k < I.N) {
                    const float d = v[j] - images[I.img_off + k];
                    acc += (double)(weights[I.img_off + k] * d * d);
                }
            }
            acc = lg_block_sum<LG_RT>(acc, red);
            if (threadIdx.x == 0) partials[P.part0 + (long long)b * I.rtiles + t] = acc;
        }
    }
}

// exact modules: 64 registers a thread, as the single-system render
#ifndef LG_RENDER_MINB
#if defined(LG_EXACT)
#define LG_RENDER_MINB (1024 / LG_RT)
#else
#define LG_RENDER_MINB 1
#endif
#endif
extern "C" __global__ void __launch_bounds__(LG_RT, LG_RENDER_MINB)
    lg_multi_render_raw(const lg_model* __restrict__ models, const lg_sysinfo* __restrict__ info,
                        const lg_sysplan* __restrict__ plan, const long long* __restrict__ hdr, float* __restrict__ raw)
{
    lg_multi_render_body<true>(models, info, plan, hdr, raw, nullptr, nullptr, nullptr);
}

extern "C" __global__ void __launch_bounds__(LG_RT, LG_RENDER_MINB)
    lg_multi_render_chi2(const lg_model* __restrict__ models, const lg_sysinfo* __restrict__ info,
                         const lg_sysplan* __restrict__ plan, const long long* __restrict__ hdr,
                         const float* __restrict__ images, const float* __restrict__ weights,
                         double* __restrict__ partials)
{
    lg_multi_render_body<false>(models, info, plan, hdr, nullptr, images, weights, partials);
}

// ----------------------------------------------------------- convolve --
// One 32x32 output tile of one candidate of one system, for a PSF shape
// known at compile time (same order and clamping as the single-system
// kernel, kernel/lensed.cl:56-103); the PSF is staged in shared memory.
template <int PW, int PH>
LG_DEV double lg_multi_conv_unit(const float* __restrict__ src, const float* __restrict__ psf_g, int W, int H,
                                 int X0, int Y0, const float* __restrict__ image, const float* __restrict__ weight,
                                 float* smem)
{
    constexpr int OX = PW - 1 - PW / 2, OY = PH - 1 - PH / 2;
    constexpr int WIN4 = (LG_CR + PW - 1 + 3) / 4 * 4;
    constexpr int NEED = LG_CTX - LG_CR + WIN4;
    constexpr int TWP = ((NEED + 27) / 32) * 32 + 4;
    constexpr int TH = LG_CTY + PH - 1;
    float* tile = smem;
    float* psf = smem + TH * TWP;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int br = Y0 + OY - (PH - 1), bc = X0 + OX - (PW - 1);
    for (int i = tid; i < TH * TWP; i += LG_CTHREADS) {
        const int r = i / TWP, c = i - r * TWP;
        int gy = br + r, gx = bc + c;
        gy = gy < 0 ? 0 : (gy > H - 1 ? H - 1 : gy);
        gx = gx < 0 ? 0 : (gx > W - 1 ? W - 1 : gx);
        tile[i] = src[gy * W + gx];
    }
    for (int i = tid; i < PW * PH; i += LG_CTHREADS) psf[i] = psf_g[i];
    __syncthreads();
    const int lx0 = threadIdx.x * LG_CR, ly = threadIdx.y;
    float acc[LG_CR];
#pragma unroll
    for (int o = 0; o < LG_CR; ++o) acc[o] = 0.0f;
#pragma unroll 1
    for (int j = 0; j < PH; ++j) {
        const float4* row = reinterpret_cast<const float4*>(tile + (ly + PH - 1 - j) * TWP + lx0);
        float win[WIN4];
#pragma unroll
        for (int t = 0; t < WIN4 / 4; ++t) {
            const float4 q = row[t];
            win[4 * t + 0] = q.x;
            win[4 * t + 1] = q.y;
            win[4 * t + 2] = q.z;
            win[4 * t + 3] = q.w;
        }
        const float* prow = psf + j * PW;
#pragma unroll
        for (int i = 0; i < PW; ++i) {
            const float p = prow[i];
#pragma unroll
            for (int o = 0; o < LG_CR; ++o) acc[o] += p * win[o + PW - 1 - i];
        }
    }
    double s = 0.0;
    const int gy = Y0 + ly;
    if (gy < H) {
#pragma unroll
        for (int o = 0; o < LG_CR; ++o) {
            const int gx = X0 + lx0 + o;
            if (gx < W) {
                const int k = gy * W + gx;
                const float d = acc[o] - image[k];
                s += (double)(weight[k] * d * d);
            }
        }
    }
    return s;
}

#if defined(LG_PAIRED)
// The paired-row unit of the fast mode for PSFs up to 49 pixels wide: a
// 32 x (2 LG_CTY) output tile, each thread LG_CR columns of rows y and
// y + LG_CTY, in the layout, order and partial-sum grouping of the
// single-system kernel (so each system's logL is identical to its own
// context's).
template <int PW, int PH>
LG_DEV double lg_multi_conv_unit_pair(const float* __restrict__ src, const float* __restrict__ psf_g, int W, int H,
                                      int X0, int Y0, const float* __restrict__ image,
                                      const float* __restrict__ weight, float* smem)
{
    constexpr int OX = PW - 1 - PW / 2, OY = PH - 1 - PH / 2;
    constexpr int CD = LG_CTY;
    constexpr int CWIN = (LG_CR + PW - 1 + 1) / 2 * 2;
    constexpr int CNC = LG_CTX - LG_CR + CWIN;
    constexpr int CROWW = 2 * (CNC - 1) + 4 * ((CNC - 1) / 8) + 2;
    constexpr int CP = (CROWW - 16 + 31) / 32 * 32 + 16;
    constexpr int CNR = CD + PH - 1;
    static_assert(LG_CR % 8 == 0, "paired convolution layout");
    float* tile = smem;
    float* psf = smem + CNR * CP;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int br = Y0 + OY - (PH - 1), bc = X0 + OX - (PW - 1);
    for (int i = tid; i < CNR * CNC; i += LG_CTHREADS) {
        const int r = i / CNC, c = i - r * CNC;
        int gy0 = br + r, gy1 = br + r + CD, gx = bc + c;
        gy0 = gy0 < 0 ? 0 : (gy0 > H - 1 ? H - 1 : gy0);
        gy1 = gy1 < 0 ? 0 : (gy1 > H - 1 ? H - 1 : gy1);
        gx = gx < 0 ? 0 : (gx > W - 1 ? W - 1 : gx);
        *reinterpret_cast<float2*>(tile + r * CP + 2 * c + 4 * (c / 8)) = make_float2(src[gy0 * W + gx], src[gy1 * W + gx]);
    }
    for (int i = tid; i < PW * PH; i += LG_CTHREADS) psf[i] = psf_g[i];
    __syncthreads();
    const int lx0 = threadIdx.x * LG_CR, ly = threadIdx.y;
    float2 acc[LG_CR];
#pragma unroll
    for (int o = 0; o < LG_CR; ++o) acc[o] = make_float2(0.0f, 0.0f);
#pragma unroll 1
    for (int j = 0; j < PH; ++j) {
        const float* row = tile + (ly + PH - 1 - j) * CP + 2 * lx0 + 4 * (lx0 / 8);
        float2 win[CWIN];
#pragma unroll
        for (int t = 0; t < CWIN / 2; ++t) {
            const float4 q = *reinterpret_cast<const float4*>(row + 4 * t + 4 * (t / 4));
            win[2 * t] = make_float2(q.x, q.y);
            win[2 * t + 1] = make_float2(q.z, q.w);
        }
        const float* prow = psf + j * PW;
#pragma unroll
        for (int i = 0; i < PW; ++i) {
            const float2 p = make_float2(prow[i], prow[i]);
#pragma unroll
            for (int o = 0; o < LG_CR; ++o) acc[o] = lg_pp_fma(p, win[o + PW - 1 - i], acc[o]);
        }
    }
    double s0 = 0.0, s1 = 0.0;
#pragma unroll
    for (int o = 0; o < LG_CR; ++o) {
        const int gx = X0 + lx0 + o;
        if (gx < W) {
            if (Y0 + ly < H) {
                const int k = (Y0 + ly) * W + gx;
                const float d = acc[o].x - image[k];
                s0 += (double)(weight[k] * d * d);
            }
            if (Y0 + ly + CD < H) {
                const int k = (Y0 + ly + CD) * W + gx;
                const float d = acc[o].y - image[k];
                s1 += (double)(weight[k] * d * d);
            }
        }
    }
    return s0 + s1;
}
#define LG_MULTI_PAIRED(w) ((w) <= 49)
#else
#define LG_MULTI_PAIRED(w) false
#endif

extern "C" __global__ void __launch_bounds__(LG_CTHREADS)
    lg_multi_conv_chi2(const float* __restrict__ raw, const lg_sysinfo* __restrict__ info,
                       const lg_sysplan* __restrict__ plan, const long long* __restrict__ hdr,
                       const float* __restrict__ images, const float* __restrict__ weights,
                       const float* __restrict__ psfs, double* __restrict__ partials)
{
    extern __shared__ float4 lg_msmem4[];
    float* smem = reinterpret_cast<float*>(lg_msmem4);
    __shared__ double red[LG_CTHREADS / 32];
    const long long U = hdr[1];
    const int nsys = (int)hdr[3];
    for (long long u = blockIdx.x; u < U; u += gridDim.x) {
        const int s = lg_find_system(plan, nsys, u, true);
        const lg_sysinfo I = info[s];
        const lg_sysplan P = plan[s];
        const long long local = u - P.c_unit0;
        const int b = (int)(local / I.ctiles), t = (int)(local - (long long)b * I.ctiles);
        const int ty = t / I.ctiles_x, tx = t - ty * I.ctiles_x;
        const float* src = raw + P.raw0 + (long long)b * I.N;
        const float* img = images + I.img_off;
        const float* wht = weights + I.img_off;
        const float* psf = psfs + I.psf_off;
        double acc = 0.0;
        switch (I.pw * 1024 + I.ph) {
#if defined(LG_PAIRED)
#define LG_PSF_CASE(w, h)                                                                                        \
    case (w) * 1024 + (h):                                                                                      \
        if constexpr (LG_MULTI_PAIRED(w))                                                                        \
            acc = lg_multi_conv_unit_pair<w, h>(src, psf, I.W, I.H, tx * LG_CTX, ty * 2 * LG_CTY, img, wht, smem); \
        else                                                                                                     \
            acc = lg_multi_conv_unit<w, h>(src, psf, I.W, I.H, tx * LG_CTX, ty * LG_CTY, img, wht, smem);        \
        break;
#else
#define LG_PSF_CASE(w, h)                                                                                 \
    case (w) * 1024 + (h):                                                                               \
        acc = lg_multi_conv_unit<w, h>(src, psf, I.W, I.H, tx * LG_CTX, ty * LG_CTY, img, wht, smem);    \
        break;
#endif
            LG_PSF_SHAPES
#undef LG_PSF_CASE
        default:
            break;
        }
        acc = lg_block_sum<LG_CTHREADS>(acc, red);
        if (threadIdx.x == 0 && threadIdx.y == 0) partials[P.part0 + (long long)b * I.ctiles + t] = acc;
    }
}

// ------------------------------------------------------------- finish --
// logL of every candidate from its partials, one warp per candidate: lane l
// sums tiles l, l + 32, ... in order, then a fixed shuffle tree -- the
// grouping of the single-system kernels, so each system's logL is identical
// to its own context's.
extern "C" __global__ void __launch_bounds__(256)
    lg_multi_finish(const double* __restrict__ partials, const lg_sysinfo* __restrict__ info,
                    const lg_sysplan* __restrict__ plan, const long long* __restrict__ hdr, int with_psf,
                    double* __restrict__ logL)
{
    const int C = (int)hdr[2], nsys = (int)hdr[3];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (int c = blockIdx.x * 8 + warp; c < C; c += gridDim.x * 8) {
        int s = 0;
        while (s + 1 < nsys && plan[s + 1].cand0 <= c) ++s;
        const int n = with_psf ? info[s].ctiles : info[s].rtiles;
        const double* p = partials + plan[s].part0 + (long long)(c - plan[s].cand0) * n;
        double acc = 0.0;
        for (int t = lane; t < n; t += 32) acc += p[t];
        acc = lg_warp_sum(acc);
        if (lane == 0) logL[c] = -0.5 * acc;
    }
}
