// Correctly rounded single-precision exp, log, atan, atanh, sin, cos, pow
// and atan2 computed in single-precision arithmetic, for the exact
// evaluation modules.
//
// The likelihood's FP32 semantics (the oracle's, and the strict modules')
// takes every elementary function as its value evaluated in double and
// rounded once to float.  GB300 executes FP64 at a small fraction of its
// FP32 rate, so per ray these functions are computed here instead with
// "double-word" arithmetic -- a value carried as an unevaluated sum hi + lo
// of two floats, with exact products and sums from fma (Dekker 1971, "A
// floating-point technique for extending the available precision") -- after
// table-driven argument reductions (Tang 1989, "Table-driven implementation
// of the exponential function in IEEE floating-point arithmetic"; Tang 1990,
// "... of the logarithm function").  The double-word result is within about
// 2^-42 of the true value (relative); Ziv's rounding test (Ziv 1991, "Fast
// evaluation of elementary mathematical functions with correctly rounded
// last bit") then rounds both ends of that error interval, and if they round
// to the same float, that float is the correctly rounded result -- which is
// also what the double evaluation rounds to, its own error being far smaller
// than the interval.  Otherwise (about one call in 2^16) the lane evaluates
// the function in double and rounds once, exactly as the strict modules do.
// So each function returns the double-then-round value for every input.
//
// The functions are written once over a lane type F: float (one value;
// also compiled for the host, with LG_CRF_HOST, for the CPU tests) or
// float2 (two rays, with the paired f32x2 instructions).  Every operation is
// a single IEEE round-to-nearest operation (no contraction is left to the
// compiler).  Tables: lg_crf_tables.cuh, generated by make_crf_tables.py.

#ifdef LG_CRF_HOST
#include <cmath>
#include <cstdint>
#include <cstring>
#define LG_CRF_DEV static inline
#define LG_CRF_COLD static
#define LG_CRF_TABLE(type, name, n) static const type name[n]
struct float2 {
    float x, y;
};
struct float4 {
    float x, y, z, w;
};
#else
#define LG_CRF_DEV static __device__ __forceinline__
#define LG_CRF_COLD static __device__ __noinline__
#define LG_CRF_TABLE(type, name, n) __device__ const type name[n]
#endif

// ------------------------------------------------------------- primitives --
#ifdef LG_CRF_HOST
LG_CRF_DEV float crf_add(float a, float b) { return a + b; }
LG_CRF_DEV float crf_sub(float a, float b) { return a - b; }
LG_CRF_DEV float crf_mul(float a, float b) { return a * b; }
LG_CRF_DEV float crf_fma(float a, float b, float c) { return std::fma(a, b, c); }
LG_CRF_DEV int crf_bits(float a)
{
    int i;
    std::memcpy(&i, &a, 4);
    return i;
}
LG_CRF_DEV float crf_from_bits(int i)
{
    float a;
    std::memcpy(&a, &i, 4);
    return a;
}
// reciprocal estimate: any value within a few ulp of 1/a serves (the
// double-word steps correct it); the host uses the IEEE quotient unless a
// test build substitutes a perturbed one (to stand in for the device's
// approximate reciprocal)
#ifndef LG_CRF_HOST_RCP
#define LG_CRF_HOST_RCP(a) (1.0f / (a))
#endif
LG_CRF_DEV float crf_rcp(float a) { return LG_CRF_HOST_RCP(a); }
// (a test build may count the lanes that take the double path)
#ifndef LG_CRF_SLOW_COUNT
#define LG_CRF_SLOW_COUNT()
#endif
// integer fields of the arguments' bit patterns (see the device versions)
LG_CRF_DEV void crf_log_fields(int b, int& e, int& j, int& mb)
{
    const int t = b - 0x3f400000;
    e = t >> 23;
    j = (t >> 13) & 1023;
    mb = b - e * 0x800000;
}
LG_CRF_DEV void crf_exp_fields(int bits, int& j, int& m)
{
    const int k = bits - 0x4b400000;
    j = k & 63;
    m = k >> 6;
}
LG_CRF_DEV int crf_pow2_bits(int e) { return (e + 127) * 0x800000; }   // bits of 2^e (normal e)
LG_CRF_DEV int crf_add_exp(int bits, int m) { return bits + m * 0x800000; }
LG_CRF_DEV float crf_slow_exp(float x) { LG_CRF_SLOW_COUNT(); return (float)std::exp((double)x); }
LG_CRF_DEV float crf_slow_log(float x) { LG_CRF_SLOW_COUNT(); return (float)std::log((double)x); }
LG_CRF_DEV float crf_slow_atan(float x) { LG_CRF_SLOW_COUNT(); return (float)std::atan((double)x); }
LG_CRF_DEV float crf_slow_atanh(float x) { LG_CRF_SLOW_COUNT(); return (float)std::atanh((double)x); }
LG_CRF_DEV float crf_slow_sin(float x) { LG_CRF_SLOW_COUNT(); return (float)std::sin((double)x); }
LG_CRF_DEV float crf_slow_cos(float x) { LG_CRF_SLOW_COUNT(); return (float)std::cos((double)x); }
LG_CRF_DEV float crf_slow_pow(float x, float y) { LG_CRF_SLOW_COUNT(); return (float)std::pow((double)x, (double)y); }
LG_CRF_DEV float crf_slow_atan2(float y, float x)
{
    LG_CRF_SLOW_COUNT();
    return (float)std::atan2((double)y, (double)x);
}
#else
LG_CRF_DEV float crf_add(float a, float b) { return __fadd_rn(a, b); }
LG_CRF_DEV float crf_sub(float a, float b) { return __fsub_rn(a, b); }
LG_CRF_DEV float crf_mul(float a, float b) { return __fmul_rn(a, b); }
LG_CRF_DEV float crf_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// paired operations: add and fma on f32x2; products lane by lane, because
// with CUDA 13.0 the assembler fused an f32x2 multiply into the following
// f32x2 add (scalar round-to-nearest multiplies are never fused), and the
// double-word steps are written for separately rounded products
LG_CRF_DEV float2 crf_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
LG_CRF_DEV float2 crf_sub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
LG_CRF_DEV float2 crf_mul(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
LG_CRF_DEV float2 crf_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
LG_CRF_DEV int crf_bits(float a) { return __float_as_int(a); }
LG_CRF_DEV float crf_from_bits(int i) { return __int_as_float(i); }
// PTX rcp.approx (within about 1 ulp; subnormal results flushed, which
// the callers tolerate: see each use)
LG_CRF_DEV float crf_rcp(float a)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
// Integer fields of the arguments' bit patterns, in inline PTX: with CUDA
// 13.0 the optimizer was seen to miscompute such per-lane shifts of paired
// values (a lane's t >> 23 came out as t), and an asm block is opaque to it.
//   log: t = b - bits(0.75); e = t >> 23 (arithmetic); j = (t >> 13) & 1023;
//        mb = b - e 2^23 (the mantissa scaled into [0.75, 1.5))
LG_CRF_DEV void crf_log_fields(int b, int& e, int& j, int& mb)
{
    asm("{\n.reg .s32 t, x;\nsub.s32 t, %3, 0x3f400000;\nshr.s32 %0, t, 23;\nshr.s32 x, t, 13;\n"
        "and.b32 %1, x, 1023;\nshl.b32 x, %0, 23;\nsub.s32 %2, %3, x;\n}"
        : "=r"(e), "=r"(j), "=r"(mb)
        : "r"(b));
}
//   exp: k = bits - bits(1.5 2^23); j = k & 63; m = k >> 6 (arithmetic)
LG_CRF_DEV void crf_exp_fields(int bits, int& j, int& m)
{
    asm("{\n.reg .s32 k;\nsub.s32 k, %2, 0x4b400000;\nand.b32 %0, k, 63;\nshr.s32 %1, k, 6;\n}"
        : "=r"(j), "=r"(m)
        : "r"(bits));
}
// bits of 2^e for a normal power of two, and bits + m 2^23 (a float scaled
// by 2^m while it stays normal)
LG_CRF_DEV int crf_pow2_bits(int e)
{
    int r;
    asm("{\n.reg .s32 x;\nadd.s32 x, %1, 127;\nshl.b32 %0, x, 23;\n}" : "=r"(r) : "r"(e));
    return r;
}
LG_CRF_DEV int crf_add_exp(int bits, int m)
{
    int r;
    asm("{\n.reg .s32 x;\nshl.b32 x, %2, 23;\nadd.s32 %0, %1, x;\n}" : "=r"(r) : "r"(bits), "r"(m));
    return r;
}
// the lanes the double-word path cannot decide: the function in double,
// rounded once (out of line: a cold path)
LG_CRF_COLD float crf_slow_exp(float x) { return (float)exp((double)x); }
LG_CRF_COLD float crf_slow_log(float x) { return (float)log((double)x); }
LG_CRF_COLD float crf_slow_atan(float x) { return (float)atan((double)x); }
LG_CRF_COLD float crf_slow_atanh(float x) { return (float)atanh((double)x); }
LG_CRF_COLD float crf_slow_sin(float x) { return (float)sin((double)x); }
LG_CRF_COLD float crf_slow_cos(float x) { return (float)cos((double)x); }
LG_CRF_COLD float crf_slow_pow(float x, float y) { return (float)pow((double)x, (double)y); }
LG_CRF_COLD float crf_slow_atan2(float y, float x) { return (float)atan2((double)y, (double)x); }
LG_CRF_DEV float crf_get(float2 v, int i) { return i ? v.y : v.x; }
LG_CRF_DEV void crf_set(float2& v, int i, float s)
{
    if (i)
        v.y = s;
    else
        v.x = s;
}
template <class T> LG_CRF_DEV T crf_ldg(const T* p) { return __ldg(p); }
#endif

#ifdef LG_CRF_HOST
template <class T> LG_CRF_DEV T crf_ldg(const T* p) { return *p; }
LG_CRF_DEV float crf_fabsf(float a) { return std::fabs(a); }
LG_CRF_DEV float crf_copysignf(float a, float b) { return std::copysign(a, b); }
#else
LG_CRF_DEV float crf_fabsf(float a) { return fabsf(a); }
LG_CRF_DEV float crf_copysignf(float a, float b) { return copysignf(a, b); }
#endif
LG_CRF_DEV float crf_get(float v, int) { return v; }
LG_CRF_DEV void crf_set(float& v, int, float s) { v = s; }

template <class F> struct crf_lanes;
template <> struct crf_lanes<float> { static const int n = 1; };
template <> struct crf_lanes<float2> { static const int n = 2; };

LG_CRF_DEV void crf_fill(float& v, float s) { v = s; }
LG_CRF_DEV void crf_fill(float2& v, float s)
{
    v.x = s;
    v.y = s;
}
// s in every lane
template <class F>
LG_CRF_DEV F crf_bc(float s)
{
    F v;
    crf_fill(v, s);
    return v;
}
LG_CRF_DEV float crf_neg(float a) { return -a; }
LG_CRF_DEV float2 crf_neg(float2 a)
{
    float2 v;
    v.x = -a.x;
    v.y = -a.y;
    return v;
}
LG_CRF_DEV float crf_abs(float a) { return crf_fabsf(a); }
LG_CRF_DEV float2 crf_abs(float2 a)
{
    float2 v;
    v.x = crf_fabsf(a.x);
    v.y = crf_fabsf(a.y);
    return v;
}

// (the library embeds the tables here for NVRTC, which has no include path)
#ifndef LG_CRF_TABLES_INLINE
#include "lg_crf_tables.cuh"
#endif

// Relative half-width of Ziv's interval: the double-word results of the
// functions below are within 2^-42 of the true value (bound from the
// error analysis in each function; tests/test_crfloat.py measures it over
// all or dense samples of the inputs), so a margin of 2^-40 leaves a factor
// of 4.
#ifndef LG_CRF_ZIV
#define LG_CRF_ZIV (0x1p-40f)
#endif

// Both ends of [hi + lo - d, hi + lo + d], d = |hi| 2^-40, rounded: equal
// means the result.  (lo +- hi 2^-40 from an fma: the product is exact, a
// power-of-two scaling; for negative hi the two ends swap, which the
// equality test does not mind.)
template <class F>
LG_CRF_DEV void crf_ziv(F hi, F lo, F& z1, F& z2)
{
    z1 = crf_add(hi, crf_fma(hi, crf_bc<F>(LG_CRF_ZIV), lo));
    z2 = crf_add(hi, crf_fma(hi, crf_bc<F>(-LG_CRF_ZIV), lo));
}

// every lane of v satisfies ok
template <class F>
LG_CRF_DEV bool crf_all(const bool (&ok)[2])
{
    bool a = true;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) a = a && ok[i];
    return a;
}

// ---------------------------------------------------------------------- exp --
// x = k ln2/64 + r, |r| <= ln2/128 (k = m 64 + j); e^x = 2^m 2^(j/64) e^r.
// r = x - k L_hi exactly (an fma: the difference is a multiple of 2^-31
// below 2^-7 in magnitude) minus k L_lo; e^r = 1 + r + r^2/2 + r^3 (1/6 +
// r/24) with r = rh + rl, the square of rh exact (fma), rl to first order
// (it reaches 2^-22), the cubic tail in float.
// Error: k L_lo rounding and the L_hi + L_lo split (2^-46 at |k| <= 9600),
// truncation r^5/120 (2^-44.6), table pairs (2^-48), evaluation (2^-47).
// Results below 2^-126 are rounded to the subnormal grid from the
// double-word value directly; e^x rounds to 0 for x <= LG_CRF_EXP_ZERO.
LG_CRF_COLD float crf_exp_low(float x, float yh0, float yl0, int m)
{
    // renormalise the pair (yl0 reaches a few ulp of yh0): |yl| <= ulp(yh)/2
    const float yh = crf_add(yh0, yl0);
    const float yl = crf_sub(yl0, crf_sub(yh, yh0));
    // the result y 2^m with m <= -126 and y < 2^(-126 - m): round y to the
    // grid g = 2^(-149 - m) with the magic number M = 2^(-126 - m), for
    // which M + y lies in [M, 2M) where floats are spaced by g
    const float M = crf_from_bits(crf_pow2_bits(-126 - m));
    const float g = crf_mul(M, 0x1p-23f), h = crf_mul(g, 0.5f);
    const float a = crf_add(M, yh);
    const float base = crf_sub(a, M);   // exact
    const float ea = crf_sub(yh, base);  // exact
    const float rho = crf_add(ea, yl);
    const float dd = crf_add(crf_mul(yh, LG_CRF_ZIV), crf_mul(h, 0x1p-22f));
    const float ar = crf_fabsf(rho);
    float q;
    if (ar < crf_sub(h, dd))
        q = base;
    else if (ar > crf_add(h, dd))
        q = crf_add(base, rho > 0.0f ? g : crf_neg(g));
    else
        return crf_slow_exp(x);
    // q 2^m, exactly, in two power-of-two steps (m + 64 >= -87)
    return crf_mul(crf_mul(q, crf_from_bits(crf_pow2_bits(m + 64))), 0x1p-64f);
}

// e^r 2^(j/64) as yh + yl for r = rh + rl (|rh| <= ln2/128 + 2^-17, rl to
// first order) and j, m (k = 64 m + j) from big = k + 1.5 2^23, per lane.
template <class F>
LG_CRF_DEV void crf_exp_tail(F big, F rh, F rl, F& yh, F& yl, int (&mm)[2])
{
    const F sh = crf_mul(rh, rh);
    const F sl = crf_fma(rh, rh, crf_neg(sh));
    const F p3 = crf_fma(rh, crf_bc<F>(0x1.555556p-5f), crf_bc<F>(0x1.555556p-3f));
    const F h = crf_mul(sh, crf_bc<F>(0.5f));
    // first order in rl (up to 2^-22 at large |k|): rl (1 + rh + rh^2/2)
    const F small = crf_fma(crf_mul(sh, rh), p3, crf_fma(sl, crf_bc<F>(0.5f), crf_fma(h, rl, crf_fma(rh, rl, rl))));
    const F uh = crf_add(rh, h);  // |rh| >= rh^2 / 2: fast two-sum
    const F ul = crf_add(crf_sub(h, crf_sub(uh, rh)), small);
    F th, tl;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        int j;
        crf_exp_fields(crf_bits(crf_get(big, i)), j, mm[i]);
        const float2 T = crf_ldg(lg_crf_exp_tab + j);
        crf_set(th, i, T.x);
        crf_set(tl, i, T.y);
    }
    // T (1 + u) = T + T uh + (T ul + tl uh + tl)
    const F ph = crf_mul(th, uh);
    const F pl = crf_fma(th, uh, crf_neg(ph));
    const F e = crf_add(crf_fma(th, ul, crf_fma(tl, uh, tl)), pl);
    yh = crf_add(th, ph);  // |th| >= 1 > |ph|: fast two-sum
    yl = crf_add(crf_sub(ph, crf_sub(yh, th)), e);
}

// The double-word e^x 2^-m as yh + yl, big = k + 1.5 2^23, and m per lane.
template <class F>
LG_CRF_DEV void crf_exp_core(F x, F& big, F& yh, F& yl, int (&mm)[2])
{
    const F S = crf_bc<F>(0x1.8p23f);
    big = crf_fma(x, crf_bc<F>(LG_CRF_EXP_INVL), S);  // k + 1.5 2^23 (|k| < 2^22)
    const F kf = crf_sub(big, S);
    const F rh = crf_fma(crf_neg(kf), crf_bc<F>(LG_CRF_EXP_LHI), x);
    const F rl = crf_mul(crf_neg(kf), crf_bc<F>(LG_CRF_EXP_LLO));
    crf_exp_tail(big, rh, rl, yh, yl, mm);
}

template <class F>
LG_CRF_DEV F lg_crf_exp(F x)
{
    F big, yh, yl, z1, z2;
    int m[2];
    crf_exp_core(x, big, yh, yl, m);
    crf_ziv(yh, yl, z1, z2);
    F out;
    // the common case for the whole pair: x in [-87, 88] (a normal result,
    // so m >= -125 or m = -126 with z1 >= 1) and the rounding decided
    bool ok[2];
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        const float xi = crf_get(x, i);
        ok[i] = xi >= -87.0f && xi <= 88.0f && crf_get(z1, i) == crf_get(z2, i);
    }
    if (crf_all<F>(ok)) {
#pragma unroll
        for (int i = 0; i < crf_lanes<F>::n; ++i)
            crf_set(out, i, crf_from_bits(crf_add_exp(crf_bits(crf_get(z1, i)), m[i])));
        return out;
    }
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        const float xi = crf_get(x, i);
        float r;
        if (xi <= 88.0f && xi > LG_CRF_EXP_ZERO) {
            const float a = crf_get(z1, i);
            if (m[i] >= -125 || (m[i] == -126 && a >= 1.0f))
                r = a == crf_get(z2, i) ? crf_from_bits(crf_add_exp(crf_bits(a), m[i])) : crf_slow_exp(xi);
            else
                r = crf_exp_low(xi, crf_get(yh, i), crf_get(yl, i), m[i]);
        } else {
            r = xi <= LG_CRF_EXP_ZERO ? 0.0f : crf_slow_exp(xi);  // NaN, x > 88: in double
        }
        crf_set(out, i, r);
    }
    return out;
}

// ---------------------------------------------------------------------- log --
// log1p of the double-word r = rh + rl (|r| <= 2^-10): r - r^2/2 + r^3
// (1/3 - r/4 + r^2/5), the square exact; truncation r^6/6 (relative 2^-52
// where the result is r itself), the cubic term in float (relative to r,
// 3 roundings of a term below 2^-21.6: 2^-44).  Out: uh + ul.
template <class F>
LG_CRF_DEV void crf_log1p_dw(F rh, F rl, F& uh, F& ul)
{
    const F sh = crf_mul(rh, rh);
    const F sl = crf_fma(rh, rh, crf_neg(sh));
    const F P = crf_fma(crf_fma(rh, crf_bc<F>(0x1.99999ap-3f), crf_bc<F>(-0.25f)), rh, crf_bc<F>(0x1.555556p-2f));
    const F t = crf_mul(crf_mul(sh, rh), P);
    // r_lo - r_h r_lo - s_lo / 2 + t
    const F small = crf_add(crf_fma(crf_neg(rh), rl, rl), crf_fma(sl, crf_bc<F>(-0.5f), t));
    const F h = crf_mul(sh, crf_bc<F>(-0.5f));
    uh = crf_add(rh, h);  // |rh| >= rh^2 / 2: fast two-sum
    ul = crf_add(crf_sub(h, crf_sub(uh, rh)), small);
}

// ln(u), u = uh + ul > 0 (uh normal, |ul| <= ulp(uh)): u = 2^e m (m in
// [0.75, 1.5)) and m c_j = 1 + r with c_j from the table of the interval of
// m (|r| <= 2^-10), so ln u = e ln2 - ln(c_j) + log1p(r).  r = m c_j - 1 is exact as
// (m_hi c_j - 1) + (the product's rounding error) + m_lo c_j (the first term
// exactly by Sterbenz); c_j = 1 next to 1, so small logarithms keep their
// relative accuracy.  Sum: e ln2 as an exact product pair plus e LN2_LO,
// then two fast two-sums (|e ln2| >= |ln c_j| >= |log1p(r)| or the larger
// term is zero).  Out: hi + lo.
template <class F, bool DW>
LG_CRF_DEV void crf_log_dw(F uh, F ul, F& hi, F& lo)
{
    F m, c, Lh, Ll, ef, ml;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        int e, j, mb;
        crf_log_fields(crf_bits(crf_get(uh, i)), e, j, mb);
        crf_set(m, i, crf_from_bits(mb));
        const float4 T = crf_ldg(lg_crf_log_tab + j);
        crf_set(c, i, T.x);
        crf_set(Lh, i, T.y);
        crf_set(Ll, i, T.z);
        // e as float: e + 1.5 2^23 has the bits 0x4b400000 + e
        crf_set(ef, i, crf_from_bits(0x4b400000 + e) - 0x1.8p23f);
        if (DW) crf_set(ml, i, crf_get(ul, i) * crf_from_bits(crf_pow2_bits(-e)));  // exact: ul 2^-e
    }
    const F ph = crf_mul(m, c);
    const F pl = crf_fma(m, c, crf_neg(ph));
    F rh = crf_sub(ph, crf_bc<F>(1.0f));  // exact
    F rl;
    if (DW) {
        // + m_lo c, then renormalise (two-sum: m_lo can exceed rh)
        const F q = crf_fma(ml, c, pl);
        const F s = crf_add(rh, q);
        const F bb = crf_sub(s, rh);
        rl = crf_add(crf_sub(rh, crf_sub(s, bb)), crf_sub(q, bb));
        rh = s;
    } else {
        // renormalise: pl (up to 2^-25) would otherwise dominate the
        // rounding errors of small r (fast two-sum: rh = 0 or |rh| >= 2^-24)
        const F s = crf_add(rh, pl);
        rl = crf_sub(pl, crf_sub(s, rh));
        rh = s;
    }
    F vh, vl;
    crf_log1p_dw(rh, rl, vh, vl);
    const F a1 = crf_mul(ef, crf_bc<F>(LG_CRF_LN2_HI));
    const F a1l = crf_fma(ef, crf_bc<F>(LG_CRF_LN2_HI), crf_neg(a1));
    const F a1l2 = crf_mul(ef, crf_bc<F>(LG_CRF_LN2_LO));
    const F s1 = crf_add(a1, Lh);
    const F e1 = crf_sub(Lh, crf_sub(s1, a1));
    hi = crf_add(s1, vh);
    const F e2 = crf_sub(vh, crf_sub(hi, s1));
    lo = crf_add(crf_add(e1, e2), crf_add(crf_add(a1l, a1l2), crf_add(Ll, vl)));
}

template <class F>
LG_CRF_DEV F lg_crf_log(F x)
{
    F hi, lo, z1, z2;
    crf_log_dw<F, false>(x, x, hi, lo);
    crf_ziv(hi, lo, z1, z2);
    // normal, positive, finite x with the rounding decided; zero, negative,
    // subnormal, infinite and NaN x in double
    bool ok[2];
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        const float xi = crf_get(x, i);
        ok[i] = xi >= 0x1p-126f && xi <= 0x1.fffffep127f && crf_get(z1, i) == crf_get(z2, i);
    }
    if (crf_all<F>(ok)) return z1;
    F out;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) crf_set(out, i, ok[i] ? crf_get(z1, i) : crf_slow_log(crf_get(x, i)));
    return out;
}

// --------------------------------------------------------------------- atan --
// a = |z|; t = a, or 1/a (as rcp(a) plus one Newton correction, a double
// word) for a > 1.  With t_j = j/512 nearest t, atan t = atan t_j +
// atan(delta), delta = (t - t_j) / (1 + t t_j) as a double word (numerator
// exact by Sterbenz; denominator 1 + t t_j from an exact product; quotient
// from rcp plus one correction step), |delta| <= 2^-10, atan(delta) = delta
// + delta^3 (-1/3 + delta^2/5), truncation delta^7/7 (relative 2^-62), the
// cubic term in float (relative to delta 2^-44).  For a > 1 the result is
// pi/2 - that.  Error about 2^-44.
// atan t for t = th + tl in [0, 1] (tl a few ulp of th at most) as s1 + lo.
template <class F>
LG_CRF_DEV void crf_atan_core(F th, F tl, F& s1, F& lo)
{
    F rd, Ah, Al;
    const F S = crf_bc<F>(0x1.8p23f);
    const F big = crf_fma(th, crf_bc<F>(512.0f), S);
    const F tj = crf_mul(crf_sub(big, S), crf_bc<F>(0x1p-9f));
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        int j = crf_bits(crf_get(big, i)) - 0x4b400000;
        j = j < 0 ? 0 : (j > 512 ? 512 : j);  // (in range for every finite t in [0, 1])
        const float2 A = crf_ldg(lg_crf_atan_tab + j);
        crf_set(Ah, i, A.x);
        crf_set(Al, i, A.y);
    }
    const F nh = crf_sub(th, tj);  // exact
    const F qh = crf_mul(th, tj);
    const F ql = crf_fma(th, tj, crf_neg(qh));
    const F dh = crf_add(crf_bc<F>(1.0f), qh);  // 1 >= qh: fast two-sum
    const F dl = crf_add(crf_sub(qh, crf_sub(dh, crf_bc<F>(1.0f))), crf_fma(tl, tj, ql));
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) crf_set(rd, i, crf_rcp(crf_get(dh, i)));  // dh in [1, 2]
    const F d0 = crf_mul(nh, rd);
    const F res = crf_add(crf_fma(crf_neg(d0), dh, nh), crf_fma(crf_neg(d0), dl, tl));
    const F d1 = crf_mul(res, rd);
    const F s = crf_mul(d0, d0);
    const F P = crf_fma(s, crf_bc<F>(0x1.99999ap-3f), crf_bc<F>(-0x1.555556p-2f));
    const F cub = crf_mul(crf_mul(s, d0), P);
    s1 = crf_add(Ah, d0);  // |atan t_j| >= |delta| or t_j = 0
    const F e1 = crf_sub(d0, crf_sub(s1, Ah));
    lo = crf_add(crf_add(e1, Al), crf_add(d1, cub));
}

template <class F>
LG_CRF_DEV F lg_crf_atan(F z)
{
    const F a = crf_abs(z);
    F th = a, tl = crf_bc<F>(0.0f);
    bool inv[2];
    bool any_inv = false;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        inv[i] = crf_get(a, i) > 1.0f;
        any_inv = any_inv || inv[i];
    }
    // the reciprocal and pi/2 - ... only where a lane needs them (the SIE
    // family's arguments rarely exceed 1)
    if (any_inv) {
        F r0;
#pragma unroll
        for (int i = 0; i < crf_lanes<F>::n; ++i)  // 1/a for a > 1 (a > 2^126 flushes to 0; atan is then RN(pi/2))
            crf_set(r0, i, inv[i] ? crf_rcp(crf_get(a, i)) : 1.0f);
        const F rho = crf_fma(crf_neg(r0), a, crf_bc<F>(1.0f));
        const F r1 = crf_mul(rho, r0);
#pragma unroll
        for (int i = 0; i < crf_lanes<F>::n; ++i) {
            crf_set(th, i, inv[i] ? crf_get(r0, i) : crf_get(a, i));
            crf_set(tl, i, inv[i] ? crf_get(r1, i) : 0.0f);
        }
    }
    F s1, lo;
    crf_atan_core(th, tl, s1, lo);
    F hi2 = s1, lo2 = lo;
    if (any_inv) {  // pi/2 - (s1 + lo)
        const F ph = crf_sub(crf_bc<F>(LG_CRF_PIO2_HI), s1);
        const F pe = crf_sub(crf_sub(crf_bc<F>(LG_CRF_PIO2_HI), ph), s1);
        const F plo = crf_add(pe, crf_sub(crf_bc<F>(LG_CRF_PIO2_LO), lo));
#pragma unroll
        for (int i = 0; i < crf_lanes<F>::n; ++i) {
            crf_set(hi2, i, inv[i] ? crf_get(ph, i) : crf_get(s1, i));
            crf_set(lo2, i, inv[i] ? crf_get(plo, i) : crf_get(lo, i));
        }
    }
    F z1, z2;
    crf_ziv(hi2, lo2, z1, z2);
    // finite z with the rounding decided; infinite and NaN z in double.  The
    // sign of z on |result| (z = +-0 gives +-0: the result is 0 there).
    bool ok[2];
    F out;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        const float zi = crf_get(z, i);
        ok[i] = crf_fabsf(zi) <= 0x1.fffffep127f && crf_get(z1, i) == crf_get(z2, i);
        crf_set(out, i, crf_copysignf(crf_get(z1, i), zi));
    }
    if (crf_all<F>(ok)) return out;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i)
        if (!ok[i]) crf_set(out, i, crf_slow_atan(crf_get(z, i)));
    return out;
}

// -------------------------------------------------------------------- atanh --
// atanh v = sign(v) atanh(a), a = |v| < 1, by two formulas:
//  * a <= 0.9: with t_j = j/512 nearest a, atanh a = atanh t_j +
//    atanh(delta), delta = (a - t_j) / (1 - a t_j) as a double word
//    (numerator exact; denominator from an exact product and a fast
//    two-sum, at least 0.19; quotient from rcp plus one correction step),
//    |delta| <= 2^-7.6, atanh(delta) = delta + delta^3 (1/3 + delta^2/5),
//    truncation delta^7/7 (relative 2^-48), the cubic term in float;
//    table pairs atanh t_j (2^-48).  Error about 2^-45;
//  * a > 0.9: ln(1 + w) / 2 with w = 2a / (1 - a) as a double word (1 - a
//    exact by a fast two-sum, the quotient from rcp plus one correction
//    step), 1 + w as a two-sum, then the double-word logarithm: 1 + w
//    carries about 2^-49 absolute error, 2^-46 of the result here.
// The SIE family's arguments stay below sqrt(1 - q^2), so its rays take the
// first formula unless q < 0.44; each branch runs only where a lane of the
// pair needs it.
template <class F>
LG_CRF_DEV F lg_crf_atanh(F v)
{
    const F a = crf_abs(v);
    const F one = crf_bc<F>(1.0f);
    bool tab[2];
    bool any_tab = false, any_large = false;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        tab[i] = crf_get(a, i) <= 0.9f;
        any_tab = any_tab || tab[i];
        any_large = any_large || !tab[i];
    }
    F hs = a, ls = a, hl = a, ll = a;
    if (any_tab) {
        const F S = crf_bc<F>(0x1.8p23f);
        const F big = crf_fma(a, crf_bc<F>(512.0f), S);
        const F tj = crf_mul(crf_sub(big, S), crf_bc<F>(0x1p-9f));
        F Ah, Al, rd;
#pragma unroll
        for (int i = 0; i < crf_lanes<F>::n; ++i) {
            int j = crf_bits(crf_get(big, i)) - 0x4b400000;
            j = j < 0 ? 0 : (j > 461 ? 461 : j);  // (in range for a <= 0.9; the other lanes are not used)
            const float2 A = crf_ldg(lg_crf_atanh_tab + j);
            crf_set(Ah, i, A.x);
            crf_set(Al, i, A.y);
        }
        const F nh = crf_sub(a, tj);  // exact
        const F qh = crf_mul(a, tj);
        const F ql = crf_fma(a, tj, crf_neg(qh));
        const F dh = crf_sub(one, qh);  // 1 >= qh: fast two-sum
        const F dl = crf_sub(crf_sub(crf_sub(one, dh), qh), ql);
#pragma unroll
        for (int i = 0; i < crf_lanes<F>::n; ++i) crf_set(rd, i, crf_rcp(crf_get(dh, i)));  // dh in [0.19, 1]
        const F d0 = crf_mul(nh, rd);
        const F res = crf_fma(crf_neg(d0), dl, crf_fma(crf_neg(d0), dh, nh));
        const F d1 = crf_mul(res, rd);
        const F s = crf_mul(d0, d0);
        const F P = crf_fma(s, crf_bc<F>(0x1.99999ap-3f), crf_bc<F>(0x1.555556p-2f));
        const F cub = crf_mul(crf_mul(s, d0), P);
        hs = crf_add(Ah, d0);  // |atanh t_j| >= |delta| or t_j = 0: fast two-sum
        const F e1 = crf_sub(d0, crf_sub(hs, Ah));
        ls = crf_add(crf_add(e1, Al), crf_add(d1, cub));
    }
    if (any_large) {
        const F dh = crf_sub(one, a);
        const F dl = crf_sub(crf_sub(one, dh), a);  // exact (1 >= a)
        const F n = crf_add(a, a);
        F rd;
#pragma unroll
        for (int i = 0; i < crf_lanes<F>::n; ++i) crf_set(rd, i, crf_rcp(crf_get(dh, i)));  // dh >= 2^-24
        const F w0 = crf_mul(n, rd);
        const F res = crf_fma(crf_neg(w0), dl, crf_fma(crf_neg(w0), dh, n));
        const F w1 = crf_mul(res, rd);
        // 1 + w0 (two-sum: w0 may exceed 1), + w1
        const F uh = crf_add(one, w0);
        const F bb = crf_sub(uh, one);
        const F ul = crf_add(crf_add(crf_sub(one, crf_sub(uh, bb)), crf_sub(w0, bb)), w1);
        crf_log_dw<F, true>(uh, ul, hl, ll);
        hl = crf_mul(hl, crf_bc<F>(0.5f));
        ll = crf_mul(ll, crf_bc<F>(0.5f));
    }
    F hi, lo;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        crf_set(hi, i, tab[i] ? crf_get(hs, i) : crf_get(hl, i));
        crf_set(lo, i, tab[i] ? crf_get(ls, i) : crf_get(ll, i));
    }
    F z1, z2;
    crf_ziv(hi, lo, z1, z2);
    // |v| < 1 with the rounding decided; |v| >= 1 and NaN v in double.  The
    // sign of v on |result| (v = +-0 gives +-0).
    bool ok2[2];
    F out;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i) {
        const float vi = crf_get(v, i);
        ok2[i] = crf_fabsf(vi) < 1.0f && crf_get(z1, i) == crf_get(z2, i);
        crf_set(out, i, crf_copysignf(crf_get(z1, i), vi));
    }
    if (crf_all<F>(ok2)) return out;
#pragma unroll
    for (int i = 0; i < crf_lanes<F>::n; ++i)
        if (!ok2[i]) crf_set(out, i, crf_slow_atanh(crf_get(v, i)));
    return out;
}

// ------------------------------------------------- sincos, pow, atan2 (scalar) --
// The EPL lens's functions, one value at a time (the exact render calls the
// correctly rounded functions lane by lane).

LG_CRF_DEV void crf_two_sum(float a, float b, float& s, float& e)
{
    s = crf_add(a, b);
    const float bb = crf_sub(s, a);
    e = crf_add(crf_sub(a, crf_sub(s, bb)), crf_sub(b, bb));
}

// Ziv's test with the margin |hi| 2^-40 + floor (floor: an absolute error
// bound of results near zero); z the rounded result when it holds
LG_CRF_DEV bool crf_ziv1(float hi, float lo, float floor_, float& z)
{
    const float m = crf_fma(crf_fabsf(hi), LG_CRF_ZIV, floor_);
    const float z1 = crf_add(hi, crf_add(lo, m)), z2 = crf_add(hi, crf_sub(lo, m));
    z = z1;
    return z1 == z2;
}

// sin x and cos x.  x = k pi/2 + r with k = rint(x 2/pi) (|x| <= 128, so
// |k| < 2^7) and r = ((x - k P1) - k P2) - k P3 as a double word: k P1 and
// k P2 exact (P1, P2 of 17 significant bits), the first difference exact by
// Sterbenz, the second by a two-sum, pi/2 - P1 - P2 - P3 below 2^-59, so
// |error| <= 2^-51 (none for k = 0).  r = a + s with a = j/256 nearest r
// (s exact, |s| <= 2^-9): sin r = sin a cos s + cos a sin s, cos r = cos a
// cos s - sin a sin s with sin a, cos a as table pairs (2^-48), sin s = s -
// s^3/6 + s^5/120 (truncation 2^-65), cos s - 1 = -s^2/2 + s^4/24 - s^6/720
// with s^2 exact; the leading products exact (fma), the sums by two-sums.
// Relative error about 2^-46 plus the reduction's 2^-51 absolute: the
// rounding test takes an absolute floor of 2^-46 when k != 0.  |x| > 128,
// infinite and NaN x, and undecided roundings in double.
LG_CRF_DEV void lg_crf_sincos(float x, float* sp, float* cp)
{
    const bool inr = crf_fabsf(x) <= 128.0f;
    const float xr = inr ? x : 0.0f;
    const float S = 0x1.8p23f;
    const float big = crf_fma(xr, LG_CRF_INV_PIO2, S);
    const float kf = crf_sub(big, S);
    const int k = crf_bits(big) - 0x4b400000;
    const float r1 = crf_fma(-kf, LG_CRF_PIO2_1, xr);  // exact
    float rh, e;
    crf_two_sum(r1, crf_mul(-kf, LG_CRF_PIO2_2), rh, e);
    const float rl = crf_fma(-kf, LG_CRF_PIO2_3, e);
    const float bj = crf_fma(rh, 256.0f, S);
    const int j = crf_bits(bj) - 0x4b400000;  // |j| <= 201
    const float a = crf_mul(crf_sub(bj, S), 0x1p-8f);
    const float s0 = crf_sub(rh, a);  // exact
    const float4 T = crf_ldg(lg_crf_sc_tab + (j + 201));
    const float sah = T.x, sal = T.y, cah = T.z, cal = T.w;
    // sin s = s0 + Sl; cos s - 1 = Ch + Cl
    const float s2 = crf_mul(s0, s0);
    const float s2l = crf_fma(crf_add(s0, s0), rl, crf_fma(s0, s0, -s2));
    const float Sl = crf_fma(crf_mul(s2, s0), crf_fma(s2, 0x1.111112p-7f, -0x1.555556p-3f), rl);
    const float Ch = crf_mul(s2, -0.5f);  // exact
    const float Cl = crf_fma(crf_mul(s2, s2), crf_fma(s2, -0x1.6c16c2p-10f, 0x1.555556p-5f), crf_mul(s2l, -0.5f));
    // sin r = sa + ca s0 + sa Ch + (sa Cl + ca Sl + cal s0 + sal)
    const float p1 = crf_mul(cah, s0), e1 = crf_fma(cah, s0, -p1);
    const float p2 = crf_mul(sah, Ch), e2 = crf_fma(sah, Ch, -p2);
    float u, eu;
    crf_two_sum(sah, p1, u, eu);
    const float sh = crf_add(u, p2);  // |u| >= |p2|: fast two-sum
    const float ev = crf_sub(p2, crf_sub(sh, u));
    const float sl = crf_add(crf_add(ev, eu),
                             crf_add(crf_add(e1, e2), crf_fma(sah, Cl, crf_fma(cah, Sl, crf_fma(cal, s0, sal)))));
    // cos r = ca - sa s0 + ca Ch + (ca Cl - sa Sl - sal s0 + cal)
    const float p3 = crf_mul(sah, s0), e3 = crf_fma(sah, s0, -p3);
    const float p4 = crf_mul(cah, Ch), e4 = crf_fma(cah, Ch, -p4);
    float u2, eu2;
    crf_two_sum(cah, -p3, u2, eu2);
    const float ch = crf_add(u2, p4);  // |u2| >= 1/2 >= |p4|: fast two-sum
    const float ev2 = crf_sub(p4, crf_sub(ch, u2));
    const float cl = crf_add(crf_add(ev2, eu2),
                             crf_add(crf_sub(e4, e3), crf_fma(cah, Cl, crf_fma(-sah, Sl, crf_fma(-sal, s0, cal)))));
    // quadrant: sin x = (sin r, cos r, -sin r, -cos r)[k & 3], cos x = (cos r,
    // -sin r, -cos r, sin r)[k & 3]
    const int q = k & 3;
    const bool swap = q & 1, sneg = q >= 2, cneg = q == 1 || q == 2;
    float xsh = swap ? ch : sh, xsl = swap ? cl : sl, xch = swap ? sh : ch, xcl = swap ? sl : cl;
    if (sneg) {
        xsh = -xsh;
        xsl = -xsl;
    }
    if (cneg) {
        xch = -xch;
        xcl = -xcl;
    }
    const float fl = k != 0 ? 0x1p-46f : 0.0f;
    float zs, zc;
    const bool oks = crf_ziv1(xsh, xsl, fl, zs) && inr, okc = crf_ziv1(xch, xcl, fl, zc) && inr;
    *sp = oks ? (x == 0.0f ? x : zs) : crf_slow_sin(x);  // (sin of -0 is -0)
    *cp = okc ? zc : crf_slow_cos(x);
}

// x^y = e^(y ln x): ln x as a double word (crf_log_dw, relative error below
// 2^-42), t = y ln x as a double word (the product exact by an fma), e^t
// from the exp tail with the low part of t added to the reduced argument by
// a two-sum.  Relative error below about |t| 2^-42 + 2^-42, so the rounding
// test's margin grows with |t|.  Positive normal x with t in [-87, 88] (a
// normal result) and the rounding decided; everything else in double.
LG_CRF_DEV float lg_crf_pow(float x, float y)
{
    const bool xin = x >= 0x1p-126f && x <= 0x1.fffffep127f;
    const float xr = xin ? x : 1.0f;
    float lh, ll;
    crf_log_dw<float, false>(xr, xr, lh, ll);
    const float th = crf_mul(y, lh);
    const float tl = crf_fma(y, ll, crf_fma(y, lh, -th));
    const bool tin = th >= -87.0f && th <= 88.0f;  // (false for NaN)
    const float t = tin ? th : 0.0f, tlo = tin ? tl : 0.0f;
    const float S = 0x1.8p23f;
    const float big = crf_fma(t, LG_CRF_EXP_INVL, S);
    const float kf = crf_sub(big, S);
    const float r0 = crf_fma(-kf, LG_CRF_EXP_LHI, t);  // exact
    float rh, e;
    crf_two_sum(r0, tlo, rh, e);
    const float rl = crf_fma(-kf, LG_CRF_EXP_LLO, e);
    float yh, yl;
    int m[2];
    crf_exp_tail(big, rh, rl, yh, yl, m);
    const float mrel = crf_fma(crf_fabsf(t), 0x1p-41f, LG_CRF_ZIV);
    const float mg = crf_mul(crf_fabsf(yh), mrel);
    const float z1 = crf_add(yh, crf_add(yl, mg)), z2 = crf_add(yh, crf_sub(yl, mg));
    if (xin && tin && z1 == z2) return crf_from_bits(crf_add_exp(crf_bits(z1), m[0]));
    return crf_slow_pow(x, y);
}

// atan2(y, x): q = min(|x|, |y|) / max(|x|, |y|) in [0, 1] as a double word
// (rcp plus one correction step, relative error 2^-46), atan q from the atan
// core, then pi/2 - that where |y| > |x| and pi - that where x < 0 (double-
// word constants; fast two-sums, the constant being the larger), the sign
// of y.  Relative error about 2^-44.  min(|x|, |y|) >= 2^-100, max(|x|, |y|)
// < 2^126, a quotient above 2^-100 (so the result is normal) and the
// rounding decided; zeros, infinities, NaN, tiny or huge arguments and the
// rest in double.
LG_CRF_DEV float lg_crf_atan2(float y, float x)
{
    const float ax = crf_fabsf(x), ay = crf_fabsf(y);
    const bool swap = ay > ax;
    float num = swap ? ax : ay, den = swap ? ay : ax;
    // the quotient's remainder exact (no underflow: num >= 2^-100), the
    // reciprocal normal (den < 2^126) and the quotient above 2^-100
    const bool in = den < 0x1p126f && num >= 0x1p-100f && num >= crf_mul(den, 0x1p-100f);
    if (!in) {
        num = 1.0f;
        den = 1.0f;
    }
    const float rd = crf_rcp(den);
    const float q0 = crf_mul(num, rd);
    const float res = crf_fma(-q0, den, num);  // exact
    const float q1 = crf_mul(res, rd);
    float s1, lo;
    crf_atan_core(q0, q1, s1, lo);
    float hi = s1;
    if (swap) {  // pi/2 - (s1 + lo)
        const float ph = crf_sub(LG_CRF_PIO2_HI, s1);
        const float pe = crf_sub(crf_sub(LG_CRF_PIO2_HI, ph), s1);
        lo = crf_add(pe, crf_sub(LG_CRF_PIO2_LO, lo));
        hi = ph;
    }
    if (x < 0.0f) {  // pi - (hi + lo)
        const float PIH = crf_mul(LG_CRF_PIO2_HI, 2.0f), PIL = crf_mul(LG_CRF_PIO2_LO, 2.0f);
        const float ph = crf_sub(PIH, hi);
        const float pe = crf_sub(crf_sub(PIH, ph), hi);
        lo = crf_add(pe, crf_sub(PIL, lo));
        hi = ph;
    }
    float z;
    if (in && crf_ziv1(hi, lo, 0.0f, z)) return crf_copysignf(z, y);
    return crf_slow_atan2(y, x);
}
