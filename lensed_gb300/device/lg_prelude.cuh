// Device prelude of the composed likelihood program (compiled by NVRTC for
// sm_103a together with the object plugins and the generated model).
//
// It provides the vocabulary the plugins are written in: float2 arithmetic,
// the 2x2 matrix type and its product (kernel/constants.cl:23-35), the
// OpenCL-style vector helpers dot/length/normalize, and the constants of
// kernel/constants.cl:6-13.  Arithmetic is IEEE single precision; the fast
// mode's build enables FMA contraction and hardware-approximate division and
// square root, the exact and strict modes' builds neither.

#define LG_LENS 'L'
#define LG_SOURCE 'S'
#define LG_FOREGROUND 'F'

#define LG_PI 3.14159265358979323846f
#define LG_PI_HALF 1.57079632679489661923f
#define LG_DEG2RAD 0.0174532925199432957692f
#define LG_LOG_10 2.30258509299404568402f
#define LG_LOG_PI 1.14472988584940017414f
#define LG_LOG_2PI 1.83787706640934548356f

#ifdef LG_HOST_SET
#define LG_INF HUGE_VALF
#else
#define LG_INF __int_as_float(0x7f800000)
#endif

#ifdef LG_HOST_SET
// the scalar part below, compiled for the host (small batches' set_params)
#define LG_DEV static inline
#define LG_DEV_MEMBER inline
#else
#define LG_DEV static __device__ __forceinline__
#define LG_DEV_MEMBER __device__ __forceinline__
#endif

LG_DEV float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
LG_DEV float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
LG_DEV float2 operator-(float2 a) { return make_float2(-a.x, -a.y); }
LG_DEV float2 operator*(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
LG_DEV float2 operator*(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
LG_DEV float2 operator*(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
LG_DEV float2 operator/(float2 a, float s) { return make_float2(a.x / s, a.y / s); }
LG_DEV float2& operator+=(float2& a, float2 b) { a = a + b; return a; }
LG_DEV float2& operator-=(float2& a, float2 b) { a = a - b; return a; }
LG_DEV float2& operator*=(float2& a, float s) { a = s * a; return a; }

LG_DEV float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
LG_DEV float length(float2 a) { return sqrtf(dot(a, a)); }
// OpenCL normalize(): a zero vector is returned unchanged.
LG_DEV float2 normalize(float2 a)
{
    float l = length(a);
    return l == 0.0f ? a : make_float2(a.x / l, a.y / l);
}

// 2x2 matrix with rows (a, b) and (c, d).
struct mat22 {
    float a, b, c, d;
};
LG_DEV mat22 make_mat22(float a, float b, float c, float d)
{
    mat22 m;
    m.a = a; m.b = b; m.c = c; m.d = d;
    return m;
}
LG_DEV mat22 operator*(float s, mat22 m) { return make_mat22(s * m.a, s * m.b, s * m.c, s * m.d); }
LG_DEV mat22 operator/(mat22 m, float s) { return make_mat22(m.a / s, m.b / s, m.c / s, m.d / s); }
// matrix-vector product: (dot(row0, v), dot(row1, v))
LG_DEV float2 mv22(mat22 m, float2 v) { return make_float2(m.a * v.x + m.b * v.y, m.c * v.x + m.d * v.y); }

// Correctly rounded single-precision elementary functions: evaluated in
// double precision and rounded once to float.  set_params always uses them
// (and strict mode uses them per ray), so that the FP32 result is defined by
// IEEE arithmetic alone and not by a particular float math library.
LG_DEV float lg_cr_expf(float x) { return (float)exp((double)x); }
LG_DEV float lg_cr_exp2f(float x) { return (float)exp2((double)x); }
LG_DEV float lg_cr_expm1f(float x) { return (float)expm1((double)x); }
LG_DEV float lg_cr_logf(float x) { return (float)log((double)x); }
LG_DEV float lg_cr_log2f(float x) { return (float)log2((double)x); }
LG_DEV float lg_cr_log10f(float x) { return (float)log10((double)x); }
LG_DEV float lg_cr_log1pf(float x) { return (float)log1p((double)x); }
LG_DEV float lg_cr_powf(float x, float y) { return (float)pow((double)x, (double)y); }
LG_DEV float lg_cr_sinf(float x) { return (float)sin((double)x); }
LG_DEV float lg_cr_cosf(float x) { return (float)cos((double)x); }
LG_DEV float lg_cr_tanf(float x) { return (float)tan((double)x); }
LG_DEV void lg_cr_sincosf(float x, float* s, float* c)
{
    *s = (float)sin((double)x);
    *c = (float)cos((double)x);
}
LG_DEV float lg_cr_asinf(float x) { return (float)asin((double)x); }
LG_DEV float lg_cr_acosf(float x) { return (float)acos((double)x); }
LG_DEV float lg_cr_atanf(float x) { return (float)atan((double)x); }
LG_DEV float lg_cr_atan2f(float y, float x) { return (float)atan2((double)y, (double)x); }
LG_DEV float lg_cr_sinhf(float x) { return (float)sinh((double)x); }
LG_DEV float lg_cr_coshf(float x) { return (float)cosh((double)x); }
LG_DEV float lg_cr_tanhf(float x) { return (float)tanh((double)x); }
LG_DEV float lg_cr_asinhf(float x) { return (float)asinh((double)x); }
LG_DEV float lg_cr_acoshf(float x) { return (float)acosh((double)x); }
LG_DEV float lg_cr_atanhf(float x) { return (float)atanh((double)x); }
LG_DEV float lg_cr_tgammaf(float x) { return (float)tgamma((double)x); }
LG_DEV float lg_cr_lgammaf(float x) { return (float)lgamma((double)x); }
LG_DEV float lg_cr_cbrtf(float x) { return (float)cbrt((double)x); }
LG_DEV float lg_cr_erff(float x) { return (float)erf((double)x); }
LG_DEV float lg_cr_erfcf(float x) { return (float)erfc((double)x); }

// Apply a lens plane's summed deflection to a ray if it is finite; rays with
// a non-finite deflection are sent far away (src/kernel.c:86-91).
LG_DEV void lg_deflect(float2& y, float2 a)
{
    y -= (dot(a, a) < LG_INF) ? a : make_float2(1E10f, 1E10f);
}

#ifndef LG_HOST_SET
// ------------------------------------------------------------ ray pairs --
// The evaluation modules of the fast and exact modes trace two rays per
// thread at once with Blackwell's paired single-precision instructions
// (add/mul/fma on f32x2): lg_pair holds the value of one scalar for both
// rays, lg_pair2 a 2-vector for both rays.  Each lane is computed exactly as
// the scalar code of the same mode computes it (the same IEEE operations; a
// product followed by a sum is fused into one fma in the fast mode, as its
// scalar build contracts it, and rounded before the sum in the exact mode).
// The plugins' evaluation functions are templates over the vector type V
// (float2 or lg_pair2) and are written once for both.
struct lg_pair {
    float2 v;  // (ray 0, ray 1)
};
// Paired single-precision add, multiply and fma.  In the exact modules a
// product must be rounded before the sum that uses it; with CUDA 13.0 the
// assembler fused an f32x2 multiply into the following f32x2 add (the
// intrinsics and explicit-rounding PTX alike, also without contraction
// enabled), while scalar round-to-nearest multiplies are never fused.  So
// the exact modules multiply lane by lane (__fmul_rn) and keep the paired
// add and fma; the fast modules use the paired intrinsics throughout.
#ifdef LG_EXACT
LG_DEV float2 lg_mul2(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
#else
LG_DEV float2 lg_mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
#endif
LG_DEV float2 lg_add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
LG_DEV float2 lg_fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// a + b c for a pending product: fused into one fma in the fast mode (as
// the scalar build contracts it); in the exact mode (LG_EXACT) the product
// is rounded first, as the reference's operation order without contraction
#ifdef LG_EXACT
LG_DEV float2 lg_pp_fma(float2 b, float2 c, float2 a) { return lg_add2(lg_mul2(b, c), a); }
#else
LG_DEV float2 lg_pp_fma(float2 b, float2 c, float2 a) { return lg_fma2(b, c, a); }
#endif
// a pending product a * b, fused into an fma by a following + or -
struct lg_pair_prod {
    float2 a, b;
    LG_DEV_MEMBER operator lg_pair() const { return lg_pair{lg_mul2(a, b)}; }
};
struct lg_pair2 {
    lg_pair x, y;
};
struct lg_pair_mat22 {
    lg_pair a, b, c, d;
};

LG_DEV float2 lg_bc(float s) { return make_float2(s, s); }
LG_DEV lg_pair lg_pair_of(float s) { return lg_pair{lg_bc(s)}; }
LG_DEV lg_pair lg_pair_of(float a, float b) { return lg_pair{make_float2(a, b)}; }
LG_DEV lg_pair lg_mat(lg_pair p) { return p; }
LG_DEV lg_pair lg_mat(lg_pair_prod p) { return p; }
LG_DEV float2 lg_neg2(float2 a) { return make_float2(-a.x, -a.y); }

// products
LG_DEV lg_pair_prod operator*(lg_pair a, lg_pair b) { return {a.v, b.v}; }
LG_DEV lg_pair_prod operator*(float a, lg_pair b) { return {lg_bc(a), b.v}; }
LG_DEV lg_pair_prod operator*(lg_pair a, float b) { return {a.v, lg_bc(b)}; }
LG_DEV lg_pair_prod operator*(lg_pair_prod a, lg_pair b) { return {lg_mul2(a.a, a.b), b.v}; }
LG_DEV lg_pair_prod operator*(lg_pair a, lg_pair_prod b) { return {a.v, lg_mul2(b.a, b.b)}; }
LG_DEV lg_pair_prod operator*(lg_pair_prod a, float b) { return {lg_mul2(a.a, a.b), lg_bc(b)}; }
LG_DEV lg_pair_prod operator*(float a, lg_pair_prod b) { return {lg_bc(a), lg_mul2(b.a, b.b)}; }
LG_DEV lg_pair_prod operator*(lg_pair_prod a, lg_pair_prod b) { return {lg_mul2(a.a, a.b), lg_mul2(b.a, b.b)}; }
// sums and differences (a product on either side is fused)
LG_DEV lg_pair operator+(lg_pair a, lg_pair b) { return {lg_add2(a.v, b.v)}; }
LG_DEV lg_pair operator+(lg_pair a, float b) { return {lg_add2(a.v, lg_bc(b))}; }
LG_DEV lg_pair operator+(float a, lg_pair b) { return {lg_add2(lg_bc(a), b.v)}; }
LG_DEV lg_pair operator+(lg_pair_prod p, lg_pair c) { return {lg_pp_fma(p.a, p.b, c.v)}; }
LG_DEV lg_pair operator+(lg_pair c, lg_pair_prod p) { return {lg_pp_fma(p.a, p.b, c.v)}; }
LG_DEV lg_pair operator+(lg_pair_prod p, float c) { return {lg_pp_fma(p.a, p.b, lg_bc(c))}; }
LG_DEV lg_pair operator+(float c, lg_pair_prod p) { return {lg_pp_fma(p.a, p.b, lg_bc(c))}; }
LG_DEV lg_pair operator+(lg_pair_prod p, lg_pair_prod q) { return {lg_pp_fma(p.a, p.b, lg_mul2(q.a, q.b))}; }
LG_DEV lg_pair operator-(lg_pair a) { return {lg_neg2(a.v)}; }
LG_DEV lg_pair_prod operator-(lg_pair_prod p) { return {lg_neg2(p.a), p.b}; }
LG_DEV lg_pair operator-(lg_pair a, lg_pair b) { return {lg_fma2(b.v, lg_bc(-1.0f), a.v)}; }
LG_DEV lg_pair operator-(lg_pair a, float b) { return {lg_add2(a.v, lg_bc(-b))}; }
LG_DEV lg_pair operator-(float a, lg_pair b) { return {lg_fma2(b.v, lg_bc(-1.0f), lg_bc(a))}; }
LG_DEV lg_pair operator-(lg_pair_prod p, lg_pair c) { return {lg_pp_fma(p.a, p.b, lg_neg2(c.v))}; }
LG_DEV lg_pair operator-(lg_pair c, lg_pair_prod p) { return {lg_pp_fma(lg_neg2(p.a), p.b, c.v)}; }
LG_DEV lg_pair operator-(lg_pair_prod p, float c) { return {lg_pp_fma(p.a, p.b, lg_bc(-c))}; }
LG_DEV lg_pair operator-(float c, lg_pair_prod p) { return {lg_pp_fma(lg_neg2(p.a), p.b, lg_bc(c))}; }
LG_DEV lg_pair operator-(lg_pair_prod p, lg_pair_prod q) { return {lg_pp_fma(p.a, p.b, lg_neg2(lg_mul2(q.a, q.b)))}; }
// quotients: a times the SFU reciprocal of b (PTX rcp.approx, the
// definition of div.approx: within 2 ulp for 2^-126 <= |b| <= 2^126)
LG_DEV float lg_sfu_rcp(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
LG_DEV float lg_sfu_sqrt(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
LG_DEV float lg_sfu_rsqrt(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
LG_DEV lg_pair lg_rcp(lg_pair b) { return {make_float2(lg_sfu_rcp(b.v.x), lg_sfu_rcp(b.v.y))}; }
#ifdef LG_IEEE_DIVSQRT
// the context asked for IEEE division and square root: lane by lane
LG_DEV lg_pair operator/(lg_pair a, lg_pair b) { return {make_float2(a.v.x / b.v.x, a.v.y / b.v.y)}; }
LG_DEV lg_pair operator/(lg_pair a, float b) { return {make_float2(a.v.x / b, a.v.y / b)}; }
LG_DEV lg_pair operator/(float a, lg_pair b) { return {make_float2(a / b.v.x, a / b.v.y)}; }
#else
LG_DEV lg_pair operator/(lg_pair a, lg_pair b) { return {lg_mul2(a.v, lg_rcp(b).v)}; }
LG_DEV lg_pair operator/(lg_pair a, float b) { return {lg_mul2(a.v, lg_bc(lg_sfu_rcp(b)))}; }
LG_DEV lg_pair operator/(float a, lg_pair b) { return {lg_mul2(lg_bc(a), lg_rcp(b).v)}; }
#endif
LG_DEV lg_pair operator/(lg_pair_prod a, lg_pair b) { return lg_pair(a) / b; }
LG_DEV lg_pair operator/(lg_pair_prod a, float b) { return lg_pair(a) / b; }
LG_DEV lg_pair operator/(lg_pair a, lg_pair_prod b) { return a / lg_pair(b); }
LG_DEV lg_pair operator/(float a, lg_pair_prod b) { return a / lg_pair(b); }
LG_DEV lg_pair& operator+=(lg_pair& a, lg_pair b) { a = a + b; return a; }
LG_DEV lg_pair& operator+=(lg_pair& a, lg_pair_prod b) { a = a + b; return a; }
LG_DEV lg_pair& operator-=(lg_pair& a, lg_pair b) { a = a - b; return a; }
LG_DEV lg_pair& operator*=(lg_pair& a, lg_pair b) { a = a * b; return a; }
LG_DEV lg_pair& operator*=(lg_pair& a, float b) { a = a * b; return a; }

// vectors of two rays
LG_DEV lg_pair2 operator+(lg_pair2 a, lg_pair2 b) { return {a.x + b.x, a.y + b.y}; }
LG_DEV lg_pair2 operator-(lg_pair2 a, lg_pair2 b) { return {a.x - b.x, a.y - b.y}; }
LG_DEV lg_pair2 operator+(lg_pair2 a, float2 b) { return {a.x + b.x, a.y + b.y}; }
LG_DEV lg_pair2 operator-(lg_pair2 a, float2 b) { return {a.x - b.x, a.y - b.y}; }
LG_DEV lg_pair2 operator-(lg_pair2 a) { return {-a.x, -a.y}; }
LG_DEV lg_pair2 operator*(float s, lg_pair2 a) { return {s * a.x, s * a.y}; }
LG_DEV lg_pair2 operator*(lg_pair2 a, float s) { return {a.x * s, a.y * s}; }
LG_DEV lg_pair2 operator*(lg_pair s, lg_pair2 a) { return {s * a.x, s * a.y}; }
LG_DEV lg_pair2 operator*(lg_pair2 a, lg_pair s) { return {a.x * s, a.y * s}; }
LG_DEV lg_pair2 operator*(lg_pair_prod s, lg_pair2 a) { return lg_pair(s) * a; }
LG_DEV lg_pair2 operator/(lg_pair2 a, float s) { return {a.x / s, a.y / s}; }
LG_DEV lg_pair2& operator+=(lg_pair2& a, lg_pair2 b) { a = a + b; return a; }
LG_DEV lg_pair2& operator-=(lg_pair2& a, lg_pair2 b) { a = a - b; return a; }
LG_DEV lg_pair2& operator-=(lg_pair2& a, float2 b) { a = a - b; return a; }
LG_DEV lg_pair2& operator*=(lg_pair2& a, float s) { a = s * a; return a; }
LG_DEV lg_pair2& operator*=(lg_pair2& a, lg_pair s) { a = s * a; return a; }
LG_DEV lg_pair2& operator*=(lg_pair2& a, lg_pair_prod s) { a = lg_pair(s) * a; return a; }
LG_DEV lg_pair dot(lg_pair2 a, lg_pair2 b) { return a.x * b.x + a.y * b.y; }
LG_DEV lg_pair dot(float2 a, lg_pair2 b) { return a.x * b.x + a.y * b.y; }
LG_DEV lg_pair2 mv22(mat22 m, lg_pair2 v) { return {m.a * v.x + m.b * v.y, m.c * v.x + m.d * v.y}; }
LG_DEV lg_pair_mat22 make_mat22(lg_pair a, lg_pair b, lg_pair c, lg_pair d) { return {a, b, c, d}; }
LG_DEV lg_pair2 mv22(lg_pair_mat22 m, lg_pair2 v) { return {m.a * v.x + m.b * v.y, m.c * v.x + m.d * v.y}; }
LG_DEV lg_pair2 lg_pair2_join(float2 r0, float2 r1) { return {lg_pair_of(r0.x, r1.x), lg_pair_of(r0.y, r1.y)}; }
LG_DEV float2 lg_lane(lg_pair2 a, int i) { return i ? make_float2(a.x.v.y, a.y.v.y) : make_float2(a.x.v.x, a.y.v.x); }

// SFU approximations (PTX ex2.approx / lg2.approx, subnormals flushed)
LG_DEV float lg_sfu_ex2(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
LG_DEV float lg_sfu_lg2(float x)
{
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// e^x for two rays: 2^t * 2^c with t = fl(x log2(e)) and c the rest of
// x log2(e) (the product's rounding error, exact through an fma -- Dekker's
// exact product (Dekker 1971) -- plus x times the rounding error of the
// constant, log2(e) split into two floats as in Cody and Waite's argument
// reduction (Cody & Waite 1980, "Software Manual for the Elementary
// Functions")); 2^t from the SFU, 2^c as 1 + c ln 2, the first-order term
// of its series (|c| <= 2^-24 |t|).  Within the SFU's few-ulp error of e^x;
// results below 2^-126 are flushed to zero; for |t| >= 128 (where 2^t is 0
// or overflows, and for infinite x) and NaN x the result is 2^t itself.
LG_DEV float lg_exp_pick(float t, float p, float r) { return fabsf(t) < 128.0f ? r : p; }
LG_DEV lg_pair expf(lg_pair x)
{
    const float2 L = lg_bc(0x1.715476p+0f), Llo = lg_bc(0x1.4ae0c0p-26f);
    const float2 t = lg_mul2(x.v, L);
    const float2 c = lg_fma2(x.v, Llo, lg_fma2(x.v, L, lg_neg2(t)));
    const float2 p = make_float2(lg_sfu_ex2(t.x), lg_sfu_ex2(t.y));
    const float2 r = lg_fma2(p, lg_mul2(c, lg_bc(0x1.62e430p-1f)), p);
    return {make_float2(lg_exp_pick(t.x, p.x, r.x), lg_exp_pick(t.y, p.y, r.y))};
}
LG_DEV lg_pair expf(lg_pair_prod x) { return expf(lg_pair(x)); }

// ln x for two rays: y ln 2 + (x 2^-y - 1) with y = lg2(x) from the SFU; the
// second term is one Newton step for u in e^u = x from u0 = y ln 2 (u1 = u0
// + x e^-u0 - 1, here with e^-u0 = 2^-y), which removes the error of y to
// first order, leaving an absolute error of about 2^-22 (the SFU's 2^-y).  Outside |y| < 120 (where 2^-y
// would leave the normal range), and for zero, infinite, negative or NaN x,
// the result is y ln 2 (subnormal x is flushed: -inf).
LG_DEV lg_pair logf(lg_pair x)
{
    const float2 y = make_float2(lg_sfu_lg2(x.v.x), lg_sfu_lg2(x.v.y));
    const float2 s = make_float2(lg_sfu_ex2(-y.x), lg_sfu_ex2(-y.y));
    const float2 u = lg_mul2(y, lg_bc(0x1.62e430p-1f));
    const float2 r = lg_fma2(y, lg_bc(0x1.62e430p-1f), lg_fma2(x.v, s, lg_bc(-1.0f)));
    return {make_float2(fabsf(y.x) < 120.0f ? r.x : u.x, fabsf(y.y) < 120.0f ? r.y : u.y)};
}
LG_DEV lg_pair logf(lg_pair_prod x) { return logf(lg_pair(x)); }

// other elementary functions, lane by lane (the module's float library)
#define LG_PAIR_FN1(fn) \
    LG_DEV lg_pair fn(lg_pair a) { return {make_float2(fn(a.v.x), fn(a.v.y))}; } \
    LG_DEV lg_pair fn(lg_pair_prod a) { return fn(lg_pair(a)); }
// square root and its reciprocal from the SFU (PTX sqrt.approx /
// rsqrt.approx, within 1 ulp; subnormal inputs flushed)
#ifdef LG_IEEE_DIVSQRT
LG_DEV lg_pair sqrtf(lg_pair a) { return {make_float2(sqrtf(a.v.x), sqrtf(a.v.y))}; }
#else
LG_DEV lg_pair sqrtf(lg_pair a) { return {make_float2(lg_sfu_sqrt(a.v.x), lg_sfu_sqrt(a.v.y))}; }
#endif
LG_DEV lg_pair sqrtf(lg_pair_prod a) { return sqrtf(lg_pair(a)); }
LG_DEV lg_pair rsqrtf(lg_pair a) { return {make_float2(lg_sfu_rsqrt(a.v.x), lg_sfu_rsqrt(a.v.y))}; }
LG_DEV lg_pair rsqrtf(lg_pair_prod a) { return rsqrtf(lg_pair(a)); }
LG_PAIR_FN1(exp2f)
LG_PAIR_FN1(log2f)
LG_PAIR_FN1(sinf)
LG_PAIR_FN1(cosf)
LG_PAIR_FN1(fabsf)
#undef LG_PAIR_FN1
// |a| with the sign of b, lane by lane (sign-bit operations)
LG_DEV float2 lg_copysign2(float2 a, float2 b) { return make_float2(copysignf(a.x, b.x), copysignf(a.y, b.y)); }
LG_DEV float2 lg_abs2(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }

// arctangent for two rays: r = min(|z|, 1/|z|) (SFU reciprocal), atan(r) =
// r P(r^2) with a degree-9 polynomial in r^2 fitted to atan on [0, 1] by
// device/fit_polynomials.py (weighted least squares for relative error,
// iterated towards minimax; max error 2.4e-9 in exact arithmetic, about
// 1 ulp evaluated in FP32),
// pi/2 - atan(1/|z|) for |z| > 1, and the sign of z.
LG_DEV lg_pair atanf(lg_pair z)
{
    const float2 a = lg_abs2(z.v);
    const bool b0 = a.x > 1.0f, b1 = a.y > 1.0f;
    const float2 r = make_float2(b0 ? lg_sfu_rcp(a.x) : a.x, b1 ? lg_sfu_rcp(a.y) : a.y);
    const float2 s = lg_mul2(r, r);
    float2 p = lg_bc(-0x1.cbc208p-10f);
    p = lg_fma2(p, s, lg_bc(0x1.5f7ca4p-7f));
    p = lg_fma2(p, s, lg_bc(-0x1.f8b096p-6f));
    p = lg_fma2(p, s, lg_bc(0x1.d775dep-5f));
    p = lg_fma2(p, s, lg_bc(-0x1.57220ap-4f));
    p = lg_fma2(p, s, lg_bc(0x1.c02f58p-4f));
    p = lg_fma2(p, s, lg_bc(-0x1.241596p-3f));
    p = lg_fma2(p, s, lg_bc(0x1.999082p-3f));
    p = lg_fma2(p, s, lg_bc(-0x1.555534p-2f));
    p = lg_fma2(lg_mul2(p, s), r, r);  // r + r s P'(s)
    const float2 q = lg_fma2(p, lg_bc(-1.0f), lg_bc(LG_PI_HALF));
    return {lg_copysign2(make_float2(b0 ? q.x : p.x, b1 ? q.y : p.y), z.v)};
}
LG_DEV lg_pair atanf(lg_pair_prod z) { return atanf(lg_pair(z)); }

// inverse hyperbolic tangent for two rays: for |v| <= 1/2, v Q(v^2) with a
// degree-6 polynomial fitted to atanh on [0, 1/2] by the same script (max
// error 1.3e-9 in exact arithmetic, about 1 ulp in FP32); above, ln((1 + |v|) / (1 - |v|)) / 2
// through the paired log (absolute error about 2e-7, i.e. within 4 ulp
// there); the sign of v.  |v| = 1 gives inf, |v| > 1 NaN.
// The two branches are taken only when a lane of the thread needs them:
// neighbouring rays mostly fall on the same side of 1/2, so whole warps skip
// the branch they do not need.
LG_DEV lg_pair atanhf(lg_pair v)
{
    const float2 a = lg_abs2(v.v);
    const bool small0 = a.x <= 0.5f, small1 = a.y <= 0.5f;
    float2 p = a, h = a;
    if (small0 || small1) {
        const float2 s = lg_mul2(a, a);
        p = lg_bc(0x1.6dad62p-3f);
        p = lg_fma2(p, s, lg_bc(0x1.986234p-5f));
        p = lg_fma2(p, s, lg_bc(0x1.e6379cp-4f));
        p = lg_fma2(p, s, lg_bc(0x1.2323c0p-3f));
        p = lg_fma2(p, s, lg_bc(0x1.99a96cp-3f));
        p = lg_fma2(p, s, lg_bc(0x1.555534p-2f));
        p = lg_fma2(lg_mul2(p, s), a, a);  // a + a s Q'(s)
    }
    if (!(small0 && small1)) {
        const float2 num = lg_add2(lg_bc(1.0f), a);
        const float2 den = lg_fma2(a, lg_bc(-1.0f), lg_bc(1.0f));
        const lg_pair l = logf(lg_pair{lg_mul2(num, make_float2(lg_sfu_rcp(den.x), lg_sfu_rcp(den.y)))});
        h = lg_mul2(l.v, lg_bc(0.5f));
    }
    return {lg_copysign2(make_float2(small0 ? p.x : h.x, small1 ? p.y : h.y), v.v)};
}
LG_DEV lg_pair atanhf(lg_pair_prod v) { return atanhf(lg_pair(v)); }

// a^b for two rays and a >= 0 (the plugins' radial power laws): exp(b ln a)
// through the paired exp and log (a few ulp; b = 0 gives 1, as powf);
// negative a falls back to the library per lane
LG_DEV lg_pair powf(lg_pair a, float b)
{
    const lg_pair r = expf(b * logf(a));
    return {make_float2(b == 0.0f ? 1.0f : (a.v.x < 0.0f ? powf(a.v.x, b) : r.v.x),
                        b == 0.0f ? 1.0f : (a.v.y < 0.0f ? powf(a.v.y, b) : r.v.y))};
}
LG_DEV lg_pair powf(lg_pair a, lg_pair b) { return {make_float2(powf(a.v.x, b.v.x), powf(a.v.y, b.v.y))}; }
LG_DEV lg_pair atan2f(lg_pair y, lg_pair x) { return {make_float2(atan2f(y.v.x, x.v.x), atan2f(y.v.y, x.v.y))}; }
LG_DEV void sincosf(lg_pair a, lg_pair* s, lg_pair* c)
{
    sincosf(a.v.x, &s->v.x, &c->v.x);
    sincosf(a.v.y, &s->v.y, &c->v.y);
}
LG_DEV lg_pair length(lg_pair2 a) { return sqrtf(dot(a, a)); }
// OpenCL normalize(), lane by lane: a zero vector is returned unchanged
LG_DEV lg_pair2 normalize(lg_pair2 a)
{
    const lg_pair l = length(a);
    const float2 r0 = lg_lane(a, 0), r1 = lg_lane(a, 1);
    return lg_pair2_join(l.v.x == 0.0f ? r0 : make_float2(r0.x / l.v.x, r0.y / l.v.x),
                         l.v.y == 0.0f ? r1 : make_float2(r1.x / l.v.y, r1.y / l.v.y));
}
LG_DEV void lg_deflect(lg_pair2& y, lg_pair2 a)
{
    const lg_pair d = dot(a, a);
    const float2 a0 = d.v.x < LG_INF ? lg_lane(a, 0) : make_float2(1E10f, 1E10f);
    const float2 a1 = d.v.y < LG_INF ? lg_lane(a, 1) : make_float2(1E10f, 1E10f);
    y -= lg_pair2_join(a0, a1);
}

// Polar angles of a plugin's frame for two rays: r = |x|, (c, s) = (cos,
// sin) of phi = atan2(x.y, x.x) and (c2, s2) of 2 phi, from the coordinates:
// c = x/r, s = y/r, c2 = c^2 - s^2, s2 = 2 s c (the values of the
// reference's atan2 and sincos to within rounding), phi = 0 at the origin.
// The one-ray version, which follows the reference's calls, sits with the
// plugin that uses it (after the strict mode's function mapping).
#ifndef LG_EXACT
LG_DEV void lg_polar(lg_pair2 x, lg_pair* r, lg_pair* c, lg_pair* s, lg_pair* c2, lg_pair* s2)
{
    *r = length(x);
    const lg_pair ir = 1.0f / *r;
    lg_pair cc = x.x * ir, ss = x.y * ir;
    if (!(r->v.x > 0.0f)) { cc.v.x = 1.0f; ss.v.x = 0.0f; }
    if (!(r->v.y > 0.0f)) { cc.v.y = 1.0f; ss.v.y = 0.0f; }
    *c = cc;
    *s = ss;
    *c2 = cc * cc - ss * ss;
    *s2 = 2.0f * ss * cc;
}
#endif  // LG_EXACT (the exact modules follow the reference's atan2 and sincos, objects/epl.cuh)

#endif  // LG_HOST_SET

// scalar type of a plugin's vector type
template <class V> struct lg_scalar_of;
template <> struct lg_scalar_of<float2> { typedef float type; };
#ifndef LG_HOST_SET
template <> struct lg_scalar_of<lg_pair2> { typedef lg_pair type; };
#endif
#define LG_SCALAR(V) typename lg_scalar_of<V>::type
