// Device prelude of the composed likelihood program (compiled by NVRTC for
// sm_103a together with the object plugins and the generated model).
//
// It provides the vocabulary the plugins are written in: float2 arithmetic,
// the 2x2 matrix type and its product (kernel/constants.cl:23-35), the
// OpenCL-style vector helpers dot/length/normalize, and the constants of
// kernel/constants.cl:6-13.  Arithmetic is IEEE single precision with
// correctly rounded division and square root; the build enables FMA
// contraction unless the context asks for strict parity mode.

#define LG_LENS 'L'
#define LG_SOURCE 'S'
#define LG_FOREGROUND 'F'

#define LG_PI 3.14159265358979323846f
#define LG_PI_HALF 1.57079632679489661923f
#define LG_DEG2RAD 0.0174532925199432957692f
#define LG_LOG_10 2.30258509299404568402f
#define LG_LOG_PI 1.14472988584940017414f
#define LG_LOG_2PI 1.83787706640934548356f

#define LG_INF __int_as_float(0x7f800000)

#define LG_DEV static __device__ __forceinline__

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
