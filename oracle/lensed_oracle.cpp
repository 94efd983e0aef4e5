// CPU oracle for the Lensed likelihood hot path -- TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++, the arithmetic of Lensed v1.3.2's
// likelihood path so that the CUDA implementation in lensed_gb300/ can be
// checked against it.  It is used by tests/, by the smoke check and by the
// CPU-baseline leg of bench.py; the product never links or calls it.
//
// Everything is templated on the scalar type:
//   * T = float  -> the FP32 oracle: same operation order as the reference's
//     OpenCL C, IEEE single precision, no FMA contraction (built with
//     -ffp-contract=off), libm float functions.
//   * T = double -> the FP64 oracle: the same formulas evaluated in double
//     precision with double constants and double parameters, used to state
//     the error of the FP32 paths.
//
// Reference files restated here (paths within the Lensed source tree):
//   objects/*.cl           lens / source / foreground plugins
//   kernel/constants.cl    constants, mat22 and mv22
//   kernel/lensed.cl       render (:9-39), loglike (:41-55), convolve (:56-103)
//   src/kernel.c           generated compute() (:65-111, :235-399) and
//                          set_params (:114-150, :401-656)
//   src/nested.c           host chi^2 sum and logL (:101-115)
//   src/lensed.c           pcs shift for even PSFs (:884-891)
//   src/data.c             PSF normalisation (:354-370), weights (:314-330)
//   src/quadrature.c       abscissa scaling (:32-43)

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- vectors --
// float2 / mat22 of kernel/constants.cl:23-35.  mat22 rows are (a,b) and
// (c,d); mv22(m, v) = (dot(m.lo, v), dot(m.hi, v)).
template <class T> struct V2 { T x, y; };
template <class T> struct M22 { T a, b, c, d; };

template <class T> inline V2<T> operator+(V2<T> u, V2<T> v) { return {u.x + v.x, u.y + v.y}; }
template <class T> inline V2<T> operator-(V2<T> u, V2<T> v) { return {u.x - v.x, u.y - v.y}; }
template <class T> inline V2<T> operator*(T s, V2<T> v) { return {s * v.x, s * v.y}; }
template <class T> inline V2<T> operator*(V2<T> u, V2<T> v) { return {u.x * v.x, u.y * v.y}; }
template <class T> inline T dot(V2<T> u, V2<T> v) { return u.x * v.x + u.y * v.y; }
template <class T> inline T length(V2<T> v) { return std::sqrt(dot(v, v)); }
// OpenCL normalize(): a zero vector is returned unchanged.
template <class T> inline V2<T> normalize(V2<T> v)
{
    T l = length(v);
    if (l == T(0)) return v;
    return {v.x / l, v.y / l};
}
template <class T> inline V2<T> mv22(M22<T> m, V2<T> v) { return {m.a * v.x + m.b * v.y, m.c * v.x + m.d * v.y}; }
template <class T> inline M22<T> operator*(T s, M22<T> m) { return {s * m.a, s * m.b, s * m.c, s * m.d}; }
template <class T> inline M22<T> operator/(M22<T> m, T s) { return {m.a / s, m.b / s, m.c / s, m.d / s}; }

// --------------------------------------------------------------- constants --
// kernel/constants.cl:6-13 (single-precision literals) and the plugins' own
// constants (objects/devauc.cl:1-4).  The FP64 oracle uses the same decimal
// expansions in double precision.
template <class T> struct K;
template <> struct K<float> {
    static constexpr float PI = 3.1415926535897932384626433832795028841971693993751f;
    static constexpr float DEG2RAD = 0.0174532925199432957692369076848861271344287188854f;
    static constexpr float LOG_10 = 2.3025850929940456840179914546843642076011014886288f;
    static constexpr float LOG_PI = 1.1447298858494001741434273513530587116472948129153f;
    static constexpr float DEVAUC_B = 7.6692494425008039044f;
    static constexpr float DEVAUC_C = 296.826303766893f;
    static constexpr float HUGEV = HUGE_VALF;
    static constexpr float FARV = 1E10f;
};
template <> struct K<double> {
    static constexpr double PI = 3.1415926535897932384626433832795028841971693993751;
    static constexpr double DEG2RAD = 0.0174532925199432957692369076848861271344287188854;
    static constexpr double LOG_10 = 2.3025850929940456840179914546843642076011014886288;
    static constexpr double LOG_PI = 1.1447298858494001741434273513530587116472948129153;
    static constexpr double DEVAUC_B = 7.6692494425008039044;
    static constexpr double DEVAUC_C = 296.826303766893;
    static constexpr double HUGEV = HUGE_VAL;
    static constexpr double FARV = 1E10;
};

// ------------------------------------------------------------------ plugins --
enum Kind { LENS = 'L', SOURCE = 'S', FOREGROUND = 'F' };
enum ParType { PARAMETER = 0, POSITION_X, POSITION_Y, RADIUS, MAGNITUDE, AXIS_RATIO, POS_ANGLE };

// Per-object data.  One struct for all plugins (the oracle does not need the
// reference's packed layout); each plugin uses the fields it names.
template <class T> struct Obj {
    V2<T> x;          // position
    M22<T> m, w, g, t;
    T q2, e, d, r, rc, r2, tt, f, n;
    T rs, norm, s2, log0, log1, mexp, bg;
    V2<T> grad;
};

// A decimal literal as the reference writes it: the float literal for the
// FP32 oracle, the same decimal in double precision for the FP64 oracle.
template <class T> inline T lit(float f, double d) { return sizeof(T) == 4 ? T(f) : T(d); }

// Elementary functions.  CR: evaluated in double precision and rounded
// once to T (correctly rounded except within a double ulp of a float
// rounding boundary); LM: the C library's function in T itself.  set_params
// always uses CR; the per-ray evaluation uses CR in strict mode (the same
// semantics as the GPU's strict mode) and LM otherwise.
template <class T> struct CR {
    static T exp(T x) { return T(std::exp((double)x)); }
    static T log(T x) { return T(std::log((double)x)); }
    static T pow(T x, T y) { return T(std::pow((double)x, (double)y)); }
    static T sin(T x) { return T(std::sin((double)x)); }
    static T cos(T x) { return T(std::cos((double)x)); }
    static T atan(T x) { return T(std::atan((double)x)); }
    static T atanh(T x) { return T(std::atanh((double)x)); }
    static T atan2(T y, T x) { return T(std::atan2((double)y, (double)x)); }
    static T tgamma(T x) { return T(std::tgamma((double)x)); }
};
int g_cr_eval = 1;
template <class T> struct EM {
    static T exp(T x) { return g_cr_eval ? CR<T>::exp(x) : std::exp(x); }
    static T log(T x) { return g_cr_eval ? CR<T>::log(x) : std::log(x); }
    static T pow(T x, T y) { return g_cr_eval ? CR<T>::pow(x, y) : std::pow(x, y); }
    static T sin(T x) { return g_cr_eval ? CR<T>::sin(x) : std::sin(x); }
    static T cos(T x) { return g_cr_eval ? CR<T>::cos(x) : std::cos(x); }
    static T atan(T x) { return g_cr_eval ? CR<T>::atan(x) : std::atan(x); }
    static T atanh(T x) { return g_cr_eval ? CR<T>::atanh(x) : std::atanh(x); }
    static T atan2(T y, T x) { return g_cr_eval ? CR<T>::atan2(y, x) : std::atan2(y, x); }
};

template <class T> using DeflFn = V2<T> (*)(const Obj<T>&, V2<T>);
template <class T> using BrightFn = T (*)(const Obj<T>&, V2<T>);
template <class T> using SetFn = void (*)(Obj<T>&, const T*);

// objects/sis.cl:19-32
template <class T> V2<T> defl_sis(const Obj<T>& o, V2<T> x) { return o.r * normalize(x - o.x); }
template <class T> void set_sis(Obj<T>& o, const T* p) { o.x = {p[0], p[1]}; o.r = p[2]; }

// objects/sis_plus_shear.cl:21-40
template <class T> V2<T> defl_sis_plus_shear(const Obj<T>& o, V2<T> x)
{
    x = x - o.x;
    return o.r * normalize(x) + mv22(o.g, x);
}
template <class T> void set_sis_plus_shear(Obj<T>& o, const T* p)
{
    o.x = {p[0], p[1]};
    o.r = p[2];
    o.g = {p[3], p[4], p[4], -p[3]};
}

// objects/nsis.cl:21-40
template <class T> V2<T> defl_nsis(const Obj<T>& o, V2<T> x)
{
    x = x - o.x;
    return (o.r / (o.rc + length(x))) * x;
}
template <class T> void set_nsis(Obj<T>& o, const T* p) { o.x = {p[0], p[1]}; o.r = p[2]; o.rc = p[3]; }

// objects/sie.cl:27-64
template <class T> V2<T> defl_sie(const Obj<T>& o, V2<T> x)
{
    x = x - o.x;
    V2<T> y = mv22(o.m, x);
    T r = o.e / std::sqrt(o.q2 * y.x * y.x + y.y * y.y);
    y = o.d * V2<T>{EM<T>::atan(y.x * r), EM<T>::atanh(y.y * r)};
    return mv22(o.w, y);
}
template <class T> void set_sie_common(Obj<T>& o, T x, T y, T r, T q, T pa)
{
    T c = CR<T>::cos(pa * K<T>::DEG2RAD);
    T s = CR<T>::sin(pa * K<T>::DEG2RAD);
    o.x = {x, y};
    o.m = {c, s, -s, c};
    o.w = {c, -s, s, c};
    o.q2 = q * q;
    o.e = std::sqrt(T(1) - q * q);
    o.d = r * std::sqrt(q) / std::sqrt(T(1) - q * q);
}
template <class T> void set_sie(Obj<T>& o, const T* p) { set_sie_common(o, p[0], p[1], p[2], p[3], p[4]); }

// objects/sie_plus_shear.cl:30-70
template <class T> V2<T> defl_sie_plus_shear(const Obj<T>& o, V2<T> x)
{
    x = x - o.x;
    V2<T> y = mv22(o.m, x);
    T r = o.e / std::sqrt(o.q2 * y.x * y.x + y.y * y.y);
    y = o.d * V2<T>{EM<T>::atan(y.x * r), EM<T>::atanh(y.y * r)};
    return mv22(o.w, y) + mv22(o.g, x);
}
template <class T> void set_sie_plus_shear(Obj<T>& o, const T* p)
{
    T c = CR<T>::cos(p[4] * K<T>::DEG2RAD);
    T s = CR<T>::sin(p[4] * K<T>::DEG2RAD);
    o.x = {p[0], p[1]};
    o.m = {c, s, -s, c};
    o.w = {c, -s, s, c};
    o.g = {p[5], p[6], p[6], -p[5]};
    o.q2 = p[3] * p[3];
    o.e = std::sqrt(T(1) - p[3] * p[3]);
    o.d = p[2] * std::sqrt(p[3]) / std::sqrt(T(1) - p[3] * p[3]);
}

// objects/nsie.cl:29-69
template <class T> V2<T> defl_nsie(const Obj<T>& o, V2<T> x)
{
    x = x - o.x;
    V2<T> y = mv22(o.m, x);
    T r = std::sqrt(o.q2 * y.x * y.x + y.y * y.y);
    y = o.d * V2<T>{EM<T>::atan(y.x * o.e / (o.rc + r)), EM<T>::atanh(y.y * o.e / (o.rc * o.q2 + r))};
    return mv22(o.w, y);
}
template <class T> void set_nsie(Obj<T>& o, const T* p)
{
    T c = CR<T>::cos(p[5] * K<T>::DEG2RAD);
    T s = CR<T>::sin(p[5] * K<T>::DEG2RAD);
    T q = p[4];
    o.x = {p[0], p[1]};
    o.m = {c, s, -s, c};
    o.w = {c, -s, s, c};
    o.rc = p[3];
    o.q2 = q * q;
    o.e = std::sqrt(T(1) - q * q);
    o.d = p[2] * std::sqrt(q) / std::sqrt(T(1) - q * q);
}

// objects/point_mass.cl:18-32
template <class T> V2<T> defl_point_mass(const Obj<T>& o, V2<T> x)
{
    x = x - o.x;
    return (o.r2 / dot(x, x)) * x;
}
template <class T> void set_point_mass(Obj<T>& o, const T* p) { o.x = {p[0], p[1]}; o.r2 = p[2] * p[2]; }

// Angular series of the elliptical power law, objects/epl.cl:25-68: ten
// terms of the Tessore & Metcalf (2015) recursion, then the radial factor.
template <class T> V2<T> epl_core(const Obj<T>& o, V2<T> x)
{
    const T TT = T(2) - o.tt;
    const T f = o.f;
    T r = length(x);
    T phi = EM<T>::atan2(x.y, x.x);
    T s = EM<T>::sin(phi), c = EM<T>::cos(phi);
    T s2 = EM<T>::sin(T(2) * phi), c2 = EM<T>::cos(T(2) * phi);
    M22<T> R = {c2, -s2, s2, c2};
    V2<T> A = {c, s};
    V2<T> a = A;
    for (int k = 1; k <= 10; ++k) {
        T coef = -f * (T(2 * k) - TT) / (T(2 * k) + TT);
        A = coef * mv22(R, A);
        a = a + A;
    }
    a = (o.n * EM<T>::pow(r, T(1) - o.tt)) * a;
    return mv22(o.w, a);
}
template <class T> V2<T> defl_epl(const Obj<T>& o, V2<T> x) { return epl_core(o, mv22(o.m, x - o.x)); }
template <class T> void set_epl_common(Obj<T>& o, const T* p)
{
    T s = CR<T>::sin(p[5] * K<T>::DEG2RAD), c = CR<T>::cos(p[5] * K<T>::DEG2RAD);
    T r = p[2], q = p[4];
    o.x = {p[0], p[1]};
    o.m = (T(1) / r / std::sqrt(q)) * M22<T>{q * c, q * s, -s, c};
    o.w = {c, -s, s, c};
    o.tt = p[3];
    o.f = (T(1) - q) / (T(1) + q);
    o.n = T(2) * r * std::sqrt(q) / (T(1) + q);
}
template <class T> void set_epl(Obj<T>& o, const T* p) { set_epl_common(o, p); }

// objects/epl_plus_shear.cl:28-104
template <class T> V2<T> defl_epl_plus_shear(const Obj<T>& o, V2<T> x)
{
    V2<T> dx = x - o.x;
    V2<T> y = epl_core(o, mv22(o.m, dx));
    return y + mv22(o.g, dx);
}
template <class T> void set_epl_plus_shear(Obj<T>& o, const T* p)
{
    set_epl_common(o, p);
    o.g = {p[6], p[7], p[7], -p[6]};
}

// objects/sersic.cl:23-47
template <class T> T bright_sersic(const Obj<T>& o, V2<T> x)
{
    V2<T> y = mv22(o.t, x - o.x);
    return EM<T>::exp(o.log0 - EM<T>::exp(o.log1 + o.mexp * EM<T>::log(dot(y, y))));
}
template <class T> void set_sersic(Obj<T>& o, const T* p)
{
    T x = p[0], y = p[1], r = p[2], mag = p[3], n = p[4], q = p[5], a = p[6];
    // MacArthur, Courteau & Holtzman (2003) expansions of b(n), :31-33
    T b = n > lit<T>(0.36f, 0.36)
        ? T(2) * n - T(1) / T(3) + T(4) / (T(405) * n) + T(46) / (T(25515) * (n * n))
              + T(131) / (T(1148175) * (n * n * n)) - T(2194697) / (T(30690717750.0) * (n * n * n * n))
        : lit<T>(0.01945f, 0.01945) - lit<T>(0.8902f, 0.8902) * n + lit<T>(10.95f, 10.95) * (n * n)
              - lit<T>(19.67f, 19.67) * (n * n * n) + lit<T>(13.43f, 13.43) * (n * n * n * n);
    T c = CR<T>::cos(a * K<T>::DEG2RAD);
    T s = CR<T>::sin(a * K<T>::DEG2RAD);
    o.x = {x, y};
    o.t = M22<T>{q * c, q * s, -s, c} / std::sqrt(q);
    o.log0 = -lit<T>(0.4f, 0.4) * mag * K<T>::LOG_10 + T(2) * n * CR<T>::log(b) - K<T>::LOG_PI - T(2) * CR<T>::log(r)
           - CR<T>::log(CR<T>::tgamma(T(2) * n + T(1)));
    o.log1 = CR<T>::log(b) - CR<T>::log(r) / n;
    o.mexp = T(0.5) / n;
}

// objects/sersic-old.cl:23-45: the same profile with the older linear b(n);
// the reference's test fixtures were rendered with it.
template <class T> void set_sersic_old(Obj<T>& o, const T* p)
{
    T x = p[0], y = p[1], r = p[2], mag = p[3], n = p[4], q = p[5], a = p[6];
    T b = lit<T>(1.9992f, 1.9992) * n - lit<T>(0.3271f, 0.3271);
    T c = CR<T>::cos(a * K<T>::DEG2RAD);
    T s = CR<T>::sin(a * K<T>::DEG2RAD);
    o.x = {x, y};
    o.t = M22<T>{q * c, q * s, -s, c} / std::sqrt(q);
    o.log0 = -lit<T>(0.4f, 0.4) * mag * K<T>::LOG_10 + T(2) * n * CR<T>::log(b) - K<T>::LOG_PI - T(2) * CR<T>::log(r)
           - CR<T>::log(CR<T>::tgamma(T(2) * n + T(1)));
    o.log1 = CR<T>::log(b) - CR<T>::log(r) / n;
    o.mexp = T(0.5) / n;
}

// objects/exponential.cl:21-43
template <class T> T bright_exponential(const Obj<T>& o, V2<T> x)
{
    return o.norm * EM<T>::exp(-length(mv22(o.t, x - o.x)) / o.rs);
}
template <class T> void set_exponential(Obj<T>& o, const T* p)
{
    T c = CR<T>::cos(p[5] * K<T>::DEG2RAD), s = CR<T>::sin(p[5] * K<T>::DEG2RAD);
    T rs = p[2], q = p[4];
    o.x = {p[0], p[1]};
    o.t = {q * c, q * s, -s, c};
    o.rs = rs;
    o.norm = CR<T>::exp(-lit<T>(0.4f, 0.4) * p[3] * K<T>::LOG_10) * T(0.5) / K<T>::PI / rs / rs / q;
}

// objects/devauc.cl:26-48
template <class T> T bright_devauc(const Obj<T>& o, V2<T> x)
{
    return o.norm * EM<T>::exp(-K<T>::DEVAUC_B * std::sqrt(std::sqrt(length(mv22(o.t, x - o.x)) / o.rs)));
}
template <class T> void set_devauc(Obj<T>& o, const T* p)
{
    T c = CR<T>::cos(p[5] * K<T>::DEG2RAD), s = CR<T>::sin(p[5] * K<T>::DEG2RAD);
    T r = p[2], q = p[4];
    o.x = {p[0], p[1]};
    o.t = {q * c, q * s, -s, c};
    o.rs = r;
    o.norm = CR<T>::exp(-lit<T>(0.4f, 0.4) * p[3] * K<T>::LOG_10) / K<T>::PI / r / r / q * K<T>::DEVAUC_C;
}

// objects/gauss.cl:21-41
template <class T> T bright_gauss(const Obj<T>& o, V2<T> x)
{
    V2<T> y = mv22(o.t, x - o.x);
    return o.norm * EM<T>::exp(-T(0.5) * dot(y, y) / o.s2);
}
template <class T> void set_gauss(Obj<T>& o, const T* p)
{
    T c = CR<T>::cos(p[5] * K<T>::DEG2RAD), s = CR<T>::sin(p[5] * K<T>::DEG2RAD);
    T sigma = p[2], q = p[4];
    o.x = {p[0], p[1]};
    o.t = {q * c, q * s, -s, c};
    o.s2 = sigma * sigma;
    o.norm = CR<T>::exp(-lit<T>(0.4f, 0.4) * p[3] * K<T>::LOG_10) * T(0.5) / K<T>::PI / o.s2 / q;
}

// objects/sky.cl:16-25 (evaluated at the unlensed position)
template <class T> T fg_sky(const Obj<T>& o, V2<T> x) { return o.bg + dot(o.grad, x - V2<T>{T(1), T(1)}); }
template <class T> void set_sky(Obj<T>& o, const T* p) { o.bg = p[0]; o.grad = {p[1], p[2]}; }

// The plugin table: name, kind, parameter count and the position of an
// (x, y) pair that may carry an image-plane prior.
struct PluginInfo {
    const char* name;
    int kind;
    int npars;
    int xpar;   // index of the POSITION_X parameter, -1 if none
};
const PluginInfo PLUGINS[] = {
    {"sis", LENS, 3, 0},        {"sis_plus_shear", LENS, 5, 0}, {"nsis", LENS, 4, 0},
    {"sie", LENS, 5, 0},        {"sie_plus_shear", LENS, 7, 0}, {"nsie", LENS, 6, 0},
    {"point_mass", LENS, 3, 0}, {"epl", LENS, 6, 0},            {"epl_plus_shear", LENS, 8, 0},
    {"sersic", SOURCE, 7, 0},   {"exponential", SOURCE, 6, 0},  {"devauc", SOURCE, 6, 0},
    {"gauss", SOURCE, 6, 0},    {"sky", FOREGROUND, 3, -1},  {"sersic_old", SOURCE, 7, 0},
};
const int NPLUGINS = sizeof(PLUGINS) / sizeof(PLUGINS[0]);

template <class T> struct Fns {
    DeflFn<T> defl = nullptr;
    BrightFn<T> bright = nullptr;
    SetFn<T> set = nullptr;
};
template <class T> Fns<T> plugin_fns(int id)
{
    Fns<T> f;
    switch (id) {
    case 0: f.defl = defl_sis<T>; f.set = set_sis<T>; break;
    case 1: f.defl = defl_sis_plus_shear<T>; f.set = set_sis_plus_shear<T>; break;
    case 2: f.defl = defl_nsis<T>; f.set = set_nsis<T>; break;
    case 3: f.defl = defl_sie<T>; f.set = set_sie<T>; break;
    case 4: f.defl = defl_sie_plus_shear<T>; f.set = set_sie_plus_shear<T>; break;
    case 5: f.defl = defl_nsie<T>; f.set = set_nsie<T>; break;
    case 6: f.defl = defl_point_mass<T>; f.set = set_point_mass<T>; break;
    case 7: f.defl = defl_epl<T>; f.set = set_epl<T>; break;
    case 8: f.defl = defl_epl_plus_shear<T>; f.set = set_epl_plus_shear<T>; break;
    case 9: f.bright = bright_sersic<T>; f.set = set_sersic<T>; break;
    case 10: f.bright = bright_exponential<T>; f.set = set_exponential<T>; break;
    case 11: f.bright = bright_devauc<T>; f.set = set_devauc<T>; break;
    case 12: f.bright = bright_gauss<T>; f.set = set_gauss<T>; break;
    case 13: f.bright = fg_sky<T>; f.set = set_sky<T>; break;
    case 14: f.bright = bright_sersic<T>; f.set = set_sersic_old<T>; break;
    }
    return f;
}

// ------------------------------------------------------------------- model --
template <class T> struct Model {
    int nobjs = 0;
    std::vector<int> ids;        // plugin index per object
    std::vector<int> kinds;
    std::vector<int> par0;       // first parameter of each object
    std::vector<int> ipp;        // object has image-plane (x,y) prior
    std::vector<Fns<T>> fns;
    int npars = 0;
    int width = 0, height = 0;
    V2<T> origin{}, scale{};     // pcs after the even-PSF shift
    std::vector<V2<T>> qq, ww;   // quadrature abscissae (pixel units) and weights
    std::vector<T> psf;          // normalised PSF, row-major
    int psfw = 0, psfh = 0;
    int nthreads = 1;

    // Generated compute(), src/kernel.c:65-111 and :235-399.  Objects in list
    // order; a run of lenses forms a plane whose summed deflection is applied
    // when the next source appears; foregrounds see the unlensed position.
    T compute(const std::vector<Obj<T>>& d, V2<T> x) const
    {
        V2<T> y = x;
        T f = T(0);
        V2<T> a{T(0), T(0)};
        int trigger = 0;
        for (int i = 0; i < nobjs; ++i) {
            int k = kinds[i];
            if (k != trigger && k != FOREGROUND) {
                if (trigger == LENS) apply(y, a);
                trigger = k;
            }
            if (k == LENS) a = a + fns[i].defl(d[i], y);
            else if (k == SOURCE) f = f + fns[i].bright(d[i], y);
            else f = f + fns[i].bright(d[i], x);
        }
        if (trigger == LENS) apply(y, a);
        return f;
    }
    // src/kernel.c:86-91: deflect the ray if the deflection is finite
    static void apply(V2<T>& y, V2<T>& a)
    {
        y = y - ((dot(a, a) < K<T>::HUGEV) ? a : V2<T>{K<T>::FARV, K<T>::FARV});
        a = {T(0), T(0)};
    }

    // Generated set_params, src/kernel.c:114-150 and :401-656, including the
    // image-plane prior deflection of (x, y) through earlier lens planes.
    void set_params(const T* params, std::vector<Obj<T>>& d) const
    {
        // image-plane deflections inside set_params use the double-evaluated
        // functions too, whatever the per-ray mode
        struct Restore {
            int v;
            ~Restore() { g_cr_eval = v; }
        } restore{g_cr_eval};
        g_cr_eval = 1;
        d.assign(nobjs, Obj<T>{});
        int trigger = 0, plane = 0;
        std::vector<T> args;
        for (int i = 0; i < nobjs; ++i) {
            int k = kinds[i];
            if (k != trigger && k != FOREGROUND) {
                if (trigger == LENS && k == SOURCE) plane = i;
                trigger = k;
            }
            int np = PLUGINS[ids[i]].npars;
            args.assign(params + par0[i], params + par0[i] + np);
            if (ipp[i]) {
                int xp = PLUGINS[ids[i]].xpar;
                V2<T> x{args[xp], args[xp + 1]};
                V2<T> a{T(0), T(0)};
                int trigger2 = 0;
                for (int j = 0; j < plane; ++j) {
                    if (kinds[j] != trigger2 && kinds[j] != FOREGROUND) {
                        if (trigger2 == LENS) apply(x, a);
                        trigger2 = kinds[j];
                    }
                    if (kinds[j] == LENS) a = a + fns[j].defl(d[j], x);
                }
                if (trigger2 == LENS) apply(x, a);
                args[xp] = x.x;
                args[xp + 1] = x.y;
            }
            fns[i].set(d[i], args.data());
        }
    }

    // kernel/lensed.cl:9-39: quadrature over each pixel
    void render(const std::vector<Obj<T>>& d, T* value, T* error) const
    {
        const long N = (long)width * height;
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (long k = 0; k < N; ++k) {
            V2<T> x = origin + scale * V2<T>{T(k % width), T(k / width)};
            T f0 = T(0), f1 = T(0);
            for (size_t n = 0; n < qq.size(); ++n) {
                T c = compute(d, x + qq[n]);
                f0 = f0 + ww[n].x * c;
                f1 = f1 + ww[n].y * c;
            }
            value[k] = f0;
            if (error) error[k] = f1;
        }
    }

    // kernel/lensed.cl:56-103: flipped direct convolution, clamp-to-edge.
    // Output pixel (gi, gj) sums psf[j][i] * in(gj + PH-1-PH/2 - j,
    // gi + PW-1-PW/2 - i) with j outer, i inner.
    void convolve(const T* in, T* out) const
    {
        const int W = width, H = height;
        const int ox = psfw - 1 - psfw / 2, oy = psfh - 1 - psfh / 2;
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int gj = 0; gj < H; ++gj)
            for (int gi = 0; gi < W; ++gi) {
                T acc = T(0);
                for (int j = 0; j < psfh; ++j) {
                    int r = gj + oy - j;
                    r = r < 0 ? 0 : (r > H - 1 ? H - 1 : r);
                    for (int i = 0; i < psfw; ++i) {
                        int c = gi + ox - i;
                        c = c < 0 ? 0 : (c > W - 1 ? W - 1 : c);
                        acc = acc + psf[j * psfw + i] * in[(long)r * W + c];
                    }
                }
                out[(long)gj * W + gi] = acc;
            }
    }
};

struct Handle {
    int precision;
    Model<float> mf;
    Model<double> md;
    std::vector<float> image, weight;
    std::string err;
};

template <class T>
int setup(Model<T>& m, int nobjs, const int* ids, const int* ipp, int width, int height, const double* pcs, int nq,
          const double* qx, const double* qy, const double* qw, const double* qe, const float* psf, int psfw, int psfh)
{
    m.nobjs = nobjs;
    m.npars = 0;
    for (int i = 0; i < nobjs; ++i) {
        if (ids[i] < 0 || ids[i] >= NPLUGINS) return -1;
        m.ids.push_back(ids[i]);
        m.kinds.push_back(PLUGINS[ids[i]].kind);
        m.par0.push_back(m.npars);
        m.ipp.push_back(ipp ? ipp[i] : 0);
        m.fns.push_back(plugin_fns<T>(ids[i]));
        m.npars += PLUGINS[ids[i]].npars;
    }
    m.width = width;
    m.height = height;
    // src/lensed.c:871-891: pcs, shifted by half a pixel for even PSF sizes
    double rx = pcs[0], ry = pcs[1];
    if (psf) {
        if (psfw % 2 == 0) rx += 0.5;
        if (psfh % 2 == 0) ry += 0.5;
    }
    m.origin = {T(rx), T(ry)};
    m.scale = {T(pcs[2]), T(pcs[3])};
    // src/quadrature.c:32-43: abscissae scaled by the pixel scale in double,
    // then stored in the device precision
    for (int n = 0; n < nq; ++n) {
        m.qq.push_back({T(pcs[2] * qx[n]), T(pcs[3] * qy[n])});
        m.ww.push_back({T(qw[n]), T(qe[n])});
    }
    if (psf) {
        // src/data.c:354-370: normalise to unit sum (double sum, divide in
        // the array's precision)
        double norm = 0;
        for (int i = 0; i < psfw * psfh; ++i) norm += psf[i];
        m.psfw = psfw;
        m.psfh = psfh;
        for (int i = 0; i < psfw * psfh; ++i)
            m.psf.push_back(sizeof(T) == 4 ? T(float(psf[i] / norm)) : T(double(psf[i]) / norm));
    }
    return 0;
}

// Per-pixel chi^2 (kernel/lensed.cl:41-55) and the host sum in double in
// pixel order (src/nested.c:101-115).
template <class T> double chi2_sum(const T* model, const float* image, const float* weight, long N)
{
    double chi2 = 0.0;
    for (long k = 0; k < N; ++k) {
        T d = model[k] - T(image[k]);
        T t = T(weight[k]) * d * d;
        chi2 += (double)t;
    }
    return chi2;
}

template <class T> double eval_one(const Handle& h, const Model<T>& m, const T* params, T* value, T* error, T* conv)
{
    std::vector<Obj<T>> d;
    m.set_params(params, d);
    m.render(d, value, error);
    const long N = (long)m.width * m.height;
    const T* model = value;
    if (!m.psf.empty()) {
        m.convolve(value, conv);
        model = conv;
    }
    return -0.5 * chi2_sum(model, h.image.data(), h.weight.data(), N);
}

}  // namespace

extern "C" {

// Plugin lookup for the Python wrapper: index of a plugin name, or -1.
int lo_plugin_index(const char* name)
{
    for (int i = 0; i < NPLUGINS; ++i)
        if (std::strcmp(PLUGINS[i].name, name) == 0) return i;
    return -1;
}
// Per-ray elementary functions of the FP32 oracle: 1 = double-evaluated
// (strict semantics, the default), 0 = the C library's float functions.
// Process-wide.
void lo_set_eval_cr(int on) { g_cr_eval = on ? 1 : 0; }

int lo_plugin_npars(int id) { return (id >= 0 && id < NPLUGINS) ? PLUGINS[id].npars : -1; }
int lo_plugin_kind(int id) { return (id >= 0 && id < NPLUGINS) ? PLUGINS[id].kind : -1; }

// Create an oracle model.  precision is 32 or 64.  pcs = (rx, ry, sx, sy).
// Quadrature abscissae are in units of the pixel (scaled by sx, sy here).
// psf may be NULL.  image/weight may be NULL when only rendering.
void* lo_create(int precision, int nobjs, const int* ids, const int* ipp, int width, int height, const double* pcs,
                int nq, const double* qx, const double* qy, const double* qw, const double* qe, const float* psf,
                int psfw, int psfh, const float* image, const float* weight, int nthreads)
{
    Handle* h = new Handle();
    h->precision = precision;
    int rc = precision == 64 ? setup(h->md, nobjs, ids, ipp, width, height, pcs, nq, qx, qy, qw, qe, psf, psfw, psfh)
                             : setup(h->mf, nobjs, ids, ipp, width, height, pcs, nq, qx, qy, qw, qe, psf, psfw, psfh);
    if (rc) {
        delete h;
        return nullptr;
    }
    h->mf.nthreads = h->md.nthreads = nthreads > 0 ? nthreads : 1;
    long N = (long)width * height;
    if (image) h->image.assign(image, image + N);
    if (weight) h->weight.assign(weight, weight + N);
    return h;
}

void lo_destroy(void* p) { delete static_cast<Handle*>(p); }

int lo_npars(void* p)
{
    Handle* h = static_cast<Handle*>(p);
    return h->precision == 64 ? h->md.npars : h->mf.npars;
}

void lo_set_threads(void* p, int n)
{
    Handle* h = static_cast<Handle*>(p);
    h->mf.nthreads = h->md.nthreads = n > 0 ? n : 1;
}

// Render one parameter vector (object order, npars values).  Outputs are
// double arrays of N pixels; conv may be NULL when there is no PSF.
int lo_render(void* p, const double* params, double* value, double* error, double* conv)
{
    Handle* h = static_cast<Handle*>(p);
    if (h->precision == 64) {
        const Model<double>& m = h->md;
        std::vector<Obj<double>> d;
        m.set_params(params, d);
        m.render(d, value, error);
        if (conv && !m.psf.empty()) m.convolve(value, conv);
        return 0;
    }
    const Model<float>& m = h->mf;
    long N = (long)m.width * m.height;
    std::vector<float> pf(params, params + m.npars);
    std::vector<float> v(N), e(N), c(N);
    std::vector<Obj<float>> d;
    m.set_params(pf.data(), d);
    m.render(d, v.data(), e.data());
    for (long k = 0; k < N; ++k) {
        value[k] = v[k];
        if (error) error[k] = e[k];
    }
    if (conv && !m.psf.empty()) {
        m.convolve(v.data(), c.data());
        for (long k = 0; k < N; ++k) conv[k] = c[k];
    }
    return 0;
}

// logL = -chi^2/2 for B parameter vectors (object order, npars each), one
// after another as the reference's callback does.
int lo_loglike_batch(void* p, const double* params, int B, double* logL)
{
    Handle* h = static_cast<Handle*>(p);
    if (h->image.empty() || h->weight.empty()) return -1;
    if (h->precision == 64) {
        const Model<double>& m = h->md;
        long N = (long)m.width * m.height;
        std::vector<double> v(N), c(N);
        for (int b = 0; b < B; ++b) logL[b] = eval_one(*h, m, params + (long)b * m.npars, v.data(), (double*)nullptr, c.data());
        return 0;
    }
    const Model<float>& m = h->mf;
    long N = (long)m.width * m.height;
    std::vector<float> v(N), c(N), pf(m.npars);
    for (int b = 0; b < B; ++b) {
        for (int i = 0; i < m.npars; ++i) pf[i] = (float)params[(long)b * m.npars + i];
        logL[b] = eval_one(*h, m, pf.data(), v.data(), (float*)nullptr, c.data());
    }
    return 0;
}

// Per-pixel weights, src/data.c:314-330 and src/lensed.c:436-486:
// w = gain/(image + offset) unless a weight map is given, times xweight,
// zero where masked.  Any of gain/weight/xweight/mask may be NULL.
void lo_make_weight(const float* image, long N, const float* weight_map, const float* gain, double gain_value,
                    double offset, const float* xweight, const int* mask, float* out)
{
    for (long i = 0; i < N; ++i) {
        float w;
        if (weight_map) w = weight_map[i];
        else {
            float g = gain ? gain[i] : (float)gain_value;
            w = (float)(g / (image[i] + offset));
        }
        if (xweight) w *= xweight[i];
        if (mask && mask[i]) w = 0;
        out[i] = w;
    }
}

}  // extern "C"
