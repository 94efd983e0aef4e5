// Elementary functions of ray pairs in the exact evaluation modules
// (LG_EXACT).  Composed after the strict function mapping (lg_crmath_on.cuh,
// which routes the plugins' expf, logf, ... to lg_cr_expf, lg_cr_logf, ...):
// these are the overloads of those names for lg_pair, so that the plugins'
// template evaluation functions, instantiated for ray pairs, compute each
// lane exactly as the one-ray strict code does -- the value of the function
// evaluated in double and rounded once.
//
// exp, log, atan and atanh (the functions of the SIE family, the Sersic,
// exponential, Gaussian and de Vaucouleurs profiles) and atan2, sincos and
// pow (the EPL lens) come from lg_crfloat.cuh, in single-precision
// arithmetic; the rest of the mapped library is evaluated lane by lane in
// double.

// one lane at a time: these functions are bound by instruction issue, and
// their per-lane parts (bit fields, tests, table loads) outweigh what f32x2
// instructions save in the double-word steps (measured 5-7% faster per lane)
LG_DEV lg_pair lg_cr_expf(lg_pair a) { return {make_float2(lg_crf_exp(a.v.x), lg_crf_exp(a.v.y))}; }
LG_DEV lg_pair lg_cr_logf(lg_pair a) { return {make_float2(lg_crf_log(a.v.x), lg_crf_log(a.v.y))}; }
LG_DEV lg_pair lg_cr_atanf(lg_pair a) { return {make_float2(lg_crf_atan(a.v.x), lg_crf_atan(a.v.y))}; }
LG_DEV lg_pair lg_cr_atanhf(lg_pair a) { return {make_float2(lg_crf_atanh(a.v.x), lg_crf_atanh(a.v.y))}; }
LG_DEV lg_pair lg_cr_expf(lg_pair_prod a) { return lg_cr_expf(lg_pair(a)); }
LG_DEV lg_pair lg_cr_logf(lg_pair_prod a) { return lg_cr_logf(lg_pair(a)); }
LG_DEV lg_pair lg_cr_atanf(lg_pair_prod a) { return lg_cr_atanf(lg_pair(a)); }
LG_DEV lg_pair lg_cr_atanhf(lg_pair_prod a) { return lg_cr_atanhf(lg_pair(a)); }

#define LG_EXACT_LANES1(fn) \
    LG_DEV lg_pair fn(lg_pair a) { return {make_float2(fn(a.v.x), fn(a.v.y))}; } \
    LG_DEV lg_pair fn(lg_pair_prod a) { return fn(lg_pair(a)); }
LG_EXACT_LANES1(lg_cr_exp2f)
LG_EXACT_LANES1(lg_cr_expm1f)
LG_EXACT_LANES1(lg_cr_log2f)
LG_EXACT_LANES1(lg_cr_log10f)
LG_EXACT_LANES1(lg_cr_log1pf)
LG_EXACT_LANES1(lg_cr_sinf)
LG_EXACT_LANES1(lg_cr_cosf)
LG_EXACT_LANES1(lg_cr_tanf)
LG_EXACT_LANES1(lg_cr_asinf)
LG_EXACT_LANES1(lg_cr_acosf)
LG_EXACT_LANES1(lg_cr_sinhf)
LG_EXACT_LANES1(lg_cr_coshf)
LG_EXACT_LANES1(lg_cr_tanhf)
LG_EXACT_LANES1(lg_cr_asinhf)
LG_EXACT_LANES1(lg_cr_acoshf)
LG_EXACT_LANES1(lg_cr_cbrtf)
LG_EXACT_LANES1(lg_cr_erff)
LG_EXACT_LANES1(lg_cr_erfcf)
LG_EXACT_LANES1(lg_cr_tgammaf)
LG_EXACT_LANES1(lg_cr_lgammaf)
#undef LG_EXACT_LANES1

// the EPL lens's atan2, sincos and pow: correctly rounded in single
// precision too (lg_crfloat.cuh), one lane at a time; the strict mapping's
// names are rebound to them for the plugins of this module (scalar calls
// included: the exact EPL polar frame runs per lane)
LG_DEV float lg_crx_powf(float a, float b) { return lg_crf_pow(a, b); }
LG_DEV lg_pair lg_crx_powf(lg_pair a, float b) { return {make_float2(lg_crf_pow(a.v.x, b), lg_crf_pow(a.v.y, b))}; }
LG_DEV lg_pair lg_crx_powf(lg_pair_prod a, float b) { return lg_crx_powf(lg_pair(a), b); }
LG_DEV lg_pair lg_crx_powf(lg_pair a, lg_pair b)
{
    return {make_float2(lg_crf_pow(a.v.x, b.v.x), lg_crf_pow(a.v.y, b.v.y))};
}
LG_DEV float lg_crx_atan2f(float y, float x) { return lg_crf_atan2(y, x); }
LG_DEV lg_pair lg_crx_atan2f(lg_pair y, lg_pair x)
{
    return {make_float2(lg_crf_atan2(y.v.x, x.v.x), lg_crf_atan2(y.v.y, x.v.y))};
}
LG_DEV void lg_crx_sincosf(float a, float* s, float* c) { lg_crf_sincos(a, s, c); }
LG_DEV void lg_crx_sincosf(lg_pair a, lg_pair* s, lg_pair* c)
{
    lg_crf_sincos(a.v.x, &s->v.x, &c->v.x);
    lg_crf_sincos(a.v.y, &s->v.y, &c->v.y);
}
#undef powf
#undef atan2f
#undef sincosf
#define powf(x, y) lg_crx_powf(x, y)
#define atan2f(y, x) lg_crx_atan2f(y, x)
#define sincosf(x, s, c) lg_crx_sincosf(x, s, c)
