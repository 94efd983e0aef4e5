// Elementary functions of ray pairs in the exact evaluation modules
// (LG_EXACT).  Composed after the strict function mapping (lg_crmath_on.cuh,
// which routes the plugins' expf, logf, ... to lg_cr_expf, lg_cr_logf, ...):
// these are the overloads of those names for lg_pair, so that the plugins'
// template evaluation functions, instantiated for ray pairs, compute each
// lane exactly as the one-ray strict code does -- the value of the function
// evaluated in double and rounded once.
//
// exp, log, atan and atanh (the functions of the SIE family, the Sersic,
// exponential, Gaussian and de Vaucouleurs profiles) come from
// lg_crfloat.cuh, in single-precision arithmetic;
// the others (those of the EPL lens: atan2, sincos, pow; and the rest of the
// mapped library) are evaluated lane by lane in double.

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

LG_DEV lg_pair lg_cr_powf(lg_pair a, float b) { return {make_float2(lg_cr_powf(a.v.x, b), lg_cr_powf(a.v.y, b))}; }
LG_DEV lg_pair lg_cr_powf(lg_pair_prod a, float b) { return lg_cr_powf(lg_pair(a), b); }
LG_DEV lg_pair lg_cr_powf(lg_pair a, lg_pair b)
{
    return {make_float2(lg_cr_powf(a.v.x, b.v.x), lg_cr_powf(a.v.y, b.v.y))};
}
LG_DEV lg_pair lg_cr_atan2f(lg_pair y, lg_pair x)
{
    return {make_float2(lg_cr_atan2f(y.v.x, x.v.x), lg_cr_atan2f(y.v.y, x.v.y))};
}
LG_DEV void lg_cr_sincosf(lg_pair a, lg_pair* s, lg_pair* c)
{
    lg_cr_sincosf(a.v.x, &s->v.x, &c->v.x);
    lg_cr_sincosf(a.v.y, &s->v.y, &c->v.y);
}
