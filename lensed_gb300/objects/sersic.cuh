// Sersic source.  Parameters (objects/sersic.cl:3-12): x, y, r (effective
// radius), mag, n (index), q, pa.  b(n) from the MacArthur, Courteau &
// Holtzman (2003) expansions; the profile is
// exp(log0 - exp(log1 + m * log|T(y - x0)|^2)).
struct lg_data_sersic {
    float2 x;
    mat22 t;
    float log0, log1, m;
};
LG_DEV void lg_sersic_setup(lg_data_sersic* o, float x, float y, float r, float mag, float n, float q, float a,
                            float b)
{
    float c = cosf(a * LG_DEG2RAD);
    float s = sinf(a * LG_DEG2RAD);
    o->x = make_float2(x, y);
    o->t = make_mat22(q * c, q * s, -s, c) / sqrtf(q);
    o->log0 = -0.4f * mag * LG_LOG_10 + 2 * n * logf(b) - LG_LOG_PI - 2 * logf(r) - logf(tgammaf(2 * n + 1));
    o->log1 = logf(b) - logf(r) / n;
    o->m = 0.5f / n;
}
LG_DEV void lg_set_sersic(lg_data_sersic* o, float x, float y, float r, float mag, float n, float q, float a)
{
    float b = n > 0.36f ? 2.0f * n - 1.0f / 3 + 4.0f / (405 * n) + 46.0f / (25515 * (n * n))
                              + 131.0f / (1148175 * (n * n * n)) - 2194697.0f / (30690717750.0f * (n * n * n * n))
                        : 0.01945f - 0.8902f * n + 10.95f * (n * n) - 19.67f * (n * n * n) + 13.43f * (n * n * n * n);
    lg_sersic_setup(o, x, y, r, mag, n, q, a, b);
}
template <class V>
LG_DEV LG_SCALAR(V) lg_brightness_sersic(const lg_data_sersic* __restrict__ o, V x)
{
    V y = mv22(o->t, x - o->x);
    return expf(o->log0 - expf(o->log1 + o->m * logf(dot(y, y))));
}
