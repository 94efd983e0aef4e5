// Elliptical Gaussian source.  Parameters (objects/gauss.cl:3-11): x, y,
// sigma, mag, q, pa.
struct lg_data_gauss {
    float2 x;
    mat22 t;
    float s2, norm;
};
LG_DEV void lg_set_gauss(lg_data_gauss* o, float x, float y, float sigma, float mag, float q, float pa)
{
    float c = cosf(pa * LG_DEG2RAD);
    float s = sinf(pa * LG_DEG2RAD);
    o->x = make_float2(x, y);
    o->t = make_mat22(q * c, q * s, -s, c);
    o->s2 = sigma * sigma;
    o->norm = expf(-0.4f * mag * LG_LOG_10) * 0.5f / LG_PI / o->s2 / q;
}
template <class V>
LG_DEV LG_SCALAR(V) lg_brightness_gauss(const lg_data_gauss* __restrict__ o, V x)
{
    V y = mv22(o->t, x - o->x);
    return o->norm * expf(-0.5f * dot(y, y) / o->s2);
}
