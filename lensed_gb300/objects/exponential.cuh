// Exponential disk source.  Parameters (objects/exponential.cl:3-11): x, y,
// rs (scale length), mag, q, pa.
struct lg_data_exponential {
    float2 x;
    mat22 t;
    float rs, norm;
};
LG_DEV void lg_set_exponential(lg_data_exponential* o, float x, float y, float rs, float mag, float q, float pa)
{
    float c = cosf(pa * LG_DEG2RAD);
    float s = sinf(pa * LG_DEG2RAD);
    o->x = make_float2(x, y);
    o->t = make_mat22(q * c, q * s, -s, c);
    o->rs = rs;
    o->norm = expf(-0.4f * mag * LG_LOG_10) * 0.5f / LG_PI / rs / rs / q;
}
template <class V>
LG_DEV LG_SCALAR(V) lg_brightness_exponential(const lg_data_exponential* __restrict__ o, V x)
{
    return o->norm * expf(-length(mv22(o->t, x - o->x)) / o->rs);
}
