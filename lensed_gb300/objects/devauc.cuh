// de Vaucouleurs source.  Parameters (objects/devauc.cl:8-16): x, y, r, mag,
// q, pa.  b = 7.66924944 and the normalisation b^8/8! of the n = 4 profile.
#define LG_DEVAUC_B 7.6692494425008039044f
#define LG_DEVAUC_C 296.826303766893f
struct lg_data_devauc {
    float2 x;
    mat22 t;
    float rs, norm;
};
LG_DEV void lg_set_devauc(lg_data_devauc* o, float x, float y, float r, float mag, float q, float pa)
{
    float c = cosf(pa * LG_DEG2RAD);
    float s = sinf(pa * LG_DEG2RAD);
    o->x = make_float2(x, y);
    o->t = make_mat22(q * c, q * s, -s, c);
    o->rs = r;
    o->norm = expf(-0.4f * mag * LG_LOG_10) / LG_PI / r / r / q * LG_DEVAUC_C;
}
template <class V>
LG_DEV LG_SCALAR(V) lg_brightness_devauc(const lg_data_devauc* __restrict__ o, V x)
{
    return o->norm * expf(-LG_DEVAUC_B * sqrtf(sqrtf(length(mv22(o->t, x - o->x)) / o->rs)));
}
