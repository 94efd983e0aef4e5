// Non-singular isothermal ellipsoid (Schneider, Kochanek & Wambsganss 2006).
// Parameters (objects/nsie.cl:6-14): x, y, r, rc (core radius), q, pa.
struct lg_data_nsie {
    float2 x;
    mat22 m, w;
    float rc, q2, e, d;
};
LG_DEV void lg_set_nsie(lg_data_nsie* o, float x, float y, float r, float rc, float q, float pa)
{
    float c = cosf(pa * LG_DEG2RAD);
    float s = sinf(pa * LG_DEG2RAD);
    o->x = make_float2(x, y);
    o->m = make_mat22(c, s, -s, c);
    o->w = make_mat22(c, -s, s, c);
    o->rc = rc;
    o->q2 = q * q;
    o->e = sqrtf(1 - q * q);
    o->d = r * sqrtf(q) / sqrtf(1 - q * q);
}
template <class V>
LG_DEV V lg_deflection_nsie(const lg_data_nsie* __restrict__ o, V x)
{
    typedef LG_SCALAR(V) T;
    x -= o->x;
    V y = mv22(o->m, x);
    T r = sqrtf(o->q2 * y.x * y.x + y.y * y.y);
    y = o->d * V{atanf(y.x * o->e / (o->rc + r)), atanhf(y.y * o->e / (o->rc * o->q2 + r))};
    return mv22(o->w, y);
}
