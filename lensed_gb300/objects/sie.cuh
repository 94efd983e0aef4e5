// Singular isothermal ellipsoid (Schneider, Kochanek & Wambsganss 2006).
// Parameters (objects/sie.cl:6-13): x, y, r (Einstein radius), q (axis
// ratio), pa (position angle, degrees).
struct lg_data_sie {
    float2 x;
    mat22 m;   // rotation into the lens frame
    mat22 w;   // rotation back
    float q2, e, d;
};
LG_DEV void lg_set_sie(lg_data_sie* o, float x, float y, float r, float q, float pa)
{
    float c = cosf(pa * LG_DEG2RAD);
    float s = sinf(pa * LG_DEG2RAD);
    o->x = make_float2(x, y);
    o->m = make_mat22(c, s, -s, c);
    o->w = make_mat22(c, -s, s, c);
    o->q2 = q * q;
    o->e = sqrtf(1 - q * q);
    o->d = r * sqrtf(q) / sqrtf(1 - q * q);
}
template <class V>
LG_DEV V lg_deflection_sie(const lg_data_sie* __restrict__ o, V x)
{
    typedef LG_SCALAR(V) T;
    x -= o->x;
    V y = mv22(o->m, x);
    T r = o->e / sqrtf(o->q2 * y.x * y.x + y.y * y.y);
    y = o->d * V{atanf(y.x * r), atanhf(y.y * r)};
    return mv22(o->w, y);
}
