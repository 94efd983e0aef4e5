// Singular isothermal ellipsoid plus external shear.  Parameters
// (objects/sie_plus_shear.cl:6-15): x, y, r, q, pa, g1, g2.
struct lg_data_sie_plus_shear {
    float2 x;
    mat22 m, w, g;
    float q2, e, d;
};
LG_DEV void lg_set_sie_plus_shear(lg_data_sie_plus_shear* o, float x, float y, float r, float q, float pa,
                                  float g1, float g2)
{
    float c = cosf(pa * LG_DEG2RAD);
    float s = sinf(pa * LG_DEG2RAD);
    o->x = make_float2(x, y);
    o->m = make_mat22(c, s, -s, c);
    o->w = make_mat22(c, -s, s, c);
    o->g = make_mat22(g1, g2, g2, -g1);
    o->q2 = q * q;
    o->e = sqrtf(1 - q * q);
    o->d = r * sqrtf(q) / sqrtf(1 - q * q);
}
template <class V>
LG_DEV V lg_deflection_sie_plus_shear(const lg_data_sie_plus_shear* __restrict__ o, V x)
{
    typedef LG_SCALAR(V) T;
    x -= o->x;
    V y = mv22(o->m, x);
    T r = o->e / sqrtf(o->q2 * y.x * y.x + y.y * y.y);
    y = o->d * V{atanf(y.x * r), atanhf(y.y * r)};
    return mv22(o->w, y) + mv22(o->g, x);
}
