// Singular isothermal sphere plus external shear.  Parameters
// (objects/sis_plus_shear.cl:5-12): x, y, r, g1, g2.
struct lg_data_sis_plus_shear {
    float2 x;
    mat22 g;   // shear matrix ((g1, g2), (g2, -g1))
    float r;
};
LG_DEV void lg_set_sis_plus_shear(lg_data_sis_plus_shear* o, float x, float y, float r, float g1, float g2)
{
    o->x = make_float2(x, y);
    o->r = r;
    o->g = make_mat22(g1, g2, g2, -g1);
}
template <class V>
LG_DEV V lg_deflection_sis_plus_shear(const lg_data_sis_plus_shear* __restrict__ o, V x)
{
    x -= o->x;
    return o->r * normalize(x) + mv22(o->g, x);
}
