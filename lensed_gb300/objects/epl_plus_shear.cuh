// Elliptical power-law lens plus external shear.  Parameters
// (objects/epl_plus_shear.cl:5-15): x, y, r, t, q, pa, g1, g2.
// Needs the epl plugin's helpers (the composer includes epl first).
struct lg_data_epl_plus_shear {
    lg_data_epl p;
    mat22 g;
};
LG_DEV void lg_set_epl_plus_shear(lg_data_epl_plus_shear* o, float x1, float x2, float r, float t, float q,
                                  float pa, float g1, float g2)
{
    lg_epl_setup(&o->p, x1, x2, r, t, q, pa);
    o->g = make_mat22(g1, g2, g2, -g1);
}
template <class V>
LG_DEV V lg_deflection_epl_plus_shear(const lg_data_epl_plus_shear* __restrict__ o, V x)
{
    V dx = x - o->p.x;
    V y = lg_epl_frame(&o->p, mv22(o->p.m, dx));
    return y + mv22(o->g, dx);
}
