// Singular isothermal sphere lens.  Parameters (objects/sis.cl:6-11):
// x, y (position), r (Einstein radius).  Deflection r * (x - x0)/|x - x0|.
struct lg_data_sis {
    float2 x;
    float r;
};
LG_DEV void lg_set_sis(lg_data_sis* o, float x, float y, float r)
{
    o->x = make_float2(x, y);
    o->r = r;
}
template <class V>
LG_DEV V lg_deflection_sis(const lg_data_sis* __restrict__ o, V x)
{
    return o->r * normalize(x - o->x);
}
