// Point-mass lens.  Parameters (objects/point_mass.cl:5-10): x, y, r
// (Einstein radius).  Singular at the centre; the plane's finite-deflection
// guard sends such rays away.
struct lg_data_point_mass {
    float2 x;
    float r2;
};
LG_DEV void lg_set_point_mass(lg_data_point_mass* o, float x, float y, float r)
{
    o->x = make_float2(x, y);
    o->r2 = r * r;
}
template <class V>
LG_DEV V lg_deflection_point_mass(const lg_data_point_mass* __restrict__ o, V x)
{
    x -= o->x;
    return (o->r2 / dot(x, x)) * x;
}
