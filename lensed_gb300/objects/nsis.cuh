// Non-singular (cored) isothermal sphere.  Parameters (objects/nsis.cl:6-12):
// x, y, r (Einstein radius), rc (core radius).
struct lg_data_nsis {
    float2 x;
    float r, rc;
};
LG_DEV void lg_set_nsis(lg_data_nsis* o, float x, float y, float r, float rc)
{
    o->x = make_float2(x, y);
    o->r = r;
    o->rc = rc;
}
template <class V>
LG_DEV V lg_deflection_nsis(const lg_data_nsis* __restrict__ o, V x)
{
    x -= o->x;
    return (o->r / (o->rc + length(x))) * x;
}
