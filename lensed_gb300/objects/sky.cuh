// Sky foreground: constant level plus a gradient, evaluated at the unlensed
// image position.  Parameters (objects/sky.cl:3-8): bg, dx, dy (the
// gradients default to -0, i.e. fixed at zero).
struct lg_data_sky {
    float bg;
    float2 grad;
};
LG_DEV void lg_set_sky(lg_data_sky* o, float bg, float dx, float dy)
{
    o->bg = bg;
    o->grad = make_float2(dx, dy);
}
template <class V>
LG_DEV LG_SCALAR(V) lg_foreground_sky(const lg_data_sky* __restrict__ o, V x)
{
    return o->bg + dot(o->grad, x - make_float2(1, 1));
}
