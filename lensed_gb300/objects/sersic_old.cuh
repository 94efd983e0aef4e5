// Sersic source with the older linear b(n) = 1.9992 n - 0.3271
// (objects/sersic-old.cl:29-45; the reference's test images were rendered
// with it).  Parameters as sersic.  Needs the sersic plugin's helpers.
typedef lg_data_sersic lg_data_sersic_old;
LG_DEV void lg_set_sersic_old(lg_data_sersic_old* o, float x, float y, float r, float mag, float n, float q,
                              float a)
{
    lg_sersic_setup(o, x, y, r, mag, n, q, a, 1.9992f * n - 0.3271f);
}
template <class V>
LG_DEV LG_SCALAR(V) lg_brightness_sersic_old(const lg_data_sersic_old* __restrict__ o, V x)
{
    return lg_brightness_sersic(o, x);
}
