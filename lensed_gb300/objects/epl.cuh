// Elliptical power-law lens (Tessore & Metcalf 2015).  Parameters
// (objects/epl.cl:5-13): x, y, r, t (2-D convergence slope, 0..2), q, pa.
// The angular part is the ten-term recursion of the hypergeometric series;
// the radial part is n * R^(1 - t) in the elliptical radius R.
struct lg_data_epl {
    float2 x;
    mat22 m;   // rotate, make elliptical, scale by 1/r
    mat22 w;   // rotate back
    float t, f, n;
    float c[10];  // the recursion's factors -f (2k - T) / (2k + T), k = 1..10, T = 2 - t
};
LG_DEV void lg_epl_setup(lg_data_epl* o, float x1, float x2, float r, float t, float q, float pa)
{
    float c = cosf(pa * LG_DEG2RAD);
    float s = sinf(pa * LG_DEG2RAD);
    o->x = make_float2(x1, x2);
    o->m = (1 / r / sqrtf(q)) * make_mat22(q * c, q * s, -s, c);
    o->w = make_mat22(c, -s, s, c);
    o->t = t;
    o->f = (1 - q) / (1 + q);
    o->n = 2 * r * sqrtf(q) / (1 + q);
    // the same expression the reference evaluates per ray (objects/epl.cl),
    // once per candidate
    const float T = 2 - o->t;
    const float f = o->f;
    for (int k = 1; k <= 10; ++k) o->c[k - 1] = -f * (2 * k - T) / (2 * k + T);
}
LG_DEV void lg_set_epl(lg_data_epl* o, float x1, float x2, float r, float t, float q, float pa)
{
    lg_epl_setup(o, x1, x2, r, t, q, pa);
}
// Deflection in the rotated frame for the elliptical coordinates x.
// r = |x|, sincos of phi = atan2(x.y, x.x) and of 2 phi, as
// objects/epl.cl computes them (the two-ray version is in the prelude)
LG_DEV void lg_polar(float2 x, float* r, float* c, float* s, float* c2, float* s2)
{
    *r = length(x);
    const float phi = atan2f(x.y, x.x);
    sincosf(phi, s, c);
    sincosf(2 * phi, s2, c2);
}
#if defined(LG_EXACT) && !defined(LG_HOST_SET)
// the exact modules trace ray pairs with the one-ray calls, lane by lane
LG_DEV void lg_polar(lg_pair2 x, lg_pair* r, lg_pair* c, lg_pair* s, lg_pair* c2, lg_pair* s2)
{
    lg_polar(lg_lane(x, 0), &r->v.x, &c->v.x, &s->v.x, &c2->v.x, &s2->v.x);
    lg_polar(lg_lane(x, 1), &r->v.y, &c->v.y, &s->v.y, &c2->v.y, &s2->v.y);
}
#endif
template <class V>
LG_DEV V lg_epl_frame(const lg_data_epl* __restrict__ o, V x)
{
    typedef LG_SCALAR(V) S;
    S r, c, s, c2, s2;
    lg_polar(x, &r, &c, &s, &c2, &s2);  // atan2, sincos(phi), sincos(2 phi)
    const auto R = make_mat22(c2, -s2, s2, c2);
    V A = V{c, s};
    V a = A;
#pragma unroll
    for (int k = 1; k <= 10; ++k) {
        A = o->c[k - 1] * mv22(R, A);
        a += A;
    }
    a *= o->n * powf(r, 1 - o->t);
    return mv22(o->w, a);
}
template <class V>
LG_DEV V lg_deflection_epl(const lg_data_epl* __restrict__ o, V x)
{
    return lg_epl_frame(o, mv22(o->m, x - o->x));
}
