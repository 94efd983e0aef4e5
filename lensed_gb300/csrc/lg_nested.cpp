// Nested sampling over the unit cube with batched likelihood calls.
//
// Lensed delegates sampling to MultiNest (src/lensed.c:1236-1288, external
// Fortran, not part of the reference).  This file provides the sampler the
// likelihood path needs in its place, written from the published method:
// nested sampling (Skilling 2004/2006) with live points bounded by one
// enlarged ellipsoid (Mukherjee, Parkinson & Liddle 2006; the single-
// ellipsoid case of Feroz & Hobson 2008).  Proposals are drawn in batches and
// evaluated with one batched likelihood call; every evaluated proposal is
// kept in a pool and used, in draw order, for later replacements while its
// logL exceeds the moving threshold (a draw uniform in the ellipsoid is still
// uniform in the ellipsoid after the threshold rises).
//
// The evidence is accumulated as a log-sum-exp in double precision, with
// Skilling's information H and the error sqrt(H / nlive).  A learned
// proposal (lg_flow.cu) can replace the ellipsoid; the ellipsoid remains the
// fallback and the yardstick of the learned sampler.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "lg_internal.h"
#include "lg_nested.h"

namespace lg {

// Bounding ellipsoid of a set of points: centre, Cholesky factor of the
// covariance scaled so that every point lies inside.
struct Ellipsoid {
    int d = 0;
    std::vector<double> mu, L;  // L lower triangular, row-major d x d
    std::vector<double> Li;     // L^-1 (lower triangular): Mahalanobis distances as mat-vecs
    double scale = 1;           // (x-mu)^T C^-1 (x-mu) <= scale defines the boundary

    bool fit(const std::vector<double>& pts, int n, int dim, double enlarge_volume)
    {
        d = dim;
        mu.assign(d, 0);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < d; ++k) mu[k] += pts[(size_t)i * d + k];
        for (auto& m : mu) m /= n;
        // centred coordinates, one row per dimension, so that each
        // covariance entry is a dot product over the points (four partial
        // sums in a fixed order)
        std::vector<double> xt((size_t)d * n);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < d; ++k) xt[(size_t)k * n + i] = pts[(size_t)i * d + k] - mu[k];
        std::vector<double> C((size_t)d * d, 0);
        for (int a = 0; a < d; ++a)
            for (int b = 0; b <= a; ++b) {
                const double* xa = &xt[(size_t)a * n];
                const double* xb = &xt[(size_t)b * n];
                double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                int i = 0;
                for (; i + 4 <= n; i += 4) {
                    s0 += xa[i] * xb[i];
                    s1 += xa[i + 1] * xb[i + 1];
                    s2 += xa[i + 2] * xb[i + 2];
                    s3 += xa[i + 3] * xb[i + 3];
                }
                for (; i < n; ++i) s0 += xa[i] * xb[i];
                C[(size_t)a * d + b] = ((s0 + s1) + (s2 + s3)) / n;
            }
        // Cholesky with a small diagonal floor for degenerate point sets
        L.assign((size_t)d * d, 0);
        for (int a = 0; a < d; ++a) {
            for (int b = 0; b <= a; ++b) {
                double s = C[(size_t)a * d + b];
                for (int k = 0; k < b; ++k) s -= L[(size_t)a * d + k] * L[(size_t)b * d + k];
                if (a == b) {
                    if (s <= 1e-30) s = 1e-30;
                    L[(size_t)a * d + a] = std::sqrt(s);
                } else {
                    L[(size_t)a * d + b] = s / L[(size_t)b * d + b];
                }
            }
        }
        invert();
        double kmax = 0;
        std::vector<double> x(d);
        for (int i = 0; i < n; ++i) {
            for (int k = 0; k < d; ++k) x[k] = xt[(size_t)k * n + i];
            kmax = std::max(kmax, centred_norm2(x.data()));
        }
        scale = kmax * std::pow(enlarge_volume, 2.0 / d);
        return std::isfinite(scale) && scale > 0;
    }
    // Li = L^-1 by forward substitution on the unit vectors
    void invert()
    {
        Li.assign((size_t)d * d, 0);
        for (int c = 0; c < d; ++c)
            for (int a = c; a < d; ++a) {
                double s = a == c ? 1.0 : 0.0;
                for (int k = c; k < a; ++k) s -= L[(size_t)a * d + k] * Li[(size_t)k * d + c];
                Li[(size_t)a * d + c] = s / L[(size_t)a * d + a];
            }
    }
    // |L^-1 x|^2 of a centred point: rows independent of each other
    double centred_norm2(const double* x) const
    {
        double m = 0;
        for (int a = 0; a < d; ++a) {
            const double* r = &Li[(size_t)a * d];
            double s = 0;
            for (int k = 0; k <= a; ++k) s += r[k] * x[k];
            m += s * s;
        }
        return m;
    }
    double mahalanobis(const double* x, std::vector<double>& y) const
    {
        for (int a = 0; a < d; ++a) y[a] = x[a] - mu[a];
        return centred_norm2(y.data());
    }
    // uniform draw inside the ellipsoid
    void sample(Rng& r, double* x, std::vector<double>& u) const
    {
        double n2 = 0;
        for (int a = 0; a < d; ++a) {
            u[a] = r.normal();
            n2 += u[a] * u[a];
        }
        const double rad = std::pow(r.uniform(), 1.0 / d) / std::sqrt(n2) * std::sqrt(scale);
        for (int a = 0; a < d; ++a) {
            double s = 0;
            for (int k = 0; k <= a; ++k) s += L[(size_t)a * d + k] * u[k];
            x[a] = mu[a] + rad * s;
        }
    }
    // log volume of the ellipsoid
    double log_volume() const
    {
        double lv = 0.5 * d * std::log(M_PI) - std::lgamma(0.5 * d + 1) + 0.5 * d * std::log(scale);
        for (int a = 0; a < d; ++a) lv += std::log(L[(size_t)a * d + a]);
        return lv;
    }
    bool contains(const double* x, std::vector<double>& y) const { return mahalanobis(x, y) <= scale; }
    // grow (never shrink) to a log volume of at least lv_min
    void enlarge_to(double lv_min)
    {
        const double lv = log_volume();
        if (lv < lv_min) scale *= std::exp(2.0 * (lv_min - lv) / d);
    }
};

// Several ellipsoids bounding the live points (the multi-ellipsoidal
// decomposition of Feroz & Hobson 2008, MultiNest's multi-modal mode): a set
// of points is split in two by 2-means (started from the extreme points
// along its principal axis) while the two enlarged ellipsoids of the halves
// have less than half the volume of the set's; each ellipsoid's volume is
// then at least its share of the live points times the expected prior
// volume X of the constrained region.  Draws are uniform in the union: an
// ellipsoid picked with probability proportional to its volume, a uniform
// point in it, kept with probability 1 / (number of ellipsoids holding it).
struct Bound {
    int d = 0;
    std::vector<Ellipsoid> ell;
    std::vector<double> logv;
    std::vector<double> cum;  // cumulative volume fractions
    double logv_sum = -HUGE_VAL;

    static double lae(double a, double b)
    {
        if (a == -HUGE_VAL) return b;
        if (b == -HUGE_VAL) return a;
        const double m = std::max(a, b);
        return m + std::log(std::exp(a - m) + std::exp(b - m));
    }

    // 2-means split of the points idx; false if a half is too small
    static bool two_means(const std::vector<double>& pts, const std::vector<int>& idx, int d, std::vector<int>& a,
                          std::vector<int>& b)
    {
        const size_t n = idx.size();
        std::vector<double> m(d, 0.0), C((size_t)d * d, 0.0), v(d, 1.0 / std::sqrt((double)d)), w(d);
        for (int i : idx)
            for (int k = 0; k < d; ++k) m[k] += pts[(size_t)i * d + k];
        for (auto& x : m) x /= (double)n;
        for (int i : idx)
            for (int k = 0; k < d; ++k)
                for (int l = 0; l < d; ++l)
                    C[(size_t)k * d + l] += (pts[(size_t)i * d + k] - m[k]) * (pts[(size_t)i * d + l] - m[l]);
        for (int it = 0; it < 30; ++it) {  // principal axis by power iteration
            double nrm = 0;
            for (int k = 0; k < d; ++k) {
                w[k] = 0;
                for (int l = 0; l < d; ++l) w[k] += C[(size_t)k * d + l] * v[l];
                nrm += w[k] * w[k];
            }
            nrm = std::sqrt(nrm);
            if (!(nrm > 0)) break;
            for (int k = 0; k < d; ++k) v[k] = w[k] / nrm;
        }
        int lo = idx[0], hi = idx[0];
        double plo = HUGE_VAL, phi = -HUGE_VAL;
        for (int i : idx) {
            double p = 0;
            for (int k = 0; k < d; ++k) p += (pts[(size_t)i * d + k] - m[k]) * v[k];
            if (p < plo) plo = p, lo = i;
            if (p > phi) phi = p, hi = i;
        }
        std::vector<double> c0(pts.begin() + (size_t)lo * d, pts.begin() + (size_t)lo * d + d);
        std::vector<double> c1(pts.begin() + (size_t)hi * d, pts.begin() + (size_t)hi * d + d);
        std::vector<char> side(n, 0);
        for (int it = 0; it < 50; ++it) {
            bool changed = false;
            std::vector<double> s0(d, 0.0), s1(d, 0.0);
            size_t n0 = 0, n1 = 0;
            for (size_t j = 0; j < n; ++j) {
                const double* x = &pts[(size_t)idx[j] * d];
                double d0 = 0, d1 = 0;
                for (int k = 0; k < d; ++k) {
                    d0 += (x[k] - c0[k]) * (x[k] - c0[k]);
                    d1 += (x[k] - c1[k]) * (x[k] - c1[k]);
                }
                const char sd = d1 < d0;
                changed = changed || sd != side[j];
                side[j] = sd;
                for (int k = 0; k < d; ++k) (sd ? s1 : s0)[k] += x[k];
                (sd ? n1 : n0)++;
            }
            if (n0 == 0 || n1 == 0) return false;
            for (int k = 0; k < d; ++k) c0[k] = s0[k] / (double)n0, c1[k] = s1[k] / (double)n1;
            if (!changed && it > 0) break;
        }
        a.clear();
        b.clear();
        for (size_t j = 0; j < n; ++j) (side[j] ? b : a).push_back(idx[j]);
        return a.size() > (size_t)d + 1 && b.size() > (size_t)d + 1;
    }

    static bool fit_subset(const std::vector<double>& pts, const std::vector<int>& idx, int d, double enlarge,
                           Ellipsoid& e)
    {
        std::vector<double> sub(idx.size() * (size_t)d);
        for (size_t j = 0; j < idx.size(); ++j)
            std::memcpy(&sub[j * d], &pts[(size_t)idx[j] * d], d * sizeof(double));
        return e.fit(sub, (int)idx.size(), d, enlarge);
    }

    void decompose(const std::vector<double>& pts, const std::vector<int>& idx, int dim, double enlarge,
                   int depth, std::vector<std::vector<int>>& members, Ellipsoid e)
    {
        std::vector<int> a, b;
        Ellipsoid ea, eb;
        if (depth > 0 && idx.size() >= 2 * ((size_t)dim + 2) && two_means(pts, idx, dim, a, b) &&
            fit_subset(pts, a, dim, enlarge, ea) && fit_subset(pts, b, dim, enlarge, eb) &&
            lae(ea.log_volume(), eb.log_volume()) < std::log(0.5) + e.log_volume()) {
            decompose(pts, a, dim, enlarge, depth - 1, members, ea);
            decompose(pts, b, dim, enlarge, depth - 1, members, eb);
            return;
        }
        ell.push_back(e);
        members.push_back(idx);
    }

    // Fit to n points; logx = ln of the expected prior volume of the
    // constrained region; at most 2^depth ellipsoids.
    bool fit(const std::vector<double>& pts, int n, int dim, double enlarge, double logx, int depth)
    {
        d = dim;
        ell.clear();
        std::vector<int> idx(n);
        for (int i = 0; i < n; ++i) idx[i] = i;
        Ellipsoid e;
        if (!fit_subset(pts, idx, dim, enlarge, e)) return false;
        std::vector<std::vector<int>> members;
        decompose(pts, idx, dim, enlarge, depth, members, e);
        return finish(logx, members, n);
    }

    bool finish(double logx, const std::vector<std::vector<int>>& members, int n)
    {
        logv.clear();
        cum.clear();
        logv_sum = -HUGE_VAL;
        for (size_t k = 0; k < ell.size(); ++k) {
            if (!members.empty()) ell[k].enlarge_to(logx + std::log((double)members[k].size() / n));
            logv.push_back(ell[k].log_volume());
            logv_sum = lae(logv_sum, logv.back());
        }
        double c = 0;
        for (double lv : logv) cum.push_back(c += std::exp(lv - logv_sum));
        return std::isfinite(logv_sum);
    }

    // one uniform draw in the union; false if the draw was rejected for
    // lying in several ellipsoids
    bool sample(Rng& r, double* x, std::vector<double>& u, std::vector<double>& y) const
    {
        const double t = r.uniform() * cum.back();
        size_t k = 0;
        while (k + 1 < cum.size() && cum[k] < t) ++k;
        ell[k].sample(r, x, u);
        int inside = 0;
        for (const Ellipsoid& e : ell) inside += e.contains(x, y);
        return inside <= 1 || r.uniform() * inside < 1.0;
    }
};

namespace {

double logaddexp(double a, double b)
{
    if (a == -HUGE_VAL) return b;
    if (b == -HUGE_VAL) return a;
    const double m = std::max(a, b);
    return m + std::log(std::exp(a - m) + std::exp(b - m));
}

}  // namespace

// The sampler's state between two iterations: written to the checkpoint
// file and read back to resume.  A resumed run with the ellipsoidal proposal
// continues exactly as the uninterrupted run would (same draws, same
// result); the learned proposal is not part of the state and is retrained
// at its next scheduled retraining.
struct SamplerState {
    int nd = 0, nl = 0, batch = 0;
    long iter = 0, ncall = 0, since_train = 0, n_flow = 0, n_ell = 0, n_flow_fail = 0;
    double logz = -HUGE_VAL, H = 0, logx = 0;
    double plat_level = HUGE_VAL;  // logL of the plateau being removed
    long plat_j = 0;               // its points removed so far
    double log_enl = 0;            // constant efficiency mode: log volume enlargement
    uint64_t pool_used = 0;        // replacements taken from the pool
    int pool_ell = 0;              // the pool came from the ellipsoidal bound
    uint64_t rng[4] = {0, 0, 0, 0};
    std::vector<double> live, llive, dead_x, dead_l, dead_lw, pool_x, pool_l;
    uint64_t pool_pos = 0;
    // multi-ellipsoid bound: [count, iteration of the fit, then per
    // ellipsoid scale, centre (d), Cholesky factor (d x d)]
    std::vector<double> bound;
};

namespace {

// format version in the last byte: bumped whenever the layout changes, so a
// state of another layout is refused instead of being read misaligned
const char kStateMagic[8] = {'L', 'G', 'N', 'S', 'T', 'A', 'T', '4'};

template <class T>
bool put(FILE* f, const T& v)
{
    return std::fwrite(&v, sizeof v, 1, f) == 1;
}
template <class T>
bool get(FILE* f, T& v)
{
    return std::fread(&v, sizeof v, 1, f) == 1;
}
bool put_vec(FILE* f, const std::vector<double>& v)
{
    const uint64_t n = v.size();
    return put(f, n) && (n == 0 || std::fwrite(v.data(), sizeof(double), n, f) == n);
}
bool get_vec(FILE* f, std::vector<double>& v)
{
    uint64_t n = 0;
    if (!get(f, n) || n > (uint64_t)1 << 34) return false;
    v.resize(n);
    return n == 0 || std::fread(v.data(), sizeof(double), n, f) == n;
}

// Write the state to path (through a temporary file renamed over it, so an
// interrupted write leaves the previous state intact).
bool save_state(const char* path, const SamplerState& s)
{
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    bool ok = std::fwrite(kStateMagic, 1, 8, f) == 8 && put(f, s.nd) && put(f, s.nl) && put(f, s.batch) &&
              put(f, s.iter) && put(f, s.ncall) && put(f, s.since_train) && put(f, s.n_flow) && put(f, s.n_ell) &&
              put(f, s.n_flow_fail) && put(f, s.logz) && put(f, s.H) && put(f, s.logx) && put(f, s.plat_level) &&
              put(f, s.plat_j) && put(f, s.log_enl) && put(f, s.pool_used) && put(f, s.pool_ell);
    for (int i = 0; i < 4 && ok; ++i) ok = put(f, s.rng[i]);
    ok = ok && put_vec(f, s.live) && put_vec(f, s.llive) && put_vec(f, s.dead_x) && put_vec(f, s.dead_l) &&
         put_vec(f, s.dead_lw) && put_vec(f, s.pool_x) && put_vec(f, s.pool_l) && put(f, s.pool_pos) &&
         put_vec(f, s.bound);
    ok = (std::fclose(f) == 0) && ok;
    return ok && std::rename(tmp.c_str(), path) == 0;
}

enum class Load { ABSENT, OK, BAD };

// Read a state written by save_state.  ABSENT if there is no file; BAD (with
// the reason in why) if the file is not a state of this run: another format
// version, truncated, or for another dimension, live-point count or batch.
Load load_state(const char* path, int nd, int nl, int batch, SamplerState& s, std::string& why)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return Load::ABSENT;
    char magic[8];
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kStateMagic, 8) != 0) {
        std::fclose(f);
        why = "not a sampler state of this format version";
        return Load::BAD;
    }
    if (!get(f, s.nd) || !get(f, s.nl) || !get(f, s.batch) || s.nd != nd || s.nl != nl || s.batch != batch) {
        std::fclose(f);
        why = "a state for another dimension, live-point count or batch size";
        return Load::BAD;
    }
    bool ok = get(f, s.iter) &&
              get(f, s.ncall) && get(f, s.since_train) && get(f, s.n_flow) && get(f, s.n_ell) &&
              get(f, s.n_flow_fail) && get(f, s.logz) && get(f, s.H) && get(f, s.logx) && get(f, s.plat_level) &&
              get(f, s.plat_j) && get(f, s.log_enl) && get(f, s.pool_used) && get(f, s.pool_ell);
    for (int i = 0; i < 4 && ok; ++i) ok = get(f, s.rng[i]);
    ok = ok && get_vec(f, s.live) && get_vec(f, s.llive) && get_vec(f, s.dead_x) && get_vec(f, s.dead_l) &&
         get_vec(f, s.dead_lw) && get_vec(f, s.pool_x) && get_vec(f, s.pool_l) && get(f, s.pool_pos) &&
         get_vec(f, s.bound);
    std::fclose(f);
    ok = ok && s.live.size() == (size_t)nl * nd && s.llive.size() == (size_t)nl &&
         s.dead_x.size() == s.dead_l.size() * nd && s.dead_lw.size() == s.dead_l.size() &&
         s.pool_x.size() == s.pool_l.size() * nd && s.pool_pos <= s.pool_l.size();
    if (!ok) why = "truncated or inconsistent state";
    return ok ? Load::OK : Load::BAD;
}

}  // namespace

int nested_sample(int nd, lg_batch_loglike fn, void* user, const lg_nested_options* o, lg_nested_result* res,
                  Proposal* learned, std::string& err, EllipsoidDrawer* drawer)
{
    const auto t0 = std::chrono::steady_clock::now();
    lg_nested_options opt = lg_nested_defaults();
    if (o) opt = *o;
    if (nd <= 0 || !fn || !res || opt.nlive < nd + 1 || opt.batch <= 0 || !(opt.efr > 0)) {
        err = "nested sampling: invalid arguments (nlive must exceed the dimension)";
        return LG_ERR_INPUT;
    }
    const int nl = opt.nlive, B = opt.batch;
    if (learned) learned->set_wrap(opt.wrap, nd);
    Rng rng((uint64_t)(opt.seed < 0 ? std::chrono::steady_clock::now().time_since_epoch().count() : opt.seed));
    std::vector<double> live((size_t)nl * nd), llive(nl);
    std::vector<double> buf((size_t)B * nd), lbuf(B);
    long ncall = 0;
    using clock = std::chrono::steady_clock;
    double t_eval = 0, t_train = 0, t_prop = 0;
    auto since = [](clock::time_point t) { return std::chrono::duration<double>(clock::now() - t).count(); };
    auto evaluate = [&](const double* x, int n, double* l) {
        const auto te = clock::now();
        int rc = fn(user, x, n, l);
        t_eval += since(te);
        ncall += n;
        return rc;
    };
    SamplerState st;
    bool resumed = false;
    if (opt.checkpoint && opt.resume) {
        std::string why;
        const Load ld = load_state(opt.checkpoint, nd, nl, B, st, why);
        if (ld == Load::BAD) {
            err = std::string("nested sampling: cannot resume from ") + opt.checkpoint + ": " + why;
            return LG_ERR_INPUT;
        }
        resumed = ld == Load::OK;
    }
    // initial live points: uniform in the cube where logL > -inf.  Draws
    // with logL = -inf (or NaN: outside the priors' bounds, say) are
    // dropped and counted, and the run starts from the prior volume
    // fraction they leave, ln X0 = ln((nlive - 1) / (draws - 1)) (the
    // unbiased estimate for draws made until nlive were kept); without such
    // draws X0 = 1 and the draws are those of a plain start.
    int have = 0;
    long ndraw = 0;
    bool dropped = false;
    const long max_draws = std::max<long>(100000000L, 1000L * nl);
    while (!resumed && have < nl) {
        if (ndraw >= max_draws) {
            err = "nested sampling: logL is -inf almost everywhere in the prior";
            return LG_ERR_INPUT;
        }
        const int n = dropped ? B : std::min(B, nl - have);
        for (size_t k = 0; k < (size_t)n * nd; ++k) buf[k] = rng.uniform();
        if (int rc = evaluate(buf.data(), n, lbuf.data())) {
            err = "likelihood callback failed";
            return rc;
        }
        for (int i = 0; i < n && have < nl; ++i) {
            ++ndraw;
            if (!(lbuf[i] > -HUGE_VAL)) {
                dropped = true;
                continue;
            }
            std::memcpy(&live[(size_t)have * nd], &buf[(size_t)i * nd], nd * sizeof(double));
            llive[have++] = lbuf[i];
        }
    }
    // dead points
    std::vector<double> dead_x;
    std::vector<double> dead_l, dead_lw;
    double logz = -HUGE_VAL, H = 0;
    double logx = !resumed && ndraw > nl ? std::log((double)(nl - 1) / (double)(ndraw - 1)) : 0.0;
    const double dlogx = 1.0 / nl;
    const double lw_step = std::log1p(-std::exp(-dlogx));  // log(1 - e^{-1/nl})
    double plat_level = HUGE_VAL;  // the lowest logL while tied points leave
    long plat_j = 0;               // tied points removed so far
    // constant efficiency mode: the bound's log volume enlargement, moved
    // after each fully used ellipsoid batch towards the target acceptance
    double log_enl = std::log(1.25);
    uint64_t pool_used = 0;
    int pool_ell = 0;
    // pool of evaluated proposals, used in draw order
    std::vector<double> pool_x;
    std::vector<double> pool_l;
    size_t pool_pos = 0;
    Ellipsoid ell;
    // multi-ellipsoid mode: the decomposition is refitted every nlive / 10
    // iterations (and kept in the checkpoint, so that resumed runs repeat it)
    const bool multi = opt.max_ellipsoids > 1;
    int depth = 0;
    while ((2 << depth) <= opt.max_ellipsoids && depth < 10) ++depth;
    Bound bound;
    long bound_iter = -1;
    const long refit_every = std::max(1, nl / 10);
    std::vector<double> u(nd), y(nd);
    long iter = 0, since_train = 0, n_flow = 0, n_ell = 0, n_flow_fail = 0;
    bool use_flow = false;
    int status = LG_OK;
    if (resumed) {
        live = st.live;
        llive = st.llive;
        dead_x = st.dead_x;
        dead_l = st.dead_l;
        dead_lw = st.dead_lw;
        pool_x = st.pool_x;
        pool_l = st.pool_l;
        pool_pos = (size_t)st.pool_pos;
        logz = st.logz;
        H = st.H;
        logx = st.logx;
        plat_level = st.plat_level;
        plat_j = st.plat_j;
        log_enl = st.log_enl;
        pool_used = st.pool_used;
        pool_ell = st.pool_ell;
        iter = st.iter;
        ncall = st.ncall;
        since_train = st.since_train;
        n_flow = st.n_flow;
        n_ell = st.n_ell;
        n_flow_fail = st.n_flow_fail;
        for (int i = 0; i < 4; ++i) rng.s[i] = st.rng[i];
        if (multi && st.bound.size() >= 2) {
            const int ne = (int)st.bound[0];
            bound_iter = (long)st.bound[1];
            size_t o = 2;
            bound.d = nd;
            for (int k = 0; k < ne && o + 1 + nd + (size_t)nd * nd <= st.bound.size(); ++k) {
                Ellipsoid e;
                e.d = nd;
                e.scale = st.bound[o++];
                e.mu.assign(st.bound.begin() + o, st.bound.begin() + o + nd);
                o += nd;
                e.L.assign(st.bound.begin() + o, st.bound.begin() + o + (size_t)nd * nd);
                e.invert();
                o += (size_t)nd * nd;
                bound.ell.push_back(e);
            }
            if (!bound.finish(0, {}, 1)) bound.ell.clear(), bound_iter = -1;
        }
    }
    // the state between iterations, for the checkpoint file
    auto checkpoint = [&]() {
        if (!opt.checkpoint) return true;
        SamplerState c;
        c.nd = nd;
        c.nl = nl;
        c.batch = B;
        c.iter = iter;
        c.ncall = ncall;
        c.since_train = since_train;
        c.n_flow = n_flow;
        c.n_ell = n_ell;
        c.n_flow_fail = n_flow_fail;
        c.logz = logz;
        c.H = H;
        c.logx = logx;
        c.plat_level = plat_level;
        c.plat_j = plat_j;
        c.log_enl = log_enl;
        c.pool_used = pool_used;
        c.pool_ell = pool_ell;
        for (int i = 0; i < 4; ++i) c.rng[i] = rng.s[i];
        c.live = live;
        c.llive = llive;
        c.dead_x = dead_x;
        c.dead_l = dead_l;
        c.dead_lw = dead_lw;
        c.pool_x = pool_x;
        c.pool_l = pool_l;
        c.pool_pos = pool_pos;
        if (multi && !bound.ell.empty()) {
            c.bound = {(double)bound.ell.size(), (double)bound_iter};
            for (const Ellipsoid& e : bound.ell) {
                c.bound.push_back(e.scale);
                c.bound.insert(c.bound.end(), e.mu.begin(), e.mu.end());
                c.bound.insert(c.bound.end(), e.L.begin(), e.L.end());
            }
        }
        return save_state(opt.checkpoint, c);
    };
    // live points ordered by logL in a binary min-heap (ties by index, the
    // point a scan for the first minimum would pick), and the largest logL:
    // O(log nlive) per iteration instead of a scan of the live set
    std::vector<std::pair<double, int>> order(nl);
    double lmax = -HUGE_VAL;
    for (int i = 0; i < nl; ++i) {
        order[i] = {llive[i], i};
        lmax = std::max(lmax, llive[i]);
    }
    const auto later = [](const std::pair<double, int>& a, const std::pair<double, int>& b) { return a > b; };
    std::make_heap(order.begin(), order.end(), later);
    for (;; ++iter) {
        if (opt.checkpoint && opt.checkpoint_every > 0 && iter > 0 && iter % opt.checkpoint_every == 0 &&
            !checkpoint()) {
            err = std::string("nested sampling: cannot write the checkpoint ") + opt.checkpoint;
            return LG_ERR_INPUT;
        }
        if (opt.maxiter > 0 && iter >= opt.maxiter) {
            if (!checkpoint()) {
                err = std::string("nested sampling: cannot write the checkpoint ") + opt.checkpoint;
                return LG_ERR_INPUT;
            }
            break;
        }
        const int imin = order.front().second;
        // termination: the live points can still add at most X * Lmax; or
        // they all share one logL (a plateau at the top: nothing above it
        // to draw, and the rest of the evidence is exactly X * L)
        if ((iter > 0 && logaddexp(logz, logx + lmax) - logz < opt.tol) || llive[imin] == lmax) {
            if (!checkpoint()) {
                err = std::string("nested sampling: cannot write the checkpoint ") + opt.checkpoint;
                return LG_ERR_INPUT;
            }
            break;
        }
        const double lmin = llive[imin];
        // live points tied at the lowest logL (a plateau, e.g. -inf where
        // the priors' bounds reject a draw): the j-th of them to leave
        // shrinks ln X by 1 / (nlive - j), as if the j before it had not
        // been replaced, so that the plateau's share of the volume is
        // estimated by its share of the live points (Fowlie, Handley & Su
        // 2021); a lone lowest point shrinks it by the usual 1 / nlive
        if (lmin == plat_level) {
            ++plat_j;
        } else {
            plat_level = lmin;
            plat_j = 0;
        }
        const double step = plat_j == 0 ? dlogx : 1.0 / (double)std::max<long>(nl - plat_j, 1);
        const double lw = logx + (plat_j == 0 ? lw_step : std::log1p(-std::exp(-step))) + lmin;
        const double lznew = logaddexp(logz, lw);
        H = (lmin == -HUGE_VAL ? 0 : std::exp(lw - lznew) * lmin) +
            (logz == -HUGE_VAL ? 0 : std::exp(logz - lznew) * (H + logz)) - lznew;
        logz = lznew;
        logx -= step;
        dead_x.insert(dead_x.end(), &live[(size_t)imin * nd], &live[(size_t)imin * nd] + nd);
        dead_l.push_back(lmin);
        dead_lw.push_back(lw);
        // learned proposal: (re)train every flow_every replacements
        if (learned && opt.flow_every > 0 && since_train >= opt.flow_every) {
            since_train = 0;
            const auto tt = clock::now();
            use_flow = learned->train(live.data(), nl, nd) == LG_OK;
            t_train += since(tt);
            if (std::getenv("LG_FLOW_DEBUG"))
                std::fprintf(stderr, "flow: iter %ld trained %d, flow batches failed so far %ld\n", iter,
                             (int)use_flow, n_flow_fail);
            pool_x.clear();
            pool_l.clear();
            pool_pos = 0;
        }
        if (learned && use_flow) {
            learned->advance(since_train);
            if (since_train > 0 && since_train % refit_every == 0) {
                const auto tt = clock::now();
                learned->refresh(live.data(), nl, nd);
                t_train += since(tt);
            }
        }
        // replacement: next pool point above the threshold, else a new batch
        bool replaced = false;
        for (int attempt = 0; attempt < 100000 && !replaced; ++attempt) {
            while (pool_pos < pool_l.size() && !(pool_l[pool_pos] > lmin)) ++pool_pos;
            if (pool_pos < pool_l.size()) {
                std::memcpy(&live[(size_t)imin * nd], &pool_x[pool_pos * nd], nd * sizeof(double));
                llive[imin] = pool_l[pool_pos];
                std::pop_heap(order.begin(), order.end(), later);
                order.back() = {llive[imin], imin};
                std::push_heap(order.begin(), order.end(), later);
                lmax = std::max(lmax, llive[imin]);
                ++pool_pos;
                ++pool_used;
                replaced = true;
                break;
            }
            // constant efficiency mode: the batch just used up accepted a
            // fraction acc of its proposals; move the enlargement halfway
            // (in log) towards the target efr, within [0.1, 10]
            if (opt.ceff && pool_ell && !pool_l.empty()) {
                const double acc = std::max((double)pool_used, 0.5) / (double)pool_l.size();
                log_enl = std::min(std::log(10.0), std::max(std::log(0.1), log_enl + 0.5 * std::log(acc / opt.efr)));
            }
            // propose a batch: the learned proposal when it is trained, the
            // ellipsoid when it is not or when it yields nothing
            int n = 0;
            const auto tp = clock::now();
            // the ellipsoid bounds the live points other than the one leaving
            std::vector<double> others;
            others.reserve((size_t)(nl - 1) * nd);
            for (int i = 0; i < nl; ++i)
                if (i != imin) others.insert(others.end(), &live[(size_t)i * nd], &live[(size_t)i * nd] + nd);
            double bound_logv;
            if (multi) {
                if (bound.ell.empty() || iter - bound_iter >= refit_every) {
                    // (constant efficiency mode lifts the floor of X on the volume)
                    if (!bound.fit(others, nl - 1, nd, opt.ceff ? std::exp(log_enl) : 1.0 / opt.efr,
                                   opt.ceff ? -HUGE_VAL : logx, depth)) {
                        err = "nested sampling: degenerate live points";
                        return LG_ERR_INPUT;
                    }
                    bound_iter = iter;
                }
                bound_logv = bound.logv_sum;
            } else {
                if (!ell.fit(others, nl - 1, nd, opt.ceff ? std::exp(log_enl) : 1.0 / opt.efr)) {
                    err = "nested sampling: degenerate live points";
                    return LG_ERR_INPUT;
                }
                bound_logv = ell.log_volume();
            }
            // the learned bound is used when it is the tighter of the two,
            // its volume weighted by the cost of drawing from it (fixed by
            // the options, so that runs repeat)
            if (use_flow && learned->log_volume() + learned->log_cost() < bound_logv) {
                n = learned->propose(live.data(), nl, nd, buf.data(), B, rng.next());
                if (n > 0) n_flow += n;
                else n = 0, ++n_flow_fail;
            }
            const int from_ell = n == 0;
            if (n == 0 && drawer) {
                // the ellipsoids' draws on the GPU
                std::vector<double> packed, logv;
                auto pack = [&](const Ellipsoid& e) {
                    packed.insert(packed.end(), e.mu.begin(), e.mu.end());
                    packed.insert(packed.end(), e.L.begin(), e.L.end());
                    packed.push_back(e.scale);
                    logv.push_back(e.log_volume());
                };
                if (multi)
                    for (const Ellipsoid& e : bound.ell) pack(e);
                else
                    pack(ell);
                n = drawer->draw(nd, (int)logv.size(), packed.data(), logv.data(), opt.wrap, buf.data(), B,
                                 rng.next());
                if (n < 0) {
                    err = "nested sampling: GPU ellipsoid draws failed";
                    return LG_ERR_CUDA;
                }
                n_ell += n;
                if (n == 0) {
                    err = "nested sampling: ellipsoid left the unit cube";
                    return LG_ERR_INPUT;
                }
            }
            if (n == 0) {
                long tries = 0;
                while (n < B && tries < 1000L * B) {
                    ++tries;
                    double* x = &buf[(size_t)n * nd];
                    if (multi) {
                        if (!bound.sample(rng, x, u, y)) continue;
                    } else {
                        ell.sample(rng, x, u);
                    }
                    bool in = true;
                    for (int a = 0; a < nd && in; ++a) {
                        if (opt.wrap && opt.wrap[a]) x[a] -= std::floor(x[a]);
                        in = x[a] >= 0 && x[a] <= 1;
                    }
                    if (in) ++n;
                }
                n_ell += n;
                if (n == 0) {
                    err = "nested sampling: ellipsoid left the unit cube";
                    return LG_ERR_INPUT;
                }
            }
            t_prop += since(tp);
            if (int rc = evaluate(buf.data(), n, lbuf.data())) {
                err = "likelihood callback failed";
                return rc;
            }
            pool_x.assign(buf.begin(), buf.begin() + (size_t)n * nd);
            pool_l.assign(lbuf.begin(), lbuf.begin() + n);
            pool_used = 0;
            pool_ell = from_ell;
            for (auto& v : pool_l)
                if (std::isnan(v)) v = -HUGE_VAL;
            pool_pos = 0;
        }
        if (!replaced) {
            status = LG_ERR_TIMEOUT;
            err = "nested sampling: no replacement found above the threshold";
            break;
        }
        ++since_train;
    }
    // remaining live points share the last prior volume
    const double lwl = logx - std::log((double)nl);
    for (int i = 0; i < nl; ++i) {
        const double lw = lwl + llive[i];
        const double lznew = logaddexp(logz, lw);
        H = (llive[i] == -HUGE_VAL ? 0 : std::exp(lw - lznew) * llive[i]) +
            (logz == -HUGE_VAL ? 0 : std::exp(logz - lznew) * (H + logz)) - lznew;
        logz = lznew;
        dead_x.insert(dead_x.end(), &live[(size_t)i * nd], &live[(size_t)i * nd] + nd);
        dead_l.push_back(llive[i]);
        dead_lw.push_back(lw);
    }
    // posterior moments in the cube
    const size_t ns = dead_l.size();
    std::vector<double> mean(nd, 0), m2(nd, 0);
    double wsum = 0, lbest = -HUGE_VAL;
    for (size_t i = 0; i < ns; ++i) {
        const double w = std::exp(dead_lw[i] - logz);
        wsum += w;
        lbest = std::max(lbest, dead_l[i]);
        for (int a = 0; a < nd; ++a) {
            mean[a] += w * dead_x[i * nd + a];
            m2[a] += w * dead_x[i * nd + a] * dead_x[i * nd + a];
        }
    }
    res->logz = logz;
    res->logz_err = std::sqrt(std::max(H, 0.0) / nl);
    res->information = H;
    res->max_logl = lbest;
    res->ncall = ncall;
    res->niter = iter;
    res->nsamples = (long)ns;
    res->n_flow_proposals = n_flow;
    res->n_ellipsoid_proposals = n_ell;
    res->wall_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    res->eval_s = t_eval;
    res->train_s = t_train;
    res->propose_s = t_prop;
    if (res->mean && res->std)
        for (int a = 0; a < nd; ++a) {
            res->mean[a] = mean[a] / wsum;
            res->std[a] = std::sqrt(std::max(m2[a] / wsum - res->mean[a] * res->mean[a], 0.0));
        }
    if (res->samples && res->sample_logwt && res->max_samples > 0) {
        const size_t n = std::min(ns, (size_t)res->max_samples);
        std::memcpy(res->samples, dead_x.data(), n * nd * sizeof(double));
        for (size_t i = 0; i < n; ++i) res->sample_logwt[i] = dead_lw[i] - logz;
    }
    return status;
}

}  // namespace lg

extern "C" {

lg_nested_options lg_nested_defaults(void)
{
    lg_nested_options o;
    std::memset(&o, 0, sizeof o);
    o.nlive = 300;     // src/input/options.c: nlive default
    o.tol = 0.1;       // src/input/options.c: tol default
    o.efr = 0.8;       // ellipsoid volume enlargement 1/efr
    o.batch = 1024;
    o.seed = 1;
    o.maxiter = 0;
    o.proposal = LG_PROPOSAL_ELLIPSOID;
    o.flow_every = 1000;
    o.wrap = nullptr;
    o.checkpoint = nullptr;
    o.checkpoint_every = 0;
    o.resume = 0;
    o.max_ellipsoids = 1;
    o.ceff = 0;
    return o;
}

int lg_nested_sample(int ndims, lg_batch_loglike fn, void* user, const lg_nested_options* opts,
                     lg_nested_result* result)
{
    std::string err;
    int rc = lg::nested_sample(ndims, fn, user, opts, result, nullptr, err);
    if (rc) lg::set_global_error(err.c_str());
    return rc;
}

}  // extern "C"

namespace {

struct CtxUser {
    lg_ctx* ctx;
    int max_batch;
};

int ctx_loglike(void* user, const double* cube, int B, double* logL)
{
    CtxUser* u = static_cast<CtxUser*>(user);
    for (int b0 = 0; b0 < B; b0 += u->max_batch) {
        const int n = std::min(u->max_batch, B - b0);
        const int nd = lg_ndims(u->ctx);
        int rc = lg_eval_cube_batch(u->ctx, cube + (size_t)b0 * nd, n, nullptr, logL + b0);
        if (rc) return rc;
    }
    return LG_OK;
}

}  // namespace

extern "C" int lg_nested_run(lg_ctx* ctx, const lg_nested_options* opts, const lg_flow_options* flow,
                             lg_nested_result* result)
{
    if (!ctx || !result) return LG_ERR_INPUT;
    lg_nested_options o = opts ? *opts : lg_nested_defaults();
    CtxUser u{ctx, lg::ctx_max_batch(ctx)};
    if (o.batch > u.max_batch) o.batch = u.max_batch;
    // periodic parameters from the priors' "wrap" keyword (src/lensed.c:1254-1259)
    std::vector<int> wrap(std::max(lg_ndims(ctx), 0), 0);
    if (!o.wrap) {
        for (int i = 0; i < (int)wrap.size(); ++i) lg_param(ctx, i, nullptr, &wrap[i], nullptr, nullptr);
        o.wrap = wrap.data();
    }
    std::string err;
    std::unique_ptr<lg::Proposal> prop;
    if (o.proposal == LG_PROPOSAL_FLOW) {
        prop.reset(lg::make_flow_proposal(lg::ctx_device(ctx), lg_ndims(ctx), flow, err));
        if (!prop) {
            lg::set_global_error(err.c_str());
            return LG_ERR_ALLOC;
        }
    }
    std::unique_ptr<lg::EllipsoidDrawer> drawer(lg::make_gpu_ellipsoid_drawer(lg::ctx_device(ctx), err));
    int rc = lg::nested_sample(lg_ndims(ctx), ctx_loglike, &u, &o, result, prop.get(), err, drawer.get());
    if (rc) lg::set_global_error(err.c_str());
    return rc;
}

extern "C" int lg_nested_sample_flow(int ndims, lg_batch_loglike fn, void* user, const lg_nested_options* opts,
                                     const lg_flow_options* flow, int device, lg_nested_result* result)
{
    std::string err;
    std::unique_ptr<lg::Proposal> prop(lg::make_flow_proposal(device, ndims, flow, err));
    if (!prop) {
        lg::set_global_error(err.c_str());
        return LG_ERR_ALLOC;
    }
    lg_nested_options o = opts ? *opts : lg_nested_defaults();
    o.proposal = LG_PROPOSAL_FLOW;
    std::unique_ptr<lg::EllipsoidDrawer> drawer(lg::make_gpu_ellipsoid_drawer(device, err));
    int rc = lg::nested_sample(ndims, fn, user, &o, result, prop.get(), err, drawer.get());
    if (rc) lg::set_global_error(err.c_str());
    return rc;
}
