// Plugin registry, priors, quadrature rules and model set-up (host side).
//
// The plugin table restates the parameter blocks of Lensed's objects/*.cl
// (names, types, bounds and defaults in the same order); the device code of
// each plugin is the CUDA source under lensed_gb300/objects/, embedded into
// this library at build time.

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>

#include "lg_internal.h"

namespace lg {

#include "lg_embed.inc"  // LG_EMBED_PRELUDE, LG_EMBED_KERNELS, LG_EMBED_OBJECTS[]

const char* prelude_source() { return LG_EMBED_PRELUDE; }
const char* kernels_source() { return LG_EMBED_KERNELS; }
const char* set_kernel_source() { return LG_EMBED_SET_KERNEL; }
const char* crmath_source() { return LG_EMBED_CRMATH; }
const char* multi_kernels_source() { return LG_EMBED_MULTI; }
const char* crf_source() { return LG_EMBED_CRF; }
const char* exact_pair_source() { return LG_EMBED_EXACT_PAIR; }

namespace {

const char* embedded_object(const char* name)
{
    for (const auto& e : LG_EMBED_OBJECTS)
        if (std::strcmp(e.name, name) == 0) return e.text;
    return nullptr;
}

ParamDef P(const char* n, int type, float lo = 0, float hi = 0, float def = 0)
{
    ParamDef p;
    p.name = n;
    p.type = type;
    p.lower = lo;
    p.upper = hi;
    p.defval = def;
    return p;
}

std::vector<Plugin> builtin_plugins()
{
    const ParamDef X = P("x", LG_POSITION_X), Y = P("y", LG_POSITION_Y), R = P("r", LG_RADIUS);
    const ParamDef Q = P("q", LG_AXIS_RATIO), PA = P("pa", LG_POS_ANGLE), MAG = P("mag", LG_MAGNITUDE);
    const ParamDef G1 = P("g1", LG_PARAMETER), G2 = P("g2", LG_PARAMETER);
    const ParamDef T = P("t", LG_PARAMETER, 0.f, 2.f), RC = P("rc", LG_RADIUS);
    std::vector<Plugin> v;
    auto add = [&](const char* name, int kind, std::vector<ParamDef> pars, std::vector<std::string> deps = {}) {
        Plugin p;
        p.name = name;
        p.kind = kind;
        p.pars = pars;
        p.deps = deps;
        p.paired = true;
        p.builtin = true;
        const char* src = embedded_object(name);
        p.source = src ? src : "";
        v.push_back(p);
    };
    add("sis", LG_LENS, {X, Y, R});                                       // objects/sis.cl:6-11
    add("sis_plus_shear", LG_LENS, {X, Y, R, G1, G2});                    // objects/sis_plus_shear.cl:5-12
    add("nsis", LG_LENS, {X, Y, R, RC});                                  // objects/nsis.cl:6-12
    add("sie", LG_LENS, {X, Y, R, Q, PA});                                // objects/sie.cl:6-13
    add("sie_plus_shear", LG_LENS, {X, Y, R, Q, PA, G1, G2});             // objects/sie_plus_shear.cl:6-15
    add("nsie", LG_LENS, {X, Y, R, RC, Q, PA});                           // objects/nsie.cl:6-14
    add("point_mass", LG_LENS, {X, Y, R});                                // objects/point_mass.cl:5-10
    add("epl", LG_LENS, {X, Y, R, T, Q, PA});                             // objects/epl.cl:5-13
    add("epl_plus_shear", LG_LENS, {X, Y, R, T, Q, PA, G1, G2}, {"epl"}); // objects/epl_plus_shear.cl:5-15
    add("sersic", LG_SOURCE, {X, Y, R, MAG, P("n", LG_PARAMETER, 0.f, FLT_MAX), Q, PA});  // objects/sersic.cl:3-12
    add("sersic_old", LG_SOURCE, {X, Y, R, MAG, P("n", LG_PARAMETER, 0.5f, 8.0f), Q, PA},
        {"sersic"});                                                      // objects/sersic-old.cl:3-12
    add("exponential", LG_SOURCE, {X, Y, P("rs", LG_RADIUS), MAG, Q, PA}); // objects/exponential.cl:3-11
    add("devauc", LG_SOURCE, {X, Y, R, MAG, Q, PA});                      // objects/devauc.cl:8-16
    add("gauss", LG_SOURCE, {X, Y, P("sigma", LG_RADIUS), MAG, Q, PA});   // objects/gauss.cl:3-11
    add("sky", LG_FOREGROUND,
        {P("bg", LG_PARAMETER), P("dx", LG_PARAMETER, 0, 0, -0.0f), P("dy", LG_PARAMETER, 0, 0, -0.0f)});  // objects/sky.cl:3-8
    return v;
}

std::mutex g_mu;
// A deque keeps references to entries valid when plugins are registered.
std::deque<Plugin>& plugins()
{
    static std::deque<Plugin> v = [] {
        std::vector<Plugin> b = builtin_plugins();
        return std::deque<Plugin>(b.begin(), b.end());
    }();
    return v;
}

}  // namespace

const Plugin* find_plugin(const std::string& name)
{
    std::lock_guard<std::mutex> lk(g_mu);
    std::string n = name;
    if (n == "sersic-old") n = "sersic_old";  // the reference's file name
    for (const auto& p : plugins())
        if (p.name == n) return &p;
    return nullptr;
}

int plugin_count()
{
    std::lock_guard<std::mutex> lk(g_mu);
    return (int)plugins().size();
}

const Plugin* plugin_at(int i)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (i < 0 || i >= (int)plugins().size()) return nullptr;
    return &plugins()[i];
}

int register_plugin(const lg_plugin_desc* d, std::string& err)
{
    if (!d || !d->name || !d->source || d->npars < 0 || (d->npars > 0 && !d->par_names)) {
        err = "register_plugin: incomplete description";
        return LG_ERR_INPUT;
    }
    for (const char* c = d->name; *c; ++c)
        if (!(std::isalnum((unsigned char)*c) || *c == '_')) {
            err = std::string("register_plugin: invalid name ") + d->name;
            return LG_ERR_INPUT;
        }
    if (d->kind != LG_LENS && d->kind != LG_SOURCE && d->kind != LG_FOREGROUND) {
        err = "register_plugin: invalid kind";
        return LG_ERR_INPUT;
    }
    Plugin p;
    p.name = d->name;
    p.kind = d->kind;
    p.source = d->source;
    for (int j = 0; j < d->npars; ++j) {
        ParamDef q;
        q.name = d->par_names[j];
        q.type = d->par_types ? d->par_types[j] : LG_PARAMETER;
        q.lower = d->par_bounds ? d->par_bounds[2 * j] : 0;
        q.upper = d->par_bounds ? d->par_bounds[2 * j + 1] : 0;
        q.defval = d->par_defaults ? d->par_defaults[j] : 0;
        p.pars.push_back(q);
    }
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& e : plugins())
        if (e.name == p.name) {
            err = "register_plugin: name already registered: " + p.name;
            return LG_ERR_INPUT;
        }
    if (plugins().size() >= 256) {
        err = "register_plugin: registry full";
        return LG_ERR_UNSUPPORTED;
    }
    plugins().push_back(p);
    return LG_OK;
}

// ------------------------------------------------------------------ priors

// Inverse normal CDF approximation of Abramowitz & Stegun 26.2.23, the
// transform of Lensed's normal prior (src/prior/norm.c:9-16).
double norm_quantile(double u)
{
    double t = (u < 0.5) ? std::sqrt(-2.0 * std::log(u)) : std::sqrt(-2.0 * std::log(1 - u));
    t = t - ((0.010328 * t + 0.802853) * t + 2.515517) / (((0.001308 * t + 0.189269) * t + 1.432788) * t + 1.);
    return (u < 0.5) ? -t : t;
}

double Prior::apply(double u) const
{
    switch (kind) {
    case DELTA: return a;                       // src/prior/delta.c
    case UNIF: return a + u * (b - a);          // src/prior/unif.c:68-73
    case NORM: return a + b * norm_quantile(u); // src/prior/norm.c:77-82
    default: return NAN;
    }
}
double Prior::lower() const
{
    switch (kind) {
    case DELTA: return a;
    case UNIF: return a;
    case NORM: return a - 7 * b;  // src/prior/norm.c:84-96
    default: return -HUGE_VAL;
    }
}
double Prior::upper() const
{
    switch (kind) {
    case DELTA: return a;
    case UNIF: return b;
    case NORM: return a + 7 * b;
    default: return HUGE_VAL;
    }
}

static bool read_real(const char* s, double& v)
{
    char* end = nullptr;
    v = std::strtod(s, &end);
    return end && end != s && *end == '\0';
}

// "[wrap] [image] <value> | unif a b | norm m s" (src/input/objects.c:330-358,
// src/prior.c:68-159).
bool parse_prior(const char* s, Prior& p, std::string& err)
{
    p = Prior();
    std::vector<std::string> tok;
    const char* ws = " \t\n\v\f\r";
    std::string str(s ? s : "");
    size_t pos = 0;
    while (pos < str.size()) {
        size_t b = str.find_first_not_of(ws, pos);
        if (b == std::string::npos) break;
        size_t e = str.find_first_of(ws, b);
        tok.push_back(str.substr(b, e == std::string::npos ? std::string::npos : e - b));
        pos = e == std::string::npos ? str.size() : e;
    }
    size_t i = 0;
    while (i < tok.size() && (tok[i] == "wrap" || tok[i] == "image")) {
        if (tok[i] == "wrap") p.wrap = true;
        else p.ipp = true;
        ++i;
    }
    std::vector<std::string> args(tok.begin() + i, tok.end());
    double v = 0, w = 0;
    if (args.empty()) {
        p.kind = Prior::NONE;
        return true;
    }
    if (args.size() == 1 && read_real(args[0].c_str(), v)) {
        p.kind = Prior::DELTA;
        p.a = v;
        return true;
    }
    if (args[0] == "unif" || args[0] == "norm") {
        if (args.size() != 3 || !read_real(args[1].c_str(), v) || !read_real(args[2].c_str(), w)) {
            err = std::string("invalid prior definition: ") + str;
            return false;
        }
        p.kind = args[0] == "unif" ? Prior::UNIF : Prior::NORM;
        p.a = v;
        p.b = w;
        return true;
    }
    if (args[0] == "delta") {
        err = std::string("invalid prior definition: ") + str;
        return false;
    }
    err = std::string("unknown prior: ") + args[0];
    return false;
}

// -------------------------------------------------------------- quadrature
typedef QuadRuleData lg_quad_rule_data;
#include "lg_quad_rules.inc"

const QuadRuleData* quad_rule(const char* name)
{
    for (const QuadRuleData* r = LG_QUAD_RULES; r->name; ++r)
        if (std::strcmp(r->name, name) == 0) return r;
    return nullptr;
}
int quad_rule_count()
{
    int n = 0;
    while (LG_QUAD_RULES[n].name) ++n;
    return n;
}
const QuadRuleData* quad_rule_at(int i) { return (i >= 0 && i < quad_rule_count()) ? &LG_QUAD_RULES[i] : nullptr; }

// ------------------------------------------------------------------- model
int build_model(const lg_image_desc* img, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                Model& m, std::string& err)
{
    m = Model();
    if (!img || img->width <= 0 || img->height <= 0) {
        err = "invalid image size";
        return LG_ERR_INPUT;
    }
    if ((long)img->width * img->height > (1L << 30)) {
        err = "image too large";
        return LG_ERR_INPUT;
    }
    if (!objs || nobjs <= 0) {
        err = "no objects were given";
        return LG_ERR_INPUT;
    }
    m.width = img->width;
    m.height = img->height;
    if (img->pcs[0] || img->pcs[1] || img->pcs[2] || img->pcs[3])
        for (int i = 0; i < 4; ++i) m.pcs[i] = img->pcs[i];
    const char* rn = (opts && opts->rule) ? opts->rule : "g3k7";
    m.rule = quad_rule(rn);
    if (!m.rule) {
        err = std::string("invalid quadrature rule: ") + rn;
        return LG_ERR_INPUT;
    }
    if (img->psf) {
        // the normalised PSF lives in constant memory next to the quadrature
        // table: up to 101 x 101 taps
        if (img->psf_width <= 0 || img->psf_height <= 0 || img->psf_width > 101 || img->psf_height > 101) {
            err = "invalid PSF size (1..101 per side)";
            return LG_ERR_INPUT;
        }
        // src/data.c:354-370: normalise to unit sum
        double norm = 0;
        const long np = (long)img->psf_width * img->psf_height;
        for (long i = 0; i < np; ++i) norm += img->psf[i];
        if (!(norm != 0) || !std::isfinite(norm)) {
            err = "PSF has no finite normalisation";
            return LG_ERR_INPUT;
        }
        m.psfw = img->psf_width;
        m.psfh = img->psf_height;
        m.psf.resize(np);
        for (long i = 0; i < np; ++i) m.psf[i] = (float)(img->psf[i] / norm);
    }
    // objects and parameters (src/input/objects.c:200-240, src/lensed.c:139-262)
    int nplanes = 0, typ = 0;
    for (int i = 0; i < nobjs; ++i) {
        ObjectInfo o;
        if (!objs[i].name) {
            err = "object without plugin name";
            return LG_ERR_INPUT;
        }
        o.plugin = find_plugin(objs[i].name);
        if (!o.plugin) {
            err = std::string("could not load object \"") + objs[i].name + "\"";
            return LG_ERR_INPUT;
        }
        if (o.plugin->source.empty()) {
            err = std::string("object \"") + objs[i].name + "\" has no device source";
            return LG_ERR_INPUT;
        }
        o.id = objs[i].id ? objs[i].id : (std::string(o.plugin->name) + std::to_string(i));
        for (const auto& q : m.objs)
            if (q.id == o.id) {
                err = "duplicate object name: " + o.id;
                return LG_ERR_INPUT;
            }
        // src/input/ini.c:243-262: one lens plane only
        if (o.plugin->kind != typ && o.plugin->kind != LG_FOREGROUND) {
            if (o.plugin->kind == LG_LENS && ++nplanes > 1) {
                err = "multiple lensing planes are not supported";
                return LG_ERR_UNSUPPORTED;
            }
            typ = o.plugin->kind;
        }
        o.par0 = (int)m.pars.size();
        const int np = (int)o.plugin->pars.size();
        for (int j = 0; j < np; ++j) {
            const ParamDef& d = o.plugin->pars[j];
            ParamInfo p;
            p.id = o.id + "." + d.name;
            p.object = i;
            p.index = j;
            p.type = d.type;
            p.lower = d.lower;
            p.upper = d.upper;
            // src/input/objects.c:225-226: a positive or negative-zero default
            // becomes a fixed (delta) prior
            if (d.defval > 0 || std::signbit(d.defval)) {
                p.prior.kind = Prior::DELTA;
                p.prior.a = d.defval;
                p.has_prior = true;
            }
            if (objs[i].priors && objs[i].priors[j]) {
                Prior pr;
                if (!parse_prior(objs[i].priors[j], pr, err)) {
                    err = p.id + ": " + err;
                    return LG_ERR_INPUT;
                }
                p.prior = pr;
                p.has_prior = pr.kind != Prior::NONE;
            }
            if (objs[i].priors && !p.has_prior) {
                err = "missing prior: " + p.id;
                return LG_ERR_INPUT;
            }
            // src/lensed.c:150-170: default bounds for radii and axis ratios
            if (!p.lower && !p.upper) {
                if (p.type == LG_RADIUS) {
                    p.lower = 0;
                    p.upper = HUGE_VAL;
                } else if (p.type == LG_AXIS_RATIO) {
                    p.lower = 0;
                    p.upper = 1;
                }
            }
            p.bounded = (p.lower || p.upper);
            // src/lensed.c:172-201: a prior entirely outside the bounds is an
            // error (a partial overlap is accepted)
            if (p.has_prior && p.bounded && (p.prior.lower() < p.lower || p.prior.upper() > p.upper) &&
                (p.prior.lower() >= p.upper || p.prior.upper() <= p.lower)) {
                err = p.id + ": prior does not include parameter bounds";
                return LG_ERR_INPUT;
            }
            p.derived = p.has_prior && p.prior.pseudo();
            m.pars.push_back(p);
        }
        // image-plane priors come in (x, y) pairs (src/lensed.c:203-239)
        for (int j = 0; j < np; ++j) {
            const ParamInfo& p = m.pars[o.par0 + j];
            if (!p.prior.ipp) continue;
            if (p.type == LG_POSITION_X) {
                if (j + 1 == np || m.pars[o.par0 + j + 1].type != LG_POSITION_Y ||
                    !m.pars[o.par0 + j + 1].prior.ipp) {
                    err = "object `" + o.id + "`: image plane prior requires pair (X,Y) of parameters";
                    return LG_ERR_INPUT;
                }
                if (j != 0) {
                    err = "object `" + o.id + "`: image plane prior supported on the leading (x, y) pair only";
                    return LG_ERR_UNSUPPORTED;
                }
                o.ipp = true;
            } else if (p.type == LG_POSITION_Y) {
                if (j == 0 || m.pars[o.par0 + j - 1].type != LG_POSITION_X || !m.pars[o.par0 + j - 1].prior.ipp) {
                    err = "object `" + o.id + "`: image plane prior requires pair (X,Y) of parameters";
                    return LG_ERR_INPUT;
                }
            } else {
                err = "prior `" + p.id + "`: cannot give image plane prior for this parameter";
                return LG_ERR_INPUT;
            }
        }
        m.objs.push_back(o);
    }
    // parameter map: free parameters first, derived (pseudo-prior) ones last
    std::vector<int> derived;
    for (int p = 0; p < (int)m.pars.size(); ++p) {
        if (m.pars[p].derived) derived.push_back(p);
        else m.pmap.push_back(p);
    }
    m.ndims = (int)m.pmap.size();
    for (int p : derived) m.pmap.push_back(p);
    return LG_OK;
}

}  // namespace lg
