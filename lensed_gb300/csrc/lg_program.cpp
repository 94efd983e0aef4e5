// Composition of the per-model device program and its NVRTC compilation.
//
// This takes the place of Lensed's kernel assembly (src/kernel.c): the
// plugins' device code, a generated model section and the kernel templates
// are concatenated into one CUDA translation unit, specialised by compile-time
// constants (image size, quadrature rule, PSF) as the reference specialises its
// OpenCL program with -D options (src/kernel.c:881-944), and compiled for
// sm_103a.

#include <nvrtc.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <set>
#include <sstream>

#include "lg_internal.h"

namespace lg {

namespace {

// Exact float literal (C++17 hexadecimal floating literal).
std::string hexf(float v)
{
    char buf[64];
    std::snprintf(buf, sizeof buf, "%af", (double)v);
    return buf;
}

void emit_plugin(std::ostringstream& o, const Plugin* p, std::set<std::string>& done)
{
    if (done.count(p->name)) return;
    for (const auto& d : p->deps) {
        const Plugin* q = find_plugin(d);
        if (q) emit_plugin(o, q, done);
    }
    done.insert(p->name);
    o << "// ---- object plugin: " << p->name << "\n" << p->source << "\n";
}

// Generated compute(): objects in list order; a lens plane's deflections are
// summed and applied when the next source appears; foregrounds see the
// unlensed position (src/kernel.c:65-111, :235-399).
void emit_compute(std::ostringstream& o, const Model& m)
{
    o << "LG_DEV float lg_compute(const lg_model& m, float2 x)\n{\n"
      << "    float2 y = x;\n    float f = 0.0f;\n    float2 a = make_float2(0.0f, 0.0f);\n";
    int trigger = 0;
    for (size_t i = 0; i < m.objs.size(); ++i) {
        const Plugin* p = m.objs[i].plugin;
        if (p->kind != trigger && p->kind != LG_FOREGROUND) {
            if (trigger == LG_LENS) o << "    lg_deflect(y, a);\n    a = make_float2(0.0f, 0.0f);\n";
            trigger = p->kind;
        }
        if (p->kind == LG_LENS)
            o << "    a += lg_deflection_" << p->name << "(&m.o" << i << ", y);\n";
        else if (p->kind == LG_SOURCE)
            o << "    f += lg_brightness_" << p->name << "(&m.o" << i << ", y);\n";
        else
            o << "    f += lg_foreground_" << p->name << "(&m.o" << i << ", x);\n";
    }
    if (trigger == LG_LENS) o << "    lg_deflect(y, a);\n";
    o << "    return f;\n}\n\n";
}

// The same sum for two rays at once (lg_pair2), for the paired ray kernels
// of the fast mode: plugins with template evaluation functions are called
// with the pair; any other plugin is called once per ray.
void emit_compute2(std::ostringstream& o, const Model& m)
{
    o << "#define LG_PAIRED 1\n";
    o << "LG_DEV lg_pair lg_compute2(const lg_model& m, lg_pair2 x)\n{\n"
      << "    lg_pair2 y = x;\n    lg_pair f = lg_pair_of(0.0f);\n"
      << "    lg_pair2 a = {lg_pair_of(0.0f), lg_pair_of(0.0f)};\n";
    int trigger = 0;
    for (size_t i = 0; i < m.objs.size(); ++i) {
        const Plugin* p = m.objs[i].plugin;
        if (p->kind != trigger && p->kind != LG_FOREGROUND) {
            if (trigger == LG_LENS) o << "    lg_deflect(y, a);\n    a = {lg_pair_of(0.0f), lg_pair_of(0.0f)};\n";
            trigger = p->kind;
        }
        const char* fn = p->kind == LG_LENS ? "lg_deflection_" : (p->kind == LG_SOURCE ? "lg_brightness_" : "lg_foreground_");
        const char* acc = p->kind == LG_LENS ? "a" : "f";
        const char* arg = p->kind == LG_FOREGROUND ? "x" : "y";
        const std::string obj = "&m.o" + std::to_string(i);
        if (p->paired) {
            o << "    " << acc << " += " << fn << p->name << "(" << obj << ", " << arg << ");\n";
        } else if (p->kind == LG_LENS) {
            o << "    a += lg_pair2_join(" << fn << p->name << "(" << obj << ", lg_lane(y, 0)), " << fn << p->name
              << "(" << obj << ", lg_lane(y, 1)));\n";
        } else {
            o << "    f += lg_pair_of(" << fn << p->name << "(" << obj << ", lg_lane(" << arg << ", 0)), " << fn
              << p->name << "(" << obj << ", lg_lane(" << arg << ", 1)));\n";
        }
    }
    if (trigger == LG_LENS) o << "    lg_deflect(y, a);\n";
    o << "    return f;\n}\n\n";
}

// Generated set_params (src/kernel.c:114-150, :401-656), including the
// deflection of image-plane (x, y) priors through the lens planes before the
// object's own plane.
void emit_set_params(std::ostringstream& o, const Model& m)
{
    o << "LG_DEV void lg_set_params(lg_model& m, const float* p)\n{\n"
      << "    float2 x = make_float2(0.0f, 0.0f);\n    float2 a = make_float2(0.0f, 0.0f);\n"
      << "    (void)x;\n    (void)a;\n";
    int trigger = 0;
    size_t plane = 0;
    for (size_t i = 0; i < m.objs.size(); ++i) {
        const ObjectInfo& ob = m.objs[i];
        const Plugin* pl = ob.plugin;
        if (pl->kind != trigger && pl->kind != LG_FOREGROUND) {
            if (trigger == LG_LENS && pl->kind == LG_SOURCE) plane = i;
            trigger = pl->kind;
        }
        const int np = (int)pl->pars.size();
        if (ob.ipp) {
            int xp = -1;
            for (int j = 0; j < np; ++j)
                if (m.pars[ob.par0 + j].prior.ipp && pl->pars[j].type == LG_POSITION_X) xp = j;
            o << "    x = make_float2(p[" << ob.par0 + xp << "], p[" << ob.par0 + xp + 1 << "]);\n";
            int trigger2 = 0;
            for (size_t k = 0; k < plane; ++k) {
                const Plugin* q = m.objs[k].plugin;
                if (q->kind != trigger2 && q->kind != LG_FOREGROUND) {
                    if (trigger2 == LG_LENS) o << "    lg_deflect(x, a);\n    a = make_float2(0.0f, 0.0f);\n";
                    trigger2 = q->kind;
                }
                if (q->kind == LG_LENS) o << "    a += lg_deflection_" << q->name << "(&m.o" << k << ", x);\n";
            }
            if (trigger2 == LG_LENS) o << "    lg_deflect(x, a);\n    a = make_float2(0.0f, 0.0f);\n";
        }
        o << "    lg_set_" << pl->name << "(&m.o" << i;
        for (int j = 0; j < np; ++j) {
            const ParamInfo& pi = m.pars[ob.par0 + j];
            if (ob.ipp && pi.prior.ipp)
                o << ", " << (pl->pars[j].type == LG_POSITION_X ? "x.x" : (pl->pars[j].type == LG_POSITION_Y ? "x.y" : "0"));
            else
                o << ", p[" << ob.par0 + j << "]";
        }
        o << ");\n";
    }
    o << "}\n\n";
    // the same, one object at a time (for the kernel that gives every object
    // its own warp): objects with image-plane priors read the lenses of
    // earlier planes, so they run in a second phase
    o << "#define LG_NOBJ " << m.objs.size() << "\n";
    o << "__constant__ int lg_obj_phase[LG_NOBJ] = {";
    for (size_t i = 0; i < m.objs.size(); ++i) o << (i ? ", " : "") << (m.objs[i].ipp ? 1 : 0);
    o << "};\n";
    o << "LG_DEV void lg_set_object(lg_model& m, const float* p, int which)\n{\n"
      << "    float2 x = make_float2(0.0f, 0.0f);\n    float2 a = make_float2(0.0f, 0.0f);\n"
      << "    (void)x;\n    (void)a;\n    switch (which) {\n";
    trigger = 0;
    plane = 0;
    for (size_t i = 0; i < m.objs.size(); ++i) {
        const ObjectInfo& ob = m.objs[i];
        const Plugin* pl = ob.plugin;
        if (pl->kind != trigger && pl->kind != LG_FOREGROUND) {
            if (trigger == LG_LENS && pl->kind == LG_SOURCE) plane = i;
            trigger = pl->kind;
        }
        const int np = (int)pl->pars.size();
        o << "    case " << i << ": {\n";
        if (ob.ipp) {
            int xp = -1;
            for (int j = 0; j < np; ++j)
                if (m.pars[ob.par0 + j].prior.ipp && pl->pars[j].type == LG_POSITION_X) xp = j;
            o << "        x = make_float2(p[" << ob.par0 + xp << "], p[" << ob.par0 + xp + 1 << "]);\n";
            int trigger2 = 0;
            for (size_t k = 0; k < plane; ++k) {
                const Plugin* q = m.objs[k].plugin;
                if (q->kind != trigger2 && q->kind != LG_FOREGROUND) {
                    if (trigger2 == LG_LENS) o << "        lg_deflect(x, a);\n        a = make_float2(0.0f, 0.0f);\n";
                    trigger2 = q->kind;
                }
                if (q->kind == LG_LENS) o << "        a += lg_deflection_" << q->name << "(&m.o" << k << ", x);\n";
            }
            if (trigger2 == LG_LENS) o << "        lg_deflect(x, a);\n";
        }
        o << "        lg_set_" << pl->name << "(&m.o" << i;
        for (int j = 0; j < np; ++j) {
            const ParamInfo& pi = m.pars[ob.par0 + j];
            if (ob.ipp && pi.prior.ipp)
                o << ", " << (pl->pars[j].type == LG_POSITION_X ? "x.x" : (pl->pars[j].type == LG_POSITION_Y ? "x.y" : "0"));
            else
                o << ", p[" << ob.par0 + j << "]";
        }
        o << ");\n        break;\n    }\n";
    }
    o << "    default: break;\n    }\n}\n\n";
}

const char* mode_name(Fp mode) { return mode == Fp::FAST ? "fast" : (mode == Fp::EXACT ? "exact" : "strict"); }

// The prelude and the elementary-function layer of a module: the set_params
// module and the strict and exact evaluation modules map the plugins'
// float functions to the double-evaluated ones; the exact modules add the
// correctly rounded single-precision functions and their ray-pair overloads.
void emit_prelude(std::ostringstream& o, Fp mode, bool set)
{
    if (!set && mode == Fp::EXACT) o << "#define LG_EXACT 1\n";
    o << "\n" << prelude_source() << "\n";
    if (set || mode != Fp::FAST) o << crmath_source() << "\n";
    if (!set && mode == Fp::EXACT) o << crf_source() << "\n" << exact_pair_source() << "\n";
}

}  // namespace

std::string compose_source(const Model& m, const Shape& s, Fp mode, Part part)
{
    const bool set = part == Part::SET;
    const bool strict = mode == Fp::STRICT;
    std::ostringstream o;
    o << "// Lensed likelihood program (" << (set ? "set_params" : "evaluation") << " module) composed for:";
    for (const auto& ob : m.objs) o << " " << ob.id << "=" << ob.plugin->name;
    o << "\n// image " << m.width << "x" << m.height << ", rule " << m.rule->name << " (" << m.rule->size
      << " points), PSF " << m.psfw << "x" << m.psfh << ", " << mode_name(mode) << " FP\n\n";
    o << "#define LG_RT " << s.rt << "\n#define LG_RPPT " << s.rppt << "\n#define LG_QS " << s.qs << "\n";
    o << "#define LG_CTX " << s.ctx << "\n#define LG_CTY " << s.cty << "\n#define LG_CR " << s.cr << "\n";
    // the paired modes with a PSF up to 49 wide pair rows unless the shape says not
    if (!strict && !s.pair_rows && m.psfw <= 49) o << "#define LG_CONV_SINGLE 1\n";
    emit_prelude(o, mode, set);
    std::set<std::string> done;
    for (const auto& ob : m.objs) emit_plugin(o, ob.plugin, done);

    o << "// ---- model section\n";
    o << "#define LG_W " << m.width << "\n#define LG_H " << m.height << "\n#define LG_N (LG_W * LG_H)\n";
    o << "#define LG_NPARS " << m.pars.size() << "\n";
    o << "struct lg_model {\n";
    for (size_t i = 0; i < m.objs.size(); ++i)
        o << "    lg_data_" << m.objs[i].plugin->name << " o" << i << ";  // " << m.objs[i].id << "\n";
    o << "};\n\n";
    if (set) {
        emit_set_params(o, m);
        // parameter upload order: params[pmap[i]] = cube[i] (src/nested.c:70-71)
        o << "LG_DEV void lg_load_params(const double* __restrict__ src, float* p)\n{\n";
        for (size_t i = 0; i < m.pmap.size(); ++i) o << "    p[" << m.pmap[i] << "] = (float)src[" << i << "];\n";
        o << "}\n\n";
        o << set_kernel_source() << "\n";
        return o.str();
    }
    // pixel coordinate system, shifted by half a pixel for even PSF sizes
    // (src/lensed.c:871-891); stored in float as the reference's float4 pcs
    double rx = m.pcs[0], ry = m.pcs[1];
    if (!m.psf.empty()) {
        if (m.psfw % 2 == 0) rx += 0.5;
        if (m.psfh % 2 == 0) ry += 0.5;
    }
    o << "#define LG_RX (" << hexf((float)rx) << ")\n#define LG_RY (" << hexf((float)ry) << ")\n";
    o << "#define LG_SX (" << hexf((float)m.pcs[2]) << ")\n#define LG_SY (" << hexf((float)m.pcs[3]) << ")\n";
    // quadrature rule: abscissae scaled by the pixel scale in double, then
    // rounded to float (src/quadrature.c:32-43)
    const int nq = m.rule->size;
    o << "#define LG_Q " << nq << "\n";
    o << "__constant__ float2 lg_qq[LG_Q] = {";
    for (int n = 0; n < nq; ++n)
        o << (n ? ", " : "") << "{" << hexf((float)(m.pcs[2] * m.rule->absc[n][0])) << ", "
          << hexf((float)(m.pcs[3] * m.rule->absc[n][1])) << "}";
    o << "};\n__constant__ float2 lg_ww[LG_Q] = {";
    for (int n = 0; n < nq; ++n)
        o << (n ? ", " : "") << "{" << hexf((float)m.rule->weig[n]) << ", " << hexf((float)m.rule->errw[n]) << "}";
    o << "};\n";
    if (!m.psf.empty()) {
        o << "#define LG_HAS_PSF 1\n#define LG_PSF_W " << m.psfw << "\n#define LG_PSF_H " << m.psfh << "\n";
        o << "__constant__ float lg_psf[LG_PSF_W * LG_PSF_H] = {";
        for (size_t i = 0; i < m.psf.size(); ++i) o << (i ? (i % 8 ? ", " : ",\n    ") : "") << hexf(m.psf[i]);
        o << "};\n";
    } else {
        o << "#define LG_HAS_PSF 0\n";
    }
    emit_compute(o, m);
    if (!strict) emit_compute2(o, m);
    o << kernels_source() << "\n";
    return o.str();
}

std::string compose_multi_source(const Model& m, const std::vector<std::pair<int, int>>& psf_shapes,
                                 const Shape& s, Fp mode)
{
    const bool strict = mode == Fp::STRICT;
    std::ostringstream o;
    o << "// Lensed likelihood program (multi-system evaluation module) composed for:";
    for (const auto& ob : m.objs) o << " " << ob.id << "=" << ob.plugin->name;
    o << "\n// rule " << m.rule->name << " (" << m.rule->size << " points), " << mode_name(mode) << " FP\n\n";
    o << "#define LG_RT " << s.rt << "\n#define LG_RPPT " << s.rppt << "\n#define LG_QS " << s.qs << "\n";
    o << "#define LG_CTX " << s.ctx << "\n#define LG_CTY " << s.cty << "\n#define LG_CR " << s.cr << "\n";
    emit_prelude(o, mode, false);
    std::set<std::string> done;
    for (const auto& ob : m.objs) emit_plugin(o, ob.plugin, done);
    o << "// ---- model section\n#define LG_NPARS " << m.pars.size() << "\n";
    o << "struct lg_model {\n";
    for (size_t i = 0; i < m.objs.size(); ++i)
        o << "    lg_data_" << m.objs[i].plugin->name << " o" << i << ";  // " << m.objs[i].id << "\n";
    o << "};\n\n";
    const int nq = m.rule->size;
    o << "#define LG_Q " << nq << "\n";
    o << "__constant__ float2 lg_qq[LG_Q] = {";
    for (int n = 0; n < nq; ++n)
        o << (n ? ", " : "") << "{" << hexf((float)(m.pcs[2] * m.rule->absc[n][0])) << ", "
          << hexf((float)(m.pcs[3] * m.rule->absc[n][1])) << "}";
    o << "};\n__constant__ float2 lg_ww[LG_Q] = {";
    for (int n = 0; n < nq; ++n)
        o << (n ? ", " : "") << "{" << hexf((float)m.rule->weig[n]) << ", " << hexf((float)m.rule->errw[n]) << "}";
    o << "};\n";
    emit_compute(o, m);
    if (!strict) emit_compute2(o, m);
    o << "#define LG_PSF_SHAPES";
    for (const auto& ps : psf_shapes) o << " LG_PSF_CASE(" << ps.first << ", " << ps.second << ")";
    o << "\n";
    o << multi_kernels_source() << "\n";
    return o.str();
}

int compile_program(const std::string& src, bool fmad, std::vector<char>& cubin, std::string& log,
                    bool ieee_divsqrt)
{
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), "lensed_model.cu", 0, nullptr, nullptr);
    if (r != NVRTC_SUCCESS) {
        log = std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r);
        return LG_ERR_COMPILE;
    }
    std::vector<const char*> opts = {"--gpu-architecture=sm_103a", "-std=c++17", "--generate-line-info",
                                     "--ftz=false", "-diag-suppress=177"};
    opts.push_back(ieee_divsqrt ? "--prec-div=true" : "--prec-div=false");
    if (ieee_divsqrt) opts.push_back("-DLG_IEEE_DIVSQRT=1");  // paired-ray division and sqrt too
    opts.push_back(ieee_divsqrt ? "--prec-sqrt=true" : "--prec-sqrt=false");
    opts.push_back(fmad ? "--fmad=true" : "--fmad=false");
    if (const char* dump = std::getenv("LG_NVRTC_DUMP")) {
        static std::atomic<int> seq{0};
        std::string path = std::string(dump) + "." + std::to_string(seq++) + ".cu";
        if (FILE* f = std::fopen(path.c_str(), "w")) {
            std::fputs(src.c_str(), f);
            std::fclose(f);
        }
    }
    if (std::getenv("LG_NVRTC_VERBOSE")) {
        std::fprintf(stderr, "lensed_gb300: nvrtc");
        for (const char* o : opts) std::fprintf(stderr, " %s", o);
        std::fprintf(stderr, "\n");
    }
    r = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string l(n, '\0');
    if (n) nvrtcGetProgramLog(prog, &l[0]);
    while (!l.empty() && (l.back() == '\0' || l.back() == '\n')) l.pop_back();
    log = l;
    if (r != NVRTC_SUCCESS) {
        log = std::string("NVRTC: ") + nvrtcGetErrorString(r) + "\n" + log;
        nvrtcDestroyProgram(&prog);
        return LG_ERR_COMPILE;
    }
    nvrtcGetCUBINSize(prog, &n);
    cubin.resize(n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    return LG_OK;
}

}  // namespace lg
