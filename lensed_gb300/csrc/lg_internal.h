// Internal declarations shared by the host sources of liblensed_gb300.
#pragma once

#include <string>
#include <vector>

#include "lensed_gb300.h"

#include <cuda.h>

namespace lg {

// Driver API entry points, resolved through the runtime so the library loads
// on machines without a CUDA driver (the compile check needs no GPU).
struct Driver {
    CUresult (*moduleLoadData)(CUmodule*, const void*) = nullptr;
    CUresult (*moduleUnload)(CUmodule) = nullptr;
    CUresult (*moduleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
    CUresult (*moduleGetGlobal)(CUdeviceptr*, size_t*, CUmodule, const char*) = nullptr;
    CUresult (*funcSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
    CUresult (*launchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                             CUstream, void**, void**) = nullptr;
    CUresult (*occupancy)(int*, CUfunction, int, size_t) = nullptr;
    bool ok = false;
};
const Driver* driver();
void set_global_error(const char* msg);
int ctx_device(const lg_ctx* c);
int ctx_max_batch(const lg_ctx* c);

// ------------------------------------------------------------------ plugins
struct ParamDef {
    std::string name;
    int type = LG_PARAMETER;
    float lower = 0, upper = 0;
    float defval = 0;
};

struct Plugin {
    std::string name;
    int kind = 0;
    std::vector<ParamDef> pars;
    std::string source;             // CUDA device source of the plugin
    std::vector<std::string> deps;  // plugins whose source must come first
    // evaluation functions are templates over the vector type (float2 or
    // lg_pair2), so the paired ray kernels can call them directly
    bool paired = false;
    bool builtin = false;  // one of the library's own plugins (host set_params exists for it)
};

const Plugin* find_plugin(const std::string& name);
int plugin_count();
const Plugin* plugin_at(int i);
int register_plugin(const lg_plugin_desc* d, std::string& err);

// Device sources embedded at build time.
const char* prelude_source();
const char* kernels_source();
const char* set_kernel_source();
const char* crmath_source();
const char* multi_kernels_source();
const char* crf_source();         // correctly rounded exp/log/atan/atanh in FP32 arithmetic
const char* exact_pair_source();  // their ray-pair overloads for the exact modules

// ------------------------------------------------------------------- priors
// Lensed's prior plugins (src/prior.c:47-51): delta (pseudo), unif, norm.
struct Prior {
    enum Kind { NONE = 0, DELTA, UNIF, NORM } kind = NONE;
    double a = 0, b = 0;   // delta: a = value; unif: [a, b]; norm: mean a, sigma b
    bool wrap = false;     // "wrap" keyword
    bool ipp = false;      // "image" keyword: image-plane prior
    double apply(double u) const;
    double lower() const;
    double upper() const;
    bool pseudo() const { return kind == DELTA; }
};
bool parse_prior(const char* s, Prior& p, std::string& err);
double norm_quantile(double u);

// ------------------------------------------------------------- quadrature
struct QuadRuleData {
    const char* name;
    const char* info;
    int size;
    const double (*absc)[2];
    const double* weig;
    const double* errw;
};
const QuadRuleData* quad_rule(const char* name);
int quad_rule_count();
const QuadRuleData* quad_rule_at(int i);

// ------------------------------------------------------------------ model
// A parameter of the model, in object order.
struct ParamInfo {
    std::string id;       // "<object>.<param>"
    int object = 0, index = 0, type = 0;
    double lower = 0, upper = 0;
    bool bounded = false;
    Prior prior;
    bool has_prior = false;
    bool derived = false;
};

struct ObjectInfo {
    std::string id;
    const Plugin* plugin = nullptr;
    int par0 = 0;         // first parameter (object order)
    bool ipp = false;     // (x, y) carry an image-plane prior
};

struct Model {
    std::vector<ObjectInfo> objs;
    std::vector<ParamInfo> pars;  // object order
    std::vector<int> pmap;        // map position -> object-order index
    int ndims = 0;
    int width = 0, height = 0;
    double pcs[4] = {1, 1, 1, 1};
    std::vector<float> psf;       // normalised
    int psfw = 0, psfh = 0;
    const QuadRuleData* rule = nullptr;
};

// Build the model from the C-ABI descriptions (priors, bounds, pmap, PSF
// normalisation); no device work.
int build_model(const lg_image_desc* img, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                Model& m, std::string& err);

// set_params on the host for small batches (lg_host_set.cpp): the built-in
// plugins' set functions compiled for the host with the same IEEE
// single-precision arithmetic (no contraction) and the same FP64-evaluated
// elementary functions as the set module, laid out as the device's
// lg_model.  ok is false when a plugin has no host code.
struct HostSetLayout {
    bool ok = false;
    size_t bytes = 0;            // sizeof(lg_model)
    std::vector<size_t> offset;  // per object
    std::vector<int> index;      // per object: entry of the host plugin table
};
HostSetLayout host_set_layout(const Model& m);
// Object data of one candidate (params: np doubles in map order) into out
// (L.bytes, zero padding).
void host_set_params(const Model& m, const HostSetLayout& L, const double* params, unsigned char* out);

// Launch-shape parameters baked into the program.
struct Shape {
    int rt = 128, rppt = 2;        // render threads / pixels per thread group
    int qs = 1;                    // threads per group splitting the quadrature points
    int ctx = 32, cty = 32, cr = 8; // convolution tile and outputs per thread
    bool pair_rows = false;        // convolution threads own two rows (f32x2)
    int conv_block_y() const { return pair_rows ? cty / 2 : cty; }
    int rtile() const { return rt / qs * rppt; }  // pixels per render block
    bool operator==(const Shape& o) const
    {
        return rt == o.rt && rppt == o.rppt && qs == o.qs && ctx == o.ctx && cty == o.cty && cr == o.cr &&
               pair_rows == o.pair_rows;
    }
    std::string str() const;
};

// Floating-point mode of the evaluation module.
//   EXACT   (default) rays traced in pairs with f32x2 instructions, no
//           contraction, IEEE division and square root, elementary functions
//           correctly rounded (lg_crfloat.cuh, or in double): every image is
//           bit-identical to the strict module's and the oracle's
//   STRICT  (LG_FLAG_STRICT_FP) one ray at a time, every elementary
//           function evaluated in double and rounded once: the definition
//           the exact mode reproduces
//   FAST    (LG_FLAG_FAST_MATH) ray pairs with FMA contraction and the
//           SFU-based functions of the prelude (a few ulp)
enum class Fp { FAST, EXACT, STRICT };
Fp fp_mode(int flags);
inline bool fp_fmad(Fp m) { return m == Fp::FAST; }
// IEEE division and square root per ray (the fast mode only with
// LG_FLAG_IEEE_DIV)
bool fp_ieee(int flags);

// Compose the NVRTC sources of a model and compile them to cubins for
// sm_103a.  The set_params module always uses the double-evaluated
// elementary functions and no FMA contraction; the evaluation module per
// its floating-point mode.
enum class Part { SET, EVAL };
std::string compose_source(const Model& m, const Shape& s, Fp mode, Part part);
// Evaluation module for a batch of systems sharing m's objects and rule; the
// PSF shapes (w, h) present in the batch get their own convolution code.
std::string compose_multi_source(const Model& m, const std::vector<std::pair<int, int>>& psf_shapes,
                                 const Shape& s, Fp mode);
int compile_program(const std::string& src, bool fmad, std::vector<char>& cubin, std::string& log,
                    bool ieee_divsqrt = true);

// ---------------------------------------------------------------- autotuner
// Candidate launch shapes around a base shape (lg_tune.cpp): render shapes
// vary threads, pixels per group and (fast mode) the quadrature split;
// convolution shapes vary the tile and outputs per thread.
std::vector<Shape> render_candidates(const Shape& base, Fp mode);
std::vector<Shape> conv_candidates(const Shape& base, bool multi = false);
// "" when the shape is valid for the program, else the reason.
std::string check_shape(const Shape& s, Fp mode, bool psf, int psfw);
// Compile several programs at once (NVRTC is thread-safe).
void compile_parallel(const std::vector<std::string>& srcs, bool fmad, bool ieee,
                      std::vector<std::vector<char>>& cubins, std::vector<int>& rcs, std::vector<std::string>& logs);
std::string device_signature(int device);
std::string tune_key(const std::string& program, int device, int batch, int flags);
bool tune_cache_get(const std::string& key, Shape& s);
void tune_cache_put(const std::string& key, const Shape& s);
void tune_cache_clear();

}  // namespace lg
