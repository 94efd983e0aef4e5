// Context management, launches and the C ABI of liblensed_gb300.
//
// One context = one lens system resident on one GPU (image, weight, PSF,
// quadrature and the composed program), with scratch sized for max_batch
// candidates.  An evaluation of B candidates is three launches on the
// context's stream -- set_params, render, convolve+chi^2 (PSF only; the
// block finishing a candidate's last tile writes its logL) -- captured once
// per B into a CUDA graph together with the parameter upload and the logL
// read-back, then replayed.  This replaces, per
// candidate, the reference's map/unmap of the parameter buffer, four OpenCL
// enqueues, a blocking read of N floats and a host double loop
// (src/nested.c:63-115).

#include <cuda.h>
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "lg_internal.h"

namespace lg {

// batches up to this size go through mapped host memory in the host API
constexpr int kZeroCopyBatch = 64;
// batches up to this size through the host API take their object data from
// the host (lg_host_set.cpp) when the context's check passed
constexpr int kHostSet = 4;

namespace {
std::mutex g_drv_mu;
Driver g_drv;

template <class F>
bool resolve(const char* name, F& f)
{
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
        return false;
    f = reinterpret_cast<F>(p);
    return true;
}
}  // namespace

const Driver* driver()
{
    std::lock_guard<std::mutex> lk(g_drv_mu);
    if (!g_drv.ok) {
        Driver d;
        bool ok = resolve("cuModuleLoadData", d.moduleLoadData) && resolve("cuModuleUnload", d.moduleUnload) &&
                  resolve("cuModuleGetFunction", d.moduleGetFunction) &&
                  resolve("cuModuleGetGlobal", d.moduleGetGlobal) &&
                  resolve("cuFuncSetAttribute", d.funcSetAttribute) && resolve("cuLaunchKernel", d.launchKernel) &&
                  resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", d.occupancy);
        if (!ok) return nullptr;
        d.ok = true;
        g_drv = d;
    }
    return &g_drv;
}

}  // namespace lg

namespace {
using lg::Driver;
using lg::driver;

thread_local std::string g_create_error;

}  // namespace

namespace lg {
// Message returned by lg_last_error(NULL) on this thread.
void set_global_error(const char* msg) { g_create_error = msg ? msg : ""; }
}  // namespace lg

struct lg_ctx {
    lg::Model model;
    lg::Shape shape;
    int flags = 0;
    int device = 0;
    int max_batch = 1024;
    long N = 0;
    long masked = 0;
    bool psf = false;
    std::string err;

    const Driver* drv = nullptr;
    CUmodule mod = nullptr;      // evaluation module
    CUmodule mod_set = nullptr;  // set_params module
    CUfunction f_setp = nullptr, f_rraw = nullptr, f_rchi2 = nullptr, f_rdump = nullptr;
    CUfunction f_setp_split = nullptr;  // small batches: one warp per object
    int nobj = 0;
    CUfunction f_cchi2 = nullptr, f_cdump = nullptr;
    size_t model_bytes = 0;
    int rtiles = 0, ctiles = 0, ctiles_x = 0, ctiles_y = 0, cthreads = 0, csmem = 0;

    std::string tune_report;  // candidates and timings of the autotuner

    cudaStream_t stream = nullptr;
    // joins calls made on caller streams into the context's order
    cudaEvent_t ev_join = nullptr;
    float* d_image = nullptr;
    float* d_weight = nullptr;
    void* d_models = nullptr;
    float* d_raw = nullptr;
    double* d_partials = nullptr;
    unsigned* d_counters = nullptr;  // tiles done per candidate (zero between launches)
    double* d_params = nullptr;
    double* d_logL = nullptr;
    float* d_model_out = nullptr;
    float* d_err_out = nullptr;
    float* d_layers = nullptr;  // 6 x N output layers of lg_dump
    // unit-cube path: priors in map order, cube staging, rejection flags
    void* d_priors = nullptr;
    double* d_cube = nullptr;
    int* d_bad = nullptr;
    double* h_cube = nullptr;  // pinned
    int* h_bad = nullptr;      // pinned
    std::map<int, cudaGraphExec_t> cube_graphs;
    double* h_params = nullptr;  // pinned staging
    double* h_logL = nullptr;
    // host API, small batches: parameters and logL in mapped pinned memory
    // that the kernels read and write directly (no copy nodes in the graph)
    double* z_params = nullptr;  // host address
    double* z_logL = nullptr;
    double* zd_params = nullptr;  // device addresses of the same memory
    double* zd_logL = nullptr;
    double *z_cube = nullptr, *z_phys = nullptr, *zd_cube = nullptr, *zd_phys = nullptr;  // unit-cube path
    int *z_bad = nullptr, *zd_bad = nullptr;
    int last_bad = 0;  // rejection flag of the first point of the last unit-cube call
    std::map<int, cudaGraphExec_t> graphs;
    // batches of up to kHostSet through the host API: object data computed
    // on the host and copied in by the replayed graph (no set_params launch)
    lg::HostSetLayout hset;
    bool host_set = false;
    unsigned char* z_models = nullptr;  // pinned, kHostSet x model_bytes
    std::map<int, cudaGraphExec_t> hgraphs;

    int fail(int code, const std::string& msg)
    {
        err = msg;
        return code;
    }
    int cuda(cudaError_t e, const char* what)
    {
        if (e == cudaSuccess) return LG_OK;
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return LG_ERR_CUDA;
    }
    int drvcall(CUresult r, const char* what)
    {
        if (r == CUDA_SUCCESS) return LG_OK;
        err = std::string(what) + ": CUDA driver error " + std::to_string((int)r);
        return LG_ERR_CUDA;
    }
    int launch(CUfunction f, dim3 g, dim3 b, unsigned smem, cudaStream_t s, void** args, const char* what)
    {
        return drvcall(drv->launchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, smem, (CUstream)s, args, nullptr), what);
    }

    // Enqueue set_params, render and (with a PSF) convolve for B
    // candidates; params and logL are device pointers (the last stage ends
    // with logL, the block finishing a candidate's last tile summing its
    // partials).  With ev != NULL, ev[0..4] are recorded before set_params,
    // render, convolve and after the last stage (twice: no separate finish).
    // set_params for B candidates into d_models: a handful of candidates
    // get the objects of a candidate side by side (one warp each); else one
    // thread per candidate
    int launch_set(int B, const double* params, cudaStream_t s)
    {
        void* a_setp[] = {&params, &B, &d_models};
        const bool split = B <= 32 && nobj > 1 && nobj <= 32;
        return split ? launch(f_setp_split, dim3(B), dim3(32 * nobj), 0, s, a_setp, "set_params")
                     : launch(f_setp, dim3((B + 127) / 128), dim3(128), 0, s, a_setp, "set_params");
    }

    // set = false: the object data are already in d_models
    int enqueue(int B, const double* params, double* logL, cudaStream_t s, cudaEvent_t* ev = nullptr,
                bool set = true)
    {
        int rc;
        auto mark = [&](int i) { return ev ? cuda(cudaEventRecord(ev[i], s), "event") : LG_OK; };
        if ((rc = mark(0)) || (set && (rc = launch_set(B, params, s))) || (rc = mark(1))) return rc;
        if (psf) {
            void* a_r[] = {&d_models, &d_raw};
            if ((rc = launch(f_rraw, dim3(rtiles, B), dim3(shape.rt), 0, s, a_r, "render")) || (rc = mark(2)))
                return rc;
            void* a_c[] = {&d_raw, &d_image, &d_weight, &d_partials, &d_counters, &logL};
            if ((rc = launch(f_cchi2, dim3(ctiles_x, ctiles_y, B), dim3(shape.ctx / shape.cr, shape.conv_block_y()),
                             csmem, s, a_c, "convolve")) ||
                (rc = mark(3)))
                return rc;
            return mark(4);
        }
        void* a_r[] = {&d_models, &d_image, &d_weight, &d_partials, &d_counters, &logL};
        if ((rc = launch(f_rchi2, dim3(rtiles, B), dim3(shape.rt), 0, s, a_r, "render")) || (rc = mark(2)) ||
            (rc = mark(3)))
            return rc;
        return mark(4);
    }

    // every captured graph (they hold the evaluation module's kernels)
    void drop_graphs()
    {
        for (auto* m : {&graphs, &cube_graphs, &hgraphs}) {
            for (auto& g : *m) cudaGraphExecDestroy(g.second);
            m->clear();
        }
    }

    void release()
    {
        drop_graphs();
        cudaFreeHost(z_models);
        z_models = nullptr;
        cudaFree(d_priors);
        cudaFree(d_cube);
        cudaFree(d_bad);
        cudaFreeHost(h_cube);
        cudaFreeHost(h_bad);
        cudaFree(d_image);
        cudaFree(d_weight);
        cudaFree(d_models);
        cudaFree(d_raw);
        cudaFree(d_partials);
        cudaFree(d_counters);
        cudaFree(d_params);
        cudaFree(d_logL);
        cudaFree(d_model_out);
        cudaFree(d_err_out);
        cudaFree(d_layers);
        cudaFreeHost(h_params);
        cudaFreeHost(h_logL);
        cudaFreeHost(z_params);
        cudaFreeHost(z_logL);
        cudaFreeHost(z_cube);
        cudaFreeHost(z_phys);
        cudaFreeHost(z_bad);
        if (mod && drv) drv->moduleUnload(mod);
        if (mod_set && drv) drv->moduleUnload(mod_set);
        mod_set = nullptr;
        if (ev_join) cudaEventDestroy(ev_join);
        ev_join = nullptr;
        if (stream) cudaStreamDestroy(stream);
        mod = nullptr;
        stream = nullptr;
    }
};

int lg::ctx_device(const lg_ctx* c) { return c ? c->device : 0; }
int lg::ctx_max_batch(const lg_ctx* c) { return c ? c->max_batch : 0; }

namespace {

// Launch shape for a model (tile sizes chosen for GB300; see the design
// notes for the measurements behind them).
lg::Shape choose_shape(const lg::Model& m, lg::Fp mode)
{
    lg::Shape s;
    // fast and exact modes: 32 x 64 convolution tiles, each thread two rows
    // (paired); the register window of a thread holds 2 (8 + PSF width - 1)
    // floats, so PSFs wider than 49 pixels keep the single-row kernel
    if (!m.psf.empty() && mode != lg::Fp::STRICT && m.psfw <= 49) {
        s.cty = 64;
        s.pair_rows = true;
    }
    return s;
}

void shape_sizes(const lg::Shape& s, const lg::Model& m, lg_ctx* c)
{
    const long N = (long)m.width * m.height;
    const int rtile = s.rtile();
    c->rtiles = (int)((N + rtile - 1) / rtile);
    if (!m.psf.empty()) {
        // the shared-memory size is read back from the compiled module
        c->cthreads = (s.ctx / s.cr) * s.conv_block_y();
        c->ctiles_x = (m.width + s.ctx - 1) / s.ctx;
        c->ctiles_y = (m.height + s.cty - 1) / s.cty;
        c->ctiles = c->ctiles_x * c->ctiles_y;
    }
}

// ------------------------------------------------------------ priors --
// A parameter's prior and bounds in map order, for the unit-cube kernels.
struct DevPrior {
    int kind;     // lg::Prior::Kind
    int bounded;  // reject values outside [lower, upper]
    double a, b, lower, upper;
};

// Inverse normal CDF of Abramowitz & Stegun 26.2.23, the transform of the
// normal prior (src/prior/norm.c:9-16), with every product, sum and quotient
// rounded separately (no contraction), as the host evaluates it; log is
// CUDA's double-precision log.
__device__ double lg_norm_quantile(double u)
{
    const double v = u < 0.5 ? u : __dadd_rn(1.0, -u);
    double t = __dsqrt_rn(__dmul_rn(-2.0, log(v)));
    const double num = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(0.010328, t), 0.802853), t), 2.515517);
    const double den = __dadd_rn(
        __dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(0.001308, t), 0.189269), t), 1.432788), t), 1.0);
    t = __dadd_rn(t, -__ddiv_rn(num, den));
    return u < 0.5 ? -t : t;
}

// Unit cube (B x nd) -> physical parameters (B x np, map order) through the
// priors: the transform of src/nested.c:42-61, one candidate per thread.
// Pseudo-prior (derived) parameters, at map positions nd..np-1, take u = 0.5
// as there.  The reference redraws while a value is out of bounds, which
// never ends since the draw is a function of u (src/nested.c:54-56); here the
// candidate is flagged instead (bad[b] = 1) and its logL is set to -inf.
__global__ void __launch_bounds__(128)
    lg_prior_transform(const double* __restrict__ cube, int B, int nd, int np, const DevPrior* __restrict__ pri,
                       double* __restrict__ params, int* __restrict__ bad)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    int out = 0;
    for (int i = 0; i < np; ++i) {
        const DevPrior p = pri[i];
        const double u = i < nd ? cube[(size_t)b * nd + i] : 0.5;
        double v;
        switch (p.kind) {
        case lg::Prior::DELTA: v = p.a; break;                                              // src/prior/delta.c:50-53
        case lg::Prior::UNIF: v = __dadd_rn(p.a, __dmul_rn(u, __dadd_rn(p.b, -p.a))); break;  // src/prior/unif.c:68-73
        case lg::Prior::NORM: v = __dadd_rn(p.a, __dmul_rn(p.b, lg_norm_quantile(u))); break;  // src/prior/norm.c:77-82
        default: v = CUDART_NAN; out = 1; break;
        }
        if (p.bounded && (v < p.lower || v > p.upper)) out = 1;
        params[(size_t)b * np + i] = v;
    }
    bad[b] = out;
}

// logL = -inf for the candidates the transform rejected; the physical
// parameters are copied out when phys is not NULL.
__global__ void __launch_bounds__(128)
    lg_prior_finish(int B, int np, const int* __restrict__ bad, const double* __restrict__ params,
                    double* __restrict__ logL, double* __restrict__ phys)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    if (bad[b]) logL[b] = -CUDART_INF;
    if (phys)
        for (int i = 0; i < np; ++i) phys[(size_t)b * np + i] = params[(size_t)b * np + i];
}

lg::Fp ctx_mode(const lg_ctx* c) { return lg::fp_mode(c->flags); }
// fast mode: hardware-approximate division and square root per ray
// (<= 2 ulp, as the reference's -cl-fast-relaxed-math build allows) unless
// LG_FLAG_IEEE_DIV; the exact and strict modes and set_params stay IEEE
bool ctx_ieee(const lg_ctx* c) { return lg::fp_ieee(c->flags); }

int compile_eval(lg_ctx* c, const lg::Shape& s, std::vector<char>& cubin)
{
    std::string log;
    const lg::Fp mode = ctx_mode(c);
    int rc = lg::compile_program(lg::compose_source(c->model, s, mode, lg::Part::EVAL), lg::fp_fmad(mode), cubin,
                                 log, ctx_ieee(c));
    return rc ? c->fail(rc, log) : LG_OK;
}

// Make the evaluation module compiled for shape s the context's: its
// kernels, the convolution's shared memory and a partial-sum buffer for
// max_batch candidates.  The previous module and the graphs captured with
// it are released first.
int load_eval(lg_ctx* c, const lg::Shape& s, const std::vector<char>& cubin)
{
    int rc;
    if (c->stream && (rc = c->cuda(cudaStreamSynchronize(c->stream), "synchronize"))) return rc;
    c->drop_graphs();
    if (c->mod) c->drv->moduleUnload(c->mod);
    c->mod = nullptr;
    cudaFree(c->d_partials);
    c->d_partials = nullptr;
    cudaFree(c->d_counters);
    c->d_counters = nullptr;
    c->shape = s;
    shape_sizes(s, c->model, c);
    if ((rc = c->drvcall(c->drv->moduleLoadData(&c->mod, cubin.data()), "cuModuleLoadData"))) return rc;
    struct {
        CUfunction* f;
        const char* n;
        bool need;
    } fns[] = {{&c->f_rraw, "lg_render_raw", true},  {&c->f_rchi2, "lg_render_chi2", true},
               {&c->f_rdump, "lg_render_dump", true},
               {&c->f_cchi2, "lg_conv_chi2", c->psf}, {&c->f_cdump, "lg_conv_dump", c->psf}};
    for (auto& f : fns)
        if (f.need && (rc = c->drvcall(c->drv->moduleGetFunction(f.f, c->mod, f.n), f.n))) return rc;
    CUdeviceptr gp;
    size_t gb;
    if (c->psf) {
        int csm = 0, cth = 0;
        if ((rc = c->drvcall(c->drv->moduleGetGlobal(&gp, &gb, c->mod, "lg_conv_smem"), "lg_conv_smem")) ||
            (rc = c->cuda(cudaMemcpy(&csm, (void*)gp, sizeof csm, cudaMemcpyDeviceToHost), "conv smem")) ||
            (rc = c->drvcall(c->drv->moduleGetGlobal(&gp, &gb, c->mod, "lg_conv_threads"), "lg_conv_threads")) ||
            (rc = c->cuda(cudaMemcpy(&cth, (void*)gp, sizeof cth, cudaMemcpyDeviceToHost), "conv threads")))
            return rc;
        if (cth != c->cthreads) return c->fail(LG_ERR_COMPILE, "convolution block size mismatch");
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
        if (csm > optin)
            return c->fail(LG_ERR_UNSUPPORTED, "convolution tile needs " + std::to_string(csm) +
                                                   " bytes of shared memory, above the device's " +
                                                   std::to_string(optin));
        c->csmem = csm;
        if (c->csmem > 48 * 1024)
            if ((rc = c->drvcall(c->drv->funcSetAttribute(c->f_cchi2, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                          c->csmem),
                                 "convolve smem")) ||
                (rc = c->drvcall(c->drv->funcSetAttribute(c->f_cdump, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                          c->csmem),
                                 "convolve smem")))
                return rc;
    }
    const size_t ntiles = (size_t)(c->psf ? c->ctiles : c->rtiles);
    if (cudaMalloc((void**)&c->d_partials, (size_t)c->max_batch * ntiles * 8) != cudaSuccess ||
        cudaMalloc((void**)&c->d_counters, (size_t)c->max_batch * sizeof(unsigned)) != cudaSuccess)
        return c->fail(LG_ERR_ALLOC, "cudaMalloc partials");
    if ((rc = c->cuda(cudaMemset(c->d_counters, 0, (size_t)c->max_batch * sizeof(unsigned)), "clear counters")))
        return rc;
    return LG_OK;
}

// Candidate parameter vectors for timing: B draws from the priors (map
// order; derived parameters at u = 0.5), from a fixed seed.
void prior_draws(const lg::Model& m, int B, double* out)
{
    uint64_t st = 0x243f6a8885a308d3ull;
    auto unif = [&]() {
        st += 0x9e3779b97f4a7c15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    const size_t np = m.pars.size();
    for (int b = 0; b < B; ++b)
        for (size_t i = 0; i < np; ++i) {
            const lg::ParamInfo& p = m.pars[m.pmap[i]];
            out[(size_t)b * np + i] = p.prior.apply((int)i < m.ndims ? unif() : 0.5);
        }
}

// Render and convolution times (ms, best of several runs) of the loaded
// module on the candidates in d_params.
int time_stages(lg_ctx* c, int B, double* render_ms, double* conv_ms)
{
    cudaEvent_t ev[5] = {};
    int rc = LG_OK;
    for (auto& e : ev)
        if (!rc) rc = c->cuda(cudaEventCreate(&e), "event");
    double best[2] = {1e30, 1e30}, total = 0;
    for (int rep = 0; !rc && rep < 40; ++rep) {
        rc = c->enqueue(B, c->d_params, c->d_logL, c->stream, ev);
        if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "tune run");
        float t[3] = {0, 0, 0};
        for (int i = 0; i < 3 && !rc; ++i) rc = c->cuda(cudaEventElapsedTime(&t[i], ev[i + 1], ev[i + 2]), "elapsed");
        if (rc || rep == 0) continue;  // the first run warms up
        best[0] = std::min(best[0], (double)t[0]);
        best[1] = std::min(best[1], (double)t[1]);
        total += t[0] + t[1];
        if (rep >= 3 && total > 30.0) break;
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    *render_ms = best[0];
    *conv_ms = best[1];
    return rc;
}

// LG_FLAG_AUTOTUNE: compile the candidate shapes in parallel, time each on
// max_batch candidates drawn from the priors, keep the fastest render and
// the fastest convolution (a cached choice for the same program, device,
// batch and flags is reused without timing).
int autotune(lg_ctx* c)
{
    const lg::Model& m = c->model;
    const lg::Fp mode = ctx_mode(c);
    const lg::Shape base = choose_shape(m, mode);
    const std::string key = lg::tune_key(lg::compose_source(m, base, mode, lg::Part::EVAL), c->device,
                                         c->max_batch, c->flags & (LG_FLAG_STRICT_FP | LG_FLAG_IEEE_DIV | LG_FLAG_FAST_MATH));
    std::ostringstream rep;
    int rc;
    lg::Shape chosen;
    if (lg::tune_cache_get(key, chosen) && lg::check_shape(chosen, mode, c->psf, m.psfw).empty()) {
        std::vector<char> cubin;
        if ((rc = compile_eval(c, chosen, cubin)) || (rc = load_eval(c, chosen, cubin))) return rc;
        c->tune_report = "cached " + key + ": " + chosen.str() + "\n";
        return LG_OK;
    }
    for (size_t i = 0; i < m.pars.size(); ++i)
        if (!m.pars[i].has_prior) {
            std::vector<char> cubin;
            if ((rc = compile_eval(c, base, cubin)) || (rc = load_eval(c, base, cubin))) return rc;
            c->tune_report = "not tuned (no prior for " + m.pars[i].id + " to draw candidates from): " +
                             base.str() + "\n";
            return LG_OK;
        }
    const int B = c->max_batch;
    const size_t np = m.pars.size();
    prior_draws(m, B, c->h_params);
    if ((rc = c->cuda(cudaMemcpy(c->d_params, c->h_params, (size_t)B * np * 8, cudaMemcpyHostToDevice), "params")))
        return rc;
    // render candidates with the base convolution, convolution candidates
    // with the base render
    std::vector<lg::Shape> cand;
    std::vector<int> is_render;
    for (const lg::Shape& s : lg::render_candidates(base, mode))
        if (lg::check_shape(s, mode, c->psf, m.psfw).empty()) cand.push_back(s), is_render.push_back(1);
    if (c->psf)
        for (const lg::Shape& s : lg::conv_candidates(base)) {
            if (!lg::check_shape(s, mode, c->psf, m.psfw).empty()) continue;
            bool dup = false;
            for (const lg::Shape& t : cand) dup = dup || t == s;
            if (!dup) cand.push_back(s), is_render.push_back(0);
        }
    std::vector<std::string> srcs;
    for (const lg::Shape& s : cand) srcs.push_back(lg::compose_source(m, s, mode, lg::Part::EVAL));
    std::vector<std::vector<char>> cubins;
    std::vector<int> rcs;
    std::vector<std::string> logs;
    lg::compile_parallel(srcs, lg::fp_fmad(mode), ctx_ieee(c), cubins, rcs, logs);
    double best_r = 1e30, best_c = 1e30;
    lg::Shape br = base, bc = base;
    for (size_t i = 0; i < cand.size(); ++i) {
        double r_ms = 0, c_ms = 0;
        if (rcs[i]) {
            rep << "  " << cand[i].str() << ": compile failed\n";
            continue;
        }
        if ((rc = load_eval(c, cand[i], cubins[i]))) {
            if (rc != LG_ERR_UNSUPPORTED) return rc;
            rep << "  " << cand[i].str() << ": " << c->err << "\n";
            c->err.clear();
            continue;
        }
        if ((rc = time_stages(c, B, &r_ms, &c_ms))) return rc;
        char line[256];
        std::snprintf(line, sizeof line, "  %s: render %.4f ms, convolve %.4f ms\n", cand[i].str().c_str(), r_ms,
                      c_ms);
        rep << line;
        // the base shape is a render candidate; its convolution time also
        // stands for the base convolution
        const bool base_conv = cand[i].ctx == base.ctx && cand[i].cty == base.cty && cand[i].cr == base.cr &&
                               cand[i].pair_rows == base.pair_rows;
        if (is_render[i] && r_ms < best_r) best_r = r_ms, br = cand[i];
        if ((!is_render[i] || base_conv) && c->psf && c_ms < best_c) best_c = c_ms, bc = cand[i];
    }
    chosen = br;
    if (c->psf) {
        chosen.ctx = bc.ctx;
        chosen.cty = bc.cty;
        chosen.cr = bc.cr;
        chosen.pair_rows = bc.pair_rows;
    }
    const std::vector<char>* cb = nullptr;
    for (size_t i = 0; i < cand.size(); ++i)
        if (!rcs[i] && cand[i] == chosen) cb = &cubins[i];
    std::vector<char> own;
    if (!cb) {
        if ((rc = compile_eval(c, chosen, own))) return rc;
        cb = &own;
    }
    if ((rc = load_eval(c, chosen, *cb))) return rc;
    lg::tune_cache_put(key, chosen);
    c->tune_report = "tuned " + key + " on " + std::to_string(B) + " candidates: " + chosen.str() + "\n" + rep.str();
    return LG_OK;
}

int create_impl(lg_ctx* c, const lg_image_desc* img, const lg_object_desc* objs, int nobjs, const lg_options* opts)
{
    int rc = lg::build_model(img, objs, nobjs, opts, c->model, c->err);
    if (rc) return rc;
    const lg::Model& m = c->model;
    c->flags = opts ? opts->flags : 0;
    c->device = opts ? opts->device : 0;
    c->max_batch = (opts && opts->max_batch > 0) ? opts->max_batch : 1024;
    if (c->max_batch > 65535) return c->fail(LG_ERR_INPUT, "max_batch above 65535");
    if (!img->image) return c->fail(LG_ERR_INPUT, "image is required");
    if (!img->weight) return c->fail(LG_ERR_INPUT, "weight is required (see lg_make_weight)");
    c->N = (long)m.width * m.height;
    c->psf = !m.psf.empty();
    for (long k = 0; k < c->N; ++k)
        if (img->weight[k] == 0) c->masked++;

    // compose and compile the programs (the reference's clBuildProgram,
    // src/lensed.c:706-776): the set_params module here, the evaluation
    // module (whose launch shape may be tuned) once the buffers exist
    const lg::Fp mode = lg::fp_mode(c->flags);
    c->shape = choose_shape(m, mode);
    std::string log;
    std::vector<char> cubin_set;
    rc = lg::compile_program(lg::compose_source(m, c->shape, mode, lg::Part::SET), false, cubin_set, log);
    if (rc) return c->fail(rc, log);

    if ((rc = c->cuda(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    if ((rc = c->cuda(cudaFree(nullptr), "CUDA context"))) return rc;
    c->drv = driver();
    if (!c->drv) return c->fail(LG_ERR_CUDA, "CUDA driver entry points unavailable");
    if ((rc = c->drvcall(c->drv->moduleLoadData(&c->mod_set, cubin_set.data()), "cuModuleLoadData"))) return rc;
    if ((rc = c->drvcall(c->drv->moduleGetFunction(&c->f_setp, c->mod_set, "lg_set_params_kernel"),
                         "lg_set_params_kernel")) ||
        (rc = c->drvcall(c->drv->moduleGetFunction(&c->f_setp_split, c->mod_set, "lg_set_params_split"),
                         "lg_set_params_split")))
        return rc;
    CUdeviceptr gp;
    size_t gb;
    if ((rc = c->drvcall(c->drv->moduleGetGlobal(&gp, &gb, c->mod_set, "lg_model_bytes"), "lg_model_bytes")))
        return rc;
    unsigned mb = 0;
    if ((rc = c->cuda(cudaMemcpy(&mb, (void*)gp, sizeof mb, cudaMemcpyDeviceToHost), "model size"))) return rc;
    c->model_bytes = mb;
    if ((rc = c->drvcall(c->drv->moduleGetGlobal(&gp, &gb, c->mod_set, "lg_model_objects"), "lg_model_objects")) ||
        (rc = c->cuda(cudaMemcpy(&c->nobj, (void*)gp, sizeof c->nobj, cudaMemcpyDeviceToHost), "object count")))
        return rc;

    if ((rc = c->cuda(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream")) ||
        (rc = c->cuda(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "event")))
        return rc;
    const size_t B = (size_t)c->max_batch, N = (size_t)c->N, np = m.pars.size();
    auto alloc = [&](void** p, size_t bytes, const char* what) {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            c->err = std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e);
            return LG_ERR_ALLOC;
        }
        return LG_OK;
    };
    if ((rc = alloc((void**)&c->d_image, N * 4, "image")) || (rc = alloc((void**)&c->d_weight, N * 4, "weight")) ||
        (rc = alloc(&c->d_models, B * c->model_bytes, "models")) ||
        (rc = alloc((void**)&c->d_params, B * np * 8, "params")) ||
        (rc = alloc((void**)&c->d_logL, B * 8, "logL")))
        return rc;
    if (c->psf && (rc = alloc((void**)&c->d_raw, B * N * 4, "raw model"))) return rc;
    if ((rc = c->cuda(cudaMallocHost((void**)&c->h_params, B * np * 8), "pinned params")) ||
        (rc = c->cuda(cudaMallocHost((void**)&c->h_logL, B * 8), "pinned logL")))
        return rc;
    {
        const size_t zb = std::min<size_t>(B, lg::kZeroCopyBatch);
        if ((rc = c->cuda(cudaHostAlloc((void**)&c->z_params, std::max<size_t>(zb * np, 1) * 8, cudaHostAllocMapped),
                          "mapped params")) ||
            (rc = c->cuda(cudaHostAlloc((void**)&c->z_logL, zb * 8, cudaHostAllocMapped), "mapped logL")) ||
            (rc = c->cuda(cudaHostGetDevicePointer((void**)&c->zd_params, c->z_params, 0), "mapped params")) ||
            (rc = c->cuda(cudaHostGetDevicePointer((void**)&c->zd_logL, c->z_logL, 0), "mapped logL")))
            return rc;
        const size_t nd = std::max<size_t>((size_t)m.ndims, 1);
        if ((rc = c->cuda(cudaHostAlloc((void**)&c->z_cube, zb * nd * 8, cudaHostAllocMapped), "mapped cube")) ||
            (rc = c->cuda(cudaHostAlloc((void**)&c->z_phys, std::max<size_t>(zb * np, 1) * 8, cudaHostAllocMapped),
                          "mapped phys")) ||
            (rc = c->cuda(cudaHostAlloc((void**)&c->z_bad, zb * 4, cudaHostAllocMapped), "mapped flags")) ||
            (rc = c->cuda(cudaHostGetDevicePointer((void**)&c->zd_cube, c->z_cube, 0), "mapped cube")) ||
            (rc = c->cuda(cudaHostGetDevicePointer((void**)&c->zd_phys, c->z_phys, 0), "mapped phys")) ||
            (rc = c->cuda(cudaHostGetDevicePointer((void**)&c->zd_bad, c->z_bad, 0), "mapped flags")))
            return rc;
    }
    // unit-cube path (priors are checked when it is called)
    const size_t nd = (size_t)m.ndims;
    std::vector<DevPrior> pri(np);
    for (size_t i = 0; i < np; ++i) {
        const lg::ParamInfo& par = m.pars[m.pmap[i]];
        pri[i] = {par.has_prior ? (int)par.prior.kind : 0, par.bounded ? 1 : 0, par.prior.a, par.prior.b, par.lower,
                  par.upper};
    }
    if ((rc = alloc(&c->d_priors, std::max<size_t>(np, 1) * sizeof(DevPrior), "priors")) ||
        (rc = alloc((void**)&c->d_cube, std::max<size_t>(B * nd, 1) * 8, "cube")) ||
        (rc = alloc((void**)&c->d_bad, B * 4, "rejection flags")))
        return rc;
    if ((rc = c->cuda(cudaMallocHost((void**)&c->h_cube, std::max<size_t>(B * nd, 1) * 8), "pinned cube")) ||
        (rc = c->cuda(cudaMallocHost((void**)&c->h_bad, B * 4), "pinned flags")))
        return rc;
    if (np && (rc = c->cuda(cudaMemcpy(c->d_priors, pri.data(), np * sizeof(DevPrior), cudaMemcpyHostToDevice),
                            "upload priors")))
        return rc;
    if ((rc = c->cuda(cudaMemcpy(c->d_image, img->image, N * 4, cudaMemcpyHostToDevice), "upload image")) ||
        (rc = c->cuda(cudaMemcpy(c->d_weight, img->weight, N * 4, cudaMemcpyHostToDevice), "upload weight")))
        return rc;
    if (c->flags & LG_FLAG_AUTOTUNE) return autotune(c);
    std::vector<char> cubin;
    if ((rc = compile_eval(c, c->shape, cubin))) return rc;
    return load_eval(c, c->shape, cubin);
}

// Host set_params for small batches: the layout of the device's lg_model
// and, on sample candidates (prior draws, else points inside the bounds),
// object data identical byte for byte to the set module's; otherwise the
// context keeps the device path.
int init_host_set(lg_ctx* c)
{
    const lg::Model& m = c->model;
    c->hset = lg::host_set_layout(m);
    if (!c->hset.ok || c->hset.bytes != c->model_bytes) return LG_OK;
    const int K = std::min(lg::kHostSet, c->max_batch);
    const size_t np = m.pars.size(), mb = c->model_bytes;
    std::vector<double> P(K * np);
    for (int k = 0; k < K; ++k)
        for (size_t i = 0; i < np; ++i) {
            const lg::ParamInfo& par = m.pars[m.pmap[i]];
            const double u = 0.2 + 0.6 * std::fmod(0.37 * (double)i + (k + 0.5) / K, 1.0);
            // without a prior or finite bounds, a value typical of the
            // parameter's kind
            double v = 0.5 + 0.5 * u;
            switch (par.type) {
            case LG_POSITION_X:
            case LG_POSITION_Y: v = 10.0 + 20.0 * u; break;
            case LG_RADIUS: v = 1.0 + 4.0 * u; break;
            case LG_MAGNITUDE: v = -3.0 + 2.0 * u; break;
            case LG_AXIS_RATIO: v = 0.5 + 0.4 * u; break;
            case LG_POS_ANGLE: v = 180.0 * u; break;
            default: break;
            }
            if (par.has_prior)
                v = par.prior.apply(u);
            else if (par.bounded && !(v >= par.lower && v <= par.upper) && std::isfinite(par.lower) &&
                     std::isfinite(par.upper))
                v = par.lower + u * (par.upper - par.lower);
            P[k * np + i] = v;
        }
    std::vector<unsigned char> host(K * mb), dev(K * mb);
    for (int k = 0; k < K; ++k) lg::host_set_params(m, c->hset, &P[k * np], &host[k * mb]);
    int rc;
    if ((rc = c->cuda(cudaMemcpyAsync(c->d_params, P.data(), K * np * 8, cudaMemcpyHostToDevice, c->stream),
                      "params upload")) ||
        (rc = c->launch_set(K, c->d_params, c->stream)) ||
        (rc = c->cuda(cudaMemcpyAsync(dev.data(), c->d_models, K * mb, cudaMemcpyDeviceToHost, c->stream),
                      "object data")) ||
        (rc = c->cuda(cudaStreamSynchronize(c->stream), "set_params check")))
        return rc;
    if (std::memcmp(host.data(), dev.data(), K * mb) != 0) return LG_OK;
    if ((rc = c->cuda(cudaHostAlloc((void**)&c->z_models, lg::kHostSet * mb, cudaHostAllocDefault), "pinned models")))
        return rc;
    c->host_set = true;
    return LG_OK;
}

// Graph of B candidates whose object data the host has put in z_models:
// their upload, render, convolution + chi^2, logL into mapped memory.
int host_graph_for(lg_ctx* c, int B, cudaGraphExec_t* out)
{
    auto it = c->hgraphs.find(B);
    if (it != c->hgraphs.end()) {
        *out = it->second;
        return LG_OK;
    }
    int rc;
    cudaGraph_t g;
    if ((rc = c->cuda(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture")))
        return rc;
    int erc = c->cuda(cudaMemcpyAsync(c->d_models, c->z_models, (size_t)B * c->model_bytes, cudaMemcpyHostToDevice,
                                      c->stream),
                      "object data upload");
    if (!erc) erc = c->enqueue(B, nullptr, c->zd_logL, c->stream, nullptr, false);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (erc) return erc;
    if ((rc = c->cuda(e, "end capture"))) return rc;
    cudaGraphExec_t ge;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if ((rc = c->cuda(e, "graph instantiate"))) return rc;
    c->hgraphs[B] = ge;
    *out = ge;
    return LG_OK;
}

// logL of B <= kHostSet candidates (physical parameters, map order) with
// the object data from the host.
int host_set_eval(lg_ctx* c, const double* params, int B, double* logL)
{
    const size_t np = c->model.pars.size(), mb = c->model_bytes;
    for (int b = 0; b < B; ++b) lg::host_set_params(c->model, c->hset, params + (size_t)b * np, c->z_models + b * mb);
    cudaGraphExec_t ge;
    int rc;
    if ((rc = host_graph_for(c, B, &ge)) || (rc = c->cuda(cudaGraphLaunch(ge, c->stream), "graph launch")) ||
        (rc = c->cuda(cudaStreamSynchronize(c->stream), "evaluate")))
        return rc;
    std::memcpy(logL, c->z_logL, (size_t)B * 8);
    return LG_OK;
}

// Graph of upload + evaluation + read-back for B candidates, built on first
// use and replayed afterwards.
int graph_for(lg_ctx* c, int B, cudaGraphExec_t* out)
{
    auto it = c->graphs.find(B);
    if (it != c->graphs.end()) {
        *out = it->second;
        return LG_OK;
    }
    const size_t np = c->model.pars.size();
    int rc;
    cudaGraph_t g;
    if ((rc = c->cuda(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture")))
        return rc;
    int erc = LG_OK;
    if (B <= lg::kZeroCopyBatch) {
        // small batches: the kernels read the parameters from and write logL
        // to mapped host memory directly
        erc = c->enqueue(B, c->zd_params, c->zd_logL, c->stream);
    } else {
        erc = c->cuda(cudaMemcpyAsync(c->d_params, c->h_params, B * np * 8, cudaMemcpyHostToDevice, c->stream),
                      "params upload");
        if (!erc) erc = c->enqueue(B, c->d_params, c->d_logL, c->stream);
        if (!erc)
            erc = c->cuda(cudaMemcpyAsync(c->h_logL, c->d_logL, B * 8, cudaMemcpyDeviceToHost, c->stream),
                          "logL read");
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (erc) return erc;
    if ((rc = c->cuda(e, "end capture"))) return rc;
    cudaGraphExec_t ge;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if ((rc = c->cuda(e, "graph instantiate"))) return rc;
    c->graphs[B] = ge;
    *out = ge;
    return LG_OK;
}

// The context's stream does not synchronise with the legacy default stream
// (it is non-blocking, so that graph capture on it stays legal).  Calls that
// take caller device pointers and run on it first wait for the work already
// queued on the legacy stream, where frameworks such as PyTorch enqueue the
// copies that fill those buffers by default.
int order_after_legacy(lg_ctx* c)
{
    cudaEvent_t e;
    int rc;
    if ((rc = c->cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event"))) return rc;
    rc = c->cuda(cudaEventRecord(e, cudaStreamLegacy), "event record");
    if (!rc) rc = c->cuda(cudaStreamWaitEvent(c->stream, e, 0), "stream wait");
    cudaEventDestroy(e);
    return rc;
}

// Calls on one context share its scratch (parameters, object data, raw
// models, partial sums, tile counters), so they run in order whatever
// stream they are made on: a call on a caller stream s first waits for the
// work queued on the context's stream, and the context's stream then waits
// for the call (the context's stream is the join point of every call).
int join_before(lg_ctx* c, cudaStream_t s)
{
    int rc;
    if (s == c->stream) return LG_OK;
    if ((rc = c->cuda(cudaEventRecord(c->ev_join, c->stream), "event record"))) return rc;
    return c->cuda(cudaStreamWaitEvent(s, c->ev_join, 0), "stream wait");
}
int join_after(lg_ctx* c, cudaStream_t s)
{
    int rc;
    if (s == c->stream) return LG_OK;
    if ((rc = c->cuda(cudaEventRecord(c->ev_join, s), "event record"))) return rc;
    return c->cuda(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "stream wait");
}

int check_priors(lg_ctx* c)
{
    const lg::Model& m = c->model;
    for (size_t i = 0; i < m.pars.size(); ++i)
        if (!m.pars[m.pmap[i]].has_prior) return c->fail(LG_ERR_INPUT, "missing prior: " + m.pars[m.pmap[i]].id);
    return LG_OK;
}

// Enqueue prior transform .. logL for B unit-cube points (device pointers):
// the physical parameters land in the context's params buffer (and in
// d_phys when not NULL), the rejection flags in bad (the context's d_bad
// when NULL).
int enqueue_cube(lg_ctx* c, int B, const double* d_cube, double* d_phys, double* d_logL, cudaStream_t s,
                 int* bad = nullptr)
{
    const int np = (int)c->model.pars.size(), nd = c->model.ndims;
    const int blocks = (B + 127) / 128;
    if (!bad) bad = c->d_bad;
    int rc;
    lg_prior_transform<<<blocks, 128, 0, s>>>(d_cube, B, nd, np, static_cast<const DevPrior*>(c->d_priors),
                                              c->d_params, bad);
    if ((rc = c->cuda(cudaGetLastError(), "prior transform"))) return rc;
    if ((rc = c->enqueue(B, c->d_params, d_logL, s))) return rc;
    lg_prior_finish<<<blocks, 128, 0, s>>>(B, np, bad, c->d_params, d_logL, d_phys);
    return c->cuda(cudaGetLastError(), "prior finish");
}

// Upload of B cube points, their evaluation and the read-back of logL, the
// physical parameters and the rejection flags.
int enqueue_cube_io(lg_ctx* c, int B, cudaStream_t s)
{
    const size_t np = c->model.pars.size(), nd = (size_t)c->model.ndims;
    int rc;
    if (nd && (rc = c->cuda(cudaMemcpyAsync(c->d_cube, c->h_cube, B * nd * 8, cudaMemcpyHostToDevice, s), "cube upload")))
        return rc;
    if ((rc = enqueue_cube(c, B, c->d_cube, nullptr, c->d_logL, s))) return rc;
    if ((rc = c->cuda(cudaMemcpyAsync(c->h_logL, c->d_logL, B * 8, cudaMemcpyDeviceToHost, s), "logL read")) ||
        (np && (rc = c->cuda(cudaMemcpyAsync(c->h_params, c->d_params, B * np * 8, cudaMemcpyDeviceToHost, s),
                             "params read"))) ||
        (rc = c->cuda(cudaMemcpyAsync(c->h_bad, c->d_bad, B * 4, cudaMemcpyDeviceToHost, s), "flags read")))
        return rc;
    return LG_OK;
}

int cube_graph_for(lg_ctx* c, int B, cudaGraphExec_t* out)
{
    auto it = c->cube_graphs.find(B);
    if (it != c->cube_graphs.end()) {
        *out = it->second;
        return LG_OK;
    }
    int rc;
    cudaGraph_t g;
    if ((rc = c->cuda(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture")))
        return rc;
    // small batches read the cube from and write logL, the physical values
    // and the flags to mapped host memory directly
    int erc = B <= lg::kZeroCopyBatch ? enqueue_cube(c, B, c->zd_cube, c->zd_phys, c->zd_logL, c->stream, c->zd_bad)
                                      : enqueue_cube_io(c, B, c->stream);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (erc) return erc;
    if ((rc = c->cuda(e, "end capture"))) return rc;
    cudaGraphExec_t ge;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if ((rc = c->cuda(e, "graph instantiate"))) return rc;
    c->cube_graphs[B] = ge;
    *out = ge;
    return LG_OK;
}

// Host unit-cube evaluation of B <= max_batch points: logL and the physical
// parameters (NaN for rejected points when nan_rejected) and flags.
int cube_eval_chunk(lg_ctx* c, const double* cube, int B, double* phys, double* logL, bool nan_rejected)
{
    const size_t np = c->model.pars.size(), nd = (size_t)c->model.ndims;
    int rc;
    if (c->host_set && B <= lg::kHostSet && !(c->flags & LG_FLAG_NO_GRAPH)) {
        // the prior transform on the host too (the arithmetic of
        // lg_prior_transform: src/nested.c:42-61)
        const lg::Model& m = c->model;
        double* P = c->h_params;
        int bad[lg::kHostSet];
        for (int b = 0; b < B; ++b) {
            bad[b] = 0;
            for (size_t i = 0; i < np; ++i) {
                const lg::ParamInfo& par = m.pars[m.pmap[i]];
                const double u = i < nd ? cube[(size_t)b * nd + i] : 0.5;
                double v = NAN;
                if (par.has_prior && par.prior.kind != lg::Prior::NONE)
                    v = par.prior.apply(u);
                else
                    bad[b] = 1;
                if (par.bounded && (v < par.lower || v > par.upper)) bad[b] = 1;
                P[(size_t)b * np + i] = v;
            }
        }
        if ((rc = host_set_eval(c, P, B, logL))) return rc;
        for (int b = 0; b < B; ++b) {
            if (bad[b]) logL[b] = -HUGE_VAL;
            if (phys)
                for (size_t i = 0; i < np; ++i)
                    phys[(size_t)b * np + i] = (nan_rejected && bad[b]) ? NAN : P[(size_t)b * np + i];
        }
        c->last_bad = bad[0];
        return LG_OK;
    }
    const bool zero_copy = !(c->flags & LG_FLAG_NO_GRAPH) && B <= lg::kZeroCopyBatch;
    if (nd) std::memcpy(zero_copy ? c->z_cube : c->h_cube, cube, (size_t)B * nd * 8);
    if (c->flags & LG_FLAG_NO_GRAPH) {
        if ((rc = enqueue_cube_io(c, B, c->stream))) return rc;
    } else {
        cudaGraphExec_t ge;
        if ((rc = cube_graph_for(c, B, &ge))) return rc;
        if ((rc = c->cuda(cudaGraphLaunch(ge, c->stream), "graph launch"))) return rc;
    }
    if ((rc = c->cuda(cudaStreamSynchronize(c->stream), "evaluate"))) return rc;
    const double* hl = zero_copy ? c->z_logL : c->h_logL;
    const double* hp = zero_copy ? c->z_phys : c->h_params;
    const int* hb = zero_copy ? c->z_bad : c->h_bad;
    std::memcpy(logL, hl, (size_t)B * 8);
    if (phys)
        for (int b = 0; b < B; ++b)
            for (size_t i = 0; i < np; ++i)
                phys[(size_t)b * np + i] = (nan_rejected && hb[b]) ? NAN : hp[(size_t)b * np + i];
    c->last_bad = hb[0];
    return LG_OK;
}

}  // namespace

extern "C" {

const char* lg_version(void) { return "lensed_gb300 0.1 (sm_103a)"; }

int lg_plugin_count(void) { return lg::plugin_count(); }

int lg_plugin_info(int i, const char** name, int* kind, int* npars)
{
    const lg::Plugin* p = lg::plugin_at(i);
    if (!p) return LG_ERR_INPUT;
    if (name) *name = p->name.c_str();
    if (kind) *kind = p->kind;
    if (npars) *npars = (int)p->pars.size();
    return LG_OK;
}

int lg_plugin_param(const char* plugin, int j, const char** name, int* type, float* lower, float* upper,
                    float* defval)
{
    const lg::Plugin* p = plugin ? lg::find_plugin(plugin) : nullptr;
    if (!p || j < 0 || j >= (int)p->pars.size()) return LG_ERR_INPUT;
    const lg::ParamDef& d = p->pars[j];
    if (name) *name = d.name.c_str();
    if (type) *type = d.type;
    if (lower) *lower = d.lower;
    if (upper) *upper = d.upper;
    if (defval) *defval = d.defval;
    return LG_OK;
}

int lg_register_plugin(const lg_plugin_desc* desc)
{
    std::string err;
    int rc = lg::register_plugin(desc, err);
    if (rc) g_create_error = err;
    return rc;
}

int lg_quad_rule_count(void) { return lg::quad_rule_count(); }

int lg_quad_rule_info(int i, const char** name, int* size, double* absc, double* weig, double* errw)
{
    const lg::QuadRuleData* r = lg::quad_rule_at(i);
    if (!r) return LG_ERR_INPUT;
    if (name) *name = r->name;
    if (size) *size = r->size;
    for (int n = 0; n < r->size; ++n) {
        if (absc) {
            absc[2 * n] = r->absc[n][0];
            absc[2 * n + 1] = r->absc[n][1];
        }
        if (weig) weig[n] = r->weig[n];
        if (errw) errw[n] = r->errw[n];
    }
    return LG_OK;
}

long lg_make_weight(const float* image, long n, const float* weight_map, const float* gain, double gain_value,
                    double offset, const float* xweight, const int* mask, float* out)
{
    if (!out || n < 0 || (!weight_map && !image)) return LG_ERR_INPUT;
    long masked = 0;
    for (long i = 0; i < n; ++i) {
        float w;
        if (weight_map) w = weight_map[i];
        else w = (float)((gain ? (double)gain[i] : (double)(float)gain_value) / ((double)image[i] + offset));
        if (xweight) w *= xweight[i];
        if (mask && mask[i]) w = 0;
        out[i] = w;
        if (w == 0) ++masked;
    }
    return masked;
}

int lg_compile_check(const lg_image_desc* image, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                     char* log, size_t log_size)
{
    lg::Model m;
    std::string err;
    int rc = lg::build_model(image, objs, nobjs, opts, m, err);
    if (!rc) {
        const int flags = opts ? opts->flags : 0;
        const lg::Fp mode = lg::fp_mode(flags);
        std::vector<char> cubin;
        lg::Shape s = choose_shape(m, mode);
        rc = lg::compile_program(lg::compose_source(m, s, mode, lg::Part::EVAL), lg::fp_fmad(mode), cubin, err,
                                 lg::fp_ieee(flags));
        if (!rc) rc = lg::compile_program(lg::compose_source(m, s, mode, lg::Part::SET), false, cubin, err);
    }
    if (log && log_size) {
        std::snprintf(log, log_size, "%s", err.c_str());
    }
    return rc;
}

int lg_tune_candidates(const lg_image_desc* image, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                       int* shapes, int max_shapes)
{
    lg::Model m;
    std::string err;
    int rc = lg::build_model(image, objs, nobjs, opts, m, err);
    if (rc) {
        g_create_error = err;
        return rc;
    }
    const lg::Fp mode = lg::fp_mode(opts ? opts->flags : 0);
    const lg::Shape base = choose_shape(m, mode);
    std::vector<lg::Shape> cand;
    for (const lg::Shape& s : lg::render_candidates(base, mode))
        if (lg::check_shape(s, mode, !m.psf.empty(), m.psfw).empty()) cand.push_back(s);
    if (!m.psf.empty())
        for (const lg::Shape& s : lg::conv_candidates(base)) {
            bool dup = false;
            for (const lg::Shape& t : cand) dup = dup || t == s;
            if (!dup && lg::check_shape(s, mode, true, m.psfw).empty()) cand.push_back(s);
        }
    for (int i = 0; i < (int)cand.size() && i < max_shapes && shapes; ++i) {
        const lg::Shape& s = cand[i];
        const int v[7] = {s.rt, s.rppt, s.qs, s.ctx, s.cty, s.cr, s.pair_rows ? 1 : 0};
        std::memcpy(shapes + 7 * i, v, sizeof v);
    }
    return (int)cand.size();
}

int lg_compile_check_shape(const lg_image_desc* image, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                           const int shape[7], char* log, size_t log_size)
{
    lg::Model m;
    std::string err;
    int rc = shape ? lg::build_model(image, objs, nobjs, opts, m, err) : LG_ERR_INPUT;
    if (!rc) {
        const int flags = opts ? opts->flags : 0;
        const lg::Fp mode = lg::fp_mode(flags);
        lg::Shape s;
        s.rt = shape[0];
        s.rppt = shape[1];
        s.qs = shape[2];
        s.ctx = shape[3];
        s.cty = shape[4];
        s.cr = shape[5];
        s.pair_rows = shape[6] != 0;
        err = lg::check_shape(s, mode, !m.psf.empty(), m.psfw);
        if (!err.empty()) {
            rc = LG_ERR_INPUT;
        } else {
            std::vector<char> cubin;
            rc = lg::compile_program(lg::compose_source(m, s, mode, lg::Part::EVAL), lg::fp_fmad(mode), cubin, err,
                                     lg::fp_ieee(flags));
        }
    }
    if (log && log_size) std::snprintf(log, log_size, "%s", err.c_str());
    return rc;
}

lg_ctx* lg_create(const lg_image_desc* image, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                  int* status)
{
    lg_ctx* c = new (std::nothrow) lg_ctx();
    if (!c) {
        if (status) *status = LG_ERR_ALLOC;
        return nullptr;
    }
    int rc = create_impl(c, image, objs, nobjs, opts);
    if (!rc) rc = init_host_set(c);
    if (status) *status = rc;
    if (rc) {
        g_create_error = c->err;
        c->release();
        delete c;
        return nullptr;
    }
    return c;
}

void lg_destroy(lg_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->release();
    delete c;
}

const char* lg_last_error(const lg_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

int lg_npars(const lg_ctx* c) { return c ? (int)c->model.pars.size() : LG_ERR_INPUT; }
int lg_ndims(const lg_ctx* c) { return c ? c->model.ndims : LG_ERR_INPUT; }
long lg_masked(const lg_ctx* c) { return c ? c->masked : LG_ERR_INPUT; }

int lg_pmap(const lg_ctx* c, int i)
{
    if (!c || i < 0 || i >= (int)c->model.pmap.size()) return LG_ERR_INPUT;
    return c->model.pmap[i];
}

int lg_param(const lg_ctx* c, int i, const char** id, int* wrap, double* lower, double* upper)
{
    if (!c || i < 0 || i >= (int)c->model.pmap.size()) return LG_ERR_INPUT;
    const lg::ParamInfo& p = c->model.pars[c->model.pmap[i]];
    if (id) *id = p.id.c_str();
    if (wrap) *wrap = p.prior.wrap;
    if (lower) *lower = p.has_prior ? p.prior.lower() : -HUGE_VAL;
    if (upper) *upper = p.has_prior ? p.prior.upper() : HUGE_VAL;
    return LG_OK;
}

int lg_eval_batch(lg_ctx* c, const double* params, int B, double* logL)
{
    if (!c || !params || !logL || B < 0) return LG_ERR_INPUT;
    if (B == 0) return LG_OK;
    if (B > c->max_batch) return c->fail(LG_ERR_INPUT, "batch larger than max_batch");
    int rc;
    if ((rc = c->cuda(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    const size_t np = c->model.pars.size();
    std::memcpy(c->h_params, params, (size_t)B * np * 8);
    if (c->flags & LG_FLAG_NO_GRAPH) {
        if ((rc = c->cuda(cudaMemcpyAsync(c->d_params, c->h_params, (size_t)B * np * 8, cudaMemcpyHostToDevice,
                                          c->stream),
                          "params upload")))
            return rc;
        if ((rc = c->enqueue(B, c->d_params, c->d_logL, c->stream))) return rc;
        if ((rc = c->cuda(cudaMemcpyAsync(c->h_logL, c->d_logL, (size_t)B * 8, cudaMemcpyDeviceToHost, c->stream),
                          "logL read")))
            return rc;
    } else {
        if (c->host_set && B <= lg::kHostSet) return host_set_eval(c, params, B, logL);
        const bool zero_copy = B <= lg::kZeroCopyBatch;
        if (zero_copy) std::memcpy(c->z_params, params, (size_t)B * np * 8);
        cudaGraphExec_t ge;
        if ((rc = graph_for(c, B, &ge))) return rc;
        if ((rc = c->cuda(cudaGraphLaunch(ge, c->stream), "graph launch"))) return rc;
        if ((rc = c->cuda(cudaStreamSynchronize(c->stream), "evaluate"))) return rc;
        std::memcpy(logL, zero_copy ? c->z_logL : c->h_logL, (size_t)B * 8);
        return LG_OK;
    }
    if ((rc = c->cuda(cudaStreamSynchronize(c->stream), "evaluate"))) return rc;
    std::memcpy(logL, c->h_logL, (size_t)B * 8);
    return LG_OK;
}

int lg_eval_batch_device(lg_ctx* c, const double* d_params, int B, double* d_logL, void* stream)
{
    if (!c || !d_params || !d_logL || B < 0) return LG_ERR_INPUT;
    if (B == 0) return LG_OK;
    if (B > c->max_batch) return c->fail(LG_ERR_INPUT, "batch larger than max_batch");
    int rc;
    if ((rc = c->cuda(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    if (!stream && (rc = order_after_legacy(c))) return rc;
    const cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    if ((rc = join_before(c, s)) || (rc = c->enqueue(B, d_params, d_logL, s))) return rc;
    return join_after(c, s);
}

int lg_eval_cube_batch(lg_ctx* c, const double* cube, int B, double* phys, double* logL)
{
    if (!c || !cube || !logL || B < 0) return LG_ERR_INPUT;
    int rc;
    if ((rc = check_priors(c))) return rc;
    if (B == 0) return LG_OK;
    if ((rc = c->cuda(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    const size_t np = c->model.pars.size(), nd = (size_t)c->model.ndims;
    for (int b0 = 0; b0 < B; b0 += c->max_batch) {
        const int nb = std::min(c->max_batch, B - b0);
        if ((rc = cube_eval_chunk(c, cube + (size_t)b0 * nd, nb, phys ? phys + (size_t)b0 * np : nullptr, logL + b0,
                                  true)))
            return rc;
    }
    return LG_OK;
}

int lg_eval_cube_batch_device(lg_ctx* c, const double* d_cube, int B, double* d_phys, double* d_logL, void* stream)
{
    if (!c || (!d_cube && c->model.ndims > 0) || !d_logL || B < 0) return LG_ERR_INPUT;
    if (B > c->max_batch) return c->fail(LG_ERR_INPUT, "batch larger than max_batch");
    int rc;
    if ((rc = check_priors(c))) return rc;
    if (B == 0) return LG_OK;
    if ((rc = c->cuda(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    if (!stream && (rc = order_after_legacy(c))) return rc;
    const cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    if ((rc = join_before(c, s)) || (rc = enqueue_cube(c, B, d_cube, d_phys, d_logL, s))) return rc;
    return join_after(c, s);
}

namespace {

// Render one parameter vector (map order) on the context's stream: the raw
// model to d_model_out, its quadrature error to d_err_out and, with a PSF,
// the convolved model to the first image of d_raw (src/nested.c:175-205).
// Returns the device pointer of the model (convolved if there is a PSF).
int render_device(lg_ctx* c, const double* params, const float** d_model)
{
    int rc;
    if ((rc = c->cuda(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    const size_t N = (size_t)c->N, np = c->model.pars.size();
    if (!c->d_model_out) {
        if ((rc = c->cuda(cudaMalloc((void**)&c->d_model_out, N * 4), "render buffer")) ||
            (rc = c->cuda(cudaMalloc((void**)&c->d_err_out, N * 4), "render buffer")))
            return rc;
    }
    float* d_val = c->d_model_out;
    if ((rc = c->cuda(cudaMemcpyAsync(c->d_params, params, np * 8, cudaMemcpyHostToDevice, c->stream), "params")))
        return rc;
    int one = 1;
    void* a_setp[] = {&c->d_params, &one, &c->d_models};
    if ((rc = c->nobj > 1 && c->nobj <= 32
                  ? c->launch(c->f_setp_split, dim3(1), dim3(32 * c->nobj), 0, c->stream, a_setp, "set_params")
                  : c->launch(c->f_setp, dim3(1), dim3(128), 0, c->stream, a_setp, "set_params")))
        return rc;
    void* a_r[] = {&c->d_models, &d_val, &c->d_err_out};
    if ((rc = c->launch(c->f_rdump, dim3(c->rtiles, 1), dim3(c->shape.rt), 0, c->stream, a_r, "render"))) return rc;
    if (c->psf) {
        void* a_c[] = {&d_val, &c->d_raw};
        if ((rc = c->launch(c->f_cdump, dim3(c->ctiles_x, c->ctiles_y, 1),
                            dim3(c->shape.ctx / c->shape.cr, c->shape.conv_block_y()),
                            c->csmem, c->stream, a_c, "convolve")))
            return rc;
    }
    *d_model = c->psf ? c->d_raw : d_val;
    return LG_OK;
}

// The six output layers of the reference's dumper (src/nested.c:217-254),
// one pixel per thread: IMG model, RES image - model, RAW unconvolved model,
// ERR error / raw, WHT weight, PVL erfc(sqrt(chi2 / 2)) with the per-pixel
// chi2 = weight * (model - image)^2 of the loglike kernel
// (kernel/lensed.cl:41-53), all in IEEE FP32 except the p-value's double
// erfc/sqrt, which the reference also evaluates in double.
__global__ void __launch_bounds__(256)
    lg_dump_layers(const float* __restrict__ model, const float* __restrict__ raw, const float* __restrict__ err,
                   const float* __restrict__ image, const float* __restrict__ weight, long N, float* __restrict__ out)
{
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < N; k += (long)gridDim.x * blockDim.x) {
        const float m = model[k], v = raw[k], d = image[k], w = weight[k];
        const float r = __fsub_rn(m, d);
        const float chi2 = __fmul_rn(__fmul_rn(w, r), r);
        out[k] = m;
        out[N + k] = __fsub_rn(d, m);
        out[2 * N + k] = v;
        out[3 * N + k] = __fdiv_rn(err[k], v);
        out[4 * N + k] = w;
        out[5 * N + k] = (float)erfc(sqrt(0.5 * (double)chi2));
    }
}

}  // namespace

int lg_render(lg_ctx* c, const double* params, float* model, float* raw, float* error)
{
    if (!c || !params) return LG_ERR_INPUT;
    int rc;
    const float* d_model = nullptr;
    if ((rc = render_device(c, params, &d_model))) return rc;
    const size_t N = (size_t)c->N;
    if (raw &&
        (rc = c->cuda(cudaMemcpyAsync(raw, c->d_model_out, N * 4, cudaMemcpyDeviceToHost, c->stream), "read raw")))
        return rc;
    if (error &&
        (rc = c->cuda(cudaMemcpyAsync(error, c->d_err_out, N * 4, cudaMemcpyDeviceToHost, c->stream), "read error")))
        return rc;
    if (model && (rc = c->cuda(cudaMemcpyAsync(model, d_model, N * 4, cudaMemcpyDeviceToHost, c->stream), "read model")))
        return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "render");
}

int lg_dump(lg_ctx* c, const double* params, float* layers)
{
    if (!c || !params || !layers) return LG_ERR_INPUT;
    int rc;
    const float* d_model = nullptr;
    if ((rc = render_device(c, params, &d_model))) return rc;
    const long N = c->N;
    if (!c->d_layers && (rc = c->cuda(cudaMalloc((void**)&c->d_layers, (size_t)N * 6 * 4), "dump buffer"))) return rc;
    const int blocks = (int)std::min<long>((N + 255) / 256, 4096);
    lg_dump_layers<<<blocks, 256, 0, c->stream>>>(d_model, c->d_model_out, c->d_err_out, c->d_image, c->d_weight, N,
                                                  c->d_layers);
    if ((rc = c->cuda(cudaGetLastError(), "dump layers"))) return rc;
    if ((rc = c->cuda(cudaMemcpyAsync(layers, c->d_layers, (size_t)N * 6 * 4, cudaMemcpyDeviceToHost, c->stream),
                      "read layers")))
        return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "dump");
}

const char* const lg_dump_names[LG_DUMP_LAYERS] = {"IMG", "RES", "RAW", "ERR", "WHT", "PVL"};

int lg_write_output(lg_ctx* c, const double* params, const char* path)
{
    if (!c || !params || !path) return LG_ERR_INPUT;
    std::vector<float> layers((size_t)c->N * LG_DUMP_LAYERS);
    int rc = lg_dump(c, params, layers.data());
    if (rc) return rc;
    const float* ptr[LG_DUMP_LAYERS];
    for (int i = 0; i < LG_DUMP_LAYERS; ++i) ptr[i] = layers.data() + (size_t)i * c->N;
    rc = lg_write_fits(path, c->model.width, c->model.height, LG_DUMP_LAYERS, ptr, lg_dump_names);
    if (rc) c->err = lg_last_error(nullptr);
    return rc;
}

int lg_launch_shape(const lg_ctx* c, int shape[7])
{
    if (!c || !shape) return LG_ERR_INPUT;
    const lg::Shape& s = c->shape;
    const int v[7] = {s.rt, s.rppt, s.qs, s.ctx, s.cty, s.cr, s.pair_rows ? 1 : 0};
    std::memcpy(shape, v, sizeof v);
    return LG_OK;
}

int lg_set_launch_shape(lg_ctx* c, const int shape[7])
{
    if (!c || !shape) return LG_ERR_INPUT;
    lg::Shape s;
    s.rt = shape[0];
    s.rppt = shape[1];
    s.qs = shape[2];
    s.ctx = shape[3];
    s.cty = shape[4];
    s.cr = shape[5];
    s.pair_rows = shape[6] != 0;
    const std::string why = lg::check_shape(s, ctx_mode(c), c->psf, c->model.psfw);
    if (!why.empty()) return c->fail(LG_ERR_INPUT, "launch shape: " + why);
    int rc;
    if ((rc = c->cuda(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    std::vector<char> cubin;
    const lg::Shape old = c->shape;
    if ((rc = compile_eval(c, s, cubin))) return rc;
    rc = load_eval(c, s, cubin);
    if (rc == LG_ERR_UNSUPPORTED) {
        // keep the context usable with its previous shape
        const std::string msg = c->err;
        std::vector<char> prev;
        if (!compile_eval(c, old, prev) && !load_eval(c, old, prev)) c->err = msg;
        else rc = LG_ERR_CUDA;
    }
    return rc;
}

const char* lg_tune_report(const lg_ctx* c) { return c ? c->tune_report.c_str() : ""; }

int lg_host_set_active(const lg_ctx* c) { return c && c->host_set ? 1 : 0; }

// Per-stage device times of one evaluation, the counterpart of the
// reference's --profile event table (src/nested.c:21-40, src/profile.c).
int lg_eval_profile(lg_ctx* c, const double* d_params, int B, double* d_logL, float* stage_ms)
{
    if (!c || !d_params || !d_logL || !stage_ms || B <= 0) return LG_ERR_INPUT;
    if (B > c->max_batch) return c->fail(LG_ERR_INPUT, "batch larger than max_batch");
    int rc;
    if ((rc = c->cuda(cudaSetDevice(c->device), "cudaSetDevice"))) return rc;
    if ((rc = order_after_legacy(c))) return rc;
    cudaEvent_t ev[5] = {};
    for (auto& e : ev)
        if ((rc = c->cuda(cudaEventCreate(&e), "event"))) return rc;
    rc = c->enqueue(B, d_params, d_logL, c->stream, ev);
    if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "profile");
    for (int i = 0; i < 4 && !rc; ++i) rc = c->cuda(cudaEventElapsedTime(&stage_ms[i], ev[i], ev[i + 1]), "elapsed");
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
}

}  // extern "C"

// FP32 FMA throughput probe: eight independent FMA chains per thread.
__global__ void lg_fma_probe(float* out, float a, float b, int iters)
{
    float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-7f, x2 = x0 + 2e-7f, x3 = x0 + 3e-7f;
    float x4 = x0 + 4e-7f, x5 = x0 + 5e-7f, x6 = x0 + 6e-7f, x7 = x0 + 7e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 12345.0f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

extern "C" {

// Measured FP32 FMA throughput of the current device in TFLOP/s (2 flops per
// FMA); the denominator of the ray-shooting roofline.
int lg_measure_fp32_peak(int device, double* tflops)
{
    if (!tflops) return LG_ERR_INPUT;
    if (cudaSetDevice(device) != cudaSuccess) return LG_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float* out = nullptr;
    const int threads = 256, blocks = sms * 8, iters = 4096;
    if (cudaMalloc(&out, (size_t)threads * blocks * 4) != cudaSuccess) return LG_ERR_ALLOC;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        lg_fma_probe<<<blocks, threads>>>(out, 0.999999f, 1e-6f, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return LG_ERR_CUDA;
    *tflops = 2.0 * 8 * 16 * (double)iters * threads * blocks / (best * 1e-3) / 1e12;
    return LG_OK;
}

// src/nested.c:17-131 with the arithmetic moved to the GPU.  The reference
// redraws a parameter until it falls inside its bounds with the same unit
// value, which never ends when the first draw is outside; here such a point
// gets logL = -inf instead.
void loglike(double cube[], int* ndim, int* npar, double* lnew, void* ctx)
{
    lg_ctx* c = static_cast<lg_ctx*>(ctx);
    *lnew = -HUGE_VAL;
    if (!c || !cube || !ndim || !npar) return;
    const lg::Model& m = c->model;
    if (*npar != (int)m.pars.size() || *ndim != m.ndims) {
        c->err = "loglike: ndim/npar do not match the context";
        return;
    }
    if (check_priors(c) || c->cuda(cudaSetDevice(c->device), "cudaSetDevice")) return;
    std::vector<double> p(*npar);
    double l;
    if (cube_eval_chunk(c, cube, 1, p.data(), &l, false)) return;
    // MultiNest records the physical values written back into cube
    for (int i = 0; i < *npar; ++i) cube[i] = p[i];
    if (c->last_bad) {
        c->err = "loglike: parameter outside its bounds";
        return;
    }
    *lnew = l;
}

}  // extern "C"
