// A batch of lens systems of uneven image and PSF sizes evaluated together:
// the counterpart of running one Lensed process per system, for samplers
// that advance many systems at once.
//
// All systems share the object list (plugins, priors, parameter map) and the
// quadrature rule.  Per call, the candidate counts of the systems may change;
// a small plan (per-system counts and work-unit offsets) is uploaded inside
// the CUDA graph, so one graph -- upload, set_params, persistent render,
// persistent convolution + chi^2, finish, read-back -- is captured once and
// replayed for any counts within the capacities given at creation.

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <cstdint>
#include <cstdio>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "lg_internal.h"

namespace {

// mirrors of the device structs in device/lg_multi_kernels.cuh
struct SysInfo {
    int W, H, N, pw, ph;
    int rtiles, ctiles_x, ctiles_y, ctiles;
    int psf_off;
    float rx, ry, sx, sy;
    long long img_off;
};
struct SysPlan {
    int count, cand0;
    long long r_unit0, c_unit0, raw0, part0;
};

}  // namespace

struct lg_systems {
    int nsys = 0, flags = 0, device = 0;
    bool psf = false;
    std::string err;
    std::vector<lg::Model> models;
    lg::Shape shape;
    std::vector<int> cap;      // capacity (max candidates) per system
    int max_total = 0;
    std::vector<SysInfo> info;
    std::vector<long long> raw0, part0;
    size_t model_bytes = 0;

    const lg::Driver* drv = nullptr;
    CUmodule mod = nullptr, mod_set = nullptr;
    CUfunction f_setp = nullptr, f_render = nullptr, f_conv = nullptr, f_finish = nullptr;
    int grid_render = 0, grid_conv = 0, grid_finish = 0, csmem = 0;

    cudaStream_t stream = nullptr;
    float *d_images = nullptr, *d_weights = nullptr, *d_psfs = nullptr, *d_raw = nullptr;
    void* d_models = nullptr;
    double *d_partials = nullptr, *d_params = nullptr, *d_logL = nullptr;
    SysInfo* d_info = nullptr;
    SysPlan* d_plan = nullptr;
    long long* d_hdr = nullptr;
    double *h_params = nullptr, *h_logL = nullptr;
    SysPlan* h_plan = nullptr;
    long long* h_hdr = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::string tune_report;
    std::vector<long long> part_count;  // partial sums per system (by capacity)

    int fail(int code, const std::string& m)
    {
        err = m;
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
    int launch(CUfunction f, dim3 g, dim3 b, unsigned smem, void** args, const char* what)
    {
        return drvcall(drv->launchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, smem, (CUstream)stream, args, nullptr),
                       what);
    }
    void release()
    {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        void* dev[] = {d_images, d_weights, d_psfs, d_raw, d_models, d_partials, d_params, d_logL, d_info, d_plan,
                       d_hdr};
        for (void* p : dev) cudaFree(p);
        void* host[] = {h_params, h_logL, h_plan, h_hdr};
        for (void* p : host) cudaFreeHost(p);
        if (mod && drv) drv->moduleUnload(mod);
        if (mod_set && drv) drv->moduleUnload(mod_set);
        if (stream) cudaStreamDestroy(stream);
        mod = mod_set = nullptr;
        stream = nullptr;
    }
};

namespace {

lg::Fp sys_mode(const lg_systems* S) { return lg::fp_mode(S->flags); }
bool sys_ieee(const lg_systems* S) { return lg::fp_ieee(S->flags); }

// Distinct PSF shapes of the batch: each gets its own convolution code.
std::vector<std::pair<int, int>> psf_shapes(const lg_systems* S)
{
    std::set<std::pair<int, int>> shapes;
    if (S->psf)
        for (const lg::Model& m : S->models) shapes.insert({m.psfw, m.psfh});
    return std::vector<std::pair<int, int>>(shapes.begin(), shapes.end());
}

std::string multi_source(const lg_systems* S, const lg::Shape& sh)
{
    return lg::compose_multi_source(S->models[0], psf_shapes(S), sh, sys_mode(S));
}

int compile_multi(lg_systems* S, const lg::Shape& sh, std::vector<char>& cubin)
{
    std::string log;
    int rc = lg::compile_program(multi_source(S, sh), lg::fp_fmad(sys_mode(S)), cubin, log, sys_ieee(S));
    return rc ? S->fail(rc, log) : LG_OK;
}

// Launch shapes of the multi-system kernels: cty counts thread rows (a
// paired-row unit covers 2 cty rows), and cr is a multiple of 8 so that
// both unit kinds compile.
std::string check_multi_shape(const lg::Shape& s, lg::Fp mode)
{
    lg::Shape t = s;
    t.pair_rows = false;
    std::string why = lg::check_shape(t, mode, true, 0);
    if (why.empty() && s.pair_rows) why = "the multi-system kernels choose paired rows per system";
    if (why.empty() && s.cr % 8) why = "multi-system convolution needs cr % 8 == 0";
    return why;
}

// Make the multi-system module compiled for shape sh current: tiles and
// partial sums per system, kernels, shared memory, persistent grids.
int apply_shape(lg_systems* S, const lg::Shape& sh, const std::vector<char>& cubin)
{
    int rc;
    if (S->stream && (rc = S->cuda(cudaStreamSynchronize(S->stream), "synchronize"))) return rc;
    if (S->graph) cudaGraphExecDestroy(S->graph);
    S->graph = nullptr;
    if (S->mod) S->drv->moduleUnload(S->mod);
    S->mod = nullptr;
    cudaFree(S->d_partials);
    S->d_partials = nullptr;
    S->shape = sh;
    const bool strict = sys_mode(S) == lg::Fp::STRICT;
    long long part = 0;
    int csmem = 0;
    S->part0.clear();
    for (int s = 0; s < S->nsys; ++s) {
        const lg::Model& m = S->models[s];
        SysInfo& I = S->info[s];
        I.rtiles = (I.N + sh.rtile() - 1) / sh.rtile();
        // fast and exact modes, PSF up to 49 wide: paired-row units of
        // 2 * cty rows, as the single-system context tiles them
        const bool paired = S->psf && !strict && m.psfw <= 49;
        const int cty = paired ? 2 * sh.cty : sh.cty;
        I.ctiles_x = (I.W + sh.ctx - 1) / sh.ctx;
        I.ctiles_y = (I.H + cty - 1) / cty;
        I.ctiles = I.ctiles_x * I.ctiles_y;
        if (S->psf) {
            if (paired) {
                // layout of lg_multi_conv_unit_pair: row pairs, pair column c at
                // float 2c + 4 floor(c/8), pitch 16 (mod 32) words
                const int cwin = (sh.cr + m.psfw - 1 + 1) / 2 * 2;
                const int cnc = sh.ctx - sh.cr + cwin;
                const int croww = 2 * (cnc - 1) + 4 * ((cnc - 1) / 8) + 2;
                const int cp = (croww - 16 + 31) / 32 * 32 + 16;
                csmem = std::max(csmem, ((sh.cty + m.psfh - 1) * cp + m.psfw * m.psfh) * 4);
            } else {
                const int win4 = (sh.cr + m.psfw - 1 + 3) / 4 * 4;
                const int twp = ((sh.ctx - sh.cr + win4 + 27) / 32) * 32 + 4;
                csmem = std::max(csmem, ((sh.cty + m.psfh - 1) * twp + m.psfw * m.psfh) * 4);
            }
        }
        S->part0.push_back(part);
        part += (long long)S->cap[s] * (S->psf ? I.ctiles : I.rtiles);
    }
    S->csmem = csmem;
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, S->device);
    if (csmem > optin)
        return S->fail(LG_ERR_UNSUPPORTED, "convolution tile needs " + std::to_string(csmem) +
                                               " bytes of shared memory, above the device's " + std::to_string(optin));
    if ((rc = S->drvcall(S->drv->moduleLoadData(&S->mod, cubin.data()), "cuModuleLoadData")) ||
        (rc = S->drvcall(S->drv->moduleGetFunction(&S->f_render, S->mod,
                                                   S->psf ? "lg_multi_render_raw" : "lg_multi_render_chi2"),
                         "render")) ||
        (rc = S->drvcall(S->drv->moduleGetFunction(&S->f_conv, S->mod, "lg_multi_conv_chi2"), "convolve")) ||
        (rc = S->drvcall(S->drv->moduleGetFunction(&S->f_finish, S->mod, "lg_multi_finish"), "finish")))
        return rc;
    if (S->csmem > 48 * 1024 &&
        (rc = S->drvcall(S->drv->funcSetAttribute(S->f_conv, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                  S->csmem),
                         "convolve smem")))
        return rc;
    // persistent grids: every SM filled to its occupancy
    int sms = 0, occ_r = 0, occ_c = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S->device);
    if ((rc = S->drvcall(S->drv->occupancy(&occ_r, S->f_render, sh.rt, 0), "occupancy")) ||
        (rc = S->drvcall(S->drv->occupancy(&occ_c, S->f_conv, (sh.ctx / sh.cr) * sh.cty, S->csmem), "occupancy")))
        return rc;
    S->grid_render = sms * std::max(occ_r, 1);
    S->grid_conv = sms * std::max(occ_c, 1);
    S->grid_finish = sms * 4;
    if (cudaMalloc((void**)&S->d_partials, std::max<long long>(part, 2) * 8) != cudaSuccess)
        return S->fail(LG_ERR_ALLOC, "cudaMalloc partials");
    return S->cuda(cudaMemcpy(S->d_info, S->info.data(), S->nsys * sizeof(SysInfo), cudaMemcpyHostToDevice),
                   "upload info");
}

// Per-call plan: the systems' candidate counts and work-unit offsets;
// returns the candidate total, or -1 for a count outside [0, capacity].
int build_plan(lg_systems* S, const int* counts)
{
    long long ru = 0, cu = 0;
    int total = 0;
    for (int s = 0; s < S->nsys; ++s) {
        if (counts[s] < 0 || counts[s] > S->cap[s]) {
            S->err = "system " + std::to_string(s) + ": count outside [0, capacity]";
            return -1;
        }
        SysPlan& P = S->h_plan[s];
        P.count = counts[s];
        P.cand0 = total;
        P.r_unit0 = ru;
        P.c_unit0 = cu;
        P.raw0 = S->raw0[s];
        P.part0 = S->part0[s];
        ru += (long long)counts[s] * S->info[s].rtiles;
        cu += (long long)counts[s] * S->info[s].ctiles;
        total += counts[s];
    }
    S->h_hdr[0] = ru;
    S->h_hdr[1] = S->psf ? cu : 0;
    S->h_hdr[2] = total;
    S->h_hdr[3] = S->nsys;
    return total;
}

int enqueue_systems(lg_systems* S, cudaEvent_t* ev = nullptr);
int autotune_systems(lg_systems* S);

int create_systems(lg_systems* S, const lg_image_desc* images, int nsys, const lg_object_desc* objs, int nobjs,
                   const lg_options* opts, const int* capacity)
{
    if (!images || nsys <= 0 || nsys > 4096 || !capacity) return S->fail(LG_ERR_INPUT, "invalid system list");
    S->nsys = nsys;
    S->flags = opts ? opts->flags : 0;
    S->device = opts ? opts->device : 0;
    S->models.resize(nsys);
    int rc;
    for (int s = 0; s < nsys; ++s) {
        if ((rc = lg::build_model(&images[s], objs, nobjs, opts, S->models[s], S->err))) {
            S->err = "system " + std::to_string(s) + ": " + S->err;
            return rc;
        }
        if (!images[s].image || !images[s].weight)
            return S->fail(LG_ERR_INPUT, "system " + std::to_string(s) + ": image and weight are required");
        if (capacity[s] < 0 || capacity[s] > 65535) return S->fail(LG_ERR_INPUT, "invalid capacity");
    }
    const lg::Model& m0 = S->models[0];
    S->psf = !m0.psf.empty();
    for (int s = 1; s < nsys; ++s) {
        const lg::Model& m = S->models[s];
        if (!m.psf.empty() != S->psf) return S->fail(LG_ERR_UNSUPPORTED, "all systems need a PSF, or none");
        if (m.pcs[2] != m0.pcs[2] || m.pcs[3] != m0.pcs[3])
            return S->fail(LG_ERR_UNSUPPORTED, "systems must share the pixel scale (quadrature offsets)");
        if (m.pmap != m0.pmap) return S->fail(LG_ERR_UNSUPPORTED, "systems must share the parameter map");
    }
    S->cap.assign(capacity, capacity + nsys);
    for (int c : S->cap) S->max_total += c;
    if (S->max_total <= 0 || S->max_total > 1 << 20) return S->fail(LG_ERR_INPUT, "invalid total capacity");

    // static layout: images, PSFs and raw models by capacity; the tiles
    // and partial sums depend on the launch shape (apply_shape)
    const lg::Fp mode = lg::fp_mode(S->flags);
    long long img = 0, raw = 0;
    int psf_off = 0;
    for (int s = 0; s < nsys; ++s) {
        const lg::Model& m = S->models[s];
        SysInfo I{};
        I.W = m.width;
        I.H = m.height;
        I.N = m.width * m.height;
        I.pw = m.psfw;
        I.ph = m.psfh;
        I.psf_off = psf_off;
        double rx = m.pcs[0], ry = m.pcs[1];
        if (S->psf) {
            if (m.psfw % 2 == 0) rx += 0.5;  // src/lensed.c:884-891
            if (m.psfh % 2 == 0) ry += 0.5;
            psf_off += m.psfw * m.psfh;
        }
        I.rx = (float)rx;
        I.ry = (float)ry;
        I.sx = (float)m.pcs[2];
        I.sy = (float)m.pcs[3];
        I.img_off = img;
        img += I.N;
        S->raw0.push_back(raw);
        raw += (long long)S->cap[s] * I.N;
        S->info.push_back(I);
    }

    // set_params module
    std::vector<char> cubin_set;
    std::string log;
    rc = lg::compile_program(lg::compose_source(m0, S->shape, mode, lg::Part::SET), false, cubin_set, log);
    if (rc) return S->fail(rc, log);
    if ((rc = S->cuda(cudaSetDevice(S->device), "cudaSetDevice")) || (rc = S->cuda(cudaFree(nullptr), "context")))
        return rc;
    S->drv = lg::driver();
    if (!S->drv) return S->fail(LG_ERR_CUDA, "CUDA driver entry points unavailable");
    if ((rc = S->drvcall(S->drv->moduleLoadData(&S->mod_set, cubin_set.data()), "cuModuleLoadData")) ||
        (rc = S->drvcall(S->drv->moduleGetFunction(&S->f_setp, S->mod_set, "lg_set_params_kernel"), "set_params")))
        return rc;
    CUdeviceptr gp;
    size_t gb;
    unsigned mb = 0;
    if ((rc = S->drvcall(S->drv->moduleGetGlobal(&gp, &gb, S->mod_set, "lg_model_bytes"), "model size")) ||
        (rc = S->cuda(cudaMemcpy(&mb, (void*)gp, sizeof mb, cudaMemcpyDeviceToHost), "model size")))
        return rc;
    S->model_bytes = mb;

    if ((rc = S->cuda(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking), "stream"))) return rc;
    const size_t np = m0.pars.size();
    auto alloc = [&](void** p, size_t bytes, const char* what) {
        cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
        if (e != cudaSuccess) {
            S->err = std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e);
            return LG_ERR_ALLOC;
        }
        return LG_OK;
    };
    if ((rc = alloc((void**)&S->d_images, img * 4, "images")) || (rc = alloc((void**)&S->d_weights, img * 4, "weights")) ||
        (rc = alloc((void**)&S->d_psfs, std::max(psf_off, 1) * 4, "psfs")) ||
        (rc = alloc((void**)&S->d_raw, S->psf ? raw * 4 : 0, "raw")) ||
        (rc = alloc(&S->d_models, (size_t)S->max_total * S->model_bytes, "models")) ||
        (rc = alloc((void**)&S->d_params, (size_t)S->max_total * np * 8, "params")) ||
        (rc = alloc((void**)&S->d_logL, (size_t)S->max_total * 8, "logL")) ||
        (rc = alloc((void**)&S->d_info, nsys * sizeof(SysInfo), "info")) ||
        (rc = alloc((void**)&S->d_plan, nsys * sizeof(SysPlan), "plan")) ||
        (rc = alloc((void**)&S->d_hdr, 4 * sizeof(long long), "header")))
        return rc;
    if ((rc = S->cuda(cudaMallocHost((void**)&S->h_params, (size_t)S->max_total * np * 8), "pinned")) ||
        (rc = S->cuda(cudaMallocHost((void**)&S->h_logL, (size_t)S->max_total * 8), "pinned")) ||
        (rc = S->cuda(cudaMallocHost((void**)&S->h_plan, nsys * sizeof(SysPlan)), "pinned")) ||
        (rc = S->cuda(cudaMallocHost((void**)&S->h_hdr, 4 * sizeof(long long)), "pinned")))
        return rc;
    std::memset(S->h_params, 0, (size_t)S->max_total * np * 8);
    for (int s = 0; s < nsys; ++s) {
        const SysInfo& I = S->info[s];
        if ((rc = S->cuda(cudaMemcpy(S->d_images + I.img_off, images[s].image, (size_t)I.N * 4,
                                     cudaMemcpyHostToDevice),
                          "upload")) ||
            (rc = S->cuda(cudaMemcpy(S->d_weights + I.img_off, images[s].weight, (size_t)I.N * 4,
                                     cudaMemcpyHostToDevice),
                          "upload")))
            return rc;
        if (S->psf &&
            (rc = S->cuda(cudaMemcpy(S->d_psfs + I.psf_off, S->models[s].psf.data(), S->models[s].psf.size() * 4,
                                     cudaMemcpyHostToDevice),
                          "upload")))
            return rc;
    }
    if ((rc = S->cuda(cudaMemset(S->d_params, 0, (size_t)S->max_total * np * 8), "clear"))) return rc;
    if (S->flags & LG_FLAG_AUTOTUNE) return autotune_systems(S);
    std::vector<char> cubin;
    if ((rc = compile_multi(S, S->shape, cubin))) return rc;
    return apply_shape(S, S->shape, cubin);
}

// Upload, set_params, render, convolution + chi^2, finish and read-back of
// the current plan; with ev != NULL, ev[0..4] are recorded around the four
// kernel stages (set_params, render, convolve, finish).
int enqueue_systems(lg_systems* S, cudaEvent_t* ev)
{
    auto mark = [&](int i) { return ev ? S->cuda(cudaEventRecord(ev[i], S->stream), "event") : LG_OK; };
    const size_t np = S->models[0].pars.size();
    int rc;
    if ((rc = S->cuda(cudaMemcpyAsync(S->d_params, S->h_params, (size_t)S->max_total * np * 8,
                                      cudaMemcpyHostToDevice, S->stream),
                      "params")) ||
        (rc = S->cuda(cudaMemcpyAsync(S->d_plan, S->h_plan, S->nsys * sizeof(SysPlan), cudaMemcpyHostToDevice,
                                      S->stream),
                      "plan")) ||
        (rc = S->cuda(cudaMemcpyAsync(S->d_hdr, S->h_hdr, 4 * sizeof(long long), cudaMemcpyHostToDevice,
                                      S->stream),
                      "header")))
        return rc;
    int total = S->max_total;
    void* a_setp[] = {&S->d_params, &total, &S->d_models};
    if ((rc = mark(0)) ||
        (rc = S->launch(S->f_setp, dim3((total + 127) / 128), dim3(128), 0, a_setp, "set_params")) ||
        (rc = mark(1)))
        return rc;
    if (S->psf) {
        void* a_r[] = {&S->d_models, &S->d_info, &S->d_plan, &S->d_hdr, &S->d_raw};
        if ((rc = S->launch(S->f_render, dim3(S->grid_render), dim3(S->shape.rt), 0, a_r, "render")) ||
            (rc = mark(2)))
            return rc;
        void* a_c[] = {&S->d_raw, &S->d_info, &S->d_plan, &S->d_hdr, &S->d_images, &S->d_weights, &S->d_psfs,
                       &S->d_partials};
        if ((rc = S->launch(S->f_conv, dim3(S->grid_conv), dim3(S->shape.ctx / S->shape.cr, S->shape.cty),
                            S->csmem, a_c, "convolve")) ||
            (rc = mark(3)))
            return rc;
    } else {
        void* a_r[] = {&S->d_models, &S->d_info, &S->d_plan, &S->d_hdr, &S->d_images, &S->d_weights,
                       &S->d_partials};
        if ((rc = S->launch(S->f_render, dim3(S->grid_render), dim3(S->shape.rt), 0, a_r, "render")) ||
            (rc = mark(2)) || (rc = mark(3)))
            return rc;
    }
    int with_psf = S->psf ? 1 : 0;
    void* a_f[] = {&S->d_partials, &S->d_info, &S->d_plan, &S->d_hdr, &with_psf, &S->d_logL};
    if ((rc = S->launch(S->f_finish, dim3(S->grid_finish), dim3(256), 0, a_f, "finish")) || (rc = mark(4)))
        return rc;
    return S->cuda(cudaMemcpyAsync(S->h_logL, S->d_logL, (size_t)S->max_total * 8, cudaMemcpyDeviceToHost,
                                   S->stream),
                   "logL");
}

// Candidate parameters for timing: every system at capacity, parameters
// drawn from the priors (map order; derived ones at u = 0.5).
int tune_params(lg_systems* S)
{
    const lg::Model& m = S->models[0];
    for (const lg::ParamInfo& p : m.pars)
        if (!p.has_prior) return S->fail(LG_ERR_INPUT, "no prior for " + p.id + " to draw candidates from");
    uint64_t st = 0x13198a2e03707344ull;
    auto unif = [&]() {
        st += 0x9e3779b97f4a7c15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    const size_t np = m.pars.size();
    for (int b = 0; b < S->max_total; ++b)
        for (size_t i = 0; i < np; ++i)
            S->h_params[(size_t)b * np + i] = m.pars[m.pmap[i]].prior.apply((int)i < m.ndims ? unif() : 0.5);
    return LG_OK;
}

// Render and convolution times (ms, best of several runs) of the current
// module on the candidates in h_params, every system at capacity.
int time_systems(lg_systems* S, double* render_ms, double* conv_ms)
{
    if (build_plan(S, S->cap.data()) < 0) return LG_ERR_INPUT;
    cudaEvent_t ev[5] = {};
    int rc = LG_OK;
    for (auto& e : ev)
        if (!rc) rc = S->cuda(cudaEventCreate(&e), "event");
    double best[2] = {1e30, 1e30}, total = 0;
    for (int rep = 0; !rc && rep < 40; ++rep) {
        rc = enqueue_systems(S, ev);
        if (!rc) rc = S->cuda(cudaStreamSynchronize(S->stream), "tune run");
        float t[2] = {0, 0};
        for (int i = 0; i < 2 && !rc; ++i) rc = S->cuda(cudaEventElapsedTime(&t[i], ev[i + 1], ev[i + 2]), "elapsed");
        if (rc || rep == 0) continue;
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

// LG_FLAG_AUTOTUNE for a batch of systems: render and convolution
// candidates compiled in parallel and timed at full capacity; the fastest
// of each are combined (cached per program, device, capacity and flags).
int autotune_systems(lg_systems* S)
{
    const lg::Fp mode = sys_mode(S);
    const lg::Shape base = S->shape;
    std::string caps;
    for (int c : S->cap) caps += std::to_string(c) + ",";
    const std::string key = lg::tune_key(multi_source(S, base) + caps, S->device, S->max_total,
                                         S->flags & (LG_FLAG_STRICT_FP | LG_FLAG_IEEE_DIV | LG_FLAG_FAST_MATH));
    int rc;
    lg::Shape chosen;
    if (lg::tune_cache_get(key, chosen) && check_multi_shape(chosen, mode).empty()) {
        std::vector<char> cubin;
        if ((rc = compile_multi(S, chosen, cubin)) || (rc = apply_shape(S, chosen, cubin))) return rc;
        S->tune_report = "cached " + key + ": " + chosen.str() + "\n";
        return LG_OK;
    }
    if ((rc = tune_params(S))) {
        std::vector<char> cubin;
        const std::string why = S->err;
        S->err.clear();
        if ((rc = compile_multi(S, base, cubin)) || (rc = apply_shape(S, base, cubin))) return rc;
        S->tune_report = "not tuned (" + why + "): " + base.str() + "\n";
        return LG_OK;
    }
    std::vector<lg::Shape> cand;
    std::vector<int> is_render;
    for (const lg::Shape& s : lg::render_candidates(base, mode))
        if (check_multi_shape(s, mode).empty()) cand.push_back(s), is_render.push_back(1);
    if (S->psf)
        for (const lg::Shape& s : lg::conv_candidates(base, true)) {
            if (!check_multi_shape(s, mode).empty()) continue;
            bool dup = false;
            for (const lg::Shape& t : cand) dup = dup || t == s;
            if (!dup) cand.push_back(s), is_render.push_back(0);
        }
    std::vector<std::string> srcs;
    for (const lg::Shape& s : cand) srcs.push_back(multi_source(S, s));
    std::vector<std::vector<char>> cubins;
    std::vector<int> rcs;
    std::vector<std::string> logs;
    lg::compile_parallel(srcs, lg::fp_fmad(mode), sys_ieee(S), cubins, rcs, logs);
    std::ostringstream rep;
    double best_r = 1e30, best_c = 1e30;
    lg::Shape br = base, bc = base;
    for (size_t i = 0; i < cand.size(); ++i) {
        if (rcs[i]) {
            rep << "  " << cand[i].str() << ": compile failed\n";
            continue;
        }
        if ((rc = apply_shape(S, cand[i], cubins[i]))) {
            if (rc != LG_ERR_UNSUPPORTED) return rc;
            rep << "  " << cand[i].str() << ": " << S->err << "\n";
            S->err.clear();
            continue;
        }
        double r_ms = 0, c_ms = 0;
        if ((rc = time_systems(S, &r_ms, &c_ms))) return rc;
        char line[256];
        std::snprintf(line, sizeof line, "  %s: render %.4f ms, convolve %.4f ms\n", cand[i].str().c_str(), r_ms,
                      c_ms);
        rep << line;
        const bool base_conv = cand[i].ctx == base.ctx && cand[i].cty == base.cty && cand[i].cr == base.cr;
        if (is_render[i] && r_ms < best_r) best_r = r_ms, br = cand[i];
        if ((!is_render[i] || base_conv) && S->psf && c_ms < best_c) best_c = c_ms, bc = cand[i];
    }
    chosen = br;
    if (S->psf) {
        chosen.ctx = bc.ctx;
        chosen.cty = bc.cty;
        chosen.cr = bc.cr;
    }
    const std::vector<char>* cb = nullptr;
    for (size_t i = 0; i < cand.size(); ++i)
        if (!rcs[i] && cand[i] == chosen) cb = &cubins[i];
    std::vector<char> own;
    if (!cb) {
        if ((rc = compile_multi(S, chosen, own))) return rc;
        cb = &own;
    }
    if ((rc = apply_shape(S, chosen, *cb))) return rc;
    std::memset(S->h_params, 0, (size_t)S->max_total * S->models[0].pars.size() * 8);
    lg::tune_cache_put(key, chosen);
    S->tune_report = "tuned " + key + " at capacity: " + chosen.str() + "\n" + rep.str();
    return LG_OK;
}

}  // namespace

extern "C" {

lg_systems* lg_systems_create(const lg_image_desc* images, int nsys, const lg_object_desc* objs, int nobjs,
                              const lg_options* opts, const int* capacity, int* status)
{
    lg_systems* S = new (std::nothrow) lg_systems();
    if (!S) {
        if (status) *status = LG_ERR_ALLOC;
        return nullptr;
    }
    int rc = create_systems(S, images, nsys, objs, nobjs, opts, capacity);
    if (status) *status = rc;
    if (rc) {
        lg::set_global_error(S->err.c_str());
        S->release();
        delete S;
        return nullptr;
    }
    return S;
}

void lg_systems_destroy(lg_systems* S)
{
    if (!S) return;
    cudaSetDevice(S->device);
    if (S->stream) cudaStreamSynchronize(S->stream);
    S->release();
    delete S;
}

const char* lg_systems_last_error(const lg_systems* S) { return S ? S->err.c_str() : ""; }

int lg_systems_launch_shape(const lg_systems* S, int shape[7])
{
    if (!S || !shape) return LG_ERR_INPUT;
    const lg::Shape& s = S->shape;
    const int v[7] = {s.rt, s.rppt, s.qs, s.ctx, s.cty, s.cr, 0};
    std::memcpy(shape, v, sizeof v);
    return LG_OK;
}

int lg_systems_set_launch_shape(lg_systems* S, const int shape[7])
{
    if (!S || !shape) return LG_ERR_INPUT;
    lg::Shape s;
    s.rt = shape[0];
    s.rppt = shape[1];
    s.qs = shape[2];
    s.ctx = shape[3];
    s.cty = shape[4];
    s.cr = shape[5];
    s.pair_rows = shape[6] != 0;
    const std::string why = check_multi_shape(s, sys_mode(S));
    if (!why.empty()) return S->fail(LG_ERR_INPUT, "launch shape: " + why);
    int rc;
    if ((rc = S->cuda(cudaSetDevice(S->device), "cudaSetDevice"))) return rc;
    const lg::Shape old = S->shape;
    std::vector<char> cubin;
    if ((rc = compile_multi(S, s, cubin))) return rc;
    rc = apply_shape(S, s, cubin);
    if (rc == LG_ERR_UNSUPPORTED) {
        const std::string msg = S->err;
        std::vector<char> prev;
        if (!compile_multi(S, old, prev) && !apply_shape(S, old, prev)) S->err = msg;
        else rc = LG_ERR_CUDA;
    }
    return rc;
}

const char* lg_systems_tune_report(const lg_systems* S) { return S ? S->tune_report.c_str() : ""; }

int lg_systems_npars(const lg_systems* S) { return S ? (int)S->models[0].pars.size() : LG_ERR_INPUT; }

int lg_systems_eval(lg_systems* S, const double* params, const int* counts, double* logL)
{
    if (!S || !params || !counts || !logL) return LG_ERR_INPUT;
    int rc;
    if ((rc = S->cuda(cudaSetDevice(S->device), "cudaSetDevice"))) return rc;
    const size_t np = S->models[0].pars.size();
    const int total = build_plan(S, counts);
    if (total < 0) return LG_ERR_INPUT;
    if (total == 0) return LG_OK;
    std::memcpy(S->h_params, params, (size_t)total * np * 8);
    if (!S->graph) {
        cudaGraph_t g;
        if ((rc = S->cuda(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal), "capture")))
            return rc;
        int erc = enqueue_systems(S);
        cudaError_t e = cudaStreamEndCapture(S->stream, &g);
        if (erc) return erc;
        if ((rc = S->cuda(e, "end capture"))) return rc;
        e = cudaGraphInstantiate(&S->graph, g, 0);
        cudaGraphDestroy(g);
        if ((rc = S->cuda(e, "graph instantiate"))) return rc;
    }
    if ((rc = S->cuda(cudaGraphLaunch(S->graph, S->stream), "graph launch")) ||
        (rc = S->cuda(cudaStreamSynchronize(S->stream), "evaluate")))
        return rc;
    std::memcpy(logL, S->h_logL, (size_t)total * 8);
    return LG_OK;
}

}  // extern "C"
