/*
 * lensed_gb300 -- C ABI of the GB300-native Lensed likelihood path.
 *
 * The library replaces Lensed's device runtime and kernel assembly
 * (src/opencl.c, src/kernel.c) and the arithmetic of its likelihood callback
 * (src/nested.c:17-131) with CUDA for sm_103a.  A context holds one lens
 * system -- image, weights, optional PSF, pixel coordinate system, quadrature
 * rule and an ordered object list -- resident on one GPU, plus a program
 * composed from the object plugins and compiled with NVRTC.  Evaluation is
 * batched: one call evaluates B candidate parameter vectors.
 *
 * Conventions
 *   - The caller owns every host buffer passed in; the context owns its
 *     device memory, stream, module and graphs.
 *   - Functions return LG_OK (0) or a negative LG_ERR_* code and never exit
 *     the process; lg_last_error() describes the last failure of a context.
 *   - A context is used by one host thread at a time.  Separate contexts are
 *     independent.
 *   - Images are row-major float32 with row 0 at the bottom (FITS order), so
 *     pixel index k = x + width * y and pixel (x, y) has coordinates
 *     (rx + sx * x, ry + sy * y) -- kernel/lensed.cl:25.
 *   - Parameter vectors are in the context's parameter-map order: the free
 *     parameters first, then the derived ones (fixed by a delta prior), each
 *     group in object order -- src/lensed.c:106-271.
 */
#ifndef LENSED_GB300_H
#define LENSED_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LG_VERSION_MAJOR 0
#define LG_VERSION_MINOR 1

/* status codes */
#define LG_OK 0
#define LG_ERR_INPUT (-1)       /* invalid argument, size, name or prior */
#define LG_ERR_COMPILE (-2)     /* NVRTC composition or compilation failed */
#define LG_ERR_CUDA (-3)        /* CUDA runtime / driver error */
#define LG_ERR_ALLOC (-4)       /* device or host allocation failed */
#define LG_ERR_TIMEOUT (-5)     /* a bounded device-side wait ran out */
#define LG_ERR_UNSUPPORTED (-6) /* valid request the library does not do */

/* object kinds (kernel/object.cl:1-6) */
#define LG_LENS 'L'
#define LG_SOURCE 'S'
#define LG_FOREGROUND 'F'

/* parameter types (kernel/object.cl:8-17) */
#define LG_PARAMETER 0
#define LG_POSITION_X 1
#define LG_POSITION_Y 2
#define LG_RADIUS 3
#define LG_MAGNITUDE 4
#define LG_AXIS_RATIO 5
#define LG_POS_ANGLE 6

/* context flags.  The floating-point mode of the per-ray arithmetic:
 *   default (exact)    IEEE single precision in the reference's operation
 *                      order, no FMA contraction, every elementary function
 *                      correctly rounded (its value in double, rounded once):
 *                      model images and logL identical to the oracle's and to
 *                      the strict mode's.  Rays are traced in pairs with
 *                      f32x2 instructions; exp, log, atan, atanh, sin, cos,
 *                      pow and atan2 are computed in single-precision
 *                      double-word arithmetic (Ziv's rounding test, double
 *                      where it cannot decide), the other functions in
 *                      double.
 *   LG_FLAG_STRICT_FP  the same results one ray at a time with every
 *                      elementary function evaluated in double (the
 *                      definition the default mode reproduces; slow on
 *                      GB300's FP64 pipe)
 *   LG_FLAG_FAST_MATH  ray pairs with FMA contraction and hardware-
 *                      approximate functions (a few ulp each; what the
 *                      reference's -cl-fast-relaxed-math build allows):
 *                      about three times the default's throughput, logL
 *                      within about 1e-3 + 2e-6 |logL| of the oracle's */
#define LG_FLAG_STRICT_FP 1  /* strict mode (above) */
#define LG_FLAG_NO_GRAPH 2   /* launch kernels directly instead of graph replay */
#define LG_FLAG_IEEE_DIV 4   /* fast mode with IEEE division and square root per ray */
#define LG_FLAG_AUTOTUNE 8   /* choose the launch shape by timing candidates at creation */
#define LG_FLAG_FAST_MATH 16 /* fast mode (above) */

typedef struct lg_ctx lg_ctx;

/* The observed data of one lens system.  weight may be NULL only if
 * lg_make_weight() output is passed instead; psf NULL means no PSF.
 * pcs = (rx, ry, sx, sy); all zero means the default (1, 1, 1, 1). */
typedef struct {
    int width, height;
    const float* image;  /* width*height */
    const float* weight; /* width*height inverse variances, 0 = masked */
    const float* psf;    /* psf_width*psf_height, normalised by lg_create */
    int psf_width, psf_height;
    double pcs[4];
} lg_image_desc;

/* One object of the model, in list order (the order decides the planes:
 * sources before the first lens are unlensed; foregrounds use the unlensed
 * position -- src/kernel.c:235-399).
 *   name    plugin name: sis, sis_plus_shear, nsis, sie, sie_plus_shear, nsie,
 *           point_mass, epl, epl_plus_shear, sersic, sersic_old, exponential,
 *           devauc, gauss, sky, or a plugin added with lg_register_plugin
 *   id      object identifier used in parameter ids "<id>.<param>"
 *   priors  NULL or one string per plugin parameter in plugin order, each in
 *           Lensed's prior syntax "[wrap] [image] <value> | unif a b |
 *           norm m s" (docs/configuration.md); NULL entries keep the
 *           plugin default (a fixed value where the plugin defines one). */
typedef struct {
    const char* name;
    const char* id;
    const char* const* priors;
} lg_object_desc;

typedef struct {
    const char* rule; /* quadrature rule name, NULL = "g3k7" (src/input/options.c:130-135) */
    int device;       /* CUDA device ordinal */
    int max_batch;    /* largest B per call (scratch sizing); 0 = 1024 */
    int flags;        /* LG_FLAG_* */
} lg_options;

/* Plugin description for lg_register_plugin (the equivalent of dropping an
 * objects/<name>.cl file into Lensed).  source is CUDA C++ defining
 * struct lg_data_<name>, lg_set_<name>(lg_data_<name>*, float...) with the
 * parameters in order, and lg_deflection_<name> (lens), lg_brightness_<name>
 * (source) or lg_foreground_<name> (foreground). */
typedef struct {
    const char* name;
    int kind;                   /* LG_LENS / LG_SOURCE / LG_FOREGROUND */
    int npars;
    const char* const* par_names;
    const int* par_types;       /* LG_PARAMETER ... LG_POS_ANGLE */
    const float* par_bounds;    /* npars x {lower, upper}; {0,0} = unbounded */
    const float* par_defaults;  /* npars; > 0 or -0.0 means fixed by default */
    const char* source;
} lg_plugin_desc;

/* ---------------------------------------------------------------- library */
const char* lg_version(void);
int lg_plugin_count(void);
/* Metadata of plugin i (0 <= i < lg_plugin_count()).  Any output may be NULL. */
int lg_plugin_info(int i, const char** name, int* kind, int* npars);
int lg_plugin_param(const char* plugin, int j, const char** name, int* type, float* lower, float* upper,
                    float* defval);
int lg_register_plugin(const lg_plugin_desc* desc);

int lg_quad_rule_count(void);
/* Rule i: name, point count and (if non-NULL) abscissae (size x 2), value
 * weights and error weights, on the unit pixel [-0.5, 0.5]^2. */
int lg_quad_rule_info(int i, const char** name, int* size, double* absc, double* weig, double* errw);

/* Weights: weight_map if given, else gain / (image + offset) with a gain map
 * or a constant gain; then times xweight; then zero where mask != 0
 * (src/lensed.c:436-486, src/data.c:314-330).  Returns the number of
 * zero-weight (masked) pixels, or a negative status. */
long lg_make_weight(const float* image, long n, const float* weight_map, const float* gain, double gain_value,
                    double offset, const float* xweight, const int* mask, float* weight_out);

/* Compose and compile the program for a model without creating a context or
 * touching a GPU (configuration check; usable on machines without a GPU). */
int lg_compile_check(const lg_image_desc* image, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                     char* log, size_t log_size);

/* ---------------------------------------------------------------- context */
/* Replaces get_lensed_cl (src/opencl.c:128-191) + main_program
 * (src/kernel.c:838-879) + the buffer and work-size set-up of
 * src/lensed.c:652-1112. */
lg_ctx* lg_create(const lg_image_desc* image, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                  int* status);
void lg_destroy(lg_ctx* ctx);
const char* lg_last_error(const lg_ctx* ctx);

int lg_npars(const lg_ctx* ctx); /* all parameters */
int lg_ndims(const lg_ctx* ctx); /* free parameters (the sampler's cube) */
/* Parameter i in map order: id "<obj>.<par>", whether it wraps, its bounds. */
int lg_param(const lg_ctx* ctx, int i, const char** id, int* wrap, double* lower, double* upper);
/* Index in object order of the parameter at map position i. */
int lg_pmap(const lg_ctx* ctx, int i);
/* Number of pixels with zero weight (for chi^2 per degree of freedom). */
long lg_masked(const lg_ctx* ctx);

/* Evaluate logL = -chi^2/2 for B parameter vectors (B x npars doubles in map
 * order, host memory) into logL[B] (host).  Replaces one call of the
 * reference's loglike() per vector (src/nested.c:63-115): parameter upload,
 * set_params, render, convolve, chi^2 and its sum.  B <= max_batch. */
int lg_eval_batch(lg_ctx* ctx, const double* params, int B, double* logL);

/* Same with device pointers on a caller stream; returns without
 * synchronising.  With stream = NULL the work runs on the context's own
 * (non-blocking) stream, after the work already queued on the legacy
 * default stream; buffers filled on any other stream must be ready first.
 * Calls on one context run in call order whatever streams they are made on
 * (they share the context's scratch): a call on a caller stream first waits
 * for the context's earlier calls, and later calls wait for it. */
int lg_eval_batch_device(lg_ctx* ctx, const double* d_params, int B, double* d_logL, void* stream);

/* Unit-cube points (B x ndims, host) -> physical parameters via the priors
 * (written to phys, B x npars, if not NULL) and logL[B].  Points whose prior
 * transform leaves the parameter bounds get logL = -inf and phys NaN. */
int lg_eval_cube_batch(lg_ctx* ctx, const double* cube, int B, double* phys, double* logL);

/* The unit-cube evaluation on the GPU with device pointers on a caller
 * stream (NULL: as lg_eval_batch_device), B <= max_batch; returns without
 * synchronising.  The prior transform of src/nested.c:42-61 runs as a
 * kernel (one candidate per thread; unif, norm, delta priors; pseudo-prior
 * parameters at u = 0.5), followed by the likelihood kernels.  d_phys
 * (B x npars, map order, may be NULL) receives the physical parameters;
 * points outside the parameter bounds get logL = -inf.  Calls on one
 * context are ordered as for lg_eval_batch_device. */
int lg_eval_cube_batch_device(lg_ctx* ctx, const double* d_cube, int B, double* d_phys, double* d_logL, void* stream);

/* Render one parameter vector (map order) for output: the model (convolved
 * if there is a PSF), the unconvolved model and the quadrature error
 * estimate (src/nested.c:175-216).  Any output may be NULL. */
int lg_render(lg_ctx* ctx, const double* params, float* model, float* raw, float* error);

/* The reference's result dumper (src/nested.c:175-257): render one
 * parameter vector (map order) and return LG_DUMP_LAYERS images of
 * width x height floats each, in this order, in `layers`
 * (LG_DUMP_LAYERS * width * height floats):
 *   IMG  the model (convolved if there is a PSF),
 *   RES  image - model,
 *   RAW  the unconvolved model,
 *   ERR  relative quadrature error, error / RAW,
 *   WHT  the weight map (0 on masked pixels),
 *   PVL  per-pixel p-value erfc(sqrt(chi2 / 2)), chi2 = WHT * (IMG - image)^2.
 * The per-pixel chi^2 is that of the rendered parameters (the reference
 * reads the per-pixel buffer of its last likelihood evaluation instead). */
#define LG_DUMP_LAYERS 6
extern const char* const lg_dump_names[LG_DUMP_LAYERS]; /* "IMG" .. "PVL" */
int lg_dump(lg_ctx* ctx, const double* params, float* layers);

/* lg_dump followed by lg_write_fits of the six layers under their names:
 * the counterpart of the dumper's write_output (src/data.c:372-391). */
int lg_write_output(lg_ctx* ctx, const double* params, const char* path);

/* FITS writer (no CFITSIO): an empty primary HDU (ORIGIN, DATE) and one
 * 2-D float32 IMAGE extension per layer, EXTNAME = names[i] when names and
 * names[i] are not NULL (src/data.c:129-165).  Errors go to
 * lg_last_error(NULL). */
int lg_write_fits(const char* path, int width, int height, int nlayers, const float* const* layers,
                  const char* const* names);

/* Same into memory (src/data.c:393-419): *size receives the file size; the
 * file is copied to buf when buf is not NULL and capacity >= *size
 * (LG_ERR_INPUT when it is smaller). */
int lg_write_fits_memory(int width, int height, int nlayers, const float* const* layers, const char* const* names,
                         void* buf, size_t capacity, size_t* size);

/* Device times (ms) of the stages of one evaluation of B candidates with
 * device pointers: set_params, render, convolve + chi^2 (0 without a PSF)
 * and a fourth entry that is 0 (the chi^2 sum ends the last stage) -- the
 * counterpart of the reference's --profile table
 * (src/nested.c:21-40, src/profile.c:36-83).  Runs on the context's stream
 * after the work queued on the legacy default stream, and synchronises. */
int lg_eval_profile(lg_ctx* ctx, const double* d_params, int B, double* d_logL, float* stage_ms);

/* Launch shape of the evaluation kernels, as 7 ints: render threads per
 * block, pixels per thread group, quadrature split (threads of a group that
 * share its pixels, each taking every split-th quadrature point; 1 in strict
 * mode), convolution tile width, tile height, outputs per thread, paired
 * rows (0/1).  The counterpart of the reference's work-group sizing
 * (src/lensed.c:866-1047), which queries the device for the render
 * work-group size and halves the convolution tile until it fits local
 * memory.  With LG_FLAG_AUTOTUNE, lg_create compiles candidate shapes in
 * parallel, times them on max_batch candidates drawn from the priors and
 * keeps the fastest render and convolution; the choice is cached per
 * program, device, batch and flags in the process, and in the text file
 * named by the environment variable LG_TUNE_CACHE when it is set.  Results
 * are the same for every shape up to the order of FP64 partial sums, and,
 * with a quadrature split above 1, of the FP32 quadrature sum. */
int lg_launch_shape(const lg_ctx* ctx, int shape[7]);
/* Recompile the evaluation module for a given shape (LG_ERR_INPUT for an
 * invalid one, LG_ERR_UNSUPPORTED when the convolution tile does not fit
 * the device's shared memory). */
int lg_set_launch_shape(lg_ctx* ctx, const int shape[7]);
/* The autotuner's candidates and their render and convolution times ("" if
 * the context was not tuned). */
const char* lg_tune_report(const lg_ctx* ctx);
/* 1 when batches of up to 4 candidates through the host entry points
 * (lg_eval_batch, lg_eval_cube_batch, loglike) take their object data and
 * prior transform from the host (the set module's arithmetic, checked
 * against it byte for byte on sample candidates at lg_create), 0 when they
 * use the set_params kernel (models with registered plugins, or a check
 * that did not match). */
int lg_host_set_active(const lg_ctx* ctx);
/* Without a GPU: the candidate shapes the autotuner would time for a model
 * (up to max_shapes x 7 ints written; returns the count), and a compile
 * check of the model's evaluation module for one shape (like
 * lg_compile_check). */
int lg_tune_candidates(const lg_image_desc* image, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                       int* shapes, int max_shapes);
int lg_compile_check_shape(const lg_image_desc* image, const lg_object_desc* objs, int nobjs, const lg_options* opts,
                           const int shape[7], char* log, size_t log_size);

/* Diagnostic: the paired-ray exp (fn = 0), log (1), square root (2),
 * reciprocal (3), atan (4) or atanh (5) of the fast evaluation modules, or
 * the correctly rounded exp (6), log (7), atan (8) or atanh (9) of the exact
 * modules, applied to x[0..n) on a device (out[i] = f(x[i])). */
int lg_probe_pair_math(int device, int fn, const float* x, int n, float* out);

/* Diagnostic: compares the exact modules' correctly rounded exp (fn = 0),
 * log (1), atan (2) or atanh (3), on ray pairs, or sin (4), cos (5),
 * pow(x, Y[u % 16]) (6: sixteen fixed exponents, those of the EPL lens among
 * them), atan2(x, p) (7) or pow(|x|, p) (8), with p the float of bit pattern
 * u * 0x9E3779B1, one value at a time, with the function evaluated in double
 * and rounded once, for every float x whose bit pattern u lies in [lo, hi)
 * (hi <= 2^32), on a device.  *mismatches receives the number of inputs
 * whose results differ (NaN matches NaN); the first nfirst of their bit
 * patterns go to first. */
int lg_probe_crf_sweep(int device, int fn, unsigned long long lo, unsigned long long hi,
                       unsigned long long* mismatches, unsigned* first, int nfirst);

/* Measured FP32 FMA throughput (TFLOP/s) of a device, for roofline
 * denominators. */
int lg_measure_fp32_peak(int device, double* tflops);

/* Capacity of the static scratch of lg_loglike_images_noalloc, in partial
 * sums (doubles): 512 KiB held on every GPU that loads the library. */
#define LG_NOALLOC_MAX_PARTIALS 65536

/* logL[b] = -chi^2/2 of B model images (d_models: B x n_pixels floats) against
 * one image and weight map (n_pixels floats each), all device pointers, on
 * the given stream (NULL = default stream), returning without synchronising.
 * No counterpart in the reference: it is the likelihood path's chi^2
 * reduction for callers that cannot allocate device memory (a host framework
 * that owns the GPU's memory through its own pool, or code running where new
 * allocations are not allowed).  It allocates nothing: its scratch is a
 * static device array of LG_NOALLOC_MAX_PARTIALS doubles shared by all calls,
 * so calls that overlap on the GPU race and must be serialised by the caller.
 * The first call in a CUDA context (per device, and again after
 * cudaDeviceReset) looks up the array's device address; with CUDA's lazy
 * module loading that first call also loads the library's kernels and places
 * the array, a one-time allocation made by the driver.  A caller that may
 * not allocate at all makes one call at its own set-up time, before any
 * stream capture; later calls allocate nothing.  B is limited to 65535; larger B, null
 * pointers or non-positive sizes return LG_ERR_INPUT (message in
 * lg_last_error(NULL)). */
int lg_loglike_images_noalloc(const float* d_image, const float* d_weight, const float* d_models, long n_pixels,
                              int B, double* d_logL, void* stream);

/* ---------------------------------------------------------------- systems */
/* A batch of lens systems of uneven image and PSF sizes that share the
 * object list (plugins, priors, parameter map) and quadrature rule,
 * evaluated together: one persistent launch per stage over (system,
 * candidate, tile) work units, replayed from one CUDA graph for any per-call
 * candidate counts up to capacity[s].  The counterpart of running one
 * reference process (src/lensed.c) per system. */
typedef struct lg_systems lg_systems;
lg_systems* lg_systems_create(const lg_image_desc* images, int nsys, const lg_object_desc* objs, int nobjs,
                              const lg_options* opts, const int* capacity, int* status);
void lg_systems_destroy(lg_systems* S);
const char* lg_systems_last_error(const lg_systems* S);
int lg_systems_npars(const lg_systems* S);
/* params: counts[0] vectors of system 0, then counts[1] of system 1, ...
 * (npars doubles each, map order); logL receives sum(counts) values in the
 * same order.  Each system's values equal those of its own lg_ctx. */
int lg_systems_eval(lg_systems* S, const double* params, const int* counts, double* logL);
/* Launch shape of the multi-system kernels (the 7 ints of lg_launch_shape;
 * the tile height counts thread rows, a paired-row unit covering two of
 * them per thread, and the paired flag is 0: paired rows are chosen per
 * system).  LG_FLAG_AUTOTUNE at creation times render and convolution
 * candidates with every system at capacity. */
int lg_systems_launch_shape(const lg_systems* S, int shape[7]);
int lg_systems_set_launch_shape(lg_systems* S, const int shape[7]);
const char* lg_systems_tune_report(const lg_systems* S);

/* ------------------------------------------------------- nested sampling */
/* The sampler that replaces MultiNest's role (src/lensed.c:1236-1288):
 * nested sampling over the unit cube with one enlarged bounding ellipsoid
 * (Mukherjee, Parkinson & Liddle 2006), proposals drawn and evaluated in
 * batches, FP64 log-sum-exp evidence; optionally a learned coupling-flow
 * proposal trained on the live points (the ellipsoid stays the fallback). */
#define LG_PROPOSAL_ELLIPSOID 0
#define LG_PROPOSAL_FLOW 1

typedef struct {
    int nlive;      /* live points (reference option nlive) */
    double tol;     /* stop when the live points can raise ln Z by less than tol */
    double efr;     /* ellipsoid volume enlargement factor 1/efr */
    int batch;      /* proposals per batched likelihood call */
    int seed;       /* random seed (-1: from the clock) */
    long maxiter;   /* 0: unlimited */
    int proposal;   /* LG_PROPOSAL_* */
    int flow_every; /* retrain the flow every this many replacements */
    const int* wrap; /* ndims flags or NULL: periodic parameters (the prior keyword "wrap", passed to
                        MultiNest by the reference, src/lensed.c:1254-1275); a proposal outside [0, 1]
                        on such a dimension is wrapped into it instead of rejected.  lg_nested_run takes
                        them from the context's priors when NULL */
    const char* checkpoint; /* state file or NULL: the counterpart of MultiNest's resume files
                               (option resume, src/input/options.c:217-221) */
    int checkpoint_every;   /* write the state every this many iterations (0: only when stopping) */
    int resume;             /* continue from the state file when it exists; an existing file that is
                               not a state of this run (another format version, truncated, another
                               dimension, nlive or batch) is an error (LG_ERR_INPUT), not a fresh
                               start */
    int max_ellipsoids;     /* 1: one bounding ellipsoid (default); more: the multi-ellipsoidal
                               decomposition of MultiNest's multi-modal mode (option mmodal,
                               src/input/options.c), up to this many ellipsoids */
    int ceff;               /* constant efficiency mode (the reference's ceff option, which then
                               passes efr = acc, src/lensed.c:1247-1248): efr is the target fraction
                               of ellipsoid proposals accepted, and the bound's volume adapts to it,
                               below the live points' enclosing volume if need be.  Faster; as in
                               MultiNest the evidence can come out biased.  0 (default): efr is the
                               fixed volume enlargement 1 / efr */
} lg_nested_options;

typedef struct {
    double logz, logz_err, information, max_logl;
    long ncall, niter, nsamples, n_flow_proposals, n_ellipsoid_proposals;
    double wall_s;
    double* mean;          /* ndims, caller-owned, or NULL: posterior means (cube) */
    double* std;           /* ndims, or NULL */
    double* samples;       /* max_samples x ndims, or NULL: dead + final live points */
    double* sample_logwt;  /* max_samples, or NULL: log posterior weights */
    long max_samples;
    /* wall time (s) spent in the likelihood callback, in training the
     * learned proposal and in drawing proposals (ellipsoid or flow) */
    double eval_s, train_s, propose_s;
} lg_nested_result;

/* Learned proposal: affine coupling layers with MLP conditioners, trained by
 * maximum likelihood on the live points with hand-written CUDA kernels. */
typedef struct {
    int layers;     /* coupling layers (default 8) */
    int width;      /* hidden units (default 128) */
    int hidden;     /* hidden layers per conditioner (default 2) */
    int epochs;     /* epochs of the first training (default 200); later retrainings start from the
                       previous weights with an eighth of them */
    int batch;      /* training batch (default 256) */
    double lr;      /* Adam learning rate (default 1e-3) */
    double expand;  /* volume enlargement of the latent ball through the farthest live point
                       (default 1.25, as the plain sampler's 1 / efr) */
    int patience;   /* epochs without held-out improvement before a retraining stops (default 4) */
    int lag;        /* replacements after a retraining starts at which the new flow takes over
                       (default 800): the retraining runs on its own stream meanwhile, and the
                       sampler waits for it there if it has not finished */
    double draw_cost; /* cost of one latent draw of the flow in likelihood calls (default 0.005, a
                         128^2 image with a 9-point rule): the flow is used when its volume times
                         1 + draw_cost x latent draws per proposal is below the ellipsoids' volume;
                         0 for expensive likelihoods.  A fixed number, so that runs repeat */
    int wait_tries;   /* polls of each bounded wait of the tensor-core kernels (inverse and
                         training step) before it gives up (0: the default 2^20; negative: none --
                         every wait gives up at once, which exercises the timeout path: the kernel
                         flags the error, lets its own copies and tensor-core work in flight
                         complete, frees its tensor memory and returns, and the sampler drops that
                         flow) */
    int train_tc;     /* 1: training steps on the tensor cores (lg_flow_step_tc: BF16 weights,
                         conditioner inputs and activations, FP32 accumulators in tensor memory)
                         when the shape allows it (width 128, two hidden layers, d <= 16, sm_100+);
                         0 (default): the FP32-weight training kernels (BF16 activations) */
} lg_flow_options;

typedef int (*lg_batch_loglike)(void* user, const double* cube, int B, double* logL);

lg_nested_options lg_nested_defaults(void);
lg_flow_options lg_flow_defaults(void);
int lg_nested_sample(int ndims, lg_batch_loglike fn, void* user, const lg_nested_options* opts,
                     lg_nested_result* result);
/* Loss and gradient of a flow with the given parameters on n points
 * (standardised coordinates), for gradient checks: bf16 = 0 the FP32
 * training kernel with FP32 hidden activations, 1 the same with BF16 hidden
 * activations, 2 the tensor-core training step (lg_flow_options.train_tc). */
long lg_flow_nparams(int d, int layers, int width, int hidden);
int lg_flow_loss_grad(int device, int d, int layers, int width, int hidden, int bf16, const float* params,
                      const float* x, int n, float* loss, float* grad);
/* Inverse flow of M latent points (M x d) with the given parameters: tc = 1
 * the tensor-core kernel of the proposals (BF16 weights and activations,
 * FP32 accumulation; width a multiple of 32), tc = 0 the FP32-weight kernel
 * (bf16 = 1: BF16 hidden activations).  u: M x d standardised points,
 * ldet: log |det du/dz|.  For checks against the CPU restatement. */
int lg_flow_inverse_check(int device, int d, int layers, int width, int hidden, int bf16, int tc,
                          const float* params, const float* z, int M, float* u, float* ldet);

/* Device time of the inverse flow (lg_flow_inverse_check's arguments; z
   uploaded once): reps launches after two warm-up launches, timed with CUDA
   events on the launching stream; *ms = milliseconds per launch. */
int lg_flow_inverse_time(int device, int d, int layers, int width, int hidden, int tc, const float* params,
                         const float* z, int M, int reps, float* ms);
/* Device time of flow training steps (forward + backward of `batch` rows
   of the n points, then the Adam step): tc = 1 the tensor-core step, 0 the
   FP32-weight step (BF16 activations); reps steps after two warm-up steps,
   CUDA events on the launching stream; *ms = milliseconds per step. */
int lg_flow_train_time(int device, int d, int layers, int width, int hidden, int tc, const float* params,
                       const float* x, int n, int batch, int reps, float* ms);
/* One retraining of the learned proposal on n points (n x d, row-major),
 * as the sampler does it on its live points: history receives the held-out
 * loss before training and after each epoch (NaN past the last epoch run);
 * returns the epochs run (negative: error; LG_ERR_TIMEOUT when a bounded
 * wait of the tensor-core training step or of the calibration's
 * tensor-core inverse ran out, see wait_tries; lg_last_error says which);
 * *efficiency = calibrated kept fraction of latent draws. */
int lg_flow_fit(int device, int d, const lg_flow_options* opts, const double* pts, int n, float* history,
                int max_history, double* efficiency);
/* The sampler's GPU draws uniform in a union of nell ellipsoids (and the
 * unit cube; periodic dimensions, wrap[a] != 0, wrapped): packed holds per
 * ellipsoid its centre (d), lower Cholesky factor of the covariance (d x d,
 * row-major) and scale (the ellipsoid is (x - mu)^T C^-1 (x - mu) <= scale),
 * logv their log volumes.  Returns the number of points written (<= B). */
int lg_ellipsoid_draw_check(int device, int d, int nell, const double* packed, const double* logv, const int* wrap,
                            double* out, int B, unsigned long long seed);
/* lg_nested_sample with the learned proposal on the given CUDA device. */
int lg_nested_sample_flow(int ndims, lg_batch_loglike fn, void* user, const lg_nested_options* opts,
                          const lg_flow_options* flow, int device, lg_nested_result* result);
/* Nested sampling of a context's posterior (cube -> priors -> GPU logL). */
int lg_nested_run(lg_ctx* ctx, const lg_nested_options* opts, const lg_flow_options* flow,
                  lg_nested_result* result);

/* Drop-in for the reference's likelihood callback (src/nested.h:3): ctx is
 * an lg_ctx*.  cube[0..ndim) holds unit-cube values and is overwritten with
 * the physical values of all npar parameters (map order); *lnew receives
 * logL.  On failure *lnew is -inf and lg_last_error() says why. */
void loglike(double cube[], int* ndim, int* npar, double* lnew, void* ctx);

#ifdef __cplusplus
}
#endif

#endif /* LENSED_GB300_H */
