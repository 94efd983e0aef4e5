// set_params module: compiled separately, without FMA contraction and with
// the double-evaluated elementary functions, so the object data of every
// candidate are the IEEE single-precision values of the plugin formulas.

// ------------------------------------------------------------ set_params --
// One thread per candidate: physical parameters (pmap order, double) ->
// object data.  src/nested.c:67-77 and the generated set_params of
// src/kernel.c:114-150.
extern "C" __global__ void lg_set_params_kernel(const double* __restrict__ params, int B,
                                                lg_model* __restrict__ models)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float p[LG_NPARS];
    lg_load_params(params + (size_t)b * LG_NPARS, p);
    lg_model m;
    memset(&m, 0, sizeof m);  // padding included: object data compare byte for byte
    lg_set_params(m, p);
    models[b] = m;
}

// Small batches: one block per candidate and one warp per object, so that
// the objects' data (each computed by one thread, with the same arithmetic
// as above) are computed side by side; objects whose positions carry
// image-plane priors follow in a second phase, once the lenses they are
// deflected through are set.
extern "C" __global__ void lg_set_params_split(const double* __restrict__ params, int B,
                                               lg_model* __restrict__ models)
{
    __shared__ lg_model m;
    __shared__ float p[LG_NPARS > 0 ? LG_NPARS : 1];
    const int b = blockIdx.x;
    if (b >= B) return;
    const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
    static_assert(sizeof(lg_model) % 4 == 0, "object data are 32-bit words");
    for (int i = threadIdx.x; i < (int)(sizeof(lg_model) / 4); i += blockDim.x) reinterpret_cast<unsigned*>(&m)[i] = 0;
    if (threadIdx.x == 0) lg_load_params(params + (size_t)b * LG_NPARS, p);
    __syncthreads();
    if (lane == 0 && w < LG_NOBJ && lg_obj_phase[w] == 0) lg_set_object(m, p, w);
    __syncthreads();
    if (lane == 0 && w < LG_NOBJ && lg_obj_phase[w] == 1) lg_set_object(m, p, w);
    __syncthreads();
    const unsigned* src = reinterpret_cast<const unsigned*>(&m);
    unsigned* dst = reinterpret_cast<unsigned*>(models + b);
    for (int i = threadIdx.x; i < (int)(sizeof(lg_model) / 4); i += blockDim.x) dst[i] = src[i];
}

extern "C" __device__ const unsigned lg_model_bytes = sizeof(lg_model);
extern "C" __device__ const int lg_model_objects = LG_NOBJ;
