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
    lg_set_params(m, p);
    models[b] = m;
}

extern "C" __device__ const unsigned lg_model_bytes = sizeof(lg_model);
