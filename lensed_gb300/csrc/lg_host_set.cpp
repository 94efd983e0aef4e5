// set_params on the host, for batches of a few candidates.
//
// One candidate's object data take 12-15 us on the GPU: the set module
// evaluates its elementary functions in FP64 (rounded once to FP32, the
// oracle's semantics), GB300 runs FP64 at a small fraction of its FP32 rate,
// and one thread per object walks a dependent chain of them.  The host's
// FP64 is fast, so for a handful of candidates the object data are computed
// here and copied to the GPU with the launch.
//
// The code is the plugins' own (lensed_gb300/objects/*.cuh and the scalar
// part of device/lg_prelude.cuh, compiled for the host with LG_HOST_SET):
// the same IEEE single-precision operations in the same order, no FMA
// contraction (the build passes -ffp-contract=off, as the set module is
// compiled with --fmad=false), IEEE division and square root, and the float
// elementary functions routed to FP64 evaluation rounded once
// (device/lg_crmath_on.cuh).  The FP64 functions are the host C library's
// instead of CUDA's; both are within an ulp of the exact value, so their
// roundings to FP32 agree except when the exact value lies within about
// 2^-29 of a rounding boundary.  The context checks both paths on sample
// candidates before it uses this one.
//
// The composition follows the generated set_params (src/kernel.c:401-656 and
// lg_program.cpp: emit_set_params): objects in model order, objects whose
// positions carry image-plane priors deflected through the lenses of the
// earlier planes first.

#include <cuda_runtime.h>  // float2, make_float2 (host functions)

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "lg_internal.h"

// the plugins' device loop hints mean nothing here
#pragma GCC diagnostic ignored "-Wunknown-pragmas"

namespace lg {
namespace hostset {

#define LG_HOST_SET 1
#include "../device/lg_prelude.cuh"
#include "../device/lg_crmath_on.cuh"
#include "../objects/sis.cuh"
#include "../objects/sis_plus_shear.cuh"
#include "../objects/nsis.cuh"
#include "../objects/sie.cuh"
#include "../objects/sie_plus_shear.cuh"
#include "../objects/nsie.cuh"
#include "../objects/point_mass.cuh"
#include "../objects/epl.cuh"
#include "../objects/epl_plus_shear.cuh"
#include "../objects/sersic.cuh"
#include "../objects/sersic_old.cuh"
#include "../objects/exponential.cuh"
#include "../objects/devauc.cuh"
#include "../objects/gauss.cuh"
#include "../objects/sky.cuh"

// A built-in plugin's data size and alignment, its set function (arguments
// in parameter order) and, for lenses, its deflection of one ray.
struct HostPlugin {
    const char* name;
    size_t size, align;
    void (*set)(void* o, const float* a);
    float2 (*deflect)(const void* o, float2 x);
};

#define LG_HP_DATA(N) sizeof(lg_data_##N), alignof(lg_data_##N)
#define LG_HP_DEFLECT(N) [](const void* o, float2 x) { return lg_deflection_##N(static_cast<const lg_data_##N*>(o), x); }

const HostPlugin kPlugins[] = {
    {"sis", LG_HP_DATA(sis), [](void* o, const float* a) { lg_set_sis(static_cast<lg_data_sis*>(o), a[0], a[1], a[2]); },
     LG_HP_DEFLECT(sis)},
    {"sis_plus_shear", LG_HP_DATA(sis_plus_shear),
     [](void* o, const float* a) {
         lg_set_sis_plus_shear(static_cast<lg_data_sis_plus_shear*>(o), a[0], a[1], a[2], a[3], a[4]);
     },
     LG_HP_DEFLECT(sis_plus_shear)},
    {"nsis", LG_HP_DATA(nsis),
     [](void* o, const float* a) { lg_set_nsis(static_cast<lg_data_nsis*>(o), a[0], a[1], a[2], a[3]); },
     LG_HP_DEFLECT(nsis)},
    {"sie", LG_HP_DATA(sie),
     [](void* o, const float* a) { lg_set_sie(static_cast<lg_data_sie*>(o), a[0], a[1], a[2], a[3], a[4]); },
     LG_HP_DEFLECT(sie)},
    {"sie_plus_shear", LG_HP_DATA(sie_plus_shear),
     [](void* o, const float* a) {
         lg_set_sie_plus_shear(static_cast<lg_data_sie_plus_shear*>(o), a[0], a[1], a[2], a[3], a[4], a[5], a[6]);
     },
     LG_HP_DEFLECT(sie_plus_shear)},
    {"nsie", LG_HP_DATA(nsie),
     [](void* o, const float* a) { lg_set_nsie(static_cast<lg_data_nsie*>(o), a[0], a[1], a[2], a[3], a[4], a[5]); },
     LG_HP_DEFLECT(nsie)},
    {"point_mass", LG_HP_DATA(point_mass),
     [](void* o, const float* a) { lg_set_point_mass(static_cast<lg_data_point_mass*>(o), a[0], a[1], a[2]); },
     LG_HP_DEFLECT(point_mass)},
    {"epl", LG_HP_DATA(epl),
     [](void* o, const float* a) { lg_set_epl(static_cast<lg_data_epl*>(o), a[0], a[1], a[2], a[3], a[4], a[5]); },
     LG_HP_DEFLECT(epl)},
    {"epl_plus_shear", LG_HP_DATA(epl_plus_shear),
     [](void* o, const float* a) {
         lg_set_epl_plus_shear(static_cast<lg_data_epl_plus_shear*>(o), a[0], a[1], a[2], a[3], a[4], a[5], a[6],
                               a[7]);
     },
     LG_HP_DEFLECT(epl_plus_shear)},
    {"sersic", LG_HP_DATA(sersic),
     [](void* o, const float* a) {
         lg_set_sersic(static_cast<lg_data_sersic*>(o), a[0], a[1], a[2], a[3], a[4], a[5], a[6]);
     },
     nullptr},
    {"sersic_old", LG_HP_DATA(sersic_old),
     [](void* o, const float* a) {
         lg_set_sersic_old(static_cast<lg_data_sersic_old*>(o), a[0], a[1], a[2], a[3], a[4], a[5], a[6]);
     },
     nullptr},
    {"exponential", LG_HP_DATA(exponential),
     [](void* o, const float* a) {
         lg_set_exponential(static_cast<lg_data_exponential*>(o), a[0], a[1], a[2], a[3], a[4], a[5]);
     },
     nullptr},
    {"devauc", LG_HP_DATA(devauc),
     [](void* o, const float* a) {
         lg_set_devauc(static_cast<lg_data_devauc*>(o), a[0], a[1], a[2], a[3], a[4], a[5]);
     },
     nullptr},
    {"gauss", LG_HP_DATA(gauss),
     [](void* o, const float* a) { lg_set_gauss(static_cast<lg_data_gauss*>(o), a[0], a[1], a[2], a[3], a[4], a[5]); },
     nullptr},
    {"sky", LG_HP_DATA(sky), [](void* o, const float* a) { lg_set_sky(static_cast<lg_data_sky*>(o), a[0], a[1], a[2]); },
     nullptr},
};

#undef LG_HP_DATA
#undef LG_HP_DEFLECT

void deflect(float2& y, float2 a) { lg_deflect(y, a); }

}  // namespace hostset

HostSetLayout host_set_layout(const Model& m)
{
    HostSetLayout L;
    size_t off = 0, maxal = 1;
    for (const ObjectInfo& ob : m.objs) {
        int k = -1;
        if (ob.plugin && ob.plugin->builtin)
            for (int i = 0; i < (int)(sizeof hostset::kPlugins / sizeof hostset::kPlugins[0]); ++i)
                if (ob.plugin->name == hostset::kPlugins[i].name) k = i;
        if (k < 0) return HostSetLayout{};  // a registered plugin: device code only
        const hostset::HostPlugin& hp = hostset::kPlugins[k];
        if (ob.plugin->pars.size() > 16 || (ob.plugin->kind == LG_LENS && !hp.deflect)) return HostSetLayout{};
        // members of struct lg_model { lg_data_<plugin> o0, o1, ...; }
        off = (off + hp.align - 1) / hp.align * hp.align;
        L.offset.push_back(off);
        L.index.push_back(k);
        off += hp.size;
        maxal = std::max(maxal, hp.align);
    }
    L.bytes = std::max<size_t>((off + maxal - 1) / maxal * maxal, 1);
    L.ok = true;
    return L;
}

void host_set_params(const Model& m, const HostSetLayout& L, const double* params, unsigned char* out)
{
    std::memset(out, 0, L.bytes);
    // parameter upload order: p[pmap[i]] = params[i] (src/nested.c:70-71)
    std::vector<float> p(m.pars.size());
    for (size_t i = 0; i < m.pmap.size(); ++i) p[m.pmap[i]] = (float)params[i];
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
        float2 x = make_float2(0.0f, 0.0f);
        if (ob.ipp) {
            // the image-plane position, deflected through the lenses of the
            // earlier planes
            int xp = -1;
            for (int j = 0; j < np; ++j)
                if (m.pars[ob.par0 + j].prior.ipp && pl->pars[j].type == LG_POSITION_X) xp = j;
            x = make_float2(p[ob.par0 + xp], p[ob.par0 + xp + 1]);
            float2 a = make_float2(0.0f, 0.0f);
            int trigger2 = 0;
            for (size_t k = 0; k < plane; ++k) {
                const Plugin* q = m.objs[k].plugin;
                if (q->kind != trigger2 && q->kind != LG_FOREGROUND) {
                    if (trigger2 == LG_LENS) {
                        hostset::deflect(x, a);
                        a = make_float2(0.0f, 0.0f);
                    }
                    trigger2 = q->kind;
                }
                if (q->kind == LG_LENS) {
                    const float2 d = hostset::kPlugins[L.index[k]].deflect(out + L.offset[k], x);
                    a = make_float2(a.x + d.x, a.y + d.y);
                }
            }
            if (trigger2 == LG_LENS) hostset::deflect(x, a);
        }
        float args[16];
        for (int j = 0; j < np; ++j) {
            const ParamInfo& pi = m.pars[ob.par0 + j];
            if (ob.ipp && pi.prior.ipp)
                args[j] = pl->pars[j].type == LG_POSITION_X ? x.x : (pl->pars[j].type == LG_POSITION_Y ? x.y : 0.0f);
            else
                args[j] = p[ob.par0 + j];
        }
        hostset::kPlugins[L.index[i]].set(out + L.offset[i], args);
    }
}

}  // namespace lg
