// Internal interface between the nested sampler and its learned proposal.
#pragma once

#include <cmath>
#include <cstdint>
#include <string>

#include "lensed_gb300.h"

namespace lg {

// xoshiro256** (Blackman & Vigna 2018) seeded by splitmix64.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed)
    {
        uint64_t z = seed + 0x9E3779B97F4A7C15ull;
        for (auto& v : s) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            v = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next()
    {
        const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    double normal()
    {
        // Marsaglia polar method
        double u, v, q;
        do {
            u = 2 * uniform() - 1;
            v = 2 * uniform() - 1;
            q = u * u + v * v;
        } while (q >= 1 || q == 0);
        return u * std::sqrt(-2 * std::log(q) / q);
    }
};


// A proposal that learns the constrained prior from the live points.
// propose() fills up to B points (unit cube, row-major) that are uniform
// within its region and returns how many; 0 or less means "not usable".
struct Proposal {
    virtual ~Proposal() {}
    virtual int train(const double* live, int n, int d) = 0;
    virtual int propose(const double* live, int n, int d, double* out, int B, uint64_t seed) = 0;
    // called before every replacement with the replacements made since the
    // last train(): a proposal that trains in the background switches to
    // its new state at a fixed count, so that runs are reproducible
    virtual void advance(long since_train) { (void)since_train; }
    // called every nlive / 10 replacements with the live points: a learned
    // bound can follow the shrinking constrained region between trainings
    virtual void refresh(const double* live, int n, int d) { (void)live, (void)n, (void)d; }
    // periodic dimensions: proposals are wrapped into [0, 1) there
    virtual void set_wrap(const int* wrap, int d) { (void)wrap, (void)d; }
    // log volume (unit-cube coordinates) of the region propose() draws from
    virtual double log_volume() const = 0;
    // log of the cost of one of its proposals in likelihood calls (>= 0:
    // the call itself plus drawing it); the sampler weighs volumes by it
    virtual double log_cost() const { return 0.0; }
};

// Uniform draws in a union of ellipsoids (and the unit cube, periodic
// dimensions wrapped) on the GPU (lg_propose.cu).  packed: per ellipsoid its
// centre (d), lower Cholesky factor (d x d) and scale; logv: log volumes.
// Returns the number of points written to out (up to B), negative on error.
struct EllipsoidDrawer {
    virtual ~EllipsoidDrawer() {}
    virtual int draw(int d, int nell, const double* packed, const double* logv, const int* wrap, double* out,
                     int B, uint64_t seed) = 0;
};
EllipsoidDrawer* make_gpu_ellipsoid_drawer(int device, std::string& err);

int nested_sample(int nd, lg_batch_loglike fn, void* user, const lg_nested_options* o, lg_nested_result* res,
                  Proposal* learned, std::string& err, EllipsoidDrawer* drawer = nullptr);

// Affine-coupling flow proposal trained and run on the GPU (lg_flow.cu).
Proposal* make_flow_proposal(int device, int d, const lg_flow_options* opts, std::string& err);

}  // namespace lg
