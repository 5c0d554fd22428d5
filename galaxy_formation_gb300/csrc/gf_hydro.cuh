// gf_hydro.cuh — the fused, device-resident force evaluation (simulation.py:61-95).
#pragma once

#include "gf_sph.cuh"

namespace gf {

struct HydroScalars {
    int ng;                          // gas particles of the last hydro call
    int fail;                        // Verlet reselection impossible
    unsigned long long amax_bits;    // max |a| (float64 bits, non-negative)
    unsigned long long dtmin_bits;   // min Courant step of the gas (float64 bits)
    unsigned long long knn_iters;    // search-radius iterations of the last full search
    double dt_grav, dt_gas;
};

struct ForceArgs {
    int n;
    const double* pos;
    const double* vel;
    const double* mass;
    const int8_t* kind;
    const double* u;
    double theta, eps, gamma, alpha, beta;
    const uint8_t* active;
    int rebuild, sph, fresh_nb;
    double* acc;     // (n,3) out
    double* dt_ind;  // (n,) out
};

struct ForceEngine {
    int n_total = -1;
    int ng = 0, ng_valid = 0;
    bool cache_valid = false, have_hprev = false;
    long long full_searches = 0, verlet_hits = 0;
    Octree knn_tree;
    SphScratch sph;
    DevBuf acc_grav, acc_sph, dt_courant, h_prev, row, loc, cache;
    DevBuf flag, scan, gidx, gpos, gvel, gmass, gu_, nb48, dsel, rguess, h, rho, gacc, dudt, dt_i;
    DevBuf scalars;
    HydroScalars* scalars_h = nullptr;  // pinned copy, valid after the stream synchronises

    void evaluate(const ForceArgs& a, cudaStream_t s);
    void hydro(const ForceArgs& a, cudaStream_t s);
};

ForceEngine& force_engine();

}  // namespace gf
