// gf_hydro.cuh — the fused, device-resident force evaluation (simulation.py:61-95).
#pragma once

#include <cstring>
#include <initializer_list>

#include "gf_sph.cuh"

namespace gf {

struct HydroScalars {
    int ng;                          // gas particles of the last hydro call
    int fail;                        // Verlet reselection impossible
    unsigned long long amax_bits;    // max |a| (float64 bits, non-negative)
    unsigned long long dtmin_bits;   // min Courant step of the gas (float64 bits)
    unsigned long long knn_iters;    // search-radius iterations of the last full search
    int nact;                        // gas due in a partial (block time-step) call
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
    // block time steps: SPH recomputed only for the gas flagged here (others keep their last
    // density, forces and Courant step); null = all gas, as in the reference
    const uint8_t* sph_active = nullptr;
    // no host synchronisation (for CUDA-graph capture): gas set, neighbour cache and tree are
    // those of the last regular call; gravity refits with device-side node counts
    int nosync = 0;
    // walk work items of <= walk_chunk active particles with their own spheres (0: the
    // reference's groups); used with an active set
    int walk_chunk = 0;
    int walk_npl = 2;  // mixed walk: nodes per lane and round (2, or 8 for walks of a few items)
    int walk_shape = -1;  // mixed walk's launch shape (kNumWalkShapes); -1: the engine's option
    // vel and u may still be arriving (copies on another stream): the hydro chain waits for
    // this event before it reads them; the gravity chain does not need them
    cudaEvent_t late_inputs = nullptr;
};

struct ForceEngine {
    // options (gf_set_option)
    int sph_float32 = 0;     // 1: mixed-precision SPH (float32 + Kahan), 0: float64
    int gravity_quad = 0;    // 1: quadrupole moments + Kahan tile sums, 0: the reference's monopole
    int walk_chunk = 0;      // walk items for active-set walks (0: the reference's groups)
    int walk_group = 64;     // mixed form: walk groups = shallowest nodes with <= this many particles
    int walk_merge = 0;      // mixed form: walk items = runs of consecutive sibling groups of <= this
                             // many particles (0: one item per group)
    int walk_shape = 0;      // mixed form: launch shape of the walk (block warps x tile size)
    // mixed form: relative opening criterion with this tolerance (0 = the geometric criterion
    // at the caller's theta). It takes the gravity of the previous evaluation of the same
    // particle set as the error scale: the first evaluation (and every one before an
    // evaluation of all particles) uses the geometric criterion; later ones a geometric floor
    // at theta = kRelFloorTheta combined with the relative test.
    double grav_rel = 0.0;
    double grav_rel_mono = 0.0;  // accepted nodes with quadrupole term below this x a_min: monopoles
    bool have_aold = false;
    static constexpr double kRelFloorTheta = 1.0;
    int hguess = 0;          // start of the neighbour-count iteration: 0 previous h, 1 cell
                             // density only, 2 the learned guess (MLP)
    long long collect_cap = 0, collect_n = 0;  // (features, log d48) training pairs kept
    bool have_divv = false;
    int n_total = -1;
    int order_ng = -1;       // gas count of the last full neighbour search
    int ng = 0, ng_valid = 0;
    bool cache_valid = false, have_hprev = false;
    const int* last_nb = nullptr;  // neighbour rows (48 columns, the 32 nearest first) of the last hydro call
    long long full_searches = 0, verlet_hits = 0;
    Octree grav;             // gravity tree of the fused path
    Octree knn_tree;
    SphScratch sph;
    Sph32Scratch sph32;
    DevBuf acc_grav, acc_sph, dt_courant, h_prev, row, loc, cache, cgidx;
    DevBuf flag, scan, gidx, gpos, gvel, gmass, gu_, nb48, dsel, rguess, h, rho, gacc, dudt, dt_i;
    DevBuf scalars;
    DevBuf divv_prev, gdivv, hX, hY, hrg, hdk, colX, colT, ghi, glo, vsel, aflag, ascan, alist;
    ScanScratch hscratch;    // scans of the hydro stream
    cudaStream_t s2 = nullptr;               // the hydro chain's stream
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaStream_t s3 = nullptr;               // a refit's moments, beside the walk items
    cudaEvent_t ev_gathered = nullptr, ev_moments = nullptr;
    HydroScalars* scalars_h = nullptr;  // pinned copy, valid after the stream synchronises

    void evaluate(const ForceArgs& a, cudaStream_t s);
    // The options a captured evaluation bakes in: a graph captured under other values is stale.
    unsigned long long option_key() const {
        unsigned long long rel_bits;
        memcpy(&rel_bits, &grav_rel, sizeof rel_bits);
        unsigned long long k = 1469598103934665603ull;
        for (unsigned long long v : {(unsigned long long)sph_float32, (unsigned long long)gravity_quad,
                                     (unsigned long long)walk_chunk, (unsigned long long)walk_group,
                                     (unsigned long long)hguess, rel_bits, (unsigned long long)have_aold,
                                     (unsigned long long)walk_merge, (unsigned long long)(grav_rel_mono * 1e12),
                                     (unsigned long long)walk_shape})
            k = (k ^ v) * 1099511628211ull;
        return k;
    }
    // allocates the buffers that only synchronisation-free evaluations touch
    // every buffer a captured (synchronisation-free) evaluation touches, at its final size
    void reserve_nosync(int n) {
        grav.reserve_graph_build();
        reserve_scan_sort(n, &hscratch);
        if (ng > 0) {
            aflag.get<int>(ng);
            ghi.get<float4>(ng);
            glo.get<float4>(ng);
            vsel.get<int>(ng);
            ascan.get<int>(ng);
            alist.get<int>(ng);
        }
    }
    void hydro(const ForceArgs& a, cudaStream_t s);
    // Autotuner of the mixed walk of full evaluations: on the tree and error scale of the last
    // evaluation, times the walk for each item size (merge cap) and launch shape and keeps the
    // fastest as walk_merge / walk_shape.
    void autotune_walk(double eps, cudaStream_t s, int* merge_out, int* shape_out, double* ms_out);
    DevBuf tune_acc;
};

ForceEngine& force_engine();

// Device-resident step loop (gf_sim.cu).
void sim_init(int n, const double* pos, const double* vel, const double* mass, const int8_t* kind, const double* u,
              double theta, double eps, double gamma, double alpha, double beta);
double sim_step(double dt_max, int* substeps);
void block_config(const int* chunk, int nbins, int rebuild_every);
void block_autotune(int nlev, int* chunk, int* rebuild_every, double* graph_ms);
double sim_updates();
void sim_read(double* pos, double* vel, double* acc, double* dt_ind, double* t);
void sim_read_u(double* u);
// t, dt_grav, dt_gas of the step loop
void sim_scalars(double* out);
// overwrites the integrator state after sim_init of a saved particle set (exact resume):
// accelerations and time-step limits of the last evaluations, times, bubble times
void sim_restore(const double* acc, const double* dt_ind, const double* birth, const double* no_cool,
                 const double* rho, const double* dudt, double t, double dt_grav, double dt_gas);
// density and du/dt of the last SPH evaluation, per particle (NaN outside its gas set)
void sim_read_hydro(double* rho, double* dudt);
// thermal update of the step loop: mode 0 off, 1 heating/compression, 2 also cooling;
// units: the 8 constants of ThermoUnits (gf_thermo.cuh), in its order
void sim_thermo(int mode, const double* units);
// star formation + supernova feedback after every step and sub-step of sim_step: params = the
// 10 values of StarParams (gf_stars.cuh) in its order; rng_words = NumPy PCG64 state
// (state high, state low, increment high, increment low)
void sim_stars(int on, const double* params, const unsigned long long* rng_words);
// copies kind, birth, no_cool (n each) and the PCG64 words out (any may be null); returns the
// number of stars formed since sim_init
long long sim_read_stars(int8_t* kind, double* birth, double* no_cool, unsigned long long* rng_words);
void sim_diagnostics(double theta, double* out);
// Block time steps (the batched form): advances nblocks blocks of 2^(nlev-1) sub-steps;
// returns the particle-updates done.
double block_run(int nblocks, int nlev);
bool simulation_ready();
void block_levels(int nlev, double* frac);

}  // namespace gf
