// gf_sim.cu — the hierarchical kick-drift-kick step of GalaxyFormation.step
// (galaxy_formation/simulation.py:114-149), device-resident, without the sub-grid physics
// hooks (_thermodynamics, _stars), which sit outside the force path.
//
// One long step D = min(dt_max, 10th percentile of dt_ind): when D <= 1.5 dt_min a global
// step; otherwise the slow particles (dt_ind >= D, not gas) get one opening and one closing
// half-kick of D, and the fast ones sub-step with dt = min(dt_ind[fast], D - tau), every
// particle drifting, forces on a refitted tree with Verlet-list neighbours; the long step
// closes with a rebuilt tree and gravity of the slow particles. Positions, velocities and
// kicks are float64 on the device; the percentile and the minima are computed on the
// device, and only those scalars cross to the host, as the reference's host loop needs them.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gf_hydro.cuh"
#include "gf_stars.cuh"
#include "gf_thermo.cuh"

namespace gf {

namespace {

constexpr int kThreads = 256;

__global__ void k_kick(int n, double* __restrict__ vel, const double* __restrict__ acc,
                       const uint8_t* __restrict__ mask, double h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (mask && !mask[i])) return;
    for (int c = 0; c < 3; ++c) vel[3 * size_t(i) + c] += h * acc[3 * size_t(i) + c];
}

__global__ void k_set(int n, double* __restrict__ a, double v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

__global__ void k_drift(int n, double* __restrict__ pos, const double* __restrict__ vel, double dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < 3; ++c) pos[3 * size_t(i) + c] += dt * vel[3 * size_t(i) + c];
}

// fast = dt_ind < D or gas; slow = the rest (simulation.py:129-130)
__global__ void k_split(int n, const double* __restrict__ dt_ind, const int8_t* __restrict__ kind, double D,
                        uint8_t* __restrict__ fast, uint8_t* __restrict__ slow) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool f = dt_ind[i] < D || kind[i] == 0;
    fast[i] = f;
    slow[i] = !f;
}

__global__ void k_keys_of(int n, const double* __restrict__ v, uint64_t* __restrict__ key, int* __restrict__ val) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = uint64_t(__double_as_longlong(v[i]));  // dt_ind > 0: bit order = value order
    val[i] = i;
}

__global__ void k_count_forced(int n, const uint8_t* __restrict__ active, const int8_t* __restrict__ kind, int sph,
                               unsigned long long* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool f = i < n && (active[i] || (sph && kind[i] == 0));
    const unsigned m = __ballot_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

__global__ void k_masked_min(int n, const double* __restrict__ v, const uint8_t* __restrict__ mask,
                             unsigned long long* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double m = INFINITY;
    if (i < n && (!mask || mask[i])) m = v[i];
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m < INFINITY) atomicMin(out, (unsigned long long)__double_as_longlong(m));
}

}  // namespace

struct Simulation {
    int n = 0;
    double t = 0, theta = 0.7, eps = 0, gamma = 5.0 / 3.0, alpha = 1, beta = 2;
    double dt_grav = 0, dt_gas = INFINITY;
    int last_substeps = 0;
    double updates = 0;  // particle-updates of the last step (forces computed)
    DevBuf pos, vel, acc, mass, kind, u, dt_ind, fast, slow, keys, keys_alt, vals, vals_alt, scal;
    unsigned long long* h_scal = nullptr;
    // thermal update at the start of every (sub-)step (simulation.py:97-104): 0 off, 1 the
    // compression / shock-heating update of u, 2 also radiative cooling (cooling.py)
    int thermo_mode = 0;
    ThermoUnits thermo_units{};
    // star formation and supernova feedback after every (sub-)step (simulation.py:106-110)
    bool stars_on = false;
    StarParams star_params{};
    DevBuf birth, no_cool, rng;   // per particle: birth time, end of the bubble; Pcg64
    long long stars_formed = 0;

    cudaStream_t s() const { return ctx().stream; }

    // _thermodynamics(dt): on the gas of the last SPH evaluation, with its du/dt and density
    void thermo(double dt) {
        if (!thermo_mode) return;
        ForceEngine& F = force_engine();
        if (F.ng_valid <= 0) return;  // rho_gas.size == 0 (simulation.py:99)
        thermo_gas(F.ng_valid, F.gidx.as<int>(), F.rho.as<double>(), F.dudt.as<double>(), u.as<double>(), dt,
                   thermo_mode, no_cool.as<double>(), t, thermo_units, s());
    }

    // _stars(dt) at the current time
    void stars(double dt) {
        if (!stars_on) return;
        ForceEngine& F = force_engine();
        if (F.ng_valid <= 0) return;  // rho_gas.size == 0 (simulation.py:107)
        stars_formed += form_stars_and_feedback(n, F.ng_valid, F.gidx.as<int>(), F.rho.as<double>(),
                                                pos.as<double>(), mass.as<double>(), kind.as<int8_t>(),
                                                u.as<double>(), birth.as<double>(), no_cool.as<double>(), dt, t,
                                                star_params, rng.as<Pcg64>(), s());
    }

    void accelerations(const uint8_t* active, int rebuild, int sph, int fresh) {
        if (active) {  // particles receiving new forces: the active ones, plus the gas under SPH
            unsigned long long* d = scal.get<unsigned long long>(2);
            GF_CUDA(cudaMemsetAsync(d + 1, 0, sizeof(unsigned long long), s()));
            k_count_forced<<<div_up(n, kThreads), kThreads, 0, s()>>>(n, active, kind.as<int8_t>(), sph, d + 1);
            GF_CHECK_LAUNCH();
            GF_CUDA(cudaMemcpyAsync(h_scal + 1, d + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s()));
        }
        ForceArgs a{n, pos.as<double>(), vel.as<double>(), mass.as<double>(), kind.as<int8_t>(), u.as<double>(),
                    theta, eps, gamma, alpha, beta, active, rebuild, sph, fresh, acc.as<double>(),
                    dt_ind.as<double>()};
        ForceEngine& F = force_engine();
        F.evaluate(a, s());
        GF_CUDA(cudaStreamSynchronize(s()));
        dt_grav = F.scalars_h->dt_grav;
        if (sph) dt_gas = F.scalars_h->dt_gas;
        updates += active ? double(h_scal[1]) : double(n);
    }

    void kick(const uint8_t* mask, double h) {
        k_kick<<<div_up(n, kThreads), kThreads, 0, s()>>>(n, vel.as<double>(), acc.as<double>(), mask, h);
        GF_CHECK_LAUNCH();
    }

    void drift(double dt) {
        k_drift<<<div_up(n, kThreads), kThreads, 0, s()>>>(n, pos.as<double>(), vel.as<double>(), dt);
        GF_CHECK_LAUNCH();
    }

    double masked_min(const uint8_t* mask) {
        unsigned long long* d = scal.get<unsigned long long>(2);
        GF_CUDA(cudaMemsetAsync(d, 0x7f, sizeof(unsigned long long), s()));
        k_masked_min<<<div_up(n, kThreads), kThreads, 0, s()>>>(n, dt_ind.as<double>(), mask, d);
        GF_CHECK_LAUNCH();
        GF_CUDA(cudaMemcpyAsync(h_scal, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s()));
        GF_CUDA(cudaStreamSynchronize(s()));
        double v;
        memcpy(&v, h_scal, sizeof v);
        return v;
    }

    // np.percentile(dt_ind, q) with numpy's default linear interpolation
    double percentile(double q) {
        uint64_t* k = keys.get<uint64_t>(n);
        int* v = vals.get<int>(n);
        k_keys_of<<<div_up(n, kThreads), kThreads, 0, s()>>>(n, dt_ind.as<double>(), k, v);
        GF_CHECK_LAUNCH();
        radix_sort_pairs(k, v, keys_alt.get<uint64_t>(n), vals_alt.get<int>(n), n, 0, 64, s());
        const double idx = q / 100.0 * (n - 1);
        const int lo = int(std::floor(idx));
        const int hi = std::min(n - 1, lo + 1);
        uint64_t b[2];
        GF_CUDA(cudaMemcpyAsync(&b[0], k + lo, sizeof(uint64_t), cudaMemcpyDeviceToHost, s()));
        GF_CUDA(cudaMemcpyAsync(&b[1], k + hi, sizeof(uint64_t), cudaMemcpyDeviceToHost, s()));
        GF_CUDA(cudaStreamSynchronize(s()));
        double a, c;
        memcpy(&a, &b[0], sizeof a);
        memcpy(&c, &b[1], sizeof c);
        const double w = idx - lo, diff = c - a;
        return w >= 0.5 ? c - diff * (1 - w) : a + diff * w;
    }

    double step(double dt_max) {
        updates = 0;
        const double dt_min = std::min(std::min(dt_gas, dt_grav), dt_max);
        const double D = std::min(dt_max, percentile(10.0));
        last_substeps = 0;
        if (D <= 1.5 * dt_min) {  // global step (simulation.py:118-127)
            thermo(dt_min);
            kick(nullptr, 0.5 * dt_min);
            drift(dt_min);
            accelerations(nullptr, 1, 1, 1);
            kick(nullptr, 0.5 * dt_min);
            t += dt_min;
            stars(dt_min);
            last_substeps = 1;
            return dt_min;
        }
        uint8_t* f = fast.get<uint8_t>(n);
        uint8_t* sl = slow.get<uint8_t>(n);
        k_split<<<div_up(n, kThreads), kThreads, 0, s()>>>(n, dt_ind.as<double>(), kind.as<int8_t>(), D, f, sl);
        GF_CHECK_LAUNCH();
        kick(sl, 0.5 * D);
        double tau = 0.0;
        bool first = true;
        while (tau < D * (1 - 1e-9)) {
            const double dt = std::min(masked_min(f), D - tau);
            thermo(dt);
            kick(f, 0.5 * dt);
            drift(dt);
            accelerations(f, 0, 1, first ? 1 : 0);
            first = false;
            kick(f, 0.5 * dt);
            tau += dt;
            t += dt;
            stars(dt);
            ++last_substeps;
        }
        accelerations(sl, 1, 0, 1);
        kick(sl, 0.5 * D);
        return D;
    }
};

static Simulation g_sim;
Simulation& simulation() { return g_sim; }
bool simulation_ready() { return g_sim.n > 0; }

// ---------------------------------------------------------------------------------------
// Block time steps (the batched form). Every particle sits on a power-of-two level j:
// its step is 2^j delta, delta = min dt_ind (the finest step), j = floor(log2(dt_ind /
// delta)) clamped to [0, nlev-1]; a block is 2^(nlev-1) finest sub-steps, so every level
// is synchronised at block boundaries. Leapfrog per particle: an opening half-kick at the
// block start, a full kick (closing + opening) at each of its force evaluations inside the
// block, a closing half-kick at the block end. Sub-step s evaluates forces (gravity on the
// refitted tree, SPH) for the particles with s mod 2^j == 0 only — from 100 % of them at
// s = 0 down to the finest level alone at odd s. The 2^(nlev-1) - 1 inner sub-steps plus the
// last drift are captured once as a CUDA graph and replayed every block; the block-end
// evaluation (rebuilt tree, fresh neighbour search, all particles) runs outside the graph.
// The graph is recaptured whenever a device buffer moved (g_alloc_generation).

namespace {

__global__ void k_levels(int n, const double* __restrict__ dt_ind, const unsigned long long* __restrict__ dbits,
                         int nlev, int8_t* __restrict__ level) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double delta = __longlong_as_double((long long)*dbits);
    int j = int(floor(log2(dt_ind[i] / delta)));
    level[i] = int8_t(min(max(j, 0), nlev - 1));
}

// mode 0: opening half-kick (all); 1: full kick of the particles active at sub-step s;
// 2: closing half-kick (all)
__global__ void k_kick_levels(int n, double* __restrict__ vel, const double* __restrict__ acc,
                              const int8_t* __restrict__ level, const unsigned long long* __restrict__ dbits,
                              int mode, int s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = level[i];
    if (mode == 1 && (s & ((1 << j) - 1))) return;
    const double step = __longlong_as_double((long long)*dbits) * double(1 << j);
    const double h = mode == 1 ? step : 0.5 * step;
    for (int c = 0; c < 3; ++c) vel[3 * size_t(i) + c] += h * acc[3 * size_t(i) + c];
}

// One pass between two sub-steps of a block: the kick of the particles due at sub-step s_kick
// (k_kick_levels' mode 1; s_kick 0: none), the drift of everybody by the finest step with the
// kicked velocities, and the flags of the particles due at sub-step s_next with their count
// (act null: none). The same float64 operations, in the same order, as the three kernels.
__global__ void k_kick_drift_active(int n, double* __restrict__ pos, double* __restrict__ vel,
                                    const double* __restrict__ acc, const int8_t* __restrict__ level,
                                    const unsigned long long* __restrict__ dbits, int s_kick, int s_next,
                                    uint8_t* __restrict__ act, unsigned long long* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool a = false;
    if (i < n) {
        const int j = level[i];
        const double dt = __longlong_as_double((long long)*dbits);
        double v[3];
        for (int c = 0; c < 3; ++c) v[c] = vel[3 * size_t(i) + c];
        if (s_kick > 0 && !(s_kick & ((1 << j) - 1))) {
            const double step = dt * double(1 << j);
            for (int c = 0; c < 3; ++c) {
                v[c] += step * acc[3 * size_t(i) + c];
                vel[3 * size_t(i) + c] = v[c];
            }
        }
        for (int c = 0; c < 3; ++c) pos[3 * size_t(i) + c] += dt * v[c];
        if (act) {
            a = !(s_next & ((1 << j) - 1));
            act[i] = a;
        }
    }
    if (act) {
        const unsigned m = __ballot_sync(0xffffffffu, a);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
    }
}

__global__ void k_active_at(int n, const int8_t* __restrict__ level, int s, uint8_t* __restrict__ act,
                            unsigned long long* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool a = i < n && !(s & ((1 << level[i]) - 1));
    if (i < n) act[i] = a;
    const unsigned m = __ballot_sync(0xffffffffu, a);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

}  // namespace

// Launch shape of the batched step, per sub-step bin (bin = number of trailing zero bits of
// the sub-step index: levels 0..bin are due). Chosen by BlockIntegrator::autotune.
struct BlockTuning {
    int chunk[8] = {4, 8, 8, 16, 16, 32, 64, 64};  // walk item code per bin (Octree::prepare_walk)
    int npl[8] = {8, 8, 8, 2, 2, 2, 2, 2};         // mixed walk: nodes per lane and round (2 or 8)
    int shape[8] = {0, 0, 0, 0, 0, 0, 0, 0};       // mixed walk with 2 per lane: launch shape
    int rebuild_every = 8;  // captured tree rebuild every this many sub-steps (0: refit only)
};

struct BlockIntegrator {
    int nlev = 7;
    bool started = false;
    DevBuf level, act, scal;  // scal: [0] delta bits, [1] active-count accumulator
    DevBuf save_pos, save_vel, save_u, tune_acc, t_block;
    double* h_tblock = nullptr;  // pinned
    unsigned long long* h_cnt = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long gen = ~0ull;
    int cap_n = -1, cap_nlev = -1;
    unsigned long long cap_key = 0;  // force-engine options the graph was captured under
    double last_updates = 0;
    int captures = 0;
    BlockTuning tune;
    bool tune_changed = true;
    double last_graph_ms = 0;  // device time of the last replayed graph

    int nsub() const { return 1 << (nlev - 1); }
    static int bin_of(int sub) { return std::min(7, __builtin_ctz(unsigned(sub))); }

    void levels_and_open(Simulation& S) {
        cudaStream_t s = S.s();
        unsigned long long* d = scal.as<unsigned long long>();
        GF_CUDA(cudaMemsetAsync(d, 0x7f, sizeof(unsigned long long), s));
        k_masked_min<<<div_up(S.n, 256), 256, 0, s>>>(S.n, S.dt_ind.as<double>(), nullptr, d);
        GF_CHECK_LAUNCH();
        k_levels<<<div_up(S.n, 256), 256, 0, s>>>(S.n, S.dt_ind.as<double>(), d, nlev, level.as<int8_t>());
        GF_CHECK_LAUNCH();
        k_kick_levels<<<div_up(S.n, 256), 256, 0, s>>>(S.n, S.vel.as<double>(), S.acc.as<double>(),
                                                       level.as<int8_t>(), d, 0, 0);
        GF_CHECK_LAUNCH();
    }

    // thermal update of the gas due at sub-step `sub` (every gas particle at sub = nsub)
    void thermo_at(Simulation& S, int sub) {
        ForceEngine& F = force_engine();
        if (!S.thermo_mode || F.ng_valid <= 0) return;
        thermo_gas_levels(F.ng_valid, F.gidx.as<int>(), level.as<int8_t>(), sub, scal.as<unsigned long long>(),
                          F.rho.as<double>(), F.dudt.as<double>(), S.u.as<double>(), S.thermo_mode,
                          S.no_cool.as<double>(), t_block.get<double>(1), S.thermo_units, S.s());
    }
    // options and gas set the graph bakes in
    unsigned long long capture_key(const Simulation& S) const {
        const ForceEngine& F = force_engine();
        return (F.option_key() * 31u + unsigned(S.thermo_mode)) * 1000003u + unsigned(F.ng_valid);
    }
    // the block's start time on the device (the thermal update's bubble test), before its replay
    void set_block_time(Simulation& S) {
        if (!h_tblock) GF_CUDA(cudaMallocHost(&h_tblock, sizeof(double)));
        *h_tblock = S.t;
        GF_CUDA(cudaMemcpyAsync(t_block.get<double>(1), h_tblock, sizeof(double), cudaMemcpyHostToDevice, S.s()));
    }

    // nosync: inside the captured graph (rebuild = captured tree rebuild, else refit);
    // otherwise a regular evaluation of everybody on a rebuilt tree with fresh neighbours
    void force(Simulation& S, const uint8_t* active, bool nosync, bool rebuild = false, int chunk = 0, int npl = 2,
               int shape = -1) {
        ForceArgs a{S.n, S.pos.as<double>(), S.vel.as<double>(), S.mass.as<double>(), S.kind.as<int8_t>(),
                    S.u.as<double>(), S.theta, S.eps, S.gamma, S.alpha, S.beta, active,
                    nosync ? (rebuild ? 1 : 0) : 1, 1, nosync ? 0 : 1, S.acc.as<double>(), S.dt_ind.as<double>()};
        a.sph_active = active;
        a.nosync = nosync ? 1 : 0;
        a.walk_chunk = chunk;
        a.walk_npl = npl;
        a.walk_shape = shape;
        force_engine().evaluate(a, S.s());
    }

    void capture(Simulation& S) {
        cudaStream_t s = S.s();
        if (exec) {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        Context& C = ctx();
        force_engine().reserve_nosync(S.n);  // nothing may allocate inside the capture
        t_block.get<double>(1);
        const bool prof = C.prof.on;
        C.prof.on = false;
        unsigned long long* d = scal.as<unsigned long long>();
        uint8_t* ac = act.as<uint8_t>();
        GF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeGlobal));
        g_no_alloc = true;
        try {
            // each sub-step opens with the kick of the previous one's particles due, the drift
            // and the flags of its own particles due, in one pass
            for (int sub = 1; sub < nsub(); ++sub) {
                k_kick_drift_active<<<div_up(S.n, 256), 256, 0, s>>>(S.n, S.pos.as<double>(), S.vel.as<double>(),
                                                                     S.acc.as<double>(), level.as<int8_t>(), d,
                                                                     sub - 1, sub, ac, d + 1);
                GF_CHECK_LAUNCH();
                const bool rb = tune.rebuild_every > 0 && sub % tune.rebuild_every == 0;
                thermo_at(S, sub);
                force(S, ac, true, rb, tune.chunk[bin_of(sub)], tune.npl[bin_of(sub)], tune.shape[bin_of(sub)]);
            }
            k_kick_drift_active<<<div_up(S.n, 256), 256, 0, s>>>(S.n, S.pos.as<double>(), S.vel.as<double>(),
                                                                 S.acc.as<double>(), level.as<int8_t>(), d,
                                                                 nsub() - 1, 0, nullptr, nullptr);
            GF_CHECK_LAUNCH();
        } catch (...) {
            g_no_alloc = false;
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            C.prof.on = prof;
            throw;
        }
        g_no_alloc = false;
        cudaGraph_t g;
        GF_CUDA(cudaStreamEndCapture(s, &g));
        GF_CUDA(cudaGraphInstantiate(&exec, g, 0));
        GF_CUDA(cudaGraphDestroy(g));
        C.prof.on = prof;
        gen = g_alloc_generation;
        cap_n = S.n;
        cap_nlev = nlev;
        cap_key = capture_key(S);
        tune_changed = false;
        ++captures;
    }

    void start(Simulation& S) {  // block start: forces of everybody on a rebuilt tree, levels, opening kicks
        level.get<int8_t>(S.n);
        act.get<uint8_t>(S.n);
        scal.get<unsigned long long>(2);
        if (!h_cnt) GF_CUDA(cudaMallocHost(&h_cnt, 2 * sizeof(unsigned long long)));
        force(S, nullptr, false);
        levels_and_open(S);
        started = true;
    }

    // Advances nblocks blocks; returns particle-updates done (forces computed).
    double run(Simulation& S, int nblocks) {
        cudaStream_t s = S.s();
        double updates = 0;
        if (!started) {
            start(S);
            updates += S.n;
        }
        Event e0, e1;
        for (int b = 0; b < nblocks; ++b) {
            if (!exec || gen != g_alloc_generation || cap_n != S.n || cap_nlev != nlev || tune_changed ||
                cap_key != capture_key(S))
                capture(S);
            unsigned long long* d = scal.as<unsigned long long>();
            GF_CUDA(cudaMemsetAsync(d + 1, 0, sizeof(unsigned long long), s));
            set_block_time(S);
            e0.record(s);
            GF_CUDA(cudaGraphLaunch(exec, s));
            e1.record(s);
            GF_CUDA(cudaMemcpyAsync(h_cnt, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
            thermo_at(S, nsub());      // every gas particle is due at the block end
            force(S, nullptr, false);  // block end: synchronised, rebuilt tree, fresh neighbours
            GF_CUDA(cudaStreamSynchronize(s));
            last_graph_ms = e1.since(e0);
            double delta;
            memcpy(&delta, &h_cnt[0], sizeof delta);
            updates += double(h_cnt[1]) + S.n;
            S.t += delta * nsub();
            k_kick_levels<<<div_up(S.n, 256), 256, 0, s>>>(S.n, S.vel.as<double>(), S.acc.as<double>(),
                                                           level.as<int8_t>(), d, 2, 0);  // closing
            GF_CHECK_LAUNCH();
            levels_and_open(S);  // new levels from the new dt_ind, opening kicks
        }
        GF_CUDA(cudaStreamSynchronize(s));
        last_updates = updates;
        return updates;
    }

    // Autotuner. The state (positions, velocities, energies, time) is saved first and restored at the
    // end; the next block then starts with a full evaluation, so tuning leaves no trace in the
    // trajectory. Two knobs:
    //   * walk items per bin: for the particles due at the first sub-step of each bin, the
    //     gravity walk alone (on the block-start tree, into a scratch array) is timed for each
    //     candidate chunk; the fastest wins;
    //   * tree rebuild cadence: one whole block per candidate, graph time compared.
    void autotune(Simulation& S, int* chunk_out, int* rebuild_out, double* graph_ms_out) {
        cudaStream_t s = S.s();
        const size_t n3 = 3 * size_t(S.n);
        double* sp = save_pos.get<double>(n3);
        double* sv = save_vel.get<double>(n3);
        GF_CUDA(cudaMemcpyAsync(sp, S.pos.as<double>(), sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
        GF_CUDA(cudaMemcpyAsync(sv, S.vel.as<double>(), sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
        double* su = save_u.get<double>(size_t(S.n));  // the thermal update changes u
        GF_CUDA(cudaMemcpyAsync(su, S.u.as<double>(), sizeof(double) * size_t(S.n), cudaMemcpyDeviceToDevice, s));
        const double t0 = S.t;
        ForceEngine& F = force_engine();
        const long long collect = F.collect_cap;
        F.collect_cap = F.collect_n;  // no training rows from trial runs
        Context& C = ctx();
        const bool prof = C.prof.on;
        C.prof.on = false;
        try {
            start(S);
            Octree& T = F.grav;
            double* ta = tune_acc.get<double>(n3);
            unsigned long long* d = scal.as<unsigned long long>();
            // chunks of one group's active particles, then sibling-group runs merged by active
            // count (codes 72, 80, 84, 96: <= 16, 32, 40, 64 active particles per item)
            static const int cand[] = {0, 2, 4, 8, 16, 32, 64, 72, 80, 84, 96};
            Event e0, e1;
            for (int bin = 0; bin < nlev - 1; ++bin) {
                k_active_at<<<div_up(S.n, 256), 256, 0, s>>>(S.n, level.as<int8_t>(), 1 << bin, act.as<uint8_t>(),
                                                             d + 1);
                GF_CHECK_LAUNCH();
                double best = INFINITY;
                int best_c = 0, best_p = 2, best_s = 0;
                for (int npl : {2, 8}) {
                    if (npl != 2 && !T.quad) continue;  // the monopole walk has one width
                    // launch shapes (block warps x tile size) of the 2-per-lane mixed walk
                    const int nshape = npl == 2 && T.quad ? kNumWalkShapes : 1;
                    for (int shape = 0; shape < nshape; ++shape) {
                        for (int c : cand) {
                            double ms[3];
                            for (int r = 0; r < 3; ++r) {
                                e0.record(s);
                                T.prepare_walk(act.as<uint8_t>(), s, c);
                                T.walk(S.eps, ta, s, nullptr, npl, shape);
                                e1.record(s);
                                GF_CUDA(cudaStreamSynchronize(s));
                                ms[r] = e1.since(e0);
                            }
                            std::sort(ms, ms + 3);
                            if (ms[1] < best * 0.97) {  // prefer the earlier candidate on near-ties
                                best = ms[1];
                                best_c = c;
                                best_p = npl;
                                best_s = shape;
                            }
                        }
                    }
                }
                tune.chunk[bin] = best_c;
                tune.npl[bin] = best_p;
                tune.shape[bin] = best_s;
            }
            for (int bin = nlev - 1; bin < 8; ++bin) {
                tune.chunk[bin] = tune.chunk[std::max(0, nlev - 2)];
                tune.npl[bin] = tune.npl[std::max(0, nlev - 2)];
                tune.shape[bin] = tune.shape[std::max(0, nlev - 2)];
            }
            // rebuild cadence: whole blocks from the same start
            static const int every[] = {0, 32, 16, 8, 4};
            double best = INFINITY;
            int best_r = 0;
            for (int r : every) {
                if (r >= nsub()) continue;
                GF_CUDA(cudaMemcpyAsync(S.pos.as<double>(), sp, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
                GF_CUDA(cudaMemcpyAsync(S.vel.as<double>(), sv, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
                GF_CUDA(cudaMemcpyAsync(S.u.as<double>(), su, sizeof(double) * size_t(S.n), cudaMemcpyDeviceToDevice,
                                        s));
                tune.rebuild_every = r;
                tune_changed = true;
                started = false;
                run(S, 1);
                if (last_graph_ms < best) {
                    best = last_graph_ms;
                    best_r = r;
                }
            }
            tune.rebuild_every = best_r;
            tune_changed = true;
            if (graph_ms_out) *graph_ms_out = best;
        } catch (...) {
            F.collect_cap = collect;
            C.prof.on = prof;
            throw;
        }
        F.collect_cap = collect;
        C.prof.on = prof;
        GF_CUDA(cudaMemcpyAsync(S.pos.as<double>(), sp, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
        GF_CUDA(cudaMemcpyAsync(S.vel.as<double>(), sv, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
        GF_CUDA(cudaMemcpyAsync(S.u.as<double>(), su, sizeof(double) * size_t(S.n), cudaMemcpyDeviceToDevice, s));
        GF_CUDA(cudaStreamSynchronize(s));
        S.t = t0;
        started = false;
        if (chunk_out)  // chunk, + 100 where the 8-nodes-per-lane walk won, + 1000 x the launch shape
            for (int b = 0; b < nlev - 1; ++b)
                chunk_out[b] = tune.chunk[b] + (tune.npl[b] > 2 ? 100 : 0) + 1000 * tune.shape[b];
        if (rebuild_out) *rebuild_out = tune.rebuild_every;
    }
};

static BlockIntegrator g_block;

double block_run(int nblocks, int nlev) {
    if (g_block.nlev != nlev) {
        g_block.nlev = nlev;
        g_block.started = false;
    }
    return g_block.run(g_sim, nblocks);
}

void block_config(const int* chunk, int nbins, int rebuild_every) {
    BlockTuning& t = g_block.tune;
    for (int b = 0; b < 8; ++b) {
        const int c = chunk ? chunk[std::min(b, nbins - 1)] : 0;
        t.chunk[b] = c % 100;
        t.npl[b] = (c % 1000) >= 100 ? 8 : 2;
        t.shape[b] = std::min(kNumWalkShapes - 1, std::max(0, c / 1000));
    }
    t.rebuild_every = rebuild_every;
    g_block.tune_changed = true;
}

void block_autotune(int nlev, int* chunk, int* rebuild_every, double* graph_ms) {
    g_block.nlev = nlev;
    g_block.autotune(g_sim, chunk, rebuild_every, graph_ms);
}

void block_reset() { g_block.started = false; }

// Fraction of particles on each level (levels 0..nlev-1) of the current block.
void block_levels(int nlev, double* frac) {
    Simulation& S = g_sim;
    std::vector<int8_t> lv(S.n);
    GF_CUDA(cudaMemcpy(lv.data(), g_block.level.p, S.n, cudaMemcpyDeviceToHost));
    for (int j = 0; j < nlev; ++j) frac[j] = 0;
    for (int8_t v : lv)
        if (v >= 0 && v < nlev) frac[v] += 1.0 / S.n;
}

void sim_init_reset_blocks() { g_block.started = false; }

void sim_init(int n, const double* pos, const double* vel, const double* mass, const int8_t* kind, const double* u,
              double theta, double eps, double gamma, double alpha, double beta) {
    Simulation& S = g_sim;
    cudaStream_t s = ctx().stream;
    S.n = n;
    S.t = 0;
    S.theta = theta;
    S.eps = eps;
    S.gamma = gamma;
    S.alpha = alpha;
    S.beta = beta;
    if (!S.h_scal) GF_CUDA(cudaMallocHost(&S.h_scal, 2 * sizeof(unsigned long long)));
    GF_CUDA(cudaMemcpyAsync(S.pos.get<double>(3 * size_t(n)), pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
    GF_CUDA(cudaMemcpyAsync(S.vel.get<double>(3 * size_t(n)), vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
    GF_CUDA(cudaMemcpyAsync(S.mass.get<double>(n), mass, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    GF_CUDA(cudaMemcpyAsync(S.kind.get<int8_t>(n), kind, n, cudaMemcpyHostToDevice, s));
    GF_CUDA(cudaMemcpyAsync(S.u.get<double>(n), u, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    S.acc.get<double>(3 * size_t(n));
    S.dt_ind.get<double>(n);
    k_set<<<div_up(n, kThreads), kThreads, 0, s>>>(n, S.birth.get<double>(n), INFINITY);       // simulation.py:36
    GF_CHECK_LAUNCH();
    k_set<<<div_up(n, kThreads), kThreads, 0, s>>>(n, S.no_cool.get<double>(n), -INFINITY);    // simulation.py:43
    GF_CHECK_LAUNCH();
    S.stars_formed = 0;
    force_engine().n_total = -1;  // fresh force state (simulation.py:51-54)
    g_block.started = false;
    S.dt_gas = INFINITY;
    S.accelerations(nullptr, 1, 1, 1);
}

double sim_updates() { return g_sim.updates; }

double sim_step(double dt_max, int* substeps) {
    const double D = g_sim.step(dt_max);
    if (substeps) *substeps = g_sim.last_substeps;
    return D;
}

// ---------------------------------------------------------------------------------------
// Conserved quantities in float64: kinetic, potential (softened, from a monopole Barnes-Hut
// walk at opening angle theta on a tree of its own), thermal energy and angular momentum.
// Between blocks of the batched form the velocities carry the opening half-kick of the next
// block; it is taken off here so the diagnostics see synchronised velocities.

namespace {

constexpr int kDiagThreads = 256;
constexpr int kDiagQ = 6;  // kinetic, potential, thermal, Lx, Ly, Lz

__global__ void __launch_bounds__(kDiagThreads) k_diag_partial(
    int n, const double* __restrict__ pos, const double* __restrict__ vel, const double* __restrict__ acc,
    const double* __restrict__ mass, const int8_t* __restrict__ kind, const double* __restrict__ u,
    const double* __restrict__ phi, const int8_t* __restrict__ level, const unsigned long long* __restrict__ dbits,
    double* __restrict__ part) {
    __shared__ double sm[kDiagQ][kDiagThreads];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double q[kDiagQ] = {0, 0, 0, 0, 0, 0};
    if (i < n) {
        const double m = mass[i];
        double v[3] = {vel[3 * size_t(i)], vel[3 * size_t(i) + 1], vel[3 * size_t(i) + 2]};
        if (level) {
            const double h = 0.5 * __longlong_as_double((long long)*dbits) * double(1 << level[i]);
            for (int c = 0; c < 3; ++c) v[c] -= h * acc[3 * size_t(i) + c];
        }
        const double x = pos[3 * size_t(i)], y = pos[3 * size_t(i) + 1], z = pos[3 * size_t(i) + 2];
        q[0] = 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        q[1] = 0.5 * m * phi[i];
        q[2] = kind[i] == 0 ? m * u[i] : 0.0;
        q[3] = m * (y * v[2] - z * v[1]);
        q[4] = m * (z * v[0] - x * v[2]);
        q[5] = m * (x * v[1] - y * v[0]);
    }
    for (int c = 0; c < kDiagQ; ++c) sm[c][threadIdx.x] = q[c];
    __syncthreads();
    for (int w = kDiagThreads / 2; w > 0; w >>= 1) {  // fixed pairing: deterministic
        if (threadIdx.x < w)
            for (int c = 0; c < kDiagQ; ++c) sm[c][threadIdx.x] += sm[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < kDiagQ) part[size_t(blockIdx.x) * kDiagQ + threadIdx.x] = sm[threadIdx.x][0];
}

__global__ void k_diag_final(int nb, const double* __restrict__ part, double* __restrict__ out) {
    const int c = threadIdx.x;
    if (c >= kDiagQ) return;
    double t = 0;
    for (int b = 0; b < nb; ++b) t += part[size_t(b) * kDiagQ + c];
    out[c] = t;
}

}  // namespace

static Octree g_diag_tree;
static DevBuf g_diag_acc, g_diag_phi, g_diag_part, g_diag_out;

void sim_diagnostics(double theta, double* out) {
    Simulation& S = g_sim;
    cudaStream_t s = ctx().stream;
    const int n = S.n;
    Octree& T = g_diag_tree;
    T.quad = false;
    T.build(n, S.pos.as<double>(), S.mass.as<double>(), theta, s);
    T.prepare_walk(nullptr, s);
    double* phi = g_diag_phi.get<double>(n);
    T.walk(S.eps, g_diag_acc.get<double>(3 * size_t(n)), s, phi);
    const int nb = div_up(n, kDiagThreads);
    double* part = g_diag_part.get<double>(size_t(nb) * kDiagQ);
    double* dout = g_diag_out.get<double>(kDiagQ);
    const bool blocks = g_block.started;
    k_diag_partial<<<nb, kDiagThreads, 0, s>>>(n, S.pos.as<double>(), S.vel.as<double>(), S.acc.as<double>(),
                                               S.mass.as<double>(), S.kind.as<int8_t>(), S.u.as<double>(), phi,
                                               blocks ? g_block.level.as<int8_t>() : nullptr,
                                               blocks ? g_block.scal.as<unsigned long long>() : nullptr, part);
    GF_CHECK_LAUNCH();
    k_diag_final<<<1, 32, 0, s>>>(nb, part, dout);
    GF_CHECK_LAUNCH();
    double q[kDiagQ];
    GF_CUDA(cudaMemcpyAsync(q, dout, sizeof q, cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaStreamSynchronize(s));
    out[0] = q[0];
    out[1] = q[1];
    out[2] = q[2];
    out[3] = q[0] + q[1] + q[2];
    out[4] = q[3];
    out[5] = q[4];
    out[6] = q[5];
    out[7] = S.t;
}

void sim_thermo(int mode, const double* units) {
    Simulation& S = g_sim;
    S.thermo_mode = mode;
    if (mode) {
        ThermoUnits& U = S.thermo_units;
        U = ThermoUnits{units[0], units[1], units[2], units[3], units[4], units[5], units[6], units[7]};
    }
}

void sim_stars(int on, const double* params, const unsigned long long* rng_words) {
    Simulation& S = g_sim;
    S.stars_on = on != 0;
    if (!on) return;
    StarParams& P = S.star_params;
    P = StarParams{params[0], params[1], params[2], params[3], params[4],
                   params[5], params[6], params[7], params[8], params[9]};
    Pcg64 R;
    for (int i = 0; i < 4; ++i) R.w[i] = rng_words[i];
    GF_CUDA(cudaMemcpyAsync(S.rng.get<Pcg64>(1), &R, sizeof(Pcg64), cudaMemcpyHostToDevice, ctx().stream));
    GF_CUDA(cudaStreamSynchronize(ctx().stream));
}

long long sim_read_stars(int8_t* kind, double* birth, double* no_cool, unsigned long long* rng_words) {
    Simulation& S = g_sim;
    cudaStream_t s = ctx().stream;
    const size_t n = S.n;
    if (kind) GF_CUDA(cudaMemcpyAsync(kind, S.kind.p, n, cudaMemcpyDeviceToHost, s));
    if (birth) GF_CUDA(cudaMemcpyAsync(birth, S.birth.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (no_cool) GF_CUDA(cudaMemcpyAsync(no_cool, S.no_cool.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (rng_words && S.rng.p) GF_CUDA(cudaMemcpyAsync(rng_words, S.rng.p, sizeof(Pcg64), cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaStreamSynchronize(s));
    return S.stars_formed;
}

void sim_scalars(double* out) {
    Simulation& S = g_sim;
    out[0] = S.t;
    out[1] = S.dt_grav;
    out[2] = S.dt_gas;
}

namespace {
__global__ void k_gas_to_particles(int ng, const int* __restrict__ gidx, const double* __restrict__ a,
                                   const double* __restrict__ b, double* __restrict__ pa, double* __restrict__ pb) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < ng) {
        pa[gidx[g]] = a[g];
        pb[gidx[g]] = b[g];
    }
}
__global__ void k_particles_to_gas(int ng, const int* __restrict__ gidx, const double* __restrict__ pa,
                                   const double* __restrict__ pb, double* __restrict__ a, double* __restrict__ b) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < ng) {
        a[g] = pa[gidx[g]];
        b[g] = pb[gidx[g]];
    }
}
}  // namespace

// density and du/dt of the last SPH evaluation (the next thermal update's inputs), per particle
// (NaN outside its gas set)
void sim_read_hydro(double* rho, double* dudt) {
    Simulation& S = g_sim;
    ForceEngine& F = force_engine();
    cudaStream_t s = ctx().stream;
    const size_t n = S.n;
    static DevBuf pr, pd;
    double* a = pr.get<double>(n);
    double* b = pd.get<double>(n);
    GF_CUDA(cudaMemsetAsync(a, 0xff, sizeof(double) * n, s));  // NaN pattern
    GF_CUDA(cudaMemsetAsync(b, 0xff, sizeof(double) * n, s));
    if (F.ng_valid > 0) {
        k_gas_to_particles<<<div_up(F.ng_valid, kThreads), kThreads, 0, s>>>(F.ng_valid, F.gidx.as<int>(),
                                                                            F.rho.as<double>(), F.dudt.as<double>(),
                                                                            a, b);
        GF_CHECK_LAUNCH();
    }
    GF_CUDA(cudaMemcpyAsync(rho, a, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaMemcpyAsync(dudt, b, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaStreamSynchronize(s));
}

void sim_restore(const double* acc, const double* dt_ind, const double* birth, const double* no_cool,
                 const double* rho, const double* dudt, double t, double dt_grav, double dt_gas) {
    Simulation& S = g_sim;
    cudaStream_t s = ctx().stream;
    const size_t n = S.n;
    ForceEngine& F = force_engine();
    if (rho && dudt && F.ng_valid > 0) {  // the gas set of sim_init's evaluation: same kinds, same order
        static DevBuf pr, pd;
        double* a = pr.get<double>(n);
        double* b = pd.get<double>(n);
        GF_CUDA(cudaMemcpyAsync(a, rho, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        GF_CUDA(cudaMemcpyAsync(b, dudt, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        k_particles_to_gas<<<div_up(F.ng_valid, kThreads), kThreads, 0, s>>>(F.ng_valid, F.gidx.as<int>(), a, b,
                                                                            F.rho.as<double>(), F.dudt.as<double>());
        GF_CHECK_LAUNCH();
    }
    GF_CUDA(cudaMemcpyAsync(S.acc.p, acc, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
    GF_CUDA(cudaMemcpyAsync(S.dt_ind.p, dt_ind, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    if (birth) GF_CUDA(cudaMemcpyAsync(S.birth.p, birth, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    if (no_cool) GF_CUDA(cudaMemcpyAsync(S.no_cool.p, no_cool, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    GF_CUDA(cudaStreamSynchronize(s));
    S.t = t;
    S.dt_grav = dt_grav;
    S.dt_gas = dt_gas;
    g_block.started = false;  // block steps restart from a full evaluation
}

void sim_read_u(double* u) {
    Simulation& S = g_sim;
    cudaStream_t s = ctx().stream;
    GF_CUDA(cudaMemcpyAsync(u, S.u.p, sizeof(double) * size_t(S.n), cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaStreamSynchronize(s));
}

void sim_read(double* pos, double* vel, double* acc, double* dt_ind, double* t) {
    Simulation& S = g_sim;
    cudaStream_t s = ctx().stream;
    const size_t n = S.n;
    if (pos) GF_CUDA(cudaMemcpyAsync(pos, S.pos.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    if (vel) GF_CUDA(cudaMemcpyAsync(vel, S.vel.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    if (acc) GF_CUDA(cudaMemcpyAsync(acc, S.acc.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    if (dt_ind) GF_CUDA(cudaMemcpyAsync(dt_ind, S.dt_ind.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    GF_CUDA(cudaStreamSynchronize(s));
    if (t) *t = S.t;
}

}  // namespace gf
