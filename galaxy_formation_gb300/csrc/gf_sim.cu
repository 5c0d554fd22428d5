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

#include "gf_hydro.cuh"

namespace gf {

namespace {

constexpr int kThreads = 256;

__global__ void k_kick(int n, double* __restrict__ vel, const double* __restrict__ acc,
                       const uint8_t* __restrict__ mask, double h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (mask && !mask[i])) return;
    for (int c = 0; c < 3; ++c) vel[3 * size_t(i) + c] += h * acc[3 * size_t(i) + c];
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
    DevBuf pos, vel, acc, mass, kind, u, dt_ind, fast, slow, keys, keys_alt, vals, vals_alt, scal;
    unsigned long long* h_scal = nullptr;

    cudaStream_t s() const { return ctx().stream; }

    void accelerations(const uint8_t* active, int rebuild, int sph, int fresh) {
        ForceArgs a{n, pos.as<double>(), vel.as<double>(), mass.as<double>(), kind.as<int8_t>(), u.as<double>(),
                    theta, eps, gamma, alpha, beta, active, rebuild, sph, fresh, acc.as<double>(),
                    dt_ind.as<double>()};
        ForceEngine& F = force_engine();
        F.evaluate(a, s());
        GF_CUDA(cudaStreamSynchronize(s()));
        dt_grav = F.scalars_h->dt_grav;
        if (sph) dt_gas = F.scalars_h->dt_gas;
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
        const double dt_min = std::min(std::min(dt_gas, dt_grav), dt_max);
        const double D = std::min(dt_max, percentile(10.0));
        last_substeps = 0;
        if (D <= 1.5 * dt_min) {  // global step (simulation.py:118-127)
            kick(nullptr, 0.5 * dt_min);
            drift(dt_min);
            accelerations(nullptr, 1, 1, 1);
            kick(nullptr, 0.5 * dt_min);
            t += dt_min;
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
            kick(f, 0.5 * dt);
            drift(dt);
            accelerations(f, 0, 1, first ? 1 : 0);
            first = false;
            kick(f, 0.5 * dt);
            tau += dt;
            t += dt;
            ++last_substeps;
        }
        accelerations(sl, 1, 0, 1);
        kick(sl, 0.5 * D);
        return D;
    }
};

static Simulation g_sim;
Simulation& simulation() { return g_sim; }

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
    force_engine().n_total = -1;  // fresh force state (simulation.py:51-54)
    S.dt_gas = INFINITY;
    S.accelerations(nullptr, 1, 1, 1);
}

double sim_step(double dt_max, int* substeps) {
    const double D = g_sim.step(dt_max);
    if (substeps) *substeps = g_sim.last_substeps;
    return D;
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
