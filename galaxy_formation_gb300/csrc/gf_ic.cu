// gf_ic.cu — seeded initial conditions generated on the device: the rotating 1/r cloud of
// galaxy_formation/initial_conditions.py:33-68 at any size, and the collapsed disk + 1/r halo
// snapshot (with optional Plummer clumps) of the benchmark workloads.
//
// Every random number is a pure function of (seed, particle or clump index, draw number):
// SplitMix64 (Steele, Lea & Flood 2014) applied to a counter, so a set is the same for any
// launch shape and any GPU, and particle i does not depend on how many others are drawn.
// The distributions are the host generators' (galaxy_formation_gb300/synthetic.py), not
// their streams: NumPy's normal and gamma deviates come from rejection samplers whose
// consumption of the stream cannot be followed cheaply in parallel, so the device sets agree
// with the host sets in distribution (mass, profile, spin and dispersion moments), not bit for
// bit. Deviates used here:
//   uniform on [0,1) ........ the top 53 bits of a SplitMix64 output;
//   normal .................. Box-Muller on two uniforms;
//   direction ............... z uniform on [-1,1], azimuth uniform (uniform on the sphere);
//   Gamma(2, Rd) ............ -Rd ln(U1 U2) (the sum of two exponentials), truncated by
//                             redrawing (bounded number of tries);
//   sech^2 height ........... z0 atanh(2U - 1) (inverse CDF);
//   Plummer radius .......... a / sqrt(U^(-2/3) - 1) (inverse CDF of the enclosed mass).
// The disk's circular velocities need the enclosed mass M(<r): the radii are sorted on the
// device (radix sort of their float64 bit patterns) and the masses accumulated in that order
// (two species of equal-mass particles, so a scan of gas counts gives it exactly).
#include <algorithm>
#include <cmath>

#include "gf_sph.cuh"

namespace gf {
namespace {

constexpr int kThreads = 256;
constexpr double kTwoPi = 6.283185307179586;

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Draw number c of stream `id` under `seed`: a uniform double on [0, 1).
__device__ __forceinline__ double uni(uint64_t seed, uint64_t id, uint32_t c) {
    const uint64_t h = splitmix64(splitmix64(seed) ^ (id * 0x100000001b3ull + c));
    return double(h >> 11) * 0x1.0p-53;
}
// (0, 1]: safe under log
__device__ __forceinline__ double uni_pos(uint64_t seed, uint64_t id, uint32_t c) {
    return 1.0 - uni(seed, id, c);
}

__device__ __forceinline__ void normal2(uint64_t seed, uint64_t id, uint32_t c, double& a, double& b) {
    const double r = sqrt(-2.0 * log(uni_pos(seed, id, c)));
    double s, co;
    sincos(kTwoPi * uni(seed, id, c + 1), &s, &co);
    a = r * co;
    b = r * s;
}

__device__ __forceinline__ void direction(uint64_t seed, uint64_t id, uint32_t c, double d[3]) {
    const double z = 2.0 * uni(seed, id, c) - 1.0;
    const double s = sqrt(fmax(0.0, 1.0 - z * z));
    double sp, cp;
    sincos(kTwoPi * uni(seed, id, c + 1), &sp, &cp);
    d[0] = s * cp;
    d[1] = s * sp;
    d[2] = z;
}

// Gamma(2, rd) below rmax: redraws up to 64 times, then takes rmax (1 - 2^-30) (probability of
// getting there: (P(R > rmax))^64, i.e. none for the truncations used here).
__device__ double gamma2_trunc(uint64_t seed, uint64_t id, uint32_t c, double rd, double rmax) {
    for (int t = 0; t < 64; ++t) {
        const double R = -rd * log(uni_pos(seed, id, c + 2 * t) * uni_pos(seed, id, c + 2 * t + 1));
        if (R < rmax) return R;
    }
    return rmax * (1.0 - 0x1.0p-30);
}

__device__ __forceinline__ double sech2_height(uint64_t seed, uint64_t id, uint32_t c, double z0) {
    const double x = fmin(fmax(2.0 * uni(seed, id, c) - 1.0, -1.0 + 1e-12), 1.0 - 1e-12);
    return z0 * atanh(x);
}

struct IcSpec {
    int kind;          // 0 rotating cloud, 1 disk + halo
    int n_gas, n_dm, n_disk, n_smooth, n_clumps, n_cl_each;
    uint64_t seed;
    double m_gas, m_dm;
    double R0;         // outer radius of the 1/r spheres
    double u_gas;      // cloud: specific energy of the gas
    double ln_u_lo, ln_u_hi;  // disk: log-uniform specific energies of the gas
    double rd, z0, a_cl;
    double kappa, M_tot, v_vir;  // cloud rotation (initial_conditions.py:55-63)
};

// Positions, masses, kinds, energies; radii for the enclosed-mass sort (disk).
__global__ void k_ic_place(IcSpec S, double* __restrict__ pos, double* __restrict__ mass, int8_t* __restrict__ kind,
                           double* __restrict__ u, uint64_t* __restrict__ rkey, int* __restrict__ ridx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = S.n_gas + S.n_dm;
    if (i >= n) return;
    const bool gas = i < S.n_gas;
    double p[3];
    if (S.kind == 1 && i < S.n_smooth) {  // smooth exponential disk
        const double R = gamma2_trunc(S.seed, i, 0, S.rd, 12.0 * S.rd);
        double sp, cp;
        sincos(kTwoPi * uni(S.seed, i, 200), &sp, &cp);
        p[0] = R * cp;
        p[1] = R * sp;
        p[2] = sech2_height(S.seed, i, 201, S.z0);
    } else if (S.kind == 1 && i < S.n_disk) {  // Plummer clump member
        const int k = (i - S.n_smooth) / S.n_cl_each;
        const uint64_t cid = uint64_t(n) + uint64_t(k);  // the clump's own stream
        const double Rc = gamma2_trunc(S.seed, cid, 0, S.rd, 6.0 * S.rd);
        double sp, cp;
        sincos(kTwoPi * uni(S.seed, cid, 200), &sp, &cp);
        const double cz = sech2_height(S.seed, cid, 201, S.z0);
        const double U = 1e-6 + (0.999 - 1e-6) * uni(S.seed, i, 0);
        const double rr = S.a_cl / sqrt(pow(U, -2.0 / 3.0) - 1.0);
        double d[3];
        direction(S.seed, i, 1, d);
        p[0] = Rc * cp + rr * d[0];
        p[1] = Rc * sp + rr * d[1];
        p[2] = cz + rr * d[2];
    } else {  // 1/r sphere: M(<r) ~ r^2, r = R0 U^(1/2) (initial_conditions.py:25-30, 39)
        double d[3];
        direction(S.seed, i, 0, d);
        const double r = S.R0 * sqrt(uni(S.seed, i, 2));
        for (int a = 0; a < 3; ++a) p[a] = r * d[a];
    }
    for (int a = 0; a < 3; ++a) pos[3 * size_t(i) + a] = p[a];
    mass[i] = gas ? S.m_gas : S.m_dm;
    kind[i] = gas ? 0 : 2;
    if (!gas)
        u[i] = 0.0;
    else if (S.kind == 0)
        u[i] = S.u_gas;
    else
        u[i] = exp(S.ln_u_lo + (S.ln_u_hi - S.ln_u_lo) * uni(S.seed, i, 300));
    if (rkey) {
        const double r = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        rkey[i] = uint64_t(__double_as_longlong(r));  // r >= 0: bit order = numeric order
        ridx[i] = i;
    }
}

// Gas flag of the particle at each sorted-radius position (the scan of these counts the gas
// inside, hence the enclosed mass).
__global__ void k_ic_gasflag(int n, int n_gas, const int* __restrict__ ridx, int* __restrict__ flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) flag[k] = ridx[k] < n_gas ? 1 : 0;
}

__global__ void k_ic_menc(int n, const int* __restrict__ ridx, const int* __restrict__ flag,
                          const int* __restrict__ gscan, double m_gas, double m_dm, double* __restrict__ menc) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const long long g = (long long)gscan[k] + flag[k];  // gas at sorted positions 0..k
    menc[ridx[k]] = m_gas * double(g) + m_dm * double((long long)k + 1 - g);
}

// Velocities: rotation about z plus 10 % Gaussian dispersion (cloud: initial_conditions.py
// :55-66; disk: circular velocity from the enclosed mass, the disk rotating at v_c, the rest
// slowly at spin 0.05).
__global__ void k_ic_vel(IcSpec S, const double* __restrict__ pos, const double* __restrict__ menc,
                         double* __restrict__ vel) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = S.n_gas + S.n_dm;
    if (i >= n) return;
    const double x = pos[3 * size_t(i)], y = pos[3 * size_t(i) + 1], z = pos[3 * size_t(i) + 2];
    const double r = sqrt(x * x + y * y + z * z), rc = fmax(r, 1e-6);
    const double Rcyl = hypot(x, y);
    const double inv = 1.0 / (Rcyl + 1e-30);  // phi_hat = (-y, x, 0) / R
    double vrot, sig;
    if (S.kind == 0) {
        const double vc = sqrt(S.M_tot * (r / S.R0) * (r / S.R0) / rc);
        vrot = S.kappa * vc * Rcyl / rc;
        sig = 0.1 * S.v_vir;
    } else {
        const double vc = sqrt(menc[i] / rc);
        vrot = (i < S.n_disk ? 1.0 : 0.05 / 0.47 * Rcyl / rc) * vc;
        sig = 0.1 * vc;
    }
    double g0, g1, g2, g3;
    normal2(S.seed, i, 400, g0, g1);
    normal2(S.seed, i, 402, g2, g3);
    const double f = sig / sqrt(3.0);
    vel[3 * size_t(i)] = -y * inv * vrot + f * g0;
    vel[3 * size_t(i) + 1] = x * inv * vrot + f * g1;
    vel[3 * size_t(i) + 2] = f * g2;
}

// Mass-weighted mean velocity (fixed-order block partials, then one block): removed so the set
// has no bulk motion.
__global__ void k_ic_momentum(int n, const double* __restrict__ vel, const double* __restrict__ mass,
                              double* __restrict__ part) {
    __shared__ double sm[4][kThreads];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double q[4] = {0, 0, 0, 0};
    if (i < n) {
        const double m = mass[i];
        q[0] = m * vel[3 * size_t(i)];
        q[1] = m * vel[3 * size_t(i) + 1];
        q[2] = m * vel[3 * size_t(i) + 2];
        q[3] = m;
    }
    for (int c = 0; c < 4; ++c) sm[c][threadIdx.x] = q[c];
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int c = 0; c < 4; ++c) sm[c][threadIdx.x] += sm[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 4) part[size_t(blockIdx.x) * 4 + threadIdx.x] = sm[threadIdx.x][0];
}

__global__ void k_ic_momentum_final(int nb, const double* __restrict__ part, double* __restrict__ mean) {
    __shared__ double sm[4][kThreads];
    double q[4] = {0, 0, 0, 0};
    for (int b = threadIdx.x; b < nb; b += kThreads)
        for (int c = 0; c < 4; ++c) q[c] += part[size_t(b) * 4 + c];
    for (int c = 0; c < 4; ++c) sm[c][threadIdx.x] = q[c];
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int c = 0; c < 4; ++c) sm[c][threadIdx.x] += sm[c][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 3) mean[threadIdx.x] = sm[threadIdx.x][0] / sm[3][0];
}

__global__ void k_ic_shift(int n, double* __restrict__ vel, const double* __restrict__ mean) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int a = 0; a < 3; ++a) vel[3 * size_t(i) + a] -= mean[a];
}

DevBuf g_ic_key, g_ic_key_alt, g_ic_idx, g_ic_idx_alt, g_ic_flag, g_ic_scan, g_ic_menc, g_ic_part;
ScanScratch g_ic_scratch;

}  // namespace

// params (code units): M_tot, f_baryon, R0, spin, u_gas, disk_frac, rd, z0, n_clumps,
// clump_frac, a_clump, u_lo, u_hi. Host-side layout arithmetic follows synthetic.disk_halo.
void ic_generate(int kind, int n_gas, int n_dm, uint64_t seed, const double* prm, double* pos, double* vel,
                 double* mass, int8_t* kind_out, double* u, cudaStream_t s) {
    const double M_tot = prm[0], f_b = prm[1], R0 = prm[2], spin = prm[3];
    IcSpec S{};
    S.kind = kind;
    S.n_gas = n_gas;
    S.n_dm = n_dm;
    S.seed = seed;
    S.R0 = R0;
    S.M_tot = M_tot;
    S.m_gas = f_b * M_tot / n_gas;
    S.m_dm = n_dm > 0 ? (1 - f_b) * M_tot / n_dm : 0.0;
    if (kind == 0) {
        S.u_gas = prm[4];
        S.kappa = spin / 0.47;
        S.v_vir = sqrt(M_tot / R0);
        S.n_disk = S.n_smooth = 0;
    } else {
        const int n_clumps = int(prm[8]);
        S.n_disk = int(std::lround(prm[5] * n_gas));
        S.n_cl_each = n_clumps ? int(std::lround(prm[9] * n_gas)) : 0;
        int n_cl = n_clumps * S.n_cl_each;
        n_cl = std::min(n_cl, S.n_disk);
        S.n_clumps = S.n_cl_each ? n_cl / S.n_cl_each : 0;
        S.n_smooth = S.n_disk - S.n_clumps * S.n_cl_each;
        S.n_disk = S.n_smooth + S.n_clumps * S.n_cl_each;
        S.rd = prm[6];
        S.z0 = prm[7];
        S.a_cl = prm[10];
        S.ln_u_lo = std::log(prm[11]);
        S.ln_u_hi = std::log(prm[12]);
    }
    const int n = n_gas + n_dm;
    const int grid = div_up(n, kThreads);
    uint64_t* key = nullptr;
    int* idx = nullptr;
    double* menc = nullptr;
    if (kind == 1) {
        key = g_ic_key.get<uint64_t>(n);
        idx = g_ic_idx.get<int>(n);
        menc = g_ic_menc.get<double>(n);
    }
    k_ic_place<<<grid, kThreads, 0, s>>>(S, pos, mass, kind_out, u, key, idx);
    GF_CHECK_LAUNCH();
    if (kind == 1) {
        radix_sort_pairs(key, idx, g_ic_key_alt.get<uint64_t>(n), g_ic_idx_alt.get<int>(n), n, 0, 64, s,
                         &g_ic_scratch);
        int* flag = g_ic_flag.get<int>(n);
        int* gscan = g_ic_scan.get<int>(n);
        k_ic_gasflag<<<grid, kThreads, 0, s>>>(n, n_gas, idx, flag);
        GF_CHECK_LAUNCH();
        exclusive_scan(flag, gscan, n, nullptr, s, &g_ic_scratch);
        k_ic_menc<<<grid, kThreads, 0, s>>>(n, idx, flag, gscan, S.m_gas, S.m_dm, menc);
        GF_CHECK_LAUNCH();
    }
    k_ic_vel<<<grid, kThreads, 0, s>>>(S, pos, menc, vel);
    GF_CHECK_LAUNCH();
    double* part = g_ic_part.get<double>(4 * size_t(grid) + 4);
    k_ic_momentum<<<grid, kThreads, 0, s>>>(n, vel, mass, part);
    GF_CHECK_LAUNCH();
    double* mean = part + 4 * size_t(grid);
    k_ic_momentum_final<<<1, kThreads, 0, s>>>(grid, part, mean);
    GF_CHECK_LAUNCH();
    k_ic_shift<<<grid, kThreads, 0, s>>>(n, vel, mean);
    GF_CHECK_LAUNCH();
}

}  // namespace gf
