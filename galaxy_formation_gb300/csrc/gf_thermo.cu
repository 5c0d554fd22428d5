// gf_thermo.cu — the thermal update of the step loop on the device:
//   * the explicit compression / shock-heating update of GalaxyFormation._thermodynamics
//     (galaxy_formation/simulation.py:97-102): u += dt du/dt, floored at the 1e4 K energy;
//   * radiative cooling of a primordial gas (galaxy_formation/cooling.py:24-43): the cooling
//     function of Cen (1992) plus bremsstrahlung, removed explicitly over dt and bounded by
//     the floor.
// Float64 throughout, with the reference's order of operations and no contracted
// multiply-adds (explicitly rounded intrinsics), so the only differences from NumPy are those
// of exp, pow and sqrt (within an ulp or two).
#include "gf_thermo.cuh"

namespace gf {

namespace {

constexpr int kThreads = 256;
constexpr double kTFloor = 1e4;  // cooling.py:21

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// cooling.py:24-31: Lambda(T) in erg cm^3 / s, 0 at or below the floor
__device__ double cooling_lambda(double T) {
    const double Tc = fmax(T, 1.0);
    const double f = dvd(1.0, add(1.0, sqrt(dvd(Tc, 1e5))));
    const double h = mul(mul(7.5e-19, exp(dvd(-118348.0, Tc))), f);
    const double he = mul(mul(mul(5.54e-17, pow(Tc, -0.397)), exp(dvd(-473638.0, Tc))), f);
    const double ff = mul(mul(1.42e-27, 1.1), sqrt(Tc));
    const double lam = add(add(h, he), ff);
    return Tc > kTFloor ? lam : 0.0;
}

// cooling.py:34-43 for one particle
__device__ double cool_one(double u, double T, double rho, double dt, bool blocked, double u_floor,
                           const ThermoUnits& U) {
    const double rho_cgs = mul(rho, U.rho_cgs);
    const double nH = dvd(mul(U.x_h, rho_cgs), U.m_h);
    const double dudt_cgs = dvd(mul(cooling_lambda(T), mul(nH, nH)), rho_cgs);
    double du = dvd(mul(mul(mul(dudt_cgs, dt), U.myr), U.sec_per_myr), U.u_cgs);
    if (blocked) du = 0.0;
    return fmax(add(u, -du), u_floor);
}

__global__ void k_cooling_function(int n, const double* __restrict__ T, double* __restrict__ lam) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) lam[i] = cooling_lambda(T[i]);
}

__global__ void k_cool(int n, const double* __restrict__ u, const double* __restrict__ T,
                       const double* __restrict__ rho, const double* __restrict__ dt,
                       const uint8_t* __restrict__ blocked, double u_floor, ThermoUnits U,
                       double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = cool_one(u[i], T[i], rho[i], dt[i], blocked && blocked[i] != 0, u_floor, U);
}

// simulation.py:97-104 for the ng gas particles of the last SPH evaluation (gas-local order,
// gidx -> particle): heating/compression, then (mode 2) cooling at the updated temperature
// no_cool (may be null): particles with no_cool > t sit in a supernova bubble and do not cool
__global__ void k_thermo_gas(int ng, const int* __restrict__ gidx, const double* __restrict__ rho,
                             const double* __restrict__ dudt, double* __restrict__ u, double dt, int mode,
                             const double* __restrict__ no_cool, double t, ThermoUnits U) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int i = gidx[g];
    double ui = fmax(add(u[i], mul(dt, dudt[g])), U.u_floor);
    if (mode == 2) ui = cool_one(ui, dvd(ui, U.u_per_k), rho[g], dt, no_cool && no_cool[i] > t, U.u_floor, U);
    u[i] = ui;
}

// Block time steps: the gas due at sub-step `sub` (level j with sub mod 2^j == 0) advances u
// over its own step 2^j delta with the rate of its last evaluation, before its evaluation at
// this sub-step (delta: float64 bits on the device)
// t_block: time at the block start (device); the sub-step's time is t_block + sub delta
__global__ void k_thermo_levels(int ng, const int* __restrict__ gidx, const int8_t* __restrict__ level, int sub,
                                const unsigned long long* __restrict__ dbits, const double* __restrict__ rho,
                                const double* __restrict__ dudt, double* __restrict__ u, int mode,
                                const double* __restrict__ no_cool, const double* __restrict__ t_block,
                                ThermoUnits U) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int i = gidx[g];
    const int j = level[i];
    if (sub & ((1 << j) - 1)) return;
    const double delta = __longlong_as_double((long long)*dbits);
    const double dt = delta * double(1 << j);
    double ui = fmax(add(u[i], mul(dt, dudt[g])), U.u_floor);
    if (mode == 2) {
        const bool blocked = no_cool && no_cool[i] > *t_block + delta * double(sub);
        ui = cool_one(ui, dvd(ui, U.u_per_k), rho[g], dt, blocked, U.u_floor, U);
    }
    u[i] = ui;
}

}  // namespace

void thermo_gas_levels(int ng, const int* gidx, const int8_t* level, int sub, const unsigned long long* dbits,
                       const double* rho, const double* dudt, double* u, int mode, const double* no_cool,
                       const double* t_block, const ThermoUnits& U, cudaStream_t s) {
    if (ng <= 0 || mode == 0) return;
    k_thermo_levels<<<div_up(ng, kThreads), kThreads, 0, s>>>(ng, gidx, level, sub, dbits, rho, dudt, u, mode,
                                                              no_cool, t_block, U);
    GF_CHECK_LAUNCH();
}

void cooling_function(int n, const double* T, double* lam, cudaStream_t s) {
    if (n <= 0) return;
    k_cooling_function<<<div_up(n, kThreads), kThreads, 0, s>>>(n, T, lam);
    GF_CHECK_LAUNCH();
}

void cool(int n, const double* u, const double* T, const double* rho, const double* dt, const uint8_t* blocked,
          double u_floor, const ThermoUnits& U, double* out, cudaStream_t s) {
    if (n <= 0) return;
    k_cool<<<div_up(n, kThreads), kThreads, 0, s>>>(n, u, T, rho, dt, blocked, u_floor, U, out);
    GF_CHECK_LAUNCH();
}

void thermo_gas(int ng, const int* gidx, const double* rho, const double* dudt, double* u, double dt, int mode,
                const double* no_cool, double t, const ThermoUnits& U, cudaStream_t s) {
    if (ng <= 0 || mode == 0) return;
    k_thermo_gas<<<div_up(ng, kThreads), kThreads, 0, s>>>(ng, gidx, rho, dudt, u, dt, mode, no_cool, t, U);
    GF_CHECK_LAUNCH();
}

}  // namespace gf
