// gf_thermo.cuh — thermal update of the step loop (simulation.py:97-104, cooling.py:24-43).
#pragma once

#include "gf_common.cuh"

namespace gf {

// Unit constants of the thermal update (galaxy_formation/units.py:17-35, simulation.py:40-42),
// supplied by the caller in this order through the C ABI.
struct ThermoUnits {
    double u_per_k;      // specific energy per kelvin (code units)
    double u_floor;      // energy at the 1e4 K floor
    double rho_cgs;      // density unit (g/cm^3)
    double x_h;          // hydrogen mass fraction
    double m_h;          // hydrogen mass (g)
    double myr;          // time unit in Myr
    double sec_per_myr;  // seconds per Myr
    double u_cgs;        // specific-energy unit (erg/g)
};

// cooling.py:24-31 elementwise
void cooling_function(int n, const double* T, double* lam, cudaStream_t s);
// cooling.py:34-43 elementwise (dt per particle; blocked may be null)
void cool(int n, const double* u, const double* T, const double* rho, const double* dt, const uint8_t* blocked,
          double u_floor, const ThermoUnits& U, double* out, cudaStream_t s);
// simulation.py:97-104 on the gas of the last SPH evaluation at time t: mode 1
// heating/compression only, mode 2 also cooling, except for particles with no_cool > t (inside a
// supernova bubble; no_cool may be null)
void thermo_gas(int ng, const int* gidx, const double* rho, const double* dudt, double* u, double dt, int mode,
                const double* no_cool, double t, const ThermoUnits& U, cudaStream_t s);

// Block time steps: the gas due at sub-step `sub` (level j, sub mod 2^j == 0) advances u over
// its step 2^j delta (delta as float64 bits at dbits) before its evaluation there; the time of
// the sub-step is *t_block + sub delta (device values)
void thermo_gas_levels(int ng, const int* gidx, const int8_t* level, int sub, const unsigned long long* dbits,
                       const double* rho, const double* dudt, double* u, int mode, const double* no_cool,
                       const double* t_block, const ThermoUnits& U, cudaStream_t s);

}  // namespace gf
