// gf_stars.cuh — star formation and supernova feedback of the step loop on the device
// (galaxy_formation/star_formation.py:35-65, GalaxyFormation._stars, simulation.py:106-110).
#pragma once

#include "gf_common.cuh"

namespace gf {

// Parameters, in the order gf_sim_stars takes them (config.py:21-26, star_formation.py:29-30,
// units.py, simulation.py:40-46): the density threshold rho_sf (code units), sf_eff, fb_eff,
// fb_ngb, the bubble lifetime fb_myr / MYR (code units), E_SN_PER_MSUN (erg), MSUN, MSUN_G,
// U_CGS, u_per_K.
struct StarParams {
    double rho_sf, sf_eff, fb_eff, fb_ngb, fb_time, e_sn_per_msun, msun, msun_g, u_cgs, u_per_k;
};

// NumPy's PCG64 bit generator (128-bit LCG, XSL-RR output) as four words: state high, state
// low, increment high, increment low. Generator.uniform draws (next_uint64 >> 11) * 2^-53.
struct Pcg64 {
    unsigned long long w[4];
};

// One call of _stars(dt) at time t (after the sub-step's time advance) for the gas of the last
// SPH evaluation (ng particles, gas-local order gidx, densities rho): form_stars with the
// uniforms of `rng` (advanced on the device by the number of dense particles, as
// rng.uniform(size=p.size)), then supernova_feedback on the current gas. kind, birth, u and
// no_cool (per particle) are updated in place. Returns the number of new stars (synchronises s).
int form_stars_and_feedback(int n, int ng, const int* gidx, const double* rho, const double* pos,
                            const double* mass, int8_t* kind, double* u, double* birth, double* no_cool,
                            double dt, double t, const StarParams& P, Pcg64* rng_dev, cudaStream_t s);

}  // namespace gf
