"""Host-side parameters of the device sub-grid physics (gf_sim_thermo, gf_sim_stars).

The constants are the reference's (galaxy_formation/config.py:21-26, units.py:17-35,
simulation.py:40-46, star_formation.py:29-30); `star_params` packs them in the order
gf_sim_stars takes. The device draws the star-formation uniforms of NumPy's PCG64 stream:
`pcg64_words` / `set_pcg64_words` move a Generator's state to and from the four 64-bit words
the library uses (state high, state low, increment high, increment low), so a run on the GPU
consumes the same stream as the reference's `rng.uniform` calls would.
"""

import numpy as np

from . import params

N_SF = 1.0             # star-formation density threshold (H atoms / cm^3), config.py:21
SF_EFF = 0.005         # efficiency per free-fall time, config.py:22
FB_EFF = 0.4           # supernova energy coupled, in units of 1e49 erg / Msun formed, config.py:23
FB_NGB = 16            # gas neighbours heated per new star, config.py:24
FB_MYR = 30.0          # bubble lifetime (Myr), config.py:25
E_SN_PER_MSUN = 1e49   # erg per Msun of stars formed, star_formation.py:30
T_SF_MAX = 3e4         # star_formation.py:29


def rho_sf(n_sf=N_SF):
    """The density threshold in code units (simulation.py:46)."""
    return n_sf * params.M_H / params.X_H / params.RHO_CGS


def star_params(n_sf=N_SF, sf_eff=SF_EFF, fb_eff=FB_EFF, fb_ngb=FB_NGB, fb_myr=FB_MYR):
    """The 10 parameters of gf_sim_stars, in its order."""
    return np.array([rho_sf(n_sf), sf_eff, fb_eff, float(fb_ngb), fb_myr / params.MYR, E_SN_PER_MSUN,
                     params.MSUN, params.MSUN_G, params.U_CGS, params.U_PER_K], dtype=np.float64)


def pcg64_words(rng):
    """The PCG64 state of a numpy Generator as 4 uint64 words (state hi, lo, inc hi, lo)."""
    st = rng.bit_generator.state
    if st["bit_generator"] != "PCG64":
        raise ValueError("the device draws NumPy's PCG64 stream only")
    s, inc = st["state"]["state"], st["state"]["inc"]
    m = (1 << 64) - 1
    return np.array([s >> 64, s & m, inc >> 64, inc & m], dtype=np.uint64)


def set_pcg64_words(rng, words):
    """Moves a numpy Generator (PCG64) to the state of 4 words."""
    w = [int(x) for x in words]
    st = rng.bit_generator.state
    st["state"] = {"state": (w[0] << 64) | w[1], "inc": (w[2] << 64) | w[3]}
    st["has_uint32"], st["uinteger"] = 0, 0
    rng.bit_generator.state = st
