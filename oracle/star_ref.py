"""CPU restatement of star formation and supernova feedback (TEST INFRASTRUCTURE ONLY).

Follows galaxy_formation/star_formation.py:35-65 (form_stars, supernova_feedback) as called
by GalaxyFormation._stars (simulation.py:106-110): stochastic conversion of dense, cold gas
with NumPy's Generator, then heating of the fb_ngb nearest gas particles of each new star
(scipy's cKDTree, the reference's own call) and their cooling switched off for fb_myr.
Float64 NumPy with the reference's order of operations.
"""

import numpy as np
from scipy.spatial import cKDTree

GAS, STAR = 0, 1
T_SF_MAX = 3e4          # star_formation.py:29


def form_stars(state, g, rho, dt, P, rng):
    """star_formation.py:35-47 on state (dict: u, kind, birth, t) for the gas g of the last
    SPH evaluation with densities rho; P: the parameter dict of star_params."""
    dense = (rho > P["rho_sf"]) & (state["u"][g] / P["u_per_K"] < T_SF_MAX)
    if not np.any(dense):
        return g[:0]
    t_ff = np.sqrt(3 * np.pi / (32 * rho[dense]))      # G = 1
    p = 1 - np.exp(-P["sf_eff"] * dt / t_ff)
    new = g[dense][rng.uniform(size=p.size) < p]
    state["kind"][new] = STAR
    state["birth"][new] = state["t"]
    return new


def supernova_feedback(state, new, P):
    """star_formation.py:50-65 on state (dict: pos, mass, kind, u, no_cool_until, t)."""
    if P["fb_eff"] <= 0 or new.size == 0:
        return
    g = np.flatnonzero(state["kind"] == GAS)
    if g.size < 10:
        return
    k = min(int(P["fb_ngb"]), g.size)
    _, nb = cKDTree(state["pos"][g]).query(state["pos"][new], k=k, workers=-1)
    targets = g[np.asarray(nb).reshape(len(new), k)]
    e_per_g = P["fb_eff"] * P["e_sn_per_msun"] / P["msun_g"]
    E = e_per_g * state["mass"][new] * P["msun"] * P["msun_g"]
    du = E[:, None] / k / (state["mass"][targets] * P["msun"] * P["msun_g"]) / P["u_cgs"]
    np.add.at(state["u"], targets.ravel(), du.ravel())
    state["no_cool_until"][targets.ravel()] = state["t"] + P["fb_time"]


def param_dict(values):
    """The 10 values of galaxy_formation_gb300.subgrid.star_params as a dict."""
    names = ("rho_sf", "sf_eff", "fb_eff", "fb_ngb", "fb_time", "e_sn_per_msun", "msun", "msun_g", "u_cgs",
             "u_per_K")
    return dict(zip(names, (float(v) for v in values)))
