"""CPU restatement of the thermal update of the step loop (TEST INFRASTRUCTURE ONLY).

Follows GalaxyFormation._thermodynamics (galaxy_formation/simulation.py:97-104) and the
radiative cooling of a primordial gas (galaxy_formation/cooling.py:24-43): the explicit
compression / shock-heating update u += dt du/dt floored at the 1e4 K energy, then the cooling
function of Cen (1992) plus bremsstrahlung, removed explicitly over dt and bounded by the
floor. Float64 NumPy with the reference's order of operations; the unit constants are the
reference's (units.py:17-35), restated in galaxy_formation_gb300/params.py.
"""

import numpy as np

T_FLOOR = 1e4


def cooling_function(T):
    """Lambda(T) in erg cm^3 / s (cooling.py:24-31)."""
    T = np.maximum(T, 1.0)
    f = 1 / (1 + np.sqrt(T / 1e5))
    lam = (7.5e-19 * np.exp(-118348 / T) * f
           + 5.54e-17 * T ** -0.397 * np.exp(-473638 / T) * f
           + 1.42e-27 * 1.1 * np.sqrt(T))
    return np.where(T > T_FLOOR, lam, 0.0)


def cool(u, T, rho, dt, blocked, u_floor, units):
    """New specific energy after dt (cooling.py:34-43); units: RHO_CGS, X_H, M_H, MYR,
    SEC_PER_MYR, U_CGS."""
    rho_cgs = rho * units["RHO_CGS"]
    nH = units["X_H"] * rho_cgs / units["M_H"]
    dudt_cgs = cooling_function(T) * nH ** 2 / rho_cgs
    du = dudt_cgs * dt * units["MYR"] * units["SEC_PER_MYR"] / units["U_CGS"]
    du = np.where(blocked, 0.0, du)
    return np.maximum(u - du, u_floor)


def units_of(params):
    """The constants cool() needs, from galaxy_formation_gb300.params."""
    return {"RHO_CGS": params.RHO_CGS, "X_H": params.X_H, "M_H": params.M_H, "MYR": params.MYR,
            "SEC_PER_MYR": params.SEC_PER_MYR, "U_CGS": params.U_CGS}


def thermodynamics(u, g, dudt, rho, dt, u_per_K, u_floor, units, mode=2, blocked=None):
    """simulation.py:97-104 on u (in place) for the gas g of the last SPH evaluation; mode 1
    stops after the compression / shock-heating update, mode 2 also cools, except where
    blocked (inside a supernova bubble: no_cool_until[g] > t)."""
    if rho.size == 0 or mode == 0:
        return
    u[g] = np.maximum(u[g] + dt * dudt, u_floor)
    if mode == 2:
        b = np.zeros(g.size, bool) if blocked is None else blocked
        u[g] = cool(u[g], u[g] / u_per_K, rho, dt, b, u_floor, units)
