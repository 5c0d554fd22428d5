"""Physical constants and force-path parameters.

Code units have G = 1, length 3.5 kpc and mass 4e10 Msun (galaxy_formation/units.py:17-21
of the reference); the defaults below are the reference's (galaxy_formation/config.py:7-38,
galaxy_formation/sph.py:26-28, galaxy_formation/simulation.py:39).
"""

import math

# unit system (units.py:17-35)
G_KPC = 4.30091e-6                      # kpc (km/s)^2 / Msun
KPC = 3.5                               # length unit in kpc
MSUN = 4e10                             # mass unit in Msun
KMS = math.sqrt(G_KPC * MSUN / KPC)     # velocity unit in km/s
MYR = KPC / KMS * 977.79                # time unit in Myr
M_H = 1.6726e-24
K_B = 1.381e-16
MSUN_G = 1.989e33
KPC_CM = 3.086e21
YR_S = 3.156e7
RHO_CGS = MSUN * MSUN_G / (KPC * KPC_CM) ** 3
U_CGS = (KMS * 1e5) ** 2
SEC_PER_MYR = 1e6 * YR_S
X_H = 0.76
MU_IONISED = 0.6

# particle kinds (initial_conditions.py:22)
GAS, STAR, DM = 0, 1, 2

# numerics (config.py:29-30) and SPH constants (sph.py:26-28, simulation.py:39)
THETA = 0.7
EPS_KPC = 0.4
EPS = EPS_KPC / KPC
N_NEIGHBOURS = 32
N_CANDIDATES = 48
ALPHA, BETA = 1.0, 2.0
GAMMA = 5.0 / 3.0
U_PER_K = K_B / ((GAMMA - 1) * MU_IONISED * M_H) / U_CGS
T_FLOOR = 1e4                            # cooling.py:21
U_FLOOR = T_FLOOR * U_PER_K              # simulation.py:42

# constants of the thermal update of the step loop, in the order gf_sim_thermo takes them
THERMO_UNITS = (U_PER_K, U_FLOOR, RHO_CGS, X_H, M_H, MYR, SEC_PER_MYR, U_CGS)
