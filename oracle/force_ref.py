"""CPU restatement of one force evaluation (TEST INFRASTRUCTURE ONLY).

Follows GalaxyFormation.accelerations / _hydro (galaxy_formation/simulation.py:61-95) and
NeighbourFinder.find (galaxy_formation/sph.py:151-170) line by line, with:
  * gravity ............ oracle.accel_active (restatement of cpp/nbody.cpp, OpenMP);
  * full neighbour search scipy.spatial.cKDTree(p).query(p, k=48, workers=-1) — the
                         reference's own call (sph.py:166);
  * Verlet reselection . oracle.knn_from_candidates (restatement of sph.py:109-135);
  * SPH forces ......... oracle.sph_forces (restatement of sph.py:57-106, OpenMP; the
                         reference runs it through numba, absent here).
Used as the checker of the fused GPU force evaluation and as the timed CPU baseline.
"""

import numpy as np
from scipy.spatial import cKDTree

import cooling_ref
import oracle
import star_ref

GAS = 0
N_NEIGHBOURS, N_CANDIDATES = 32, 48


class ForceOracle:
    def __init__(self, n, theta, eps, gamma=5.0 / 3.0, alpha=1.0, beta=2.0, use_ckdtree=True):
        self.n, self.theta, self.eps = n, theta, eps
        self.gamma, self.alpha, self.beta = gamma, alpha, beta
        self.acc_grav = np.zeros((n, 3))
        self.acc_sph = np.zeros((n, 3))
        self.dt_courant = np.full(n, np.inf)
        self.cache = None
        self.use_ckdtree = use_ckdtree
        self.full_searches = 0

    def _find(self, g, p, fresh):
        k = N_NEIGHBOURS
        if not fresh and self.cache is not None:
            row = self.cache["row"][g]
            if (row >= 0).all():
                loc = np.full(self.n, -1, np.int64)
                loc[g] = np.arange(g.size)
                cand = loc[self.cache["cand"][row]]
                nb = np.empty((g.size, k), np.int64)
                d = np.empty((g.size, k))
                if oracle.knn_from_candidates(p, cand, k, nb, d):
                    return d, nb
        kq = min(N_CANDIDATES, g.size)
        if self.use_ckdtree:
            d, nb = cKDTree(p).query(p, k=kq, workers=-1)
        else:
            d, nb = oracle.knn_brute(p, kq)
        self.full_searches += 1
        row = np.full(self.n, -1, np.int64)
        row[g] = np.arange(g.size)
        self.cache = {"row": row, "cand": g[nb]}
        return d[:, :k], np.ascontiguousarray(nb[:, :k])

    def _hydro(self, pos, vel, mass, kind, u, fresh):
        self.acc_sph[:] = 0.0
        self.dt_courant[:] = np.inf
        self.dt_gas = np.inf
        self.rho = np.zeros(0)  # simulation.py:78
        g = np.flatnonzero(kind == GAS)
        self.n_gas = g.size
        if g.size <= 40:
            return
        p = np.ascontiguousarray(pos[g])
        d, nb = self._find(g, p, fresh)
        h = np.maximum(0.5 * d[:, -1], 0.5 * self.eps)
        rho, a, dudt, dt_i = oracle.sph_forces(p, np.ascontiguousarray(vel[g]),
                                               np.ascontiguousarray(mass[g]), nb, h,
                                               np.ascontiguousarray(u[g]), self.gamma,
                                               self.alpha, self.beta)
        self.acc_sph[g] = a
        self.dt_courant[g] = dt_i
        self.dt_gas = dt_i.min()
        self.h, self.rho, self.dudt, self.nb, self.gas_idx = h, rho, dudt, nb, g

    def accelerations(self, pos, vel, mass, kind, u, active=None, rebuild=True, sph=True,
                      fresh_nb=True):
        oracle.accel_active(pos, mass, self.acc_grav, self.theta, self.eps, active, rebuild)
        if sph:
            self._hydro(pos, vel, mass, kind, u, fresh_nb)
        acc = self.acc_grav + self.acc_sph
        a_mag = np.sqrt(np.einsum("ij,ij->i", acc, acc))
        self.dt_ind = np.minimum(0.3 * np.sqrt(self.eps / np.maximum(a_mag, 1e-30)), self.dt_courant)
        self.dt_grav = 0.3 * np.sqrt(self.eps / max(a_mag.max(), 1e-30))
        return acc


class StepOracle:
    """GalaxyFormation.step (galaxy_formation/simulation.py:114-149) restated on ForceOracle.
    thermo = 0 leaves out _thermodynamics; 1 applies its compression / shock-heating update, 2
    also cooling (oracle/cooling_ref.py), with thermo_units = (u_per_K, u_floor, RHO_CGS, X_H,
    M_H, MYR, SEC_PER_MYR, U_CGS). stars (the 10 values of subgrid.star_params) with rng (a
    NumPy Generator) adds _stars (oracle/star_ref.py). State: pos, vel, mass, kind, u, birth,
    no_cool_until (float64; mass is shared, the others are copies)."""

    def __init__(self, pos, vel, mass, kind, u, theta, eps, thermo=0, thermo_units=None, stars=None, rng=None,
                 **kw):
        self.pos, self.vel = pos.copy(), vel.copy()
        self.mass, self.kind, self.u = mass, kind.copy(), u.copy()
        self.birth = np.full(len(mass), np.inf)            # simulation.py:36
        self.no_cool_until = np.full(len(mass), -np.inf)   # simulation.py:43
        self.eps = eps
        self.thermo = thermo
        self.stars = None if stars is None else star_ref.param_dict(stars)
        self.rng = rng
        if thermo:
            u_per_K, u_floor, rho_cgs, x_h, m_h, myr, sec_per_myr, u_cgs = thermo_units
            self.u_per_K, self.u_floor = u_per_K, u_floor
            self.units = {"RHO_CGS": rho_cgs, "X_H": x_h, "M_H": m_h, "MYR": myr,
                          "SEC_PER_MYR": sec_per_myr, "U_CGS": u_cgs}
        self.f = ForceOracle(len(mass), theta, eps, **kw)
        self.t = 0.0
        self.acc = self.accelerations()

    def _thermodynamics(self, dt):
        """simulation.py:97-104 on the gas of the last SPH evaluation."""
        if self.thermo and self.f.rho.size:
            g = self.f.gas_idx
            cooling_ref.thermodynamics(self.u, g, self.f.dudt, self.f.rho, dt, self.u_per_K, self.u_floor,
                                       self.units, self.thermo, blocked=self.no_cool_until[g] > self.t)

    def _stars(self, dt):
        """simulation.py:106-110."""
        if self.stars is None or self.f.rho.size == 0:
            return
        st = {"pos": self.pos, "mass": self.mass, "kind": self.kind, "u": self.u, "birth": self.birth,
              "no_cool_until": self.no_cool_until, "t": self.t}
        new = star_ref.form_stars(st, self.f.gas_idx, self.f.rho, dt, self.stars, self.rng)
        star_ref.supernova_feedback(st, new, self.stars)

    def accelerations(self, active=None, rebuild=True, sph=True, fresh_nb=True):
        acc = self.f.accelerations(self.pos, self.vel, self.mass, self.kind, self.u, active, rebuild,
                                   sph, fresh_nb)
        self.dt_ind, self.dt_grav = self.f.dt_ind, self.f.dt_grav
        self.dt_gas = self.f.dt_gas if sph else self.dt_gas
        return acc

    def step(self, dt_max):
        dt_min = min(self.dt_gas, self.dt_grav, dt_max)
        D = min(dt_max, np.percentile(self.dt_ind, 10))
        self.substeps = 0
        if D <= 1.5 * dt_min:
            self._thermodynamics(dt_min)
            self.vel += 0.5 * dt_min * self.acc
            self.pos += dt_min * self.vel
            self.acc = self.accelerations()
            self.vel += 0.5 * dt_min * self.acc
            self.t += dt_min
            self._stars(dt_min)
            self.substeps = 1
            return dt_min
        fast = (self.dt_ind < D) | (self.kind == GAS)
        slow = ~fast
        self.vel[slow] += 0.5 * D * self.acc[slow]
        tau = 0.0
        first = True
        while tau < D * (1 - 1e-9):
            dt = min(self.dt_ind[fast].min(), D - tau)
            self._thermodynamics(dt)
            self.vel[fast] += 0.5 * dt * self.acc[fast]
            self.pos += dt * self.vel
            self.acc = self.accelerations(active=fast, rebuild=False, fresh_nb=first)
            first = False
            self.vel[fast] += 0.5 * dt * self.acc[fast]
            tau += dt
            self.t += dt
            self._stars(dt)
            self.substeps += 1
        self.acc = self.accelerations(active=slow, rebuild=True, sph=False)
        self.vel[slow] += 0.5 * D * self.acc[slow]
        return D


class BlockOracle:
    """CPU restatement of the block time-step scheme of the library's batched form (power-of-two
    levels, gravity of the particles due at each sub-step on a refitted tree — or a rebuilt one
    every `rebuild_every` sub-steps — opening / full / closing kicks).

    With gas (kind given, more than 40 gas particles) each evaluation also runs the hydro step:
    the block-start and block-end evaluations are full ones (cKDTree search of 48 candidates,
    h, sph_forces of every gas particle: simulation.py:74-95); at a sub-step only the gas due
    gets its 32 neighbours re-selected among its cached candidates (sph.py:155-164), a new h,
    density, pressure and viscous forces (oracle/sph_ref.py), its neighbours that are not due
    entering with their density and h of their own last evaluation; the others keep their SPH
    acceleration and Courant step. u stays fixed (no thermal update)."""

    def __init__(self, pos, vel, mass, theta, eps, nlev, rebuild_every=0, chunk=None, kind=None, u=None,
                 gamma=5.0 / 3.0, alpha=1.0, beta=2.0):
        self.pos, self.vel, self.mass = pos.copy(), vel.copy(), mass
        self.theta, self.eps, self.nlev = theta, eps, nlev
        self.rebuild_every = rebuild_every  # tree rebuilt at sub-steps s % rebuild_every == 0
        # walk items per sub-step bin (trailing zero bits of the sub-step index); None: groups
        self.chunk = chunk
        self.acc = np.zeros_like(pos)
        self.t = 0.0
        self.gas = np.zeros(0, np.int64) if kind is None else np.flatnonzero(kind == GAS)
        self.hydro = self.gas.size > 40
        if self.hydro:
            ng = self.gas.size
            self.u = u
            self.gamma, self.alpha, self.beta = gamma, alpha, beta
            self.acc_grav = np.zeros_like(pos)
            self.acc_sph = np.zeros_like(pos)
            self.dt_courant = np.full(len(mass), np.inf)
            self.h, self.rho = np.zeros(ng), np.zeros(ng)
            self.nb = np.zeros((ng, N_NEIGHBOURS), np.int64)
        self._force(None, True)
        self._levels_and_open()

    def _hydro(self, active):
        import sph_ref

        g = self.gas
        p, v = np.ascontiguousarray(self.pos[g]), np.ascontiguousarray(self.vel[g])
        m, u = self.mass[g], self.u[g]
        if active is None:  # full search (sph.py:165-169)
            d, nb = cKDTree(p).query(p, k=min(N_CANDIDATES, g.size), workers=-1)
            self.cand = nb
            rows = np.arange(g.size)
            self.nb[:] = nb[:, :N_NEIGHBOURS]
            self.h[:] = np.maximum(0.5 * d[:, N_NEIGHBOURS - 1], 0.5 * self.eps)
        else:  # the gas due: Verlet reselection among the cached candidates
            rows = np.flatnonzero(active[g])
            sel = sph_ref.reselect(p, self.cand, rows, N_NEIGHBOURS)
            assert sel is not None, "a gas particle lost its candidates"
            self.nb[rows] = sel[0]
            self.h[rows] = np.maximum(0.5 * sel[1], 0.5 * self.eps)
        self.rho[rows] = sph_ref.density(p, m, self.nb, self.h, rows)
        a, _, dt_i, _, _ = sph_ref.forces(p, v, m, self.nb, self.h, u, self.rho, rows, self.gamma, self.alpha,
                                       self.beta)
        self.acc_sph[g[rows]] = a
        self.dt_courant[g[rows]] = dt_i

    def _force(self, active, rebuild):
        if not self.hydro:
            oracle.accel_active(self.pos, self.mass, self.acc, self.theta, self.eps, active, rebuild)
            a = np.sqrt(np.einsum("ij,ij->i", self.acc, self.acc))
            self.dt_ind = 0.3 * np.sqrt(self.eps / np.maximum(a, 1e-30))
            return
        oracle.accel_active(self.pos, self.mass, self.acc_grav, self.theta, self.eps, active, rebuild)
        self._hydro(active)
        self.acc = self.acc_grav + self.acc_sph
        a = np.sqrt(np.einsum("ij,ij->i", self.acc, self.acc))
        self.dt_ind = np.minimum(0.3 * np.sqrt(self.eps / np.maximum(a, 1e-30)), self.dt_courant)

    def _levels_and_open(self):
        self.delta = self.dt_ind.min()
        j = np.floor(np.log2(self.dt_ind / self.delta)).astype(int)
        self.level = np.clip(j, 0, self.nlev - 1)
        self.vel += (0.5 * self.delta * 2.0 ** self.level)[:, None] * self.acc

    def block(self):
        nsub = 1 << (self.nlev - 1)
        step = self.delta * 2.0 ** self.level
        for s in range(1, nsub):
            self.pos += self.delta * self.vel
            act = (s % (1 << self.level)) == 0
            rebuild = self.rebuild_every > 0 and s % self.rebuild_every == 0
            if self.chunk is not None:
                tz = (s & -s).bit_length() - 1
                oracle.set_walk_chunk(self.chunk[min(tz, len(self.chunk) - 1)])
            self._force(act.astype(np.uint8), rebuild)
            oracle.set_walk_chunk(0)
            self.vel[act] += step[act][:, None] * self.acc[act]
        self.pos += self.delta * self.vel
        self._force(None, True)
        self.vel += (0.5 * step)[:, None] * self.acc
        self.t += self.delta * nsub
        self._levels_and_open()
