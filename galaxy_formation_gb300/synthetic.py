"""Seeded synthetic particle sets for the force path (all float64, code units).

* `rotating_cloud` restates the reference's initial cloud (galaxy_formation/
  initial_conditions.py:25-68): random directions, radii with M(<r) ~ r^2 (density ~ 1/r)
  inside R0, rotation from the spin parameter, 10 % velocity dispersion and no bulk motion.
  With the reference's defaults (5,000 gas + 5,000 dark matter, seed 3) it reproduces the
  reference's arrays bit for bit (checked against a committed fixture). `solid_body=True`
  gives the variant with solid-body rotation scaled to the spin parameter and no
  dispersion.
* `disk_halo` (no reference counterpart): a dark-matter halo with density ~ 1/r out to
  100 kpc, an exponential gas disk (scale length 3 kpc, sech^2 scale height 0.3 kpc)
  holding 60 % of the baryons and the rest of the gas in a 1/r cloud; circular velocities
  from the enclosed mass plus 10 % Gaussian dispersion; gas temperatures log-uniform over
  1e4-1e6 K. `clumps` adds seeded Plummer spheres (each `clump_frac` of the gas mass,
  radius `clump_kpc`) carved out of the disk gas.

Each generator returns a dict with pos (n,3), vel (n,3), mass (n,), kind (n,) int8 and
u (n,) specific internal energy; gas comes first, then dark matter.

`make_config_device` draws the same workloads on the GPU (gf_ic_generate: counter-based
random numbers, the same distributions, not the same streams), for sizes where the host
generators take long (4M particles and up).
"""

import numpy as np

from .params import DM, GAS, KPC, MSUN, U_PER_K


def _random_ball(n, R0, exponent, rng):
    # initial_conditions.py:25-30
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v * R0 * rng.uniform(0, 1, n)[:, None] ** exponent


def rotating_cloud(n_gas=5000, n_dm=5000, seed=3, mass=2.8e11, f_baryon=0.16, r0=100.0,
                   spin=0.05, t_gas=1e4, profile="extended", solid_body=False, rng=None):
    """The reference's cold rotating cloud (initial_conditions.py:33-68)."""
    rng = np.random.default_rng(seed) if rng is None else rng
    M_tot = mass / MSUN
    R0 = r0 / KPC
    exponent = 1 / 3 if profile == "uniform" else 1 / 2
    pos = np.ascontiguousarray(np.concatenate([_random_ball(n_gas, R0, exponent, rng),
                                               _random_ball(n_dm, R0, exponent, rng)]))
    m = np.concatenate([np.full(n_gas, f_baryon * M_tot / n_gas),
                        np.full(n_dm, (1 - f_baryon) * M_tot / n_dm)])
    kind = np.concatenate([np.full(n_gas, GAS, np.int8), np.full(n_dm, DM, np.int8)])
    ez = np.array([0.0, 0.0, 1.0])
    r = np.linalg.norm(pos, axis=1)
    if profile == "uniform" or solid_body:
        if profile == "uniform":
            Om = spin * np.sqrt(M_tot) / (0.4 * np.sqrt(0.6) * R0 ** 1.5)
        else:
            # solid body in a 1/r sphere: J = (1/3) M R0^2 Omega and |E| = 2 G M^2 / (3 R0)
            # (M(<r) ~ r^2); lambda = J |E|^1/2 / (G M^5/2) gives Omega below.
            Om = spin * np.sqrt(M_tot) / ((1 / 3) * np.sqrt(2 / 3) * R0 ** 1.5)
        vel = np.cross(Om * ez, pos)
    else:
        kappa = spin / 0.47
        vc = np.sqrt(M_tot * (r / R0) ** 2 / np.maximum(r, 1e-6))
        phi_hat = np.cross(ez, pos)
        phi_hat /= np.linalg.norm(phi_hat, axis=1, keepdims=True) + 1e-30
        R_cyl = np.hypot(pos[:, 0], pos[:, 1])
        vel = (kappa * vc * R_cyl / np.maximum(r, 1e-6))[:, None] * phi_hat
    if not solid_body:
        v_vir = np.sqrt(M_tot / R0)
        vel += 0.1 * v_vir * rng.normal(size=pos.shape) / np.sqrt(3)
    vel = np.ascontiguousarray(vel - np.average(vel, axis=0, weights=m))
    u = np.zeros(len(m))
    u[:n_gas] = t_gas * U_PER_K
    return {"pos": pos, "vel": vel, "mass": m, "kind": kind, "u": u}


def _sech2_heights(n, z0, rng):
    # p(z) ~ sech^2(z / z0): inverse CDF z = z0 atanh(2 U - 1)
    return z0 * np.arctanh(np.clip(2 * rng.uniform(size=n) - 1, -1 + 1e-12, 1 - 1e-12))


def _exp_disk_radii(n, Rd, Rmax, rng):
    # surface density ~ exp(-R/Rd): R = Rd * Gamma(2) deviate, truncated at Rmax
    R = np.empty(0)
    while R.size < n:
        x = rng.gamma(2.0, Rd, size=2 * (n - R.size) + 16)
        R = np.concatenate([R, x[x < Rmax]])
    return R[:n]


def disk_halo(n_gas=100_000, n_dm=100_000, seed=3, mass=2.8e11, f_baryon=0.16, r0=100.0,
              disk_frac=0.6, rd_kpc=3.0, z0_kpc=0.3, n_clumps=0, clump_frac=1e-3,
              clump_kpc=0.2, t_lo=1e4, t_hi=1e6):
    """Collapsed disk + 1/r halo snapshot (optionally with Plummer clumps)."""
    rng = np.random.default_rng(seed)
    M_tot = mass / MSUN
    R0 = r0 / KPC
    Rd, z0, a_cl = rd_kpc / KPC, z0_kpc / KPC, clump_kpc / KPC
    m_gas = f_baryon * M_tot / n_gas
    m_dm = (1 - f_baryon) * M_tot / max(n_dm, 1)

    n_disk = int(round(disk_frac * n_gas))
    n_cl_each = int(round(clump_frac * n_gas)) if n_clumps else 0
    n_cl = n_clumps * n_cl_each
    n_cl = min(n_cl, n_disk)
    n_smooth_disk = n_disk - n_cl
    n_cloud = n_gas - n_disk

    # smooth exponential disk
    R = _exp_disk_radii(n_smooth_disk, Rd, 12 * Rd, rng)
    ph = rng.uniform(0, 2 * np.pi, n_smooth_disk)
    disk = np.stack([R * np.cos(ph), R * np.sin(ph), _sech2_heights(n_smooth_disk, z0, rng)], 1)
    parts = [disk]
    if n_cl:
        # clump centres drawn from the disk itself; Plummer radii r = a / sqrt(U^-2/3 - 1)
        Rc = _exp_disk_radii(n_clumps, Rd, 6 * Rd, rng)
        phc = rng.uniform(0, 2 * np.pi, n_clumps)
        cen = np.stack([Rc * np.cos(phc), Rc * np.sin(phc), _sech2_heights(n_clumps, z0, rng)], 1)
        U = rng.uniform(1e-6, 0.999, size=(n_clumps, n_cl_each))
        rr = a_cl / np.sqrt(U ** (-2.0 / 3.0) - 1.0)
        d = rng.normal(size=(n_clumps, n_cl_each, 3))
        d /= np.linalg.norm(d, axis=2, keepdims=True)
        parts.append((cen[:, None, :] + d * rr[..., None]).reshape(-1, 3))
    parts.append(_random_ball(n_cloud, R0, 0.5, rng))
    gas = np.concatenate(parts)
    dm = _random_ball(n_dm, R0, 0.5, rng)
    pos = np.ascontiguousarray(np.concatenate([gas, dm]))
    m = np.concatenate([np.full(n_gas, m_gas), np.full(n_dm, m_dm)])
    kind = np.concatenate([np.full(n_gas, GAS, np.int8), np.full(n_dm, DM, np.int8)])

    # circular velocity from the spherically averaged enclosed mass
    r = np.linalg.norm(pos, axis=1)
    order = np.argsort(r, kind="stable")
    menc = np.empty_like(r)
    menc[order] = np.cumsum(m[order])
    vc = np.sqrt(menc / np.maximum(r, 1e-6))
    ez = np.array([0.0, 0.0, 1.0])
    phi_hat = np.cross(ez, pos)
    phi_hat /= np.linalg.norm(phi_hat, axis=1, keepdims=True) + 1e-30
    R_cyl = np.hypot(pos[:, 0], pos[:, 1])
    # disk gas rotates at v_c; halo and cloud particles carry a slow rotation (spin 0.05)
    rot = np.where(np.arange(len(m)) < n_disk, 1.0, 0.05 / 0.47 * R_cyl / np.maximum(r, 1e-6))
    vel = (rot * vc)[:, None] * phi_hat
    vel += 0.1 * vc[:, None] * rng.normal(size=pos.shape) / np.sqrt(3)
    vel = np.ascontiguousarray(vel - np.average(vel, axis=0, weights=m))

    u = np.zeros(len(m))
    u[:n_gas] = np.exp(rng.uniform(np.log(t_lo), np.log(t_hi), n_gas)) * U_PER_K
    return {"pos": pos, "vel": vel, "mass": m, "kind": kind, "u": u}


# The five workloads of the benchmark description (particle counts and generators).
CONFIGS = {
    0: dict(gen="cloud", n_gas=5_000, n_dm=5_000),
    1: dict(gen="disk", n_gas=100_000, n_dm=100_000),
    2: dict(gen="disk", n_gas=500_000, n_dm=500_000),
    3: dict(gen="disk", n_gas=1_000_000, n_dm=0, n_clumps=200),
    4: dict(gen="cloud", n_gas=2_000_000, n_dm=2_000_000),
}


# defaults of the two generators above, in their units
CLOUD_DEFAULTS = dict(mass=2.8e11, f_baryon=0.16, r0=100.0, spin=0.05, t_gas=1e4)
DISK_DEFAULTS = dict(mass=2.8e11, f_baryon=0.16, r0=100.0, disk_frac=0.6, rd_kpc=3.0, z0_kpc=0.3,
                     n_clumps=0, clump_frac=1e-3, clump_kpc=0.2, t_lo=1e4, t_hi=1e6)


def device_params(gen, **kw):
    """(kind, the 13 code-unit parameters of gf_ic_generate) of a generator and overrides."""
    if gen == "cloud":
        c = dict(CLOUD_DEFAULTS, **kw)
        return 0, np.array([c["mass"] / MSUN, c["f_baryon"], c["r0"] / KPC, c["spin"], c["t_gas"] * U_PER_K,
                            0, 1, 1, 0, 0, 1, 1, 1], np.float64)
    c = dict(DISK_DEFAULTS, **kw)
    return 1, np.array([c["mass"] / MSUN, c["f_baryon"], c["r0"] / KPC, 0.05, 0.0, c["disk_frac"],
                        c["rd_kpc"] / KPC, c["z0_kpc"] / KPC, c["n_clumps"], c["clump_frac"],
                        c["clump_kpc"] / KPC, c["t_lo"] * U_PER_K, c["t_hi"] * U_PER_K], np.float64)


def make_config_device(idx, seed=3, scale=1.0, lib=None):
    """Workload `idx` drawn on the GPU (gf_ic_generate), returned in host arrays."""
    from . import _lib

    lib = lib or _lib.load()
    c = dict(CONFIGS[idx])
    gen = c.pop("gen")
    n_gas = max(1, int(c.pop("n_gas") * scale))
    n_dm = int(c.pop("n_dm") * scale)
    kind, prm = device_params(gen, **c)
    n = n_gas + n_dm
    out = {"pos": np.empty((n, 3)), "vel": np.empty((n, 3)), "mass": np.empty(n), "kind": np.empty(n, np.int8),
           "u": np.empty(n)}
    _lib.check(lib.gf_ic_generate(kind, n_gas, n_dm, seed, prm, len(prm), out["pos"], out["vel"], out["mass"],
                                  out["kind"], out["u"]))
    return out


def make_config(idx, seed=3, scale=1.0):
    """Particle set of workload `idx` (0-4); `scale` shrinks the particle counts for tests."""
    c = dict(CONFIGS[idx])
    gen = c.pop("gen")
    c["n_gas"] = max(1, int(c["n_gas"] * scale))
    c["n_dm"] = int(c["n_dm"] * scale)
    if gen == "cloud":
        return rotating_cloud(seed=seed, **c)
    return disk_halo(seed=seed, **c)
