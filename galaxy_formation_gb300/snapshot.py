"""Snapshots: particle sets and step-loop checkpoints as .npz files (no reference counterpart).

* `save` / `load`: a particle set (pos, vel, mass, kind, u) with optional extra arrays and
  scalars — the inputs of a force evaluation, for regression cases and replays.
* `checkpoint` / `resume`: the device step loop (gf_sim_*). A checkpoint holds the particle
  state plus what the next step starts from (accelerations and time-step limits of the last
  evaluations, the density and du/dt of the last SPH evaluation that the next thermal update
  uses, time, star-formation times, the PCG64 words of the star-formation draws);
  `resume` re-initialises the library with it (gf_sim_init at the saved positions, which
  rebuilds the same tree, then gf_sim_restore), so the run continues exactly as if it had not
  stopped. The thermal and star-formation settings are the caller's to set again, as the
  generator state is returned to it.
"""

import ctypes

import numpy as np

from . import _lib

PARTICLE_KEYS = ("pos", "vel", "mass", "kind", "u")


def save(path, pos, vel, mass, kind, u, **extra):
    """Writes a particle set (and any extra arrays / scalars) to path (.npz, compressed)."""
    arrays = {"pos": np.asarray(pos, np.float64), "vel": np.asarray(vel, np.float64),
              "mass": np.asarray(mass, np.float64), "kind": np.asarray(kind, np.int8),
              "u": np.asarray(u, np.float64)}
    n = len(arrays["mass"])
    if arrays["pos"].shape != (n, 3) or arrays["vel"].shape != (n, 3) or len(arrays["kind"]) != n \
            or len(arrays["u"]) != n:
        raise ValueError("pos/vel (n,3), mass/kind/u (n,) expected")
    np.savez_compressed(path, **arrays, **{k: np.asarray(v) for k, v in extra.items()})


def load(path):
    """Reads a snapshot: a dict of C-contiguous arrays (scalars as 0-d arrays)."""
    with np.load(path) as f:
        out = {k: (f[k] if f[k].ndim == 0 else np.ascontiguousarray(f[k])) for k in f.files}
    missing = [k for k in PARTICLE_KEYS if k not in out]
    if missing:
        raise ValueError(f"not a snapshot: missing {missing}")
    return out


def checkpoint(lib, path, mass, theta, eps, gamma, alpha, beta):
    """Saves the device step loop's state (after gf_sim_step) to path. mass is the caller's
    array (the library keeps no host copy); theta .. beta are stored for `resume`."""
    n = len(mass)
    pos, vel, acc, dt_ind = np.empty((n, 3)), np.empty((n, 3)), np.empty((n, 3)), np.empty(n)
    t = ctypes.c_double()
    _lib.check(lib.gf_sim_read(pos.ctypes.data, vel.ctypes.data, acc.ctypes.data, dt_ind.ctypes.data,
                               ctypes.byref(t)))
    u = np.empty(n)
    _lib.check(lib.gf_sim_read_u(u))
    kind = np.empty(n, np.int8)
    birth, no_cool = np.empty(n), np.empty(n)
    words = np.zeros(4, np.uint64)
    formed = lib.gf_sim_read_stars(kind.ctypes.data, birth.ctypes.data, no_cool.ctypes.data, words.ctypes.data)
    if formed < 0:
        _lib.check(int(-formed))
    sc = np.zeros(3)
    _lib.check(lib.gf_sim_read_scalars(sc))
    rho, dudt = np.empty(n), np.empty(n)
    _lib.check(lib.gf_sim_read_hydro(rho, dudt))
    save(path, pos, vel, mass, kind, u, acc=acc, dt_ind=dt_ind, birth=birth, no_cool_until=no_cool,
         rho_gas=rho, dudt_gas=dudt, rng_words=words, t=sc[0], dt_grav=sc[1], dt_gas=sc[2],
         run=np.array([theta, eps, gamma, alpha, beta]))


def resume(lib, path):
    """Restores a checkpoint into the library's step loop; returns the snapshot dict (its
    rng_words are the star-formation generator's state at the checkpoint)."""
    s = load(path)
    theta, eps, gamma, alpha, beta = (float(x) for x in s["run"])
    n = len(s["mass"])
    _lib.check(lib.gf_sim_init(n, s["pos"], s["vel"], s["mass"], s["kind"], s["u"], theta, eps, gamma, alpha,
                               beta))
    _lib.check(lib.gf_sim_restore(s["acc"], s["dt_ind"], s["birth"].ctypes.data, s["no_cool_until"].ctypes.data,
                                  s["rho_gas"].ctypes.data, s["dudt_gas"].ctypes.data, float(s["t"]),
                                  float(s["dt_grav"]), float(s["dt_gas"])))
    return s
