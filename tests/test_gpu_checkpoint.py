"""Checkpoint and exact resume of the device step loop (galaxy_formation_gb300/snapshot.py):
a run that stops, saves, restarts from the file and goes on matches the uninterrupted run."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_resume_continues_exactly(gpulib, tmp_path):
    from galaxy_formation_gb300 import _lib, params, snapshot, subgrid, synthetic

    lib = gpulib
    for key in (_lib.OPT_SPH_FLOAT32, _lib.OPT_GRAVITY_QUAD, _lib.OPT_HGUESS, _lib.OPT_WALK_CHUNK):
        lib.gf_set_option(key, 0)
    d = synthetic.make_config(1, scale=0.02)
    n = len(d["mass"])
    units = np.array(params.THERMO_UNITS)
    sp = subgrid.star_params(sf_eff=0.5)
    run = (params.THETA, params.EPS, params.GAMMA, params.ALPHA, params.BETA)
    taken, subs = ctypes.c_double(), ctypes.c_int()

    def state():
        pos, vel = np.empty((n, 3)), np.empty((n, 3))
        t = ctypes.c_double()
        _lib.check(lib.gf_sim_read(pos.ctypes.data, vel.ctypes.data, None, None, ctypes.byref(t)))
        u = np.empty(n)
        _lib.check(lib.gf_sim_read_u(u))
        kind = np.empty(n, np.int8)
        lib.gf_sim_read_stars(kind.ctypes.data, None, None, None)
        return pos, vel, u, kind, t.value

    try:
        _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], *run))
        _lib.check(lib.gf_sim_thermo(2, units.ctypes.data))
        _lib.check(lib.gf_sim_stars(1, sp.ctypes.data, subgrid.pcg64_words(np.random.default_rng(4)).ctypes.data))
        for _ in range(2):
            _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
        path = tmp_path / "ckpt.npz"
        snapshot.checkpoint(lib, path, d["mass"], *run)
        for _ in range(2):
            _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
        a = state()
        s = snapshot.resume(lib, path)
        _lib.check(lib.gf_sim_thermo(2, units.ctypes.data))
        _lib.check(lib.gf_sim_stars(1, sp.ctypes.data, s["rng_words"].ctypes.data))
        for _ in range(2):
            _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
        b = state()
    finally:
        lib.gf_sim_stars(0, None, None)
        lib.gf_sim_thermo(0, None)
    pa, va, ua, ka, ta = a
    pb, vb, ub, kb, tb = b
    assert tb == ta
    assert np.array_equal(kb, ka)
    assert np.array_equal(pb, pa) and np.array_equal(vb, va) and np.array_equal(ub, ua)
