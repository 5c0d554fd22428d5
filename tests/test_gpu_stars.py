"""Star formation and supernova feedback on the device (gf_sim_stars: star_formation.py:35-65
called after every step and sub-step, simulation.py:106-110) against the CPU restatement
(oracle/star_ref.py in StepOracle) with the same NumPy generator state: the same particles
become stars at the same times, the same gas is heated and blocked from cooling, and the
generator ends in the same state."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_star_formation_matches_cpu(gpulib, oracle):
    from force_ref import StepOracle

    from galaxy_formation_gb300 import _lib, params, subgrid, synthetic

    lib = gpulib
    for key in (_lib.OPT_SPH_FLOAT32, _lib.OPT_GRAVITY_QUAD, _lib.OPT_HGUESS, _lib.OPT_WALK_CHUNK):
        lib.gf_set_option(key, 0)
    d = synthetic.make_config(1, scale=0.02)   # 2k gas + 2k DM disk + halo, T 1e4-1e6 K
    n = len(d["mass"])
    units = np.array(params.THERMO_UNITS)
    sp = subgrid.star_params(sf_eff=0.5)      # 100x the default efficiency: stars in a few steps
    rng_gpu = np.random.default_rng(11)
    words = subgrid.pcg64_words(rng_gpu)
    try:
        _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                                   params.GAMMA, params.ALPHA, params.BETA))
        _lib.check(lib.gf_sim_thermo(2, units.ctypes.data))
        _lib.check(lib.gf_sim_stars(1, sp.ctypes.data, words.ctypes.data))
        ref = StepOracle(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS, thermo=2,
                         thermo_units=params.THERMO_UNITS, stars=sp, rng=np.random.default_rng(11))
        taken, subs = ctypes.c_double(), ctypes.c_int()
        for _ in range(3):
            _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
            D = ref.step(1.0)
            assert abs(taken.value - D) <= 1e-6 * D, (taken.value, D)
            assert subs.value == ref.substeps
        kind = np.empty(n, np.int8)
        birth, no_cool, u = np.empty(n), np.empty(n), np.empty(n)
        w_end = np.zeros(4, np.uint64)
        formed = lib.gf_sim_read_stars(kind.ctypes.data, birth.ctypes.data, no_cool.ctypes.data, w_end.ctypes.data)
        _lib.check(lib.gf_sim_read_u(u))
    finally:
        lib.gf_sim_stars(0, None, None)
        lib.gf_sim_thermo(0, None)
    stars = ref.kind == 1
    assert stars.sum() >= 10, stars.sum()          # the case exercises the feature
    assert formed == stars.sum()
    assert np.array_equal(kind, ref.kind)
    assert np.allclose(birth[stars], ref.birth[stars], rtol=1e-6) and np.all(np.isinf(birth[~stars]))
    bub = ref.no_cool_until > -np.inf
    assert np.array_equal(no_cool > -np.inf, bub) and np.allclose(no_cool[bub], ref.no_cool_until[bub], rtol=1e-6)
    assert np.array_equal(w_end, subgrid.pcg64_words(ref.rng))
    dm = d["kind"] == params.DM
    assert np.array_equal(u[dm], d["u"][dm])
    e = np.abs(u[~dm] - ref.u[~dm]) / ref.u[~dm]
    assert np.percentile(e, 99) < 1e-5 and e.max() < 1e-3, (np.percentile(e, 99), e.max())
