"""The mixed-precision case at full size: one force evaluation of the 200,000-particle disk+halo
snapshot (100k gas + 100k DM), float32-compensated SPH against the float64 SPH of the
reference form, and the quadrupole gravity against the float64 direct sum."""

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _evaluate(lib, d, theta, sph32, quad):
    from galaxy_formation_gb300 import _lib, params

    lib.gf_set_option(_lib.OPT_SPH_FLOAT32, sph32)
    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, quad)
    n = len(d["mass"])
    acc, dt = np.empty((n, 3)), np.empty(n)
    _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], theta, params.EPS,
                                    params.GAMMA, params.ALPHA, params.BETA, None, 1, 1, 1, acc, dt))
    return acc, dt


def test_mixed_precision_200k(gpulib):
    from galaxy_formation_gb300 import _lib, params, synthetic
    from galaxy_formation_gb300.engine import Engine

    lib = gpulib
    for key in (_lib.OPT_HGUESS, _lib.OPT_WALK_CHUNK, _lib.OPT_GRAVITY_REL, _lib.OPT_WALK_MERGE,
                _lib.OPT_GRAVITY_REL_MONO):
        lib.gf_set_option(key, 0)
    d = synthetic.make_config(1)
    n = len(d["mass"])
    gas = d["kind"] == params.GAS
    assert n == 200_000 and gas.sum() == 100_000
    try:
        a64, dt64 = _evaluate(lib, d, params.THETA, 0, 0)   # reference arithmetic
        a32, dt32 = _evaluate(lib, d, params.THETA, 1, 0)   # float32 + Kahan SPH, same gravity
        aq, _ = _evaluate(lib, d, 0.55, 1, 1)               # and quadrupole gravity
    finally:
        lib.gf_set_option(_lib.OPT_SPH_FLOAT32, 0)
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
    # same gravity, so the difference is the SPH arithmetic: within 1e-5 relative
    assert np.percentile(rel_err(a32[gas], a64[gas]), 99) < 1e-5
    assert np.array_equal(a32[~gas], a64[~gas])
    assert np.percentile(np.abs(dt32[gas] - dt64[gas]) / dt64[gas], 99) < 1e-5
    # quadrupole gravity of the DM (no SPH term) against the float64 direct sum
    dm = np.flatnonzero(~gas)
    tgt = np.random.default_rng(4).choice(dm, 1000, replace=False)
    exact = Engine().gravity_direct_targets(d["pos"], d["mass"], tgt, params.EPS)
    assert np.percentile(rel_err(aq[tgt], exact), 99) < 1e-3
