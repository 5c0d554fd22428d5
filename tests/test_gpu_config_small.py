"""The reference's own CPU-runnable case on the device: its default cloud (5,000 gas + 5,000
dark matter, seed 3, the reference's make_cloud bit for bit), one full gravity + SPH force
evaluation, then 100 hierarchical-leapfrog steps with the reference's default theta, softening
and neighbour count. The first steps match the CPU restatement of the step loop; over the 100
steps the float64 energy (with the thermal update closing the budget) and angular momentum
stay conserved."""

import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_default_cloud_100_steps(gpulib, oracle):
    from force_ref import ForceOracle, StepOracle

    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    for key in (_lib.OPT_SPH_FLOAT32, _lib.OPT_GRAVITY_QUAD, _lib.OPT_HGUESS, _lib.OPT_WALK_CHUNK,
                _lib.OPT_GRAVITY_REL, _lib.OPT_WALK_MERGE, _lib.OPT_GRAVITY_REL_MONO):
        lib.gf_set_option(key, 0)
    d = synthetic.rotating_cloud(5000, 5000, seed=3)
    n = len(d["mass"])
    # one full evaluation against the CPU restatement
    acc, dt = np.empty((n, 3)), np.empty(n)
    _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                                    params.GAMMA, params.ALPHA, params.BETA, None, 1, 1, 1, acc, dt))
    f = ForceOracle(n, params.THETA, params.EPS)
    ref = f.accelerations(d["pos"], d["vel"], d["mass"], d["kind"], d["u"])
    assert np.percentile(rel_err(acc, ref), 99) < 1e-4
    # 100 steps; the first 3 against the CPU step loop
    units = np.array(params.THERMO_UNITS)
    _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                               params.GAMMA, params.ALPHA, params.BETA))
    _lib.check(lib.gf_sim_thermo(1, units.ctypes.data))
    try:
        step_ref = StepOracle(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS, thermo=1,
                              thermo_units=params.THERMO_UNITS)
        q0 = np.zeros(8)
        _lib.check(lib.gf_sim_diagnostics(0.3, q0))
        taken, subs = ctypes.c_double(), ctypes.c_int()
        total_subs = 0
        for k in range(100):
            _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
            total_subs += subs.value
            if k < 3:
                D = step_ref.step(1.0)
                assert abs(taken.value - D) <= 1e-6 * D and subs.value == step_ref.substeps
        q1 = np.zeros(8)
        _lib.check(lib.gf_sim_diagnostics(0.3, q1))
        pos, vel = np.empty((n, 3)), np.empty((n, 3))
        t = ctypes.c_double()
        _lib.check(lib.gf_sim_read(pos.ctypes.data, vel.ctypes.data, None, None, ctypes.byref(t)))
    finally:
        lib.gf_sim_thermo(0, None)
    assert np.all(np.isfinite(pos)) and np.all(np.isfinite(vel)) and t.value > 0 and total_subs >= 100
    dE = abs(q1[3] - q0[3]) / abs(q0[3])
    dL = np.linalg.norm(q1[4:7] - q0[4:7]) / np.linalg.norm(q0[4:7])
    assert dE < 1e-2 and dL < 1e-3, (dE, dL, t.value, total_subs)
