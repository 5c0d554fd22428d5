"""The device-resident step loop (gf_sim_step, simulation.py:114-149) against the CPU
restatement (oracle/force_ref.py StepOracle) over several long steps: same long-step
lengths, same sub-step counts, positions and velocities agreeing to the float32 rounding
of the Barnes-Hut sums propagated through a few steps."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_steps_match_cpu(gpulib, oracle):
    from force_ref import StepOracle

    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.rotating_cloud(2000, 2000, seed=5)
    n = len(d["mass"])
    lib = gpulib
    _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                               params.GAMMA, params.ALPHA, params.BETA))
    ref = StepOracle(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS)
    taken, subs = ctypes.c_double(), ctypes.c_int()
    for _ in range(3):
        _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
        D = ref.step(1.0)
        assert abs(taken.value - D) <= 1e-6 * D, (taken.value, D)
        assert subs.value == ref.substeps
    pos, vel, acc = np.empty((n, 3)), np.empty((n, 3)), np.empty((n, 3))
    t = ctypes.c_double()
    _lib.check(lib.gf_sim_read(pos.ctypes.data, vel.ctypes.data, acc.ctypes.data, None, ctypes.byref(t)))
    assert abs(t.value - ref.t) <= 1e-6 * ref.t
    scale = np.linalg.norm(ref.pos, axis=1).mean()
    assert np.percentile(np.linalg.norm(pos - ref.pos, axis=1), 99) < 1e-5 * scale
    vs = np.linalg.norm(ref.vel, axis=1).mean()
    assert np.percentile(np.linalg.norm(vel - ref.vel, axis=1), 99) < 1e-4 * vs


def test_steps_match_cpu_mixed_sph(gpulib, oracle):
    """The same with the mixed form's float32 + Kahan SPH, whose neighbour reselection works in
    float32 from hi + lo positions (here on the synchronised path, where the gas set is checked
    against the cached one at every call): positions and velocities agree with the float64 CPU
    restatement to the float32 rounding of the SPH and Barnes-Hut sums."""
    from force_ref import StepOracle

    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.rotating_cloud(2000, 2000, seed=5)
    n = len(d["mass"])
    lib = gpulib
    lib.gf_set_option(_lib.OPT_SPH_FLOAT32, 1)
    try:
        _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                                   params.GAMMA, params.ALPHA, params.BETA))
        ref = StepOracle(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS)
        taken, subs = ctypes.c_double(), ctypes.c_int()
        for _ in range(3):
            _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
            D = ref.step(1.0)
            assert abs(taken.value - D) <= 1e-5 * D, (taken.value, D)
            assert subs.value == ref.substeps
        pos, vel = np.empty((n, 3)), np.empty((n, 3))
        t = ctypes.c_double()
        _lib.check(lib.gf_sim_read(pos.ctypes.data, vel.ctypes.data, None, None, ctypes.byref(t)))
        st = np.zeros(9)
        _lib.check(lib.gf_force_stats(st, 9))
        assert st[6] > 0  # sub-steps reselected from the cached candidates
    finally:
        lib.gf_set_option(_lib.OPT_SPH_FLOAT32, 0)
    assert abs(t.value - ref.t) <= 1e-5 * ref.t
    scale = np.linalg.norm(ref.pos, axis=1).mean()
    assert np.percentile(np.linalg.norm(pos - ref.pos, axis=1), 99) < 1e-5 * scale
    vs = np.linalg.norm(ref.vel, axis=1).mean()
    assert np.percentile(np.linalg.norm(vel - ref.vel, axis=1), 99) < 1e-4 * vs
