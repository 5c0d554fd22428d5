"""The thermal update on the device against the reference's cooling.py (golden vectors) and
the step loop with _thermodynamics (simulation.py:97-104) against its CPU restatement."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cooling_matches_reference(gpulib, golden):
    """cooling_function and cool on the GPU against the reference's outputs: float64 with the
    reference's order of operations, so only exp / pow / sqrt rounding (an ulp or two) differs."""
    from galaxy_formation_gb300 import _lib, params

    c = golden("cooling.npz")
    units = np.array(params.THERMO_UNITS)
    lam = np.empty_like(c["T"])
    _lib.check(gpulib.gf_cooling_function(len(lam), c["T"], lam))
    assert np.all(lam[c["T"] <= 1e4] == 0)
    on = c["lam"] > 0
    assert np.max(np.abs(lam[on] - c["lam"][on]) / c["lam"][on]) < 1e-14
    out = np.empty_like(c["u"])
    blocked = c["blocked"].astype(np.uint8)
    _lib.check(gpulib.gf_cool(len(out), c["u"], c["u"] / c["u_per_K"], c["rho"], c["dt"], blocked.ctypes.data,
                              float(c["u_floor"]), units, out))
    assert np.max(np.abs(out - c["u_new"]) / c["u_new"]) < 1e-13
    floored = c["u_new"] == c["u_floor"]
    assert np.array_equal(out[floored], c["u_new"][floored])


@pytest.mark.parametrize("mode", [1, 2])
def test_steps_with_thermodynamics_match_cpu(gpulib, oracle, mode):
    """gf_sim_step with the thermal update against StepOracle with the same update: the same
    step lengths and sub-step counts, u within float32 rounding of the forces it came from."""
    from force_ref import StepOracle

    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    d = synthetic.rotating_cloud(2000, 2000, seed=5)
    # warm gas so that cooling matters (1e4-1e6 K, log-uniform)
    gas = d["kind"] == params.GAS
    d["u"][gas] = params.U_PER_K * np.exp(np.random.default_rng(2).uniform(np.log(1e4), np.log(1e6), gas.sum()))
    n = len(d["mass"])
    units = np.array(params.THERMO_UNITS)
    try:
        _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                                   params.GAMMA, params.ALPHA, params.BETA))
        _lib.check(lib.gf_sim_thermo(mode, units.ctypes.data))
        ref = StepOracle(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS, thermo=mode,
                         thermo_units=params.THERMO_UNITS)
        taken, subs = ctypes.c_double(), ctypes.c_int()
        for _ in range(3):
            _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
            D = ref.step(1.0)
            assert abs(taken.value - D) <= 1e-6 * D, (taken.value, D)
            assert subs.value == ref.substeps
        u = np.empty(n)
        _lib.check(lib.gf_sim_read_u(u))
    finally:
        lib.gf_sim_thermo(0, None)
    assert np.array_equal(u[~gas], d["u"][~gas])
    assert not np.array_equal(u[gas], d["u"][gas])
    assert np.all(u[gas] >= params.U_FLOOR)
    e = np.abs(u[gas] - ref.u[gas]) / ref.u[gas]
    assert np.percentile(e, 99) < 1e-5 and e.max() < 1e-3, (np.percentile(e, 99), e.max())


def _energy_drift(lib, d, mode, blocks):
    from galaxy_formation_gb300 import _lib, params

    n = len(d["mass"])
    units = np.array(params.THERMO_UNITS)
    _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                               params.GAMMA, params.ALPHA, params.BETA))
    _lib.check(lib.gf_sim_thermo(mode, units.ctypes.data if mode else None))
    e = np.zeros(8)
    _lib.check(lib.gf_sim_diagnostics(0.3, e))
    taken, subs, upd = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
    if blocks:
        _lib.check(lib.gf_sim_blocks(blocks, 4, ctypes.byref(upd)))
    else:
        for _ in range(6):
            _lib.check(lib.gf_sim_step(1.0, ctypes.byref(taken), ctypes.byref(subs)))
    e1 = np.zeros(8)
    _lib.check(lib.gf_sim_diagnostics(0.3, e1))
    lib.gf_sim_thermo(0, None)
    return abs(e1[3] - e[3]) / abs(e[3]), e1[2] - e[2]


@pytest.mark.parametrize("blocks", [0, 3])
def test_thermal_update_closes_the_energy_budget(gpulib, blocks):
    """With u += dt du/dt the work of the pressure and viscous forces goes into thermal energy:
    the total energy drifts less than with u frozen, in the step loop and in block steps."""
    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    for key in (_lib.OPT_SPH_FLOAT32, _lib.OPT_GRAVITY_QUAD, _lib.OPT_HGUESS, _lib.OPT_WALK_CHUNK):
        lib.gf_set_option(key, 0)
    d = synthetic.rotating_cloud(3000, 3000, seed=4)
    gas = d["kind"] == params.GAS
    d["u"][gas] = 1e5 * params.U_PER_K
    drift0, dth0 = _energy_drift(lib, d, 0, blocks)
    drift1, dth1 = _energy_drift(lib, d, 1, blocks)
    assert dth0 == 0 and dth1 != 0
    assert drift1 < drift0, (drift1, drift0)
