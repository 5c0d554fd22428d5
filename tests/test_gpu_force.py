"""The fused device force evaluation (gf_accelerations, simulation.py:61-95) against the
CPU restatement (oracle/force_ref.py, with the reference's cKDTree call) over a sequence
that exercises every branch: full evaluation, sub-steps with an active subset on a
refitted tree and Verlet-reselected neighbours, gas turning into stars, and the closing
gravity-only rebuild that keeps the previous SPH accelerations."""

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(gpulib):
    return gpulib


def gpu_acc(lib, d, active, rebuild, sph, fresh):
    from galaxy_formation_gb300 import _lib, params

    n = len(d["mass"])
    acc = np.empty((n, 3))
    dt = np.empty(n)
    act = None if active is None else np.ascontiguousarray(active, np.uint8).ctypes.data
    st = lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA,
                              params.EPS, params.GAMMA, params.ALPHA, params.BETA, act,
                              int(rebuild), int(sph), int(fresh), acc, dt)
    _lib.check(st)
    return acc, dt


def test_force_sequence_matches_cpu(lib, oracle):
    import ctypes

    from force_ref import ForceOracle

    from galaxy_formation_gb300 import params, synthetic

    d = synthetic.make_config(1, scale=0.1)    # 10k gas + 10k DM disk + halo
    n = len(d["mass"])
    fo = ForceOracle(n, params.THETA, params.EPS, use_ckdtree=True)
    rng = np.random.default_rng(2)

    def check(a_g, dt_g, a_c, tol=1e-4):
        err = rel_err(a_g, a_c)
        assert np.percentile(err, 99) <= tol, np.percentile(err, 99)
        r = np.abs(dt_g - fo.dt_ind) / fo.dt_ind
        assert np.percentile(r, 99) <= tol
        ng, dtg, dtgas, it = ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        lib.gf_force_info(ctypes.byref(ng), ctypes.byref(dtg), ctypes.byref(dtgas), ctypes.byref(it))
        assert abs(dtg.value - fo.dt_grav) <= 1e-4 * fo.dt_grav
        if fo.n_gas > 40:
            assert ng.value == fo.n_gas
            assert abs(dtgas.value - fo.dt_gas) <= 1e-5 * fo.dt_gas

    # 1. full evaluation
    a_g, dt_g = gpu_acc(lib, d, None, True, True, True)
    a_c = fo.accelerations(d["pos"], d["vel"], d["mass"], d["kind"], d["u"])
    check(a_g, dt_g, a_c)
    # 2. sub-steps: drift, fast set active, refit, Verlet neighbours
    fast = (fo.dt_ind < np.percentile(fo.dt_ind, 10)) | (d["kind"] == params.GAS)
    for _ in range(2):
        d["pos"] = np.ascontiguousarray(d["pos"] + 0.002 * d["vel"])
        a_g, dt_g = gpu_acc(lib, d, fast, False, True, False)
        a_c = fo.accelerations(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], fast, False, True, False)
        check(a_g, dt_g, a_c)
    # 3. some gas turns into stars (kind changes in place; the Verlet cache survives)
    gas = np.flatnonzero(d["kind"] == params.GAS)
    d["kind"][rng.choice(gas, 50, replace=False)] = params.STAR
    a_g, dt_g = gpu_acc(lib, d, fast, False, True, False)
    a_c = fo.accelerations(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], fast, False, True, False)
    check(a_g, dt_g, a_c)
    # 4. closing evaluation: rebuild, slow particles only, no SPH (acc_sph kept)
    slow = ~fast
    a_g, dt_g = gpu_acc(lib, d, slow, True, False, True)
    a_c = fo.accelerations(d["pos"], d["vel"], d["mass"], d["kind"], d["u"], slow, True, False, True)
    check(a_g, dt_g, a_c)


def test_force_few_gas_skips_hydro(lib, oracle):
    from force_ref import ForceOracle

    from galaxy_formation_gb300 import params, synthetic

    d = synthetic.rotating_cloud(30, 3000, seed=4)   # <= 40 gas: no hydro (simulation.py:80)
    n = len(d["mass"])
    fo = ForceOracle(n, params.THETA, params.EPS)
    a_g, dt_g = gpu_acc(lib, d, None, True, True, True)
    a_c = fo.accelerations(d["pos"], d["vel"], d["mass"], d["kind"], d["u"])
    assert np.percentile(rel_err(a_g, a_c), 99) <= 1e-4
    assert np.all(np.isfinite(dt_g))
