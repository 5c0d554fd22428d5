"""Block time steps (gf_sim_blocks, the batched form; its inner sub-steps replay a captured
CUDA graph) against the CPU restatement of the same scheme (oracle/force_ref.py
BlockOracle) on a gas-free particle set, and a run with gas for sanity (finite state,
update counts, level populations)."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(lib, n):
    from galaxy_formation_gb300 import _lib

    pos, vel = np.empty((n, 3)), np.empty((n, 3))
    t = ctypes.c_double()
    _lib.check(lib.gf_sim_read(pos.ctypes.data, vel.ctypes.data, None, None, ctypes.byref(t)))
    return pos, vel, t.value


def test_blocks_match_cpu_gravity_only(gpulib, oracle):
    from force_ref import BlockOracle

    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.rotating_cloud(1500, 1500, seed=6)
    d["kind"][:] = params.DM
    d["u"][:] = 0.0
    n = len(d["mass"])
    lib = gpulib
    _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                               params.GAMMA, params.ALPHA, params.BETA))
    ref = BlockOracle(d["pos"], d["vel"], d["mass"], params.THETA, params.EPS, nlev=3)
    upd = ctypes.c_double()
    for _ in range(3):
        _lib.check(lib.gf_sim_blocks(1, 3, ctypes.byref(upd)))
        ref.block()
        assert upd.value >= n
    pos, vel, t = _state(lib, n)
    assert abs(t - ref.t) <= 1e-6 * ref.t
    scale = np.linalg.norm(ref.pos, axis=1).mean()
    assert np.percentile(np.linalg.norm(pos - ref.pos, axis=1), 99) < 1e-5 * scale
    vs = np.linalg.norm(ref.vel, axis=1).mean()
    assert np.percentile(np.linalg.norm(vel - ref.vel, axis=1), 99) < 1e-4 * vs


def test_blocks_with_gas(gpulib):
    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.make_config(1, scale=0.05)
    n = len(d["mass"])
    lib = gpulib
    _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                               params.GAMMA, params.ALPHA, params.BETA))
    upd = ctypes.c_double()
    total = 0.0
    for _ in range(3):
        _lib.check(lib.gf_sim_blocks(1, 4, ctypes.byref(upd)))
        total += upd.value
    frac = np.zeros(4)
    _lib.check(lib.gf_sim_levels(4, frac))
    assert abs(frac.sum() - 1) < 1e-9
    pos, vel, t = _state(lib, n)
    assert np.all(np.isfinite(pos)) and np.all(np.isfinite(vel)) and t > 0
    # at least one evaluation of everybody per block, at most one per sub-step
    assert 3 * n <= total <= 3 * n * 8 + n
