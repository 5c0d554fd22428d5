"""The two remaining configurations at reduced size, on the GPU.

* Learned smoothing-length guess on the clumped disk (disk + 200 Plummer clumps, densities over
  six decades): a network trained on pairs that the simulator produced on a disk+halo snapshot
  (no clumps) starts the first neighbour search of the clumped snapshot in fewer radius
  iterations than the cell-density start, and the converged neighbours, hence accelerations and
  time steps, are identical.
* Long steps of the rotating cloud drawn on the GPU: the reference's step loop (plain form)
  and block time steps (mixed + batched + learned form) integrate the same simulated time with
  the thermal update on; float64 total energy (kinetic + potential + thermal) and angular
  momentum stay conserved in both.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _train(lib):
    """Collects (features, log d48) pairs from evaluations of a 0.1-scale disk+halo snapshot
    and fits the network on the GPU."""
    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.make_config(1, scale=0.1)
    n = len(d["mass"])
    acc, dt = np.empty((n, 3)), np.empty(n)

    def force():
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA,
                                        params.EPS, params.GAMMA, 1.0, 2.0, None, 1, 1, 1, acc, dt))

    lib.gf_set_option(_lib.OPT_HGUESS, 0)
    force()
    lib.gf_set_option(_lib.OPT_COLLECT, 200_000)
    for _ in range(4):
        d["pos"] = np.ascontiguousarray(d["pos"] + 0.5 * dt[:, None] * d["vel"])
        force()
    rows = lib.gf_mlp_collected(None, None, 0)
    X = np.zeros((rows, 4), np.float32)
    T = np.zeros(rows, np.float32)
    lib.gf_mlp_collected(X.ctypes.data, T.ctypes.data, rows)
    _lib.check(lib.gf_mlp_init(3))
    mu, sd = X.mean(0), X.std(0) + 1e-6
    _lib.check(lib.gf_mlp_set_norm(mu.astype(np.float32), sd.astype(np.float32), float(T.mean()), float(T.std())))
    loss = ctypes.c_double()
    _lib.check(lib.gf_mlp_train(1500, 4096, 2e-3, ctypes.byref(loss)))  # on the collected rows
    lib.gf_set_option(_lib.OPT_COLLECT, 0)  # (this clears them)


def test_learned_guess_on_the_clumped_disk(gpulib):
    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    for key in (_lib.OPT_SPH_FLOAT32, _lib.OPT_GRAVITY_QUAD, _lib.OPT_GRAVITY_REL, _lib.OPT_WALK_MERGE):
        lib.gf_set_option(key, 0)
    _train(lib)
    d = synthetic.make_config(3, scale=0.02)
    n = len(d["mass"])
    assert (d["kind"] == params.GAS).sum() >= 20_000
    st = np.zeros(8)
    res = {}
    for mode in (1, 2):  # cell density, learned
        acc, dt = np.empty((n, 3)), np.empty(n)
        lib.gf_set_option(_lib.OPT_HGUESS, mode)
        lib.gf_set_option(_lib.OPT_FORGET_H, 1)
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA,
                                        params.EPS, params.GAMMA, 1.0, 2.0, None, 1, 1, 1, acc, dt))
        lib.gf_force_stats(st, 8)
        res[mode] = (st[3] / st[0], acc, dt)
    lib.gf_set_option(_lib.OPT_HGUESS, 0)
    print("clumped disk, first search: cell density %.4f, learned %.4f radius iterations" % (res[1][0], res[2][0]))
    assert res[2][0] < res[1][0], (res[1][0], res[2][0])
    assert np.array_equal(res[2][1], res[1][1]) and np.array_equal(res[2][2], res[1][2])


def _diag(lib):
    from galaxy_formation_gb300 import _lib

    q = np.zeros(8)
    _lib.check(lib.gf_sim_diagnostics(0.5, q))
    return q


def test_rotating_cloud_long_steps_both_forms(gpulib):
    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    d = synthetic.make_config_device(4, seed=3, scale=0.025, lib=lib)  # 100k particles
    n = len(d["mass"])
    assert n >= 90_000 and np.all(np.isfinite(d["pos"]))
    units = np.array(params.THERMO_UNITS)

    def init(quad):
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, quad)
        lib.gf_set_option(_lib.OPT_SPH_FLOAT32, quad)
        lib.gf_set_option(_lib.OPT_GRAVITY_REL, 0)
        lib.gf_set_option(_lib.OPT_HGUESS, 0)
        _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                                   params.GAMMA, params.ALPHA, params.BETA))
        _lib.check(lib.gf_sim_thermo(1, units.ctypes.data))

    try:
        init(0)  # plain: the reference's step loop
        q0 = _diag(lib)
        tk, sub = ctypes.c_double(), ctypes.c_int()
        for _ in range(4):
            _lib.check(lib.gf_sim_step(1e30, ctypes.byref(tk), ctypes.byref(sub)))
        q1 = _diag(lib)
        t_end = q1[7]
        assert t_end > q0[7]
        init(1)  # mixed: block time steps
        b0 = _diag(lib)
        _lib.check(lib.gf_sim_block_config(None, 0, 8))
        upd = ctypes.c_double()
        blocks = 0
        while blocks < 40:
            _lib.check(lib.gf_sim_blocks(1, 5, ctypes.byref(upd)))
            blocks += 1
            if _diag(lib)[7] >= t_end:
                break
        b1 = _diag(lib)
        assert b1[7] >= t_end, (b1[7], t_end)
        for a, b in ((q0, q1), (b0, b1)):
            assert abs(b[3] - a[3]) <= 5e-3 * abs(a[3]), (a[3], b[3])
            assert np.linalg.norm(b[4:7] - a[4:7]) <= 1e-3 * np.linalg.norm(a[4:7])
    finally:
        lib.gf_sim_thermo(0, None)
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
        lib.gf_set_option(_lib.OPT_SPH_FLOAT32, 0)
