"""Conserved-quantity diagnostics (gf_sim_diagnostics): float64 kinetic / thermal energy and
angular momentum exactly as numpy sums them, the Barnes-Hut potential energy against the
float64 direct pair sum, and energy conservation over steps of both integrators."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _init(lib, d):
    from galaxy_formation_gb300 import _lib, params

    for key in (_lib.OPT_SPH_FLOAT32, _lib.OPT_GRAVITY_QUAD, _lib.OPT_HGUESS, _lib.OPT_WALK_CHUNK):
        lib.gf_set_option(key, 0)
    _lib.check(lib.gf_sim_init(len(d["mass"]), d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA,
                               params.EPS, params.GAMMA, params.ALPHA, params.BETA))


def _diag(lib, theta=0.5):
    from galaxy_formation_gb300 import _lib

    out = np.zeros(8)
    _lib.check(lib.gf_sim_diagnostics(theta, out))
    return out


def test_diagnostics_match_direct_sums(gpulib):
    from galaxy_formation_gb300 import params, synthetic

    d = synthetic.rotating_cloud(1500, 1500, seed=9)
    lib = gpulib
    _init(lib, d)
    out = _diag(lib, 0.3)
    m, x, v = d["mass"], d["pos"], d["vel"]
    ke = 0.5 * np.sum(m * np.einsum("ij,ij->i", v, v))
    th = np.sum((m * d["u"])[d["kind"] == 0])
    L = np.sum(m[:, None] * np.cross(x, v), axis=0)
    r2 = np.sum((x[:, None, :] - x[None, :, :]) ** 2, axis=2) + params.EPS ** 2
    inv = 1.0 / np.sqrt(r2)
    np.fill_diagonal(inv, 0.0)
    pe = -0.5 * np.sum(m[:, None] * m[None, :] * inv)
    assert abs(out[0] - ke) <= 1e-12 * abs(ke)
    assert abs(out[2] - th) <= 1e-12 * abs(th)
    assert np.allclose(out[4:7], L, rtol=1e-12, atol=1e-12 * np.abs(L).max())
    assert abs(out[1] - pe) <= 1e-3 * abs(pe), (out[1], pe)
    assert abs(out[3] - (out[0] + out[1] + out[2])) <= 1e-12 * abs(out[3])


def test_energy_conserved_by_both_integrators(gpulib):
    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.rotating_cloud(1500, 1500, seed=10)
    d["kind"][:] = params.DM
    d["u"][:] = 0.0
    lib = gpulib
    _init(lib, d)
    e0 = _diag(lib)
    tk, sub = ctypes.c_double(), ctypes.c_int()
    for _ in range(5):
        _lib.check(lib.gf_sim_step(1e30, ctypes.byref(tk), ctypes.byref(sub)))
    e1 = _diag(lib)
    assert e1[7] > e0[7]
    assert abs(e1[3] - e0[3]) <= 1e-3 * abs(e0[3]), (e0[3], e1[3])
    assert np.linalg.norm(e1[4:7] - e0[4:7]) <= 1e-3 * np.linalg.norm(e0[4:7])
    # the batched form: diagnostics between blocks see synchronised velocities
    _init(lib, d)
    _lib.check(lib.gf_sim_block_config(None, 0, 0))
    upd = ctypes.c_double()
    _lib.check(lib.gf_sim_blocks(1, 4, ctypes.byref(upd)))
    b0 = _diag(lib)
    _lib.check(lib.gf_sim_blocks(3, 4, ctypes.byref(upd)))
    b1 = _diag(lib)
    assert b1[7] > b0[7]
    assert abs(b1[3] - b0[3]) <= 1e-3 * abs(b0[3]), (b0[3], b1[3])
    assert np.linalg.norm(b1[4:7] - b0[4:7]) <= 1e-3 * np.linalg.norm(b0[4:7])
