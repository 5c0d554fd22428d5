"""The mixed-precision form against float64 references.

* SPH (gf_sph_forces_mixed): float32 arithmetic with hi/lo positions and Kahan sums vs the
  float64 oracle restatement of sph.py. Densities and time steps within 1e-5 relative;
  accelerations within 1e-5 relative at p99 (a pressure force is a sum of 31 terms that
  partly cancel; rare particles with near-total cancellation are bounded separately).
* Gravity (GF_OPT_GRAVITY_QUAD in the fused evaluation): quadrupole moments and Kahan tile
  sums; the error against the float64 direct sum must stay well below the monopole
  reference's at the same theta.
"""

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _gas(scale=0.05):
    from galaxy_formation_gb300 import params, synthetic

    d = synthetic.make_config(1, scale=scale)
    gas = d["kind"] == params.GAS
    return {k: np.ascontiguousarray(d[k][gas]) for k in ("pos", "vel", "mass", "u")}


def test_mixed_sph_matches_float64(gpulib, oracle, golden):
    from galaxy_formation_gb300 import _lib, params

    for data in (golden("sph2k.npz"), _gas()):
        p, v, m, u = data["pos"], data["vel"], data["mass"], data["u"]
        if "nb" in data:
            nb, h = data["nb"].astype(np.int64), data["h"]
        else:
            dist, nb = oracle.knn_brute(p, 32)
            h = np.maximum(0.5 * dist[:, -1], 0.5 * params.EPS)
        n = len(p)
        rho, acc, dudt, dt = np.empty(n), np.empty((n, 3)), np.empty(n), np.empty(n)
        _lib.check(gpulib.gf_sph_forces_mixed(n, 32, p, v, m, nb, h, u, params.GAMMA, 1.0, 2.0,
                                              rho, acc, dudt, dt))
        r_rho, r_acc, r_dudt, r_dt = oracle.sph_forces(p, v, m, nb, h, u, params.GAMMA, 1.0, 2.0)
        assert np.max(np.abs(rho - r_rho) / r_rho) < 1e-5
        assert np.max(np.abs(dt - r_dt) / r_dt) < 1e-5
        e = rel_err(acc, r_acc)
        assert np.percentile(e, 99) < 1e-5, np.percentile(e, 99)
        scale = np.linalg.norm(r_acc, axis=1).mean()
        assert np.max(np.linalg.norm(acc - r_acc, axis=1)) < 1e-4 * scale
        assert np.max(np.abs(dudt - r_dudt)) < 1e-4 * np.abs(r_dudt).mean()


def _fused(lib, d, theta, quad):
    from galaxy_formation_gb300 import _lib, params

    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, quad)
    n = len(d["mass"])
    acc = np.empty((n, 3))
    dt = np.empty(n)
    try:
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], theta,
                                        params.EPS, params.GAMMA, 1.0, 2.0, None, 1, 0, 1, acc, dt))
    finally:
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
    return acc


def test_quadrupole_gravity_accuracy(gpulib):
    from galaxy_formation_gb300 import params, synthetic
    from galaxy_formation_gb300.engine import Engine

    d = synthetic.make_config(2, scale=0.05)   # 25k gas + 25k DM disk + halo
    n = len(d["mass"])
    tgt = np.random.default_rng(3).choice(n, 1000, replace=False)
    exact = Engine().gravity_direct_targets(d["pos"], d["mass"], tgt, params.EPS)
    p99 = {}
    for quad in (0, 1):
        for theta in (0.5, 0.7):
            a = _fused(gpulib, d, theta, quad)
            p99[quad, theta] = np.percentile(rel_err(a[tgt], exact), 99)
    # observed on this 50k disk: 4.6e-3 vs 1.1e-2 at theta 0.7, 3.0e-3 vs 6.7e-3 at 0.5
    assert p99[1, 0.7] < 0.6 * p99[0, 0.7], p99
    assert p99[1, 0.5] < 0.6 * p99[0, 0.5], p99


def test_quadrupole_refit_and_active(gpulib):
    """Mixed gravity on a refitted tree with an active subset: inactive rows untouched,
    active rows close to a fresh quadrupole build."""
    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.make_config(1, scale=0.05)
    n = len(d["mass"])
    lib = gpulib
    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 1)
    try:
        acc = np.empty((n, 3))
        dt = np.empty(n)
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.6, params.EPS,
                                        params.GAMMA, 1.0, 2.0, None, 1, 0, 1, acc, dt))
        d["pos"] = np.ascontiguousarray(d["pos"] + 1e-3 * d["vel"])
        act = (np.random.default_rng(1).uniform(size=n) < 0.3).astype(np.uint8)
        a_ref = np.empty((n, 3))
        acc2 = np.empty((n, 3))
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.6, params.EPS,
                                        params.GAMMA, 1.0, 2.0, act.ctypes.data, 0, 0, 1, acc2, dt))
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.6, params.EPS,
                                        params.GAMMA, 1.0, 2.0, None, 1, 0, 1, a_ref, dt))
    finally:
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
    on = act != 0
    assert np.array_equal(acc2[~on], acc[~on])
    # a refit opens more cells than a rebuild (inflated radii): close, not identical
    assert np.percentile(rel_err(acc2[on], a_ref[on]), 99) < 2e-3


def test_relative_opening_criterion(gpulib):
    """GF_OPT_GRAVITY_REL: the first evaluation is the geometric walk at theta (bit for bit);
    the next one takes the previous gravity as its error scale and walks fewer interactions
    at the same accuracy against the float64 direct sum."""
    from galaxy_formation_gb300 import _lib, params, synthetic
    from galaxy_formation_gb300.engine import Engine

    lib = gpulib
    d = synthetic.make_config(2, scale=0.05)   # 25k gas + 25k DM disk + halo
    n = len(d["mass"])
    tgt = np.random.default_rng(3).choice(n, 1000, replace=False)
    exact = Engine().gravity_direct_targets(d["pos"], d["mass"], tgt, params.EPS)
    dt = np.empty(n)

    def run():
        acc = np.empty((n, 3))
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.55, params.EPS,
                                        params.GAMMA, 1.0, 2.0, None, 1, 0, 1, acc, dt))
        return acc, lib.gf_walk_pairs()

    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 1)
    try:
        lib.gf_set_option(_lib.OPT_GRAVITY_REL, 0)
        a_geo, pairs_geo = run()
        lib.gf_set_option(_lib.OPT_GRAVITY_REL, 2.5e-3)
        a_first, _ = run()
        a_rel, pairs_rel = run()
        a_rel2, _ = run()
    finally:
        lib.gf_set_option(_lib.OPT_GRAVITY_REL, 0)
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
    assert np.array_equal(a_first, a_geo)
    e_geo = np.percentile(rel_err(a_geo[tgt], exact), 99)
    e_rel = np.percentile(rel_err(a_rel[tgt], exact), 99)
    # observed with the float64 restatement of both criteria on this set: 1501 vs 1100
    # interactions per particle, p99 7.5e-4 vs 7.2e-4
    assert pairs_rel < 0.85 * pairs_geo, (pairs_rel, pairs_geo)
    assert e_rel < 1e-3 and e_rel < 1.3 * e_geo, (e_rel, e_geo)
    # the error scale of the third call is the second's result: the same lists to rounding
    assert np.percentile(rel_err(a_rel2[tgt], a_rel[tgt]), 99) < 1e-4


def test_relative_opening_active_subset(gpulib):
    """The relative criterion on a refitted tree with an active subset: inactive rows keep
    their values, active rows within the accuracy bar of a fresh evaluation."""
    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    d = synthetic.make_config(1, scale=0.05)
    n = len(d["mass"])
    dt = np.empty(n)
    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 1)
    lib.gf_set_option(_lib.OPT_GRAVITY_REL, 2.5e-3)
    try:
        acc = np.empty((n, 3))
        for _ in range(2):
            _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.55, params.EPS,
                                            params.GAMMA, 1.0, 2.0, None, 1, 0, 1, acc, dt))
        d["pos"] = np.ascontiguousarray(d["pos"] + 1e-3 * d["vel"])
        act = (np.random.default_rng(1).uniform(size=n) < 0.3).astype(np.uint8)
        acc2 = np.empty((n, 3))
        a_ref = np.empty((n, 3))
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.55, params.EPS,
                                        params.GAMMA, 1.0, 2.0, act.ctypes.data, 0, 0, 1, acc2, dt))
        _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.55, params.EPS,
                                        params.GAMMA, 1.0, 2.0, None, 1, 0, 1, a_ref, dt))
    finally:
        lib.gf_set_option(_lib.OPT_GRAVITY_REL, 0)
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
    on = act != 0
    assert np.array_equal(acc2[~on], acc[~on])
    assert np.percentile(rel_err(acc2[on], a_ref[on]), 99) < 2e-3


def test_merged_walk_items(gpulib):
    """GF_OPT_WALK_MERGE: runs of sibling groups walked as one item (up to 64 and up to 128
    particles, the largest batch of one walk) keep the accuracy of the group walk against the
    float64 direct sum."""
    from galaxy_formation_gb300 import _lib, params, synthetic
    from galaxy_formation_gb300.engine import Engine

    lib = gpulib
    d = synthetic.make_config(2, scale=0.05)
    n = len(d["mass"])
    tgt = np.random.default_rng(5).choice(n, 1000, replace=False)
    exact = Engine().gravity_direct_targets(d["pos"], d["mass"], tgt, params.EPS)
    dt = np.empty(n)
    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 1)
    lib.gf_set_option(_lib.OPT_GRAVITY_REL, 3e-3)
    errs = {}
    try:
        for merge in (0, 64, 128):
            lib.gf_set_option(_lib.OPT_WALK_MERGE, merge)
            acc = np.empty((n, 3))
            for _ in range(2):
                _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.55,
                                                params.EPS, params.GAMMA, 1.0, 2.0, None, 1, 0, 1, acc, dt))
            e = rel_err(acc[tgt], exact)
            errs[merge] = (np.percentile(e, 99), e.max())
    finally:
        lib.gf_set_option(_lib.OPT_WALK_MERGE, 0)
        lib.gf_set_option(_lib.OPT_GRAVITY_REL, 0)
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
    # larger items have larger spheres: each particle's criterion only gets stricter
    for merge in (64, 128):
        assert errs[merge][0] < 1e-3 and errs[merge][0] <= 1.1 * errs[0][0], errs
        assert errs[merge][1] < 5e-3, errs



def test_monopole_tolerance_for_far_nodes(gpulib):
    """GF_OPT_GRAVITY_REL_MONO: accepted nodes whose quadrupole term is below alpha_q a_min are
    taken as monopoles; fewer quadrupole interactions, the same interaction count, and the
    accuracy bar against the float64 direct sum kept."""
    from galaxy_formation_gb300 import _lib, params, synthetic
    from galaxy_formation_gb300.engine import Engine

    lib = gpulib
    d = synthetic.make_config(2, scale=0.05)
    n = len(d["mass"])
    tgt = np.random.default_rng(6).choice(n, 1000, replace=False)
    exact = Engine().gravity_direct_targets(d["pos"], d["mass"], tgt, params.EPS)
    dt = np.empty(n)
    res = {}
    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 1)
    lib.gf_set_option(_lib.OPT_GRAVITY_REL, 4e-3)
    lib.gf_set_option(_lib.OPT_WALK_MERGE, 40)
    try:
        for relq in (0.0, 2e-4):
            lib.gf_set_option(_lib.OPT_GRAVITY_REL_MONO, relq)
            acc = np.empty((n, 3))
            for _ in range(2):
                _lib.check(lib.gf_accelerations(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.55,
                                                params.EPS, params.GAMMA, 1.0, 2.0, None, 1, 0, 1, acc, dt))
            res[relq] = (np.percentile(rel_err(acc[tgt], exact), 99), lib.gf_walk_pairs(), lib.gf_walk_quad_pairs())
    finally:
        for key in (_lib.OPT_GRAVITY_REL_MONO, _lib.OPT_WALK_MERGE, _lib.OPT_GRAVITY_REL, _lib.OPT_GRAVITY_QUAD):
            lib.gf_set_option(key, 0)
    (e0, p0, q0), (e1, p1, q1) = res[0.0], res[2e-4]
    # the same acceptance (to the rounding of the error scale, which each run takes from the
    # one before), fewer quadrupoles
    assert abs(p1 - p0) <= 1e-3 * p0 and q1 < 0.85 * q0, res
    assert e1 < 1e-3 and e1 < 1.2 * e0, res
