"""The reference's own tests (tests/test_physics.py:20-38) restated on the oracle, so the
oracle satisfies the same acceptance checks the reference holds itself to."""

import numpy as np


def test_barnes_hut_matches_direct_sum(oracle):
    """tests/test_physics.py:20-30: theta 0.7, median relative error < 1 %."""
    rng = np.random.default_rng(0)
    pos = np.ascontiguousarray(rng.normal(size=(20000, 3)))
    mass = np.full(len(pos), 1.0 / len(pos))
    acc = np.zeros_like(pos)
    oracle.accel_active(pos, mass, acc, 0.7, 0.01)
    exact = oracle.accel_direct(pos, mass, 0.01)
    err = np.linalg.norm(acc - exact, axis=1) / np.linalg.norm(exact, axis=1)
    assert np.median(err) < 1e-2


def test_kernel_is_normalised(oracle):
    """tests/test_physics.py:33-38 (np.trapz is np.trapezoid in numpy >= 2)."""
    h = 0.7
    r = np.linspace(0, 2 * h, 20001)
    w = np.array([oracle.sph_kernel(x, h) for x in r])
    assert abs(np.trapezoid(4 * np.pi * r ** 2 * w, r) - 1) < 1e-4
