"""Block time steps (gf_sim_blocks, the batched form; its inner sub-steps replay a captured
CUDA graph) against the CPU restatement of the same scheme (oracle/force_ref.py
BlockOracle): gravity alone on a gas-free particle set, and with gas (partial SPH of the gas
due at each sub-step, Verlet reselection inside the graph)."""

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


def _plain(lib):
    from galaxy_formation_gb300 import _lib

    for key in (_lib.OPT_SPH_FLOAT32, _lib.OPT_GRAVITY_QUAD, _lib.OPT_HGUESS, _lib.OPT_WALK_CHUNK,
                _lib.OPT_GRAVITY_REL, _lib.OPT_WALK_MERGE, _lib.OPT_GRAVITY_REL_MONO):
        lib.gf_set_option(key, 0)


@pytest.mark.parametrize("rebuild_every,chunk", [(0, None), (2, None), (2, [1, 4]), (2, [4, 80])])
def test_blocks_match_cpu_gravity_only(gpulib, oracle, rebuild_every, chunk):
    """Against the CPU restatement: the reference's walk groups with the tree refitted at
    every sub-step; rebuilt inside the captured graph every other sub-step; walk items of a
    few active particles per bin; and sibling groups merged into items of <= 32 active
    particles (code 80) on the coarser bin."""
    from force_ref import BlockOracle

    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.rotating_cloud(1500, 1500, seed=6)
    d["kind"][:] = params.DM
    d["u"][:] = 0.0
    n = len(d["mass"])
    lib = gpulib
    _plain(lib)
    ch = None if chunk is None else np.array(chunk, np.int32)
    _lib.check(lib.gf_sim_block_config(None if ch is None else ch.ctypes.data, 0 if ch is None else len(ch),
                                       rebuild_every))
    _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                               params.GAMMA, params.ALPHA, params.BETA))
    ref = BlockOracle(d["pos"], d["vel"], d["mass"], params.THETA, params.EPS, nlev=3, rebuild_every=rebuild_every,
                      chunk=chunk)
    upd = ctypes.c_double()
    for _ in range(3):
        _lib.check(lib.gf_sim_blocks(1, 3, ctypes.byref(upd)))
        ref.block()
        assert upd.value >= n
    pos, vel, t = _state(lib, n)
    # the block length is set by the largest |a| (float32 walk sums): equal to ~1e-6
    assert abs(t - ref.t) <= 1e-5 * ref.t
    scale = np.linalg.norm(ref.pos, axis=1).mean()
    assert np.percentile(np.linalg.norm(pos - ref.pos, axis=1), 99) < 1e-5 * scale
    vs = np.linalg.norm(ref.vel, axis=1).mean()
    assert np.percentile(np.linalg.norm(vel - ref.vel, axis=1), 99) < 1e-4 * vs


@pytest.mark.parametrize("rebuild_every,sph32", [(0, 0), (4, 0), (4, 1)])
def test_blocks_with_gas_match_cpu(gpulib, oracle, rebuild_every, sph32):
    """Block steps with gas against the CPU restatement (BlockOracle with its hydro path):
    at every sub-step the gas due is compacted, re-selects its 32 neighbours among its cached
    candidates, and gets a new h, density and SPH forces, its neighbours that are not due
    entering with their last density and h; the block ends with a full evaluation (new tree,
    fresh search). Positions, velocities, time, level populations and the final gas state
    (h, neighbour sets, densities) match; also with the float32 + Kahan SPH of the mixed form
    (sph32) against the float64 restatement."""
    from force_ref import BlockOracle

    from galaxy_formation_gb300 import _lib, params, synthetic

    d = synthetic.make_config(1, scale=0.05)  # 5k gas + 5k DM disk + halo
    n = len(d["mass"])
    lib = gpulib
    _plain(lib)
    lib.gf_set_option(_lib.OPT_SPH_FLOAT32, sph32)
    chunk = [4, 8, 16, 64]
    ch = np.array(chunk, np.int32)
    _lib.check(lib.gf_sim_block_config(ch.ctypes.data, len(ch), rebuild_every))
    _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                               params.GAMMA, params.ALPHA, params.BETA))
    ref = BlockOracle(d["pos"], d["vel"], d["mass"], params.THETA, params.EPS, nlev=4, rebuild_every=rebuild_every,
                      chunk=chunk, kind=d["kind"], u=d["u"], gamma=params.GAMMA, alpha=params.ALPHA,
                      beta=params.BETA)
    assert ref.hydro
    upd = ctypes.c_double()
    total = 0.0
    try:
        for _ in range(3):
            _lib.check(lib.gf_sim_blocks(1, 4, ctypes.byref(upd)))
            ref.block()
            total += upd.value
    finally:
        lib.gf_set_option(_lib.OPT_SPH_FLOAT32, 0)
    frac = np.zeros(4)
    _lib.check(lib.gf_sim_levels(4, frac))
    ref_frac = np.bincount(ref.level, minlength=4) / n
    assert np.abs(frac - ref_frac).max() <= 2e-3, (frac, ref_frac)
    pos, vel, t = _state(lib, n)
    assert abs(t - ref.t) <= 1e-5 * ref.t
    scale = np.linalg.norm(ref.pos, axis=1).mean()
    assert np.percentile(np.linalg.norm(pos - ref.pos, axis=1), 99) < 1e-5 * scale
    vs = np.linalg.norm(ref.vel, axis=1).mean()
    assert np.percentile(np.linalg.norm(vel - ref.vel, axis=1), 99) < 1e-4 * vs
    # the block-end evaluation's gas state against the restatement's (same positions up to the
    # trajectories' float32-gravity differences)
    gs = _lib.read_gas(lib)
    assert np.array_equal(gs["gidx"], ref.gas)
    assert np.percentile(np.abs(gs["h"] - ref.h) / ref.h, 99) < 1e-4
    assert np.percentile(np.abs(gs["rho"] - ref.rho) / ref.rho, 99) < 1e-4
    same = np.all(np.sort(gs["nb"], axis=1) == np.sort(ref.nb, axis=1), axis=1)
    assert same.mean() > 0.98, same.mean()
    # at least one evaluation of everybody per block, at most one per sub-step
    assert 3 * n <= total <= 3 * n * 8 + n


def test_chunked_walk_accuracy(gpulib, oracle):
    """Walk items of a few active particles with their own spheres (chunks of one group, or
    sibling groups merged by active count: codes 72 and 96, <= 16 and <= 64 active particles):
    the same interaction lists as the CPU restatement of those items, and every particle still
    meets the opening criterion, so the error against the float64 direct sum stays at the
    per-particle level."""
    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    _plain(lib)
    d = synthetic.make_config(1, scale=0.2)
    n = len(d["mass"])
    rng = np.random.default_rng(3)
    active = (rng.random(n) < 0.02).astype(np.uint8)
    idx = np.flatnonzero(active)
    ref = oracle.accel_direct_targets(d["pos"], d["mass"], idx, params.EPS)
    errs = {}
    for chunk in (0, 1, 4, 16, 72, 96):
        lib.gf_set_option(_lib.OPT_WALK_CHUNK, chunk)
        acc = np.zeros((n, 3))
        lib.nbody_accel_active(n, d["pos"], d["mass"], acc, params.THETA, params.EPS, active, 1)
        assert lib.gf_last_status() == 0
        assert np.all(acc[active == 0] == 0)
        # the CPU restatement of the same items
        oracle.set_walk_chunk(chunk)
        acc_o = np.zeros((n, 3))
        oracle.accel_active(d["pos"], d["mass"], acc_o, params.THETA, params.EPS, active, True)
        oracle.set_walk_chunk(0)
        r = np.linalg.norm(acc[idx] - acc_o[idx], axis=1) / np.linalg.norm(acc_o[idx], axis=1)
        assert np.percentile(r, 99) <= 1e-4 and r.max() < 1e-3, (chunk, np.percentile(r, 99), r.max())
        e = np.linalg.norm(acc[idx] - ref, axis=1) / np.linalg.norm(ref, axis=1)
        errs[chunk] = np.percentile(e, 99)
    lib.gf_set_option(_lib.OPT_WALK_CHUNK, 0)
    # items drop the group's extra margin: the error is the per-particle criterion's
    for chunk in (1, 4, 16, 72, 96):
        assert errs[chunk] <= 2.0 * errs[0], errs


def test_block_autotune_restores_state(gpulib):
    """The autotuner's trial blocks (with the thermal update on) leave positions, velocities,
    energies and time as they were."""
    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    _plain(lib)
    d = synthetic.make_config(1, scale=0.05)
    n = len(d["mass"])
    _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], params.THETA, params.EPS,
                               params.GAMMA, params.ALPHA, params.BETA))
    units = np.array(params.THERMO_UNITS)
    _lib.check(lib.gf_sim_thermo(2, units.ctypes.data))
    try:
        upd = ctypes.c_double()
        _lib.check(lib.gf_sim_blocks(1, 4, ctypes.byref(upd)))
        p0, v0, t0 = _state(lib, n)
        u0 = np.empty(n)
        _lib.check(lib.gf_sim_read_u(u0))
        chunk = np.zeros(3, np.int32)
        every = ctypes.c_int()
        ms = ctypes.c_double()
        _lib.check(lib.gf_sim_block_autotune(4, chunk.ctypes.data, ctypes.byref(every), ctypes.byref(ms)))
        # walk items: chunks of one group, or sibling runs merged by active count
        assert {c % 100 for c in chunk.tolist()} <= {0, 2, 4, 8, 16, 32, 64, 72, 80, 84, 96}
        assert every.value in (0, 4) and ms.value > 0
        p1, v1, t1 = _state(lib, n)
        u1 = np.empty(n)
        _lib.check(lib.gf_sim_read_u(u1))
        assert t1 == t0
        assert np.array_equal(p1, p0) and np.array_equal(v1, v0) and np.array_equal(u1, u0)
        _lib.check(lib.gf_sim_blocks(2, 4, ctypes.byref(upd)))
        p2, v2, t2 = _state(lib, n)
        assert t2 > t1 and np.all(np.isfinite(p2)) and np.all(np.isfinite(v2))
    finally:
        lib.gf_sim_thermo(0, None)


def test_wide_rounds_walk_matches(gpulib):
    """The mixed walk with 8 nodes per lane and round (bins of a few items) evaluates the same
    interactions as the 2-per-lane walk: block runs of the two agree to float32 summation
    order."""
    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    _plain(lib)
    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 1)
    d = synthetic.rotating_cloud(3000, 3000, seed=12)
    d["kind"][:] = params.DM
    d["u"][:] = 0.0
    n = len(d["mass"])
    out = {}
    for name, chunk in (("two", [4, 8, 16]), ("eight", [104, 108, 116])):
        ch = np.array(chunk, np.int32)
        _lib.check(lib.gf_sim_block_config(ch.ctypes.data, 3, 0))
        _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.55, params.EPS,
                                   params.GAMMA, params.ALPHA, params.BETA))
        upd = ctypes.c_double()
        _lib.check(lib.gf_sim_blocks(2, 4, ctypes.byref(upd)))
        out[name] = _state(lib, n)
    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
    (p2, v2, t2), (p8, v8, t8) = out["two"], out["eight"]
    assert abs(t2 - t8) <= 1e-6 * t2
    scale = np.linalg.norm(p2, axis=1).mean()
    assert np.percentile(np.linalg.norm(p8 - p2, axis=1), 99) < 1e-5 * scale
    vs = np.linalg.norm(v2, axis=1).mean()
    assert np.percentile(np.linalg.norm(v8 - v2, axis=1), 99) < 1e-4 * vs


def test_blocks_relative_opening(gpulib):
    """Block time steps with the relative opening criterion (its error scale is every
    particle's last gravity, kept on the device across the captured sub-steps) stay within
    the criterion's accuracy of the geometric walk."""
    from galaxy_formation_gb300 import _lib, params, synthetic

    lib = gpulib
    _plain(lib)
    lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 1)
    d = synthetic.rotating_cloud(3000, 3000, seed=12)
    d["kind"][:] = params.DM
    d["u"][:] = 0.0
    n = len(d["mass"])
    out = {}
    try:
        for rel in (0.0, 2.5e-3):
            lib.gf_set_option(_lib.OPT_GRAVITY_REL, rel)
            ch = np.array([4, 8, 16], np.int32)
            _lib.check(lib.gf_sim_block_config(ch.ctypes.data, 3, 2))
            _lib.check(lib.gf_sim_init(n, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], 0.55, params.EPS,
                                       params.GAMMA, params.ALPHA, params.BETA))
            upd = ctypes.c_double()
            _lib.check(lib.gf_sim_blocks(2, 4, ctypes.byref(upd)))
            out[rel] = _state(lib, n)
    finally:
        lib.gf_set_option(_lib.OPT_GRAVITY_REL, 0)
        lib.gf_set_option(_lib.OPT_GRAVITY_QUAD, 0)
    (pg, vg, tg), (pr, vr, tr) = out[0.0], out[2.5e-3]
    assert np.all(np.isfinite(pr)) and np.all(np.isfinite(vr))
    assert abs(tr - tg) <= 1e-3 * tg
    moved = np.percentile(np.linalg.norm(pg - d["pos"], axis=1), 99)
    assert np.percentile(np.linalg.norm(pr - pg, axis=1), 99) < 1e-2 * moved
    dv = np.percentile(np.linalg.norm(vg - d["vel"], axis=1), 99)
    assert np.percentile(np.linalg.norm(vr - vg, axis=1), 99) < 2e-2 * dv
