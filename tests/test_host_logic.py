"""Host-side logic that needs no GPU: synthetic inputs, the drop-in modules' constants and
the NeighbourFinder cache logic (driven here with the oracle's search functions)."""

import numpy as np
import pytest

from galaxy_formation_gb300 import params, synthetic


def test_params_match_reference_defaults():
    assert params.THETA == 0.7 and params.EPS_KPC == 0.4 and params.KPC == 3.5
    assert params.N_NEIGHBOURS == 32 and params.N_CANDIDATES == 48
    assert (params.ALPHA, params.BETA) == (1.0, 2.0)


@pytest.mark.parametrize("idx", [0, 1, 2, 3, 4])
def test_configs_shape_and_mass(idx):
    d = synthetic.make_config(idx, scale=0.01)
    n = len(d["mass"])
    assert d["pos"].shape == (n, 3) and d["vel"].shape == (n, 3)
    assert d["pos"].dtype == np.float64 and d["pos"].flags.c_contiguous
    gas = d["kind"] == params.GAS
    assert np.all(d["u"][gas] > 0) and np.all(d["u"][~gas] == 0)
    if idx in (0, 1, 2, 4):
        assert np.isclose(d["mass"].sum() * params.MSUN, 2.8e11)
        assert np.isclose(d["mass"][gas].sum() / d["mass"].sum(), 0.16)
    # no bulk motion
    p = np.average(d["vel"], axis=0, weights=d["mass"])
    assert np.abs(p).max() < 1e-10


def test_cloud_radius_and_spin():
    """tests/test_physics.py:56-64 of the reference, on the restated generator."""
    d = synthetic.rotating_cloud(2000, 2000)
    assert np.linalg.norm(d["pos"], axis=1).max() * 3.5 <= 100.0 + 1e-9
    J = np.sum(d["mass"][:, None] * np.cross(d["pos"], d["vel"]), axis=0)
    assert J[2] > 0 and abs(J[2]) > 5 * np.hypot(J[0], J[1])


def test_disk_temperatures_and_clumps():
    d = synthetic.disk_halo(n_gas=20000, n_dm=0, n_clumps=10, clump_frac=1e-3)
    gas = d["kind"] == params.GAS
    T = d["u"][gas] / params.U_PER_K
    assert T.min() >= 1e4 * (1 - 1e-9) and T.max() <= 1e6 * (1 + 1e-9)
    R = np.hypot(d["pos"][:, 0], d["pos"][:, 1])
    assert np.median(np.abs(d["pos"][:12000, 2])) < 0.5 / params.KPC  # thin disk part
    assert np.median(R[:12000]) < 10 / params.KPC


def test_neighbour_finder_cache_logic(oracle, monkeypatch):
    """NeighbourFinder.find (sph.py:151-170): full search caches 48 global candidates;
    sub-steps reselect among the candidates that are still gas; a particle outside the
    cache forces a full search."""
    from galaxy_formation_gb300 import sph

    calls = {"full": 0}

    def fake_knn(p, k):
        calls["full"] += 1
        return oracle.knn_brute(p, k)

    monkeypatch.setattr(sph, "knn", fake_knn)
    monkeypatch.setattr(sph, "knn_from_candidates", oracle.knn_from_candidates)
    d = synthetic.rotating_cloud(600, 400, seed=1)
    n = len(d["mass"])
    g = np.flatnonzero(d["kind"] == params.GAS)
    f = sph.NeighbourFinder(n)
    dist, nb = f.find(g, d["pos"][g], True)
    assert calls["full"] == 1 and dist.shape == (g.size, 32) and nb.shape == (g.size, 32)
    assert f.cache["cand"].shape == (g.size, 48)
    assert np.array_equal(f.cache["cand"][:, :32], g[nb])
    # drift a little: Verlet reselection, no new full search
    p1 = d["pos"][g] + 1e-3
    dist1, nb1 = f.find(g, p1, False)
    assert calls["full"] == 1
    dd, nbb = oracle.knn_brute(p1, 32)
    assert np.array_equal(nb1, nbb)
    # a gas particle turns into a star: candidates map to -1, still enough of them
    g2 = g[1:]
    dist2, nb2 = f.find(g2, d["pos"][g2], False)
    assert calls["full"] == 1 and nb2.max() < g2.size
    # fresh=True always searches again
    f.find(g, d["pos"][g], True)
    assert calls["full"] == 2


def test_pcg64_words_round_trip():
    """The generator state handed to the device's star formation is NumPy's PCG64 state."""
    import numpy as np

    from galaxy_formation_gb300 import subgrid

    g = np.random.default_rng(3)
    g.uniform(size=5)
    w = subgrid.pcg64_words(g)
    h = np.random.default_rng(0)
    subgrid.set_pcg64_words(h, w)
    assert np.array_equal(g.uniform(size=9), h.uniform(size=9))
    assert int(w[3]) & 1 == 1   # PCG increments are odd


def test_snapshot_round_trip(tmp_path):
    """A particle set and extra arrays survive save / load bit for bit."""
    import numpy as np

    from galaxy_formation_gb300 import snapshot, synthetic

    d = synthetic.rotating_cloud(300, 200, seed=2)
    p = tmp_path / "snap.npz"
    snapshot.save(p, d["pos"], d["vel"], d["mass"], d["kind"], d["u"], t=1.25, extra=np.arange(3))
    s = snapshot.load(p)
    for k in snapshot.PARTICLE_KEYS:
        assert np.array_equal(s[k], d[k]) and s[k].dtype == np.asarray(d[k]).dtype
    assert float(s["t"]) == 1.25 and np.array_equal(s["extra"], np.arange(3))
    import pytest
    with pytest.raises(ValueError):
        snapshot.save(p, d["pos"][:10], d["vel"], d["mass"], d["kind"], d["u"])
