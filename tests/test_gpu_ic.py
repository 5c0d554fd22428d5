"""Initial conditions drawn on the GPU (gf_ic_generate) against the host generators of
galaxy_formation_gb300/synthetic.py: the 4M rotating cloud of the drift workload and a 16M
variant, the 1M disk + halo snapshot and the 1M-gas disk with 200 Plummer clumps.

The device sets use counter-based random numbers, so they match the host sets in
distribution, not draw for draw: masses exactly; radial profiles against the analytic ones
(Kolmogorov-Smirnov distance within 2/sqrt(N)); spin, dispersion and disk moments against the
host set's within a few per cent; no bulk motion; the same set again for the same seed and
another set for another seed.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ks_r2(r, R0):
    """KS distance of radii against M(<r) ~ r^2 (the 1/r sphere: P(r < x R0) = x^2)."""
    x = np.sort(r / R0)
    emp = np.arange(1, len(x) + 1) / len(x)
    return np.max(np.abs(emp - x ** 2))


def _lz_per_mass(d):
    p, v, m = d["pos"], d["vel"], d["mass"]
    return float(np.sum(m * (p[:, 0] * v[:, 1] - p[:, 1] * v[:, 0])) / m.sum())


def test_device_cloud_matches_host(gpulib):
    from galaxy_formation_gb300 import params, synthetic

    host = synthetic.make_config(4)  # 2M gas + 2M dark matter
    R0 = synthetic.CLOUD_DEFAULTS["r0"] / params.KPC
    M = synthetic.CLOUD_DEFAULTS["mass"] / params.MSUN
    v_vir = np.sqrt(M / R0)
    for scale in (1.0, 4.0):  # 4M, and a 16M variant
        d = synthetic.make_config_device(4, seed=3, scale=scale, lib=gpulib)
        n_gas = int(2_000_000 * scale)
        n = len(d["mass"])
        assert n == 2 * n_gas
        assert np.all(d["kind"][:n_gas] == params.GAS) and np.all(d["kind"][n_gas:] == params.DM)
        assert abs(d["mass"].sum() - M) <= 1e-9 * M
        assert abs(d["mass"][:n_gas].sum() - 0.16 * M) <= 1e-9 * M
        for sl in (slice(0, n_gas), slice(n_gas, n)):
            r = np.linalg.norm(d["pos"][sl], axis=1)
            assert r.max() <= R0 * (1 + 1e-12)
            assert _ks_r2(r, R0) < 2.0 / np.sqrt(len(r))
            dirs = d["pos"][sl] / r[:, None]
            assert np.abs(dirs.mean(axis=0)).max() < 4.0 / np.sqrt(len(r))
        # no bulk motion; the host set's spin and dispersion
        p_tot = np.sum(d["mass"][:, None] * d["vel"], axis=0)
        assert np.abs(p_tot).max() <= 1e-9 * M * v_vir
        assert abs(_lz_per_mass(d) / _lz_per_mass(host) - 1) < 0.01
        sz = np.std(d["vel"][:, 2])
        assert abs(sz / np.std(host["vel"][:, 2]) - 1) < 0.01
        assert np.all(d["u"][:n_gas] == host["u"][0]) and np.all(d["u"][n_gas:] == 0)
    # a pure function of its arguments
    a = synthetic.make_config_device(4, seed=3, scale=0.05, lib=gpulib)
    b = synthetic.make_config_device(4, seed=3, scale=0.05, lib=gpulib)
    c = synthetic.make_config_device(4, seed=4, scale=0.05, lib=gpulib)
    for k in ("pos", "vel", "mass", "kind", "u"):
        assert np.array_equal(a[k], b[k])
    assert not np.array_equal(a["pos"], c["pos"])


def _disk_moments(d, n_disk, n_smooth):
    p = d["pos"][:n_smooth]
    R = np.hypot(p[:, 0], p[:, 1])
    return {"mean_R": R.mean(), "mean_absz": np.abs(p[:, 2]).mean(), "lz": _lz_per_mass(d),
            "disk_vphi": np.mean((p[:, 0] * d["vel"][:n_smooth, 1] - p[:, 1] * d["vel"][:n_smooth, 0]) / R)}


@pytest.mark.parametrize("idx", [2, 3])
def test_device_disk_matches_host(gpulib, idx):
    from galaxy_formation_gb300 import params, synthetic

    host = synthetic.make_config(idx)
    d = synthetic.make_config_device(idx, seed=3, lib=gpulib)
    c = dict(synthetic.CONFIGS[idx])
    n_gas, n_dm, n_clumps = c["n_gas"], c["n_dm"], c.get("n_clumps", 0)
    n_disk = int(round(0.6 * n_gas))
    n_each = int(round(1e-3 * n_gas)) if n_clumps else 0
    n_smooth = n_disk - n_clumps * n_each
    M = synthetic.DISK_DEFAULTS["mass"] / params.MSUN
    assert len(d["mass"]) == n_gas + n_dm
    assert abs(d["mass"].sum() - (M if n_dm else 0.16 * M)) <= 1e-9 * M
    assert np.array_equal(d["kind"], host["kind"])
    # the smooth disk: scale length, sech^2 height, rotation at v_c
    mh, md = _disk_moments(host, n_disk, n_smooth), _disk_moments(d, n_disk, n_smooth)
    for k in ("mean_R", "mean_absz", "disk_vphi"):
        assert abs(md[k] / mh[k] - 1) < 0.02, (k, md[k], mh[k])
    z0 = synthetic.DISK_DEFAULTS["z0_kpc"] / params.KPC
    assert abs(md["mean_absz"] / (z0 * np.log(2)) - 1) < 0.02  # E|z| of sech^2 = z0 ln 2
    assert abs(md["lz"] / mh["lz"] - 1) < 0.03
    # the 1/r components
    R0 = synthetic.DISK_DEFAULTS["r0"] / params.KPC
    for sl in (slice(n_disk, n_gas), slice(n_gas, n_gas + n_dm)):
        if sl.stop > sl.start:
            r = np.linalg.norm(d["pos"][sl], axis=1)
            assert _ks_r2(r, R0) < 2.0 / np.sqrt(len(r))
    # Plummer clumps: members around their centre, median radius a / sqrt(2^(2/3) - 1) for the
    # uniform draw on [1e-6, 0.999) (the median of the truncated law within 1 %)
    if n_clumps:
        a = synthetic.DISK_DEFAULTS["clump_kpc"] / params.KPC
        mem = d["pos"][n_smooth:n_disk].reshape(n_clumps, n_each, 3)
        cen = np.median(mem, axis=1)
        rr = np.linalg.norm(mem - cen[:, None, :], axis=2)
        u_med = 1e-6 + (0.999 - 1e-6) * 0.5
        expect = a / np.sqrt(u_med ** (-2.0 / 3.0) - 1.0)
        assert abs(np.median(rr) / expect - 1) < 0.05
    # gas energies log-uniform between the bounds
    lu = np.log(d["u"][:n_gas])
    lo, hi = np.log(1e4 * params.U_PER_K), np.log(1e6 * params.U_PER_K)
    assert lu.min() >= lo - 1e-12 and lu.max() <= hi + 1e-12
    assert abs(lu.mean() - 0.5 * (lo + hi)) < 4 * (hi - lo) / np.sqrt(12 * n_gas)
    p_tot = np.sum(d["mass"][:, None] * d["vel"], axis=0)
    assert np.abs(p_tot).max() <= 1e-9 * M * np.abs(d["vel"]).max()
