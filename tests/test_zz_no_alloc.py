"""gf_sph_forces_noalloc_dev: the SPH force entry point that allocates no device memory.

It exists for callers that cannot call cudaMalloc (a host whose memory pool owns the GPU,
or a step loop that must not allocate because cudaMalloc/cudaFree synchronise the
device). Here it is called through the C ABI on caller-owned device buffers and compared
with gf_sph_forces_dev, the allocating entry point, on two calls in a row: first a larger
particle set, then a smaller one written into output buffers with spare rows, which must
stay untouched (the call writes rows 0..n-1 only); around the second call the device's free
memory must not change. It must refuse a particle count above its fixed scratch size, and a
neighbour index outside [0, n) gives that particle NaN outputs instead of a read out of
bounds.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5   # the SPH parity tolerance of tests/test_gpu_sph.py


def _sets(golden, oracle):
    from galaxy_formation_gb300 import params, synthetic

    s = golden("sph2k.npz")
    a = dict(pos=s["pos"], vel=s["vel"], mass=s["mass"], nb=s["nb"].astype(np.int64), h=s["h"],
             u=s["u"])
    d = synthetic.make_config(1, scale=0.05)
    gas = d["kind"] == params.GAS
    p = np.ascontiguousarray(d["pos"][gas])
    dist, nb = oracle.knn_brute(p, 32)
    b = dict(pos=p, vel=np.ascontiguousarray(d["vel"][gas]), mass=np.ascontiguousarray(d["mass"][gas]),
             nb=nb, h=np.maximum(0.5 * dist[:, -1], 0.5 * params.EPS), u=np.ascontiguousarray(d["u"][gas]))
    return a, b


def _run(lib, torch, fn, data, spare=0, expect_finite=True, check_free=False):
    from galaxy_formation_gb300 import params

    dev = torch.device("cuda")
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in data.items()}
    n, k = data["nb"].shape
    m = n + spare  # output rows: the n the call writes, then spare ones it must leave alone
    out = {"rho": torch.full((m,), np.nan, dtype=torch.float64, device=dev),
           "acc": torch.full((m, 3), np.nan, dtype=torch.float64, device=dev),
           "dudt": torch.full((m,), np.nan, dtype=torch.float64, device=dev),
           "dt": torch.full((m,), np.nan, dtype=torch.float64, device=dev)}
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]  # every buffer of the call exists already
    st = fn(n, k, t["pos"].data_ptr(), t["vel"].data_ptr(), t["mass"].data_ptr(), t["nb"].data_ptr(),
            t["h"].data_ptr(), t["u"].data_ptr(), params.GAMMA, params.ALPHA, params.BETA,
            out["rho"].data_ptr(), out["acc"].data_ptr(), out["dudt"].data_ptr(), out["dt"].data_ptr(),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st == 0, (st, lib.gf_last_error())
    if check_free:  # the call took no device memory
        assert torch.cuda.mem_get_info()[0] == free0
    res = {k: v.cpu().numpy() for k, v in out.items()}
    for v in res.values():
        assert np.all(np.isnan(v[n:]))
    return {k: v[:n] for k, v in res.items()}


def _close(x, y):
    x = np.asarray(x).reshape(len(x), -1)
    y = np.asarray(y).reshape(len(y), -1)
    err = np.linalg.norm(x - y, axis=1) / np.maximum(np.linalg.norm(y, axis=1), 1e-300)
    return np.all(np.isfinite(x)) and err.max() < TOL


def test_noalloc_matches_allocating_entry_twice(gpulib, golden, oracle):
    torch = pytest.importorskip("torch")
    lib = gpulib
    small, large = _sets(golden, oracle)
    assert len(large["pos"]) > len(small["pos"])
    for data, spare in ((large, 0), (small, 1000)):
        # the second call on this device: its one-time set-up (the scratch address) is done
        got = _run(lib, torch, lib.gf_sph_forces_noalloc_dev, data, spare, check_free=spare > 0)
        ref = _run(lib, torch, lib.gf_sph_forces_dev, data)
        for key in ("rho", "acc", "dudt", "dt"):
            assert _close(got[key], ref[key]), key


def test_noalloc_out_of_range_neighbour_gives_nan(gpulib, golden, oracle):
    """A neighbour row holding an index past the particle count: that particle's outputs are
    NaN (the kernels check every row before reading through it), and so are those of the
    particles that have it as a neighbour; every other particle is unaffected."""
    torch = pytest.importorskip("torch")
    lib = gpulib
    small, _ = _sets(golden, oracle)
    bad = dict(small)
    bad["nb"] = small["nb"].copy()
    n = len(bad["nb"])
    bad["nb"][5, 3] = n
    got = _run(lib, torch, lib.gf_sph_forces_noalloc_dev, bad)
    assert np.isnan(got["rho"][5]) and np.all(np.isnan(got["acc"][5])) and np.isnan(got["dt"][5])
    clean = np.flatnonzero(~np.any(bad["nb"] == 5, axis=1) & (np.arange(n) != 5))
    assert clean.size > n // 2
    ref = _run(lib, torch, lib.gf_sph_forces_dev, small)
    for key in ("rho", "acc", "dudt", "dt"):
        assert _close(got[key][clean], ref[key][clean]), key


def test_noalloc_rejects_more_particles_than_its_scratch(gpulib):
    torch = pytest.importorskip("torch")
    lib = gpulib
    from galaxy_formation_gb300 import params

    limit = 262144  # GF_SPH_NOALLOC_MAX_N
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    st = lib.gf_sph_forces_noalloc_dev(limit + 1, 32, p, p, p, p, p, p, params.GAMMA, params.ALPHA,
                                       params.BETA, p, p, p, p, None)
    assert st == 128  # GF_ERR_CAPACITY
    assert b"exceeds" in lib.gf_last_error()
    torch.cuda.synchronize()
    assert torch.all(buf == 0)
