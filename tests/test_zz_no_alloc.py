"""gf_sph_forces_noalloc_dev: the SPH force entry point that allocates no device memory.

It exists for callers that cannot call cudaMalloc (a host whose memory pool owns the GPU,
or a step loop that must not allocate because cudaMalloc/cudaFree synchronise the
device). Here it is called through the C ABI on caller-owned device buffers and compared
with gf_sph_forces_dev, the allocating entry point, on two calls in a row (the second with
a different particle set, so leftovers of the first call in the shared scratch would
show), and it must refuse a particle count above its fixed scratch size.
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


def _run(lib, torch, fn, data):
    from galaxy_formation_gb300 import params

    dev = torch.device("cuda")
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in data.items()}
    n, k = data["nb"].shape
    out = {"rho": torch.full((n,), np.nan, dtype=torch.float64, device=dev),
           "acc": torch.full((n, 3), np.nan, dtype=torch.float64, device=dev),
           "dudt": torch.full((n,), np.nan, dtype=torch.float64, device=dev),
           "dt": torch.full((n,), np.nan, dtype=torch.float64, device=dev)}
    st = fn(n, k, t["pos"].data_ptr(), t["vel"].data_ptr(), t["mass"].data_ptr(), t["nb"].data_ptr(),
            t["h"].data_ptr(), t["u"].data_ptr(), params.GAMMA, params.ALPHA, params.BETA,
            out["rho"].data_ptr(), out["acc"].data_ptr(), out["dudt"].data_ptr(), out["dt"].data_ptr(),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st == 0, (st, lib.gf_last_error())
    return {k: v.cpu().numpy() for k, v in out.items()}


def _close(x, y):
    x = np.asarray(x).reshape(len(x), -1)
    y = np.asarray(y).reshape(len(y), -1)
    err = np.linalg.norm(x - y, axis=1) / np.maximum(np.linalg.norm(y, axis=1), 1e-300)
    return np.all(np.isfinite(x)) and err.max() < TOL


def test_noalloc_matches_allocating_entry_twice(gpulib, golden, oracle):
    torch = pytest.importorskip("torch")
    lib = gpulib
    for data in _sets(golden, oracle):
        got = _run(lib, torch, lib.gf_sph_forces_noalloc_dev, data)
        ref = _run(lib, torch, lib.gf_sph_forces_dev, data)
        for key in ("rho", "acc", "dudt", "dt"):
            assert _close(got[key], ref[key]), key


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
