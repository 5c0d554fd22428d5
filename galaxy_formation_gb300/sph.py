"""Drop-in for the reference's galaxy_formation/sph.py, backed by libgfgpu.so.

Same module constants, functions and signatures (galaxy_formation/sph.py:26-170):
`kernel`, `kernel_grad`, `sph_forces` (outputs written in place), `knn_from_candidates`
(returns False when some particle lacks candidates) and `NeighbourFinder(n_total).find(g,
p, fresh)` with its Verlet-list cache keyed by global particle index. The numerics run in
CUDA kernels (float64 arithmetic, as in the reference); numba is not needed.
"""

import numpy as np

from . import _lib

N_NEIGHBOURS = 32
N_CANDIDATES = 48   # Verlet-list size: candidates kept between two full searches
ALPHA, BETA = 1.0, 2.0


def _kernel_values(r, h, which):
    lib = _lib.load()
    scalar = np.ndim(r) == 0 and np.ndim(h) == 0
    rr, hh = np.broadcast_arrays(np.asarray(r, np.float64), np.asarray(h, np.float64))
    rr = np.ascontiguousarray(rr.ravel())
    hh = np.ascontiguousarray(hh.ravel())
    out = np.empty(rr.size)
    w = out.ctypes.data if which == 0 else None
    dw = out.ctypes.data if which == 1 else None
    _lib.check(lib.gf_sph_kernel(rr.size, rr, hh, w, dw))
    return float(out[0]) if scalar else out.reshape(np.broadcast(np.asarray(r), np.asarray(h)).shape)


def kernel(r, h):
    """Cubic spline (M4) kernel with support 2h (sph.py:31-40); scalars or arrays."""
    return _kernel_values(r, h, 0)


def kernel_grad(r, h):
    """(1/r) dW/dr (sph.py:43-54): multiply by the separation vector to get grad W."""
    return _kernel_values(r, h, 1)


def sph_forces(pos, vel, mass, nb, h, u, gamma, alpha, beta, rho, acc, dudt, dt_i):
    """Density, pressure + viscosity acceleration, du/dt and Courant time step of every gas
    particle (sph.py:57-106). nb holds the neighbour indices (the particle itself
    included). Outputs: rho, acc, dudt, dt_i (written in place)."""
    n, k = nb.shape
    st = _lib.load().gf_sph_forces(
        n, k, np.ascontiguousarray(pos, np.float64), np.ascontiguousarray(vel, np.float64),
        np.ascontiguousarray(mass, np.float64), np.ascontiguousarray(nb, np.int64),
        np.ascontiguousarray(h, np.float64), np.ascontiguousarray(u, np.float64),
        float(gamma), float(alpha), float(beta), rho, acc, dudt, dt_i)
    _lib.check(st)


def knn_from_candidates(pos, cand, k, nb, dist):
    """k nearest neighbours of each particle among its candidates (local indices, -1 =
    none), sph.py:109-135. Returns False if some particle does not have enough candidates."""
    n, m = cand.shape
    r = _lib.load().gf_knn_from_candidates(n, m, np.ascontiguousarray(pos, np.float64),
                                           np.ascontiguousarray(cand, np.int64), int(k), nb, dist)
    if r < 0:
        _lib.check(-r)
    return bool(r)


def knn(p, k):
    """Exact k nearest points of every point (itself included), ascending: the
    `cKDTree(p).query(p, k=k)` of sph.py:166. Returns (dist (n,k), nb (n,k) int64)."""
    p = np.ascontiguousarray(p, np.float64)
    n = len(p)
    dist = np.empty((n, k))
    nb = np.empty((n, k), np.int64)
    _lib.check(_lib.load().gf_knn(n, p, int(k), dist, nb))
    return dist, nb


class NeighbourFinder:
    """The caching neighbour finder of sph.py:138-170, with the searches on the GPU.

    fresh=True, or a gas particle missing from the cache, or one left with fewer than 32
    usable candidates: an exact search of the 48 nearest (gf_knn), whose rows become the new
    cache. Otherwise each particle's 32 nearest are picked again from its cached 48 at the
    current positions (gf_knn_from_candidates). The cache stores global particle indices and
    a row per global index, so it stays valid when some gas has turned into stars since."""

    def __init__(self, n_total):
        self.n_total = n_total
        self.cache = None

    def find(self, g, p, fresh):
        """Neighbours of the gas particles with global indices g at positions p (len(g), 3):
        returns (dist (len(g), 32) ascending, nb (len(g), 32) int64 as positions in g)."""
        k = N_NEIGHBOURS
        if not fresh and self.cache is not None:
            row = self.cache["row"][g]
            if (row >= 0).all():
                loc = np.full(self.n_total, -1, np.int64)
                loc[g] = np.arange(g.size)
                cand = loc[self.cache["cand"][row]]      # -1 where a candidate is no longer gas
                nb = np.empty((g.size, k), np.int64)
                d = np.empty((g.size, k))
                if knn_from_candidates(p, cand, k, nb, d):
                    return d, nb
        kq = min(N_CANDIDATES, g.size)
        d, nb = knn(p, kq)
        row = np.full(self.n_total, -1, np.int64)
        row[g] = np.arange(g.size)
        self.cache = {"row": row, "cand": g[nb]}
        return d[:, :k], np.ascontiguousarray(nb[:, :k])
