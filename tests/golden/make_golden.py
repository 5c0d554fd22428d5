"""Generates the golden fixtures under tests/golden/ from the reference itself.

Run once in a container that has the reference sources (at $GALAXY_FORMATION_REFERENCE,
by default /root/reference):

    make -C oracle ref          # compiles the reference's cpp/nbody.cpp into oracle/_ref/
    python tests/golden/make_golden.py

Gravity comes from the reference's nbody.cpp (built from its sources with its own flags,
loaded through ctypes with the signatures of galaxy_formation/engine.py:30-35). SPH comes
from the reference's galaxy_formation/sph.py, imported with a numba stand-in
(oracle/numba_shim: njit = identity, prange = range), so it runs as plain NumPy in float64.
Initial conditions come from the reference's own make_cloud (initial_conditions.py:33-68).

Fixtures (npz):
  bh_gauss20k.npz  the reference test case (tests/test_physics.py:20-30): 20,000 Gaussian
                   points, m = 1/N, theta 0.7, eps 0.01; Barnes-Hut accelerations (float32
                   sums stored exactly) and direct-sum accelerations of 2,000 targets.
  cloud10k.npz     the default cloud (5k gas + 5k DM, seed 3): inputs, Barnes-Hut at the
                   default theta/eps, then a refit call after a drift with half the
                   particles active.
  sph2k.npz        a 2k + 2k cloud: the 48-candidate neighbour search, h, sph_forces
                   outputs, and a Verlet reselection after a drift.
  cooling.npz      the reference's cooling_function on a temperature grid spanning the floor,
                   and cool() on random (u, rho, dt, blocked) with the simulator's floor
                   (cooling.py:24-43, simulation.py:38-42).
  render.npz       the default cloud splatted by the reference's nbody_render into three
                   colour groups of a 160 x 120 image (cpp/nbody.cpp:445-469), and its
                   nbody_tonemap of that image with a glow derived from it as
                   rendering.py:115-124 does (cpp/nbody.cpp:474-503).

Pass fixture names (bh_gauss cloud sph cooling render) to regenerate only those.
"""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.environ.get("GALAXY_FORMATION_REFERENCE", "/root/reference")
OUT = os.path.dirname(os.path.abspath(__file__))

sys.path.insert(0, os.path.join(ROOT, "oracle", "numba_shim"))
sys.path.insert(0, REF)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from galaxy_formation.config import Config  # noqa: E402
from galaxy_formation.initial_conditions import make_cloud  # noqa: E402
from galaxy_formation import sph as ref_sph  # noqa: E402
from galaxy_formation.units import K_B, KPC, M_H, MU_IONISED, U_CGS  # noqa: E402
from galaxy_formation import cooling as ref_cooling  # noqa: E402


def bh_gauss():
    ref = oracle.RefNbody()
    rng = np.random.default_rng(0)
    pos = np.ascontiguousarray(rng.normal(size=(20000, 3)))
    mass = np.full(len(pos), 1.0 / len(pos))
    acc = np.zeros_like(pos)
    ref.gravity(pos, mass, acc, theta=0.7, eps=0.01)
    exact = ref.gravity_direct(pos, mass, eps=0.01)
    tgt = np.random.default_rng(1).choice(len(pos), 2000, replace=False)
    assert np.array_equal(acc.astype(np.float32).astype(np.float64), acc)
    np.savez_compressed(os.path.join(OUT, "bh_gauss20k.npz"), pos=pos, mass=mass,
                        acc_bh=acc.astype(np.float32), targets=tgt, acc_direct=exact[tgt],
                        theta=0.7, eps=0.01)


def cloud():
    ref = oracle.RefNbody()
    cfg = Config()
    rng = np.random.default_rng(cfg.seed)
    pos, vel, mass, kind = make_cloud(cfg, rng)
    eps = cfg.eps / KPC
    acc = np.zeros_like(pos)
    ref.gravity(pos, mass, acc, cfg.theta, eps)
    # refit: drift everybody, then only half of the particles are active
    pos1 = np.ascontiguousarray(pos + 0.05 * vel)
    act = (np.random.default_rng(5).uniform(size=len(mass)) < 0.5).astype(np.uint8)
    acc1 = acc.copy()
    ref.gravity(pos1, mass, acc1, cfg.theta, eps, active=act, rebuild=False)
    for a in (acc, acc1):
        assert np.array_equal(a.astype(np.float32).astype(np.float64), a)
    np.savez_compressed(os.path.join(OUT, "cloud10k.npz"), pos=pos, vel=vel, mass=mass,
                        kind=kind, theta=cfg.theta, eps=eps, acc_bh=acc.astype(np.float32),
                        pos1=pos1, active1=act, acc_refit=acc1.astype(np.float32))


def sph():
    cfg = Config(n_gas=2000, n_dm=2000)
    rng = np.random.default_rng(cfg.seed)
    pos, vel, mass, kind = make_cloud(cfg, rng)
    eps = cfg.eps / KPC
    gamma = 5.0 / 3.0
    g = np.flatnonzero(kind == 0)
    p = np.ascontiguousarray(pos[g])
    finder = ref_sph.NeighbourFinder(len(mass))
    d, nb = finder.find(g, p, True)
    cand = finder.cache["cand"][finder.cache["row"][g]]
    h = np.maximum(0.5 * d[:, -1], 0.5 * eps)
    # log-uniform temperatures so that pressure and viscosity terms both matter
    u = np.exp(np.random.default_rng(7).uniform(np.log(1e4), np.log(1e6), len(g))) * 1.9e-4
    v = np.ascontiguousarray(vel[g])
    m = np.ascontiguousarray(mass[g])
    rho, a = np.empty(len(g)), np.empty((len(g), 3))
    dudt, dt_i = np.empty(len(g)), np.empty(len(g))
    ref_sph.sph_forces(p, v, m, nb, h, u, gamma, ref_sph.ALPHA, ref_sph.BETA, rho, a, dudt, dt_i)
    # Verlet reselection after a drift (sub-step search)
    p1 = np.ascontiguousarray(p + 0.02 * v)
    d1, nb1 = finder.find(g, p1, False)
    np.savez_compressed(os.path.join(OUT, "sph2k.npz"), pos=p, vel=v, mass=m, u=u, eps=eps,
                        gamma=gamma, dist=d, nb=nb.astype(np.int32), cand=cand.astype(np.int32),
                        h=h, rho=rho, acc=a, dudt=dudt, dt_i=dt_i, pos1=p1, dist1=d1,
                        nb1=nb1.astype(np.int32), kernel_r=np.linspace(0, 1.5, 61),
                        kernel_w=np.array([ref_sph.kernel(r, 0.7) for r in np.linspace(0, 1.5, 61)]),
                        kernel_g=np.array([ref_sph.kernel_grad(r, 0.7)
                                           for r in np.linspace(0, 1.5, 61)]))


def cooling():
    T = np.concatenate([np.logspace(3, 9, 241), [5e3, 1e4, np.nextafter(1e4, 2e4), 2e4, 1e5, 1e6, 1e8]])
    lam = ref_cooling.cooling_function(T)
    gamma = 5.0 / 3.0
    u_per_K = K_B / ((gamma - 1) * MU_IONISED * M_H) / U_CGS
    u_floor = ref_cooling.T_FLOOR * u_per_K
    rng = np.random.default_rng(11)
    n = 4000
    u = np.exp(rng.uniform(np.log(0.5e4), np.log(1e8), n)) * u_per_K
    rho = np.exp(rng.uniform(np.log(1e-7), np.log(1e1), n))
    dt = np.exp(rng.uniform(np.log(1e-6), np.log(1e-2), n))
    blocked = rng.uniform(size=n) < 0.1
    u_new = ref_cooling.cool(u, u / u_per_K, rho, dt, blocked, u_floor)
    np.savez_compressed(os.path.join(OUT, "cooling.npz"), T=T, lam=lam, u_per_K=u_per_K, u_floor=u_floor,
                        u=u, rho=rho, dt=dt, blocked=blocked, u_new=u_new)


def render():
    from scipy.ndimage import gaussian_filter

    ref = oracle.RefNbody()
    cfg = Config()
    rng = np.random.default_rng(cfg.seed)
    pos, _, _, kind = make_cloud(cfg, rng)
    group = np.ascontiguousarray(np.random.default_rng(13).integers(0, 3, len(kind)), np.uint8)
    a, e = np.radians(30.0), np.radians(25.0)  # the screen axes of an azimuth / elevation view
    d = np.array([np.cos(e) * np.cos(a), np.cos(e) * np.sin(a), np.sin(e)])
    right = np.array([-np.sin(a), np.cos(a), 0.0])
    rot = np.ascontiguousarray(np.stack([right, np.cross(d, right), d]))
    center = np.zeros(3)
    W, H, K, exposure, glow_gain = 160, 120, 40.0, 1.6, 0.5
    scale = W / (2 * 1.2 * np.abs(pos).max())
    img = np.zeros((3, H, W), np.float32)
    ref.lib.nbody_render(len(kind), np.ascontiguousarray(pos), group, 3, rot, center, scale, W, H, img)
    small = img.reshape(3, H // 4, 4, W // 4, 4).mean(axis=(2, 4))
    level = max(np.percentile(small.sum(axis=0), 99.9), 1e-3)
    glow = gaussian_filter(small / level, sigma=(0, 3, 3))
    glow = np.ascontiguousarray(glow_gain * np.log1p(K * glow) / np.log1p(K), np.float32)
    colors = np.array([[1.0, 0.55, 0.25], [0.35, 0.6, 1.0], [0.9, 0.9, 0.85]], np.float32)
    rgb = np.zeros((H, W, 3), np.uint8)
    ref.lib.nbody_tonemap(W, H, 3, img, glow, W // 4, H // 4, colors, np.float32(1 / level), np.float32(K),
                          np.float32(exposure), rgb)
    np.savez_compressed(os.path.join(OUT, "render.npz"), pos=pos, group=group, rot=rot, center=center,
                        scale=scale, img=img, glow=glow, colors=colors, inv_ref=np.float32(1 / level), K=K,
                        exposure=exposure, rgb=rgb)


if __name__ == "__main__":
    oracle.build()
    names = sys.argv[1:] or ["bh_gauss", "cloud", "sph", "cooling", "render"]
    for name in names:
        globals()[name]()
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))
