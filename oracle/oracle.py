"""Python bindings of the test oracle (TEST INFRASTRUCTURE ONLY).

`liborc.so` (oracle/gf_oracle.cpp) is a CPU restatement of the reference's Barnes-Hut
engine (cpp/nbody.cpp) and SPH module (galaxy_formation/sph.py). Only tests/, the smoke
check in __graft_entry__.py and bench.py's CPU-baseline legs use it, always as the checker
or the timed CPU baseline, never as part of the product path.

`RefNbody` loads the reference's own cpp/nbody.cpp compiled from its sources into
oracle/_ref/ (present only where the reference sources were available at build time); it is
used to pin the restatement and to generate the committed golden fixtures.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
REF_LIB = os.path.join(HERE, "_ref", "libnbody.so")
SRC = os.path.join(HERE, "gf_oracle.cpp")
# Where the reference's sources live (only in the container that builds the pinned copy);
# override with the GALAXY_FORMATION_REFERENCE environment variable.
REFERENCE_ROOT = os.environ.get("GALAXY_FORMATION_REFERENCE", "/root/reference")

_dbl = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_ci, _cd = ctypes.c_int, ctypes.c_double


def build(force=False):
    """Compiles liborc.so (and oracle/_ref when the reference sources exist)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.run(["make", "-C", HERE, "liborc.so"], check=True,
                       stdout=subprocess.DEVNULL)
    ref_src = os.path.join(REFERENCE_ROOT, "cpp", "nbody.cpp")
    if os.path.exists(ref_src) and not os.path.exists(REF_LIB):
        subprocess.run(["make", "-C", HERE, "ref", f"REF_SRC={ref_src}"], check=True, stdout=subprocess.DEVNULL)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.orc_num_threads.restype = _ci
        L.orc_set_threads.argtypes = [_ci]
        L.orc_set_walk_chunk.argtypes = [_ci]
        L.orc_accel_active.argtypes = [_ci, _dbl, _dbl, _dbl, _cd, _cd, ctypes.c_void_p, _ci]
        L.orc_accel_direct.argtypes = [_ci, _dbl, _dbl, _dbl, _cd]
        L.orc_accel_direct_targets.argtypes = [_ci, _dbl, _dbl, _ci, _i64, _dbl, _cd]
        L.orc_tree_num_nodes.restype = _ci
        L.orc_tree_num_groups.restype = _ci
        L.orc_tree_export.argtypes = [_i32, _f32, _i32, _i32]
        L.orc_sph_kernel.argtypes = [_cd, _cd]
        L.orc_sph_kernel.restype = _cd
        L.orc_sph_kernel_grad.argtypes = [_cd, _cd]
        L.orc_sph_kernel_grad.restype = _cd
        L.orc_sph_forces.argtypes = [_ci, _ci, _dbl, _dbl, _dbl, _i64, _dbl, _dbl, _cd, _cd, _cd,
                                     _dbl, _dbl, _dbl, _dbl]
        L.orc_knn_from_candidates.argtypes = [_ci, _ci, _dbl, _i64, _ci, _i64, _dbl]
        L.orc_knn_from_candidates.restype = _ci
        L.orc_knn_brute.argtypes = [_ci, _dbl, _ci, _dbl, _i64]
        L.orc_render.argtypes = [_ci, _dbl, _u8, _ci, _dbl, _dbl, _cd, _ci, _ci, _f32]
        L.orc_tonemap.argtypes = [_ci, _ci, _ci, _f32, _f32, _ci, _ci, _f32, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, _u8]
        _lib = L
    return _lib


def num_threads():
    return lib().orc_num_threads()


def set_threads(t):
    lib().orc_set_threads(int(t))


def set_walk_chunk(c):
    """Walk items of <= c active particles with their own spheres (0: the reference's groups)."""
    lib().orc_set_walk_chunk(int(c))


def accel_active(pos, mass, acc, theta, eps, active=None, rebuild=True):
    """Restatement of nbody_accel_active (cpp/nbody.cpp:422). acc is updated in place."""
    n = len(mass)
    act = None
    if active is not None:
        act = np.ascontiguousarray(active, dtype=np.uint8)
    lib().orc_accel_active(n, pos, mass, acc, theta, eps,
                           None if act is None else act.ctypes.data, int(rebuild))
    return acc


def accel_direct(pos, mass, eps):
    acc = np.zeros_like(pos)
    lib().orc_accel_direct(len(mass), pos, mass, acc, eps)
    return acc


def accel_direct_targets(pos, mass, targets, eps):
    t = np.ascontiguousarray(targets, dtype=np.int64)
    acc = np.zeros((len(t), 3))
    lib().orc_accel_direct_targets(len(mass), pos, mass, len(t), t, acc, eps)
    return acc


def tree_export():
    """The last tree: dict of ints (nn,4), floats (nn,9), order (n,), groups (ng,)."""
    L = lib()
    nn, ng = L.orc_tree_num_nodes(), L.orc_tree_num_groups()
    n = _last_n[0]
    ints = np.zeros((nn, 4), np.int32)
    floats = np.zeros((nn, 9), np.float32)
    order = np.zeros(n, np.int32)
    groups = np.zeros(ng, np.int32)
    L.orc_tree_export(ints, floats, order, groups)
    return {"start": ints[:, 0], "count": ints[:, 1], "next": ints[:, 2], "leaf": ints[:, 3],
            "cx": floats[:, 0], "cy": floats[:, 1], "cz": floats[:, 2], "m": floats[:, 3],
            "open_r": floats[:, 4], "gx": floats[:, 5], "gy": floats[:, 6], "gz": floats[:, 7],
            "half": floats[:, 8], "order": order, "groups": groups}


_last_n = [0]


def build_tree(pos, mass, theta):
    """Builds the oracle tree for (pos, mass) and returns tree_export()."""
    acc = np.zeros_like(pos)
    _last_n[0] = len(mass)
    # an all-zero active mask builds the tree and skips every walk
    accel_active(pos, mass, acc, theta, 0.1, np.zeros(len(mass), np.uint8), True)
    return tree_export()


def sph_kernel(r, h):
    return lib().orc_sph_kernel(float(r), float(h))


def sph_kernel_grad(r, h):
    return lib().orc_sph_kernel_grad(float(r), float(h))


def sph_forces(pos, vel, mass, nb, h, u, gamma, alpha, beta):
    """Restatement of sph.sph_forces (sph.py:58); returns rho, acc, dudt, dt_i."""
    n, k = nb.shape
    rho, dudt, dt_i = np.empty(n), np.empty(n), np.empty(n)
    acc = np.empty((n, 3))
    lib().orc_sph_forces(n, k, np.ascontiguousarray(pos), np.ascontiguousarray(vel),
                         np.ascontiguousarray(mass), np.ascontiguousarray(nb, dtype=np.int64),
                         np.ascontiguousarray(h), np.ascontiguousarray(u), gamma, alpha, beta,
                         rho, acc, dudt, dt_i)
    return rho, acc, dudt, dt_i


def knn_from_candidates(pos, cand, k, nb, dist):
    """Restatement of sph.knn_from_candidates (sph.py:110); returns ok."""
    n, m = cand.shape
    return bool(lib().orc_knn_from_candidates(n, m, np.ascontiguousarray(pos),
                                              np.ascontiguousarray(cand, dtype=np.int64),
                                              k, nb, dist))


def knn_brute(pos, k):
    """Exact k nearest (self included), ascending; returns dist (n,k), nb (n,k)."""
    n = len(pos)
    dist = np.zeros((n, k))
    nb = np.zeros((n, k), np.int64)
    lib().orc_knn_brute(n, np.ascontiguousarray(pos), k, dist, nb)
    return dist, nb


def render(pos, group, ngroups, rot, center, scale, W, H):
    """Restatement of nbody_render (cpp/nbody.cpp:445-469); returns img (ngroups, H, W)."""
    img = np.zeros((ngroups, H, W), np.float32)
    lib().orc_render(len(pos), np.ascontiguousarray(pos), np.ascontiguousarray(group, np.uint8), ngroups,
                     np.ascontiguousarray(rot, np.float64), np.ascontiguousarray(center, np.float64), scale, W, H, img)
    return img


def tonemap(img, glow, colors, inv_ref, K, exposure):
    """Restatement of nbody_tonemap (cpp/nbody.cpp:474-503); returns (H, W, 3) uint8."""
    ng, H, W = img.shape
    gh, gw = glow.shape[1:]
    out = np.zeros((H, W, 3), np.uint8)
    lib().orc_tonemap(W, H, ng, np.ascontiguousarray(img, np.float32), np.ascontiguousarray(glow, np.float32), gw, gh,
                      np.ascontiguousarray(colors, np.float32), inv_ref, K, exposure, out)
    return out


class RefNbody:
    """The reference's cpp/nbody.cpp built from its own sources (oracle/_ref/)."""

    def __init__(self):
        if not os.path.exists(REF_LIB):
            raise FileNotFoundError(REF_LIB)
        L = ctypes.CDLL(REF_LIB)
        L.nbody_render.argtypes = [_ci, _dbl, _u8, _ci, _dbl, _dbl, _cd, _ci, _ci, _f32]
        L.nbody_tonemap.argtypes = [_ci, _ci, _ci, _f32, _f32, _ci, _ci, _f32, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, _u8]
        L.nbody_accel_active.argtypes = [_ci, _dbl, _dbl, _dbl, _cd, _cd, _u8, _ci]
        L.nbody_accel_direct.argtypes = [_ci, _dbl, _dbl, _dbl, _cd]
        L.nbody_num_threads.restype = _ci
        self.lib = L

    def gravity(self, pos, mass, acc, theta, eps, active=None, rebuild=True):
        n = len(mass)
        act = np.ones(n, np.uint8) if active is None else np.ascontiguousarray(active, np.uint8)
        self.lib.nbody_accel_active(n, pos, mass, acc, theta, eps, act, int(rebuild))

    def gravity_direct(self, pos, mass, eps):
        acc = np.zeros_like(pos)
        self.lib.nbody_accel_direct(len(mass), pos, mass, acc, eps)
        return acc
