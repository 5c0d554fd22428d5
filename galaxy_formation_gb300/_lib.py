"""ctypes binding of libgfgpu.so (C ABI declared in include/gfgpu.h).

The library is built in-tree by galaxy_formation_gb300/build.py. Loading fails loudly when
it is missing or when no GPU is usable: there is no CPU fallback.
"""

import ctypes
import os

import numpy as np

from . import build as _build

_dbl = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_ci, _cd, _cf, _vp = ctypes.c_int, ctypes.c_double, ctypes.c_float, ctypes.c_void_p

# Every exported symbol with (argtypes, restype); include/gfgpu.h is the source of truth
# and tests/test_capi.py checks that the two agree.
SIGNATURES = {
    "nbody_num_threads": ([], _ci),
    "nbody_accel_active": ([_ci, _dbl, _dbl, _dbl, _cd, _cd, _u8, _ci], None),
    "nbody_accel_direct": ([_ci, _dbl, _dbl, _dbl, _cd], None),
    "nbody_render": ([_ci, _dbl, _u8, _ci, _dbl, _dbl, _cd, _ci, _ci, _f32], None),
    "nbody_tonemap": ([_ci, _ci, _ci, _f32, _f32, _ci, _ci, _f32, _cf, _cf, _cf, _u8], None),
    "gf_last_status": ([], _ci),
    "gf_last_error": ([], ctypes.c_char_p),
    "gf_tree_size": ([ctypes.POINTER(_ci), ctypes.POINTER(_ci)], _ci),
    "gf_tree_export": ([_i32, _f32, _i32, _i32], _ci),
    "gf_tree_rebuild_captured": ([_ci, _dbl, _dbl, _cd], _ci),
    "gf_accel_active_dev": ([_ci, _vp, _vp, _vp, _cd, _cd, _vp, _ci, _vp], _ci),
    "gf_accel_direct_dev": ([_ci, _vp, _vp, _vp, _cd, _vp], _ci),
    "gf_accel_direct_targets": ([_ci, _dbl, _dbl, _ci, _i64, _dbl, _cd], _ci),
    "gf_sph_kernel": ([_ci, _dbl, _dbl, _vp, _vp], _ci),
    "gf_sph_forces": ([_ci, _ci, _dbl, _dbl, _dbl, _i64, _dbl, _dbl, _cd, _cd, _cd,
                       _dbl, _dbl, _dbl, _dbl], _ci),
    "gf_sph_forces_mixed": ([_ci, _ci, _dbl, _dbl, _dbl, _i64, _dbl, _dbl, _cd, _cd, _cd,
                             _dbl, _dbl, _dbl, _dbl], _ci),
    "gf_sph_forces_dev": ([_ci, _ci, _vp, _vp, _vp, _vp, _vp, _vp, _cd, _cd, _cd,
                           _vp, _vp, _vp, _vp, _vp], _ci),
    "gf_sph_forces_noalloc_dev": ([_ci, _ci, _vp, _vp, _vp, _vp, _vp, _vp, _cd, _cd, _cd,
                                   _vp, _vp, _vp, _vp, _vp], _ci),
    "gf_knn_from_candidates": ([_ci, _ci, _dbl, _i64, _ci, _i64, _dbl], _ci),
    "gf_knn": ([_ci, _dbl, _ci, _dbl, _i64], _ci),
    "gf_knn_iterations": ([], ctypes.c_longlong),
    "gf_accelerations_dev": ([_ci, _vp, _vp, _vp, _vp, _vp, _cd, _cd, _cd, _cd, _cd, _vp, _ci, _ci,
                              _ci, _vp, _vp, _vp], _ci),
    "gf_accelerations": ([_ci, _dbl, _dbl, _dbl, np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS"),
                          _dbl, _cd, _cd, _cd, _cd, _cd, _vp, _ci, _ci, _ci, _dbl, _dbl], _ci),
    "gf_ic_generate_dev": ([_ci, _ci, _ci, ctypes.c_ulonglong, _dbl, _ci, _vp, _vp, _vp, _vp, _vp, _vp], _ci),
    "gf_ic_generate": ([_ci, _ci, _ci, ctypes.c_ulonglong, _dbl, _ci, _dbl, _dbl, _dbl,
                        np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS"), _dbl], _ci),
    "gf_force_autotune": ([_cd, ctypes.POINTER(_ci), ctypes.POINTER(_ci), ctypes.POINTER(_cd)], _ci),
    "gf_force_read_gas": ([_ci, ctypes.POINTER(_ci), _vp, _vp, _vp, _vp, _vp, _vp, _vp], _ci),
    "gf_force_info": ([ctypes.POINTER(_ci), ctypes.POINTER(_cd), ctypes.POINTER(_cd),
                       ctypes.POINTER(ctypes.c_longlong)], _ci),
    "gf_sim_init": ([_ci, _dbl, _dbl, _dbl, np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS"), _dbl,
                     _cd, _cd, _cd, _cd, _cd], _ci),
    "gf_sim_step": ([_cd, ctypes.POINTER(_cd), ctypes.POINTER(_ci)], _ci),
    "gf_sim_read": ([_vp, _vp, _vp, _vp, ctypes.POINTER(_cd)], _ci),
    "gf_sim_diagnostics": ([_cd, _dbl], _ci),
    "gf_sim_read_u": ([_dbl], _ci),
    "gf_sim_read_scalars": ([_dbl], _ci),
    "gf_sim_read_hydro": ([_dbl, _dbl], _ci),
    "gf_sim_restore": ([_dbl, _dbl, _vp, _vp, _vp, _vp, _cd, _cd, _cd], _ci),
    "gf_sim_stars": ([_ci, _vp, _vp], _ci),
    "gf_sim_read_stars": ([_vp, _vp, _vp, _vp], ctypes.c_longlong),
    "gf_sim_thermo": ([_ci, _vp], _ci),
    "gf_cooling_function": ([_ci, _dbl, _dbl], _ci),
    "gf_cool": ([_ci, _dbl, _dbl, _dbl, _dbl, _vp, _cd, _dbl, _dbl], _ci),
    "gf_sim_blocks": ([_ci, _ci, ctypes.POINTER(_cd)], _ci),
    "gf_sim_updates": ([], _cd),
    "gf_sim_block_config": ([_vp, _ci, _ci], _ci),
    "gf_sim_block_autotune": ([_ci, _vp, _vp, _vp], _ci),
    "gf_stream": ([], _vp),
    "gf_sim_levels": ([_ci, _dbl], _ci),
    "gf_set_option": ([_ci, _cd], _ci),
    "gf_get_option": ([_ci], _cd),
    "gf_force_stats": ([_dbl, _ci], _ci),
    "gf_mlp_tensor_cores": ([], _ci),
    "gf_mlp_init": ([_ci], _ci),
    "gf_mlp_set_params": ([_f32], _ci),
    "gf_mlp_get_params": ([_f32], _ci),
    "gf_mlp_set_norm": ([_f32, _f32, _cd, _cd], _ci),
    "gf_mlp_predict": ([_ci, _f32, _f32], _ci),
    "gf_mlp_gradient": ([_ci, _f32, _f32, _f32], _ci),
    "gf_mlp_collected": ([_vp, _vp, ctypes.c_longlong], ctypes.c_longlong),
    "gf_mlp_train": ([_ci, _ci, _cd, ctypes.POINTER(_cd)], _ci),
    "gf_profile": ([_ci], _ci),
    "gf_profile_stage": ([_ci, ctypes.POINTER(_cd), ctypes.POINTER(_ci)], _ci),
    "gf_launch_count": ([], ctypes.c_longlong),
    "gf_walk_pairs": ([], ctypes.c_longlong),
    "gf_walk_quad_pairs": ([], ctypes.c_longlong),
    "gf_fp32_peak": ([ctypes.POINTER(_cd)], _ci),
}

# status bits (include/gfgpu.h)
GF_ERR_CUDA, GF_ERR_ARG, GF_ERR_NONFINITE, GF_ERR_WALK_STACK = 1, 2, 4, 8
GF_ERR_DEEP_CELL, GF_ERR_KNN, GF_ERR_NO_DEVICE, GF_ERR_CAPACITY = 16, 32, 64, 128
GF_ERR_TIMEOUT = 256

OPT_SPH_FLOAT32 = 0
OPT_GRAVITY_QUAD = 1
OPT_HGUESS = 2
OPT_COLLECT = 3
OPT_WALK_CHUNK = 4
OPT_WALK_GROUP = 5
OPT_GRAVITY_REL = 6
OPT_WALK_MERGE = 7
OPT_GRAVITY_REL_MONO = 8
OPT_WALK_SHAPE = 9
OPT_FORGET_H = 10
MLP_PARAMS = 4545

STAGES = ["tree_build", "tree_refit", "walk", "group_prep", "knn", "knn_tree", "sph_density",
          "sph_force", "verlet", "force", "tree_sort", "tree_emit", "tree_moments"]

LIB_PATH = _build.LIB
_lib = None


class GpuError(RuntimeError):
    """A libgfgpu call reported a non-zero status (GF_ERR_* bits in .status)."""

    def __init__(self, status, msg):
        super().__init__(f"libgfgpu status {status}: {msg}")
        self.status = status


def load(path=None):
    """Loads (once) and returns the library with argtypes set."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run galaxy_formation_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    if path == LIB_PATH:
        _lib = lib
    return lib


def read_gas(lib):
    """The gas state of the last hydro step (gf_force_read_gas) as numpy arrays: dict of gidx,
    h, rho, dudt, dt_i, acc_sph (ng,3), nb (ng,32); empty dict when it had no hydro."""
    ng = ctypes.c_int()
    check(lib.gf_force_read_gas(0, ctypes.byref(ng), None, None, None, None, None, None, None))
    m = ng.value
    if m <= 0:
        return {}
    out = {"gidx": np.empty(m, np.int32), "h": np.empty(m), "rho": np.empty(m), "dudt": np.empty(m),
           "dt_i": np.empty(m), "acc_sph": np.empty((m, 3)), "nb": np.empty((m, 32), np.int32)}
    check(lib.gf_force_read_gas(m, ctypes.byref(ng), *(out[k].ctypes.data for k in
                                                       ("gidx", "h", "rho", "dudt", "dt_i", "acc_sph", "nb"))))
    return out


def check(status=None):
    """Raises GpuError when the last call failed."""
    lib = load()
    st = lib.gf_last_status() if status is None else status
    if st:
        raise GpuError(st, (lib.gf_last_error() or b"").decode())
    return st
