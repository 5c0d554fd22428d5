"""The C ABI: libgfgpu.so builds, loads without a GPU and exports every function that
include/gfgpu.h declares; the ctypes table covers the same set (no compute calls here)."""

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "gfgpu.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"^[A-Za-z_][\w \*]*?\b((?:nbody|gf)_\w+)\s*\(", text, flags=re.M))


@pytest.fixture(scope="module")
def lib():
    from galaxy_formation_gb300 import build

    return ctypes.CDLL(build.build())


def test_header_declares_reference_exports():
    names = declared()
    # the five exports the reference's engine.py binds (galaxy_formation/engine.py:30-35)
    for f in ("nbody_num_threads", "nbody_accel_active", "nbody_accel_direct", "nbody_render",
              "nbody_tonemap"):
        assert f in names


def test_library_exports_every_declared_symbol(lib):
    missing = [f for f in sorted(declared()) if not hasattr(lib, f)]
    assert not missing, missing


def test_ctypes_table_matches_header():
    from galaxy_formation_gb300 import _lib

    assert set(_lib.SIGNATURES) == declared()


def test_reference_signatures_unchanged():
    """Argument lists of the five drop-in functions equal cpp/nbody.cpp:417-474."""
    text = re.sub(r"\s+", " ", open(HEADER).read())
    for sig in (
        "int nbody_num_threads(void);",
        "void nbody_accel_active(int n, const double* pos, const double* mass, double* acc, "
        "double theta, double eps, const uint8_t* active, int rebuild);",
        "void nbody_accel_direct(int n, const double* pos, const double* mass, double* acc, "
        "double eps);",
        "void nbody_render(int n, const double* pos, const uint8_t* group, int ngroups, "
        "const double* rot, const double* center, double scale, int W, int H, float* img);",
        "void nbody_tonemap(int W, int H, int ngroups, const float* img, const float* glow, int gw, "
        "int gh, const float* colors, float inv_ref, float K, float exposure, uint8_t* out);",
    ):
        assert sig in text, sig
