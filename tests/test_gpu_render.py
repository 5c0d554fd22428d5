"""Splat and tone map (nbody_render / nbody_tonemap, cpp/nbody.cpp:445-503) on the GPU against
the reference's own outputs (tests/golden/render.npz) and the oracle's restatement: the
splatted images to float rounding (the deposit order of atomic adds differs), the 8-bit
colours within one step at a rounding boundary (CUDA's log1pf / expf against the host's);
a group index without an image plane is refused."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_splat_and_tonemap_match_reference(gpulib, oracle, golden):
    r = golden("render.npz")
    ng, H, W = r["img"].shape
    img = np.zeros((ng, H, W), np.float32)
    gpulib.nbody_render(len(r["group"]), r["pos"], r["group"], ng, r["rot"], r["center"], float(r["scale"]), W, H,
                        img)
    assert gpulib.gf_last_status() == 0
    assert np.abs(img - r["img"]).max() <= 1e-5 * r["img"].max()
    assert abs(float(img.sum()) - float(r["img"].sum())) <= 1e-6 * float(r["img"].sum())
    ref = oracle.render(r["pos"], r["group"], ng, r["rot"], r["center"], float(r["scale"]), W, H)
    assert np.abs(img - ref).max() <= 1e-5 * ref.max()
    gh, gw = r["glow"].shape[1:]
    rgb = np.zeros((H, W, 3), np.uint8)
    gpulib.nbody_tonemap(W, H, ng, r["img"], r["glow"], gw, gh, r["colors"], float(r["inv_ref"]), float(r["K"]),
                         float(r["exposure"]), rgb)
    assert gpulib.gf_last_status() == 0
    d = np.abs(rgb.astype(int) - r["rgb"].astype(int))
    assert d.max() <= 1 and (d > 0).mean() < 1e-2, (d.max(), (d > 0).mean())


def test_splat_refuses_group_without_plane(gpulib, golden):
    from galaxy_formation_gb300 import _lib

    r = golden("render.npz")
    ng, H, W = r["img"].shape
    group = r["group"].copy()
    group[7] = ng  # one past the planes the image holds
    img = np.full((ng, H, W), -1.0, np.float32)
    gpulib.nbody_render(len(group), r["pos"], group, ng, r["rot"], r["center"], float(r["scale"]), W, H, img)
    assert gpulib.gf_last_status() & _lib.GF_ERR_ARG
