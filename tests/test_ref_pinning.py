"""Pins the oracle to the reference: ugu's own Rasterizer (src/renderer/cpu/
rasterizer.cc, util_private.cc, pixel_shader.h, camera.h -- compiled
unmodified against the Eigen-compatible shim into oracle/_ref) and the
oracle's C restatement must agree bit for bit.  Runs on the CPU wherever the
reference checkout exists; skipped elsewhere."""
import dataclasses

import numpy as np
import pytest

import adversarial as adv
from ugu_gb300 import scenes

ref_build = pytest.importorskip("oracle.ref_build")
if not ref_build.available():
    pytest.skip("reference sources not present", allow_module_level=True)


@pytest.fixture(scope="module")
def ref():
    ref_build.build_if_available()
    return ref_build


def same(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                          np.ascontiguousarray(b).view(np.uint8))


def check(ref, oracle_lib, m, cam, opt, name):
    rc, r_out, camf = ref.render(m, cam, opt)
    assert rc == 0, name
    for k in camf:  # the host-side camera floats agree with the reference's
        assert np.array_equal(camf[k], getattr(cam, k)), (name, k)
    rc, o_out, st = oracle_lib.render(m, cam, opt)
    assert rc == 0
    for k in r_out:
        assert same(r_out[k], o_out[k]), f"{name}: {k} differs from the reference"
    return st


@pytest.mark.parametrize("optname", list(adv.OPTIONS))
@pytest.mark.parametrize("scene", [s for s in adv.ALL_SMALL if s != "texture_border"])
def test_small_scenes_match_reference(ref, oracle_lib, scene, optname):
    cam = adv.identity_camera()
    m = adv.ALL_SMALL[scene](cam)
    check(ref, oracle_lib, m, cam, adv.OPTIONS[optname], f"{scene}/{optname}")


def test_texture_border_inside_allocation(ref, oracle_lib):
    """uv.x = 1 makes the reference read texel (y, cols), i.e. (y + 1, 0);
    the oracle's linear addressing reproduces that while the read stays
    inside the texture.  (uv.y = 0 would read past its end: not run.)"""
    cam = adv.identity_camera()
    m = adv.texture_border(cam)
    m.uv = np.array([[0, 0.5], [1, 0.5], [1, 0.2], [0, 0.2], [0, 0.3], [0, 0.3], [0, 0.3]],
                    dtype=np.float32)
    st = check(ref, oracle_lib, m, cam, adv.option(1, 1, 1, 0, True), "border")
    assert st.texel_clamps == 0


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_triangle_soups_match_reference(ref, oracle_lib, seed):
    cam = adv.identity_camera(W=120, H=90, f=80.0)
    m = adv.triangle_soup(cam, n_faces=1500, seed=seed)
    for opt in (adv.option(2, 1, 1, 1, False), adv.option(1, 0, 0, 2, True)):
        check(ref, oracle_lib, m, cam, opt, f"soup{seed}")


def test_uv_sphere_640x480_matches_reference(ref, oracle_lib):
    m, cam = scenes.scene_uv_sphere_vertex_color()
    check(ref, oracle_lib, m, cam, adv.option(2, 1, 1, 0, True), "uv_sphere")
    check(ref, oracle_lib, m, cam, adv.option(2, 1, 0, 1, False), "uv_sphere_lambert")


def test_ring_views_match_reference(ref, oracle_lib):
    m = scenes.icosphere_textured(5, 256)
    sizes = scenes.seeded_sizes(8, 4, [(160, 120), (320, 240), (200, 150), (120, 160)])
    cams = scenes.ring_cameras(8, 3.0, sizes)
    for i, cam in enumerate(cams):
        check(ref, oracle_lib, m, cam, adv.option(1, 1, 1, 0, True), f"ring{i}")
    for i, cam in enumerate(scenes.fibonacci_cameras(6, 3.0, 160, 90, 125.0)):
        check(ref, oracle_lib, m, cam, adv.option(2, 0, 1, 1, True), f"fib{i}")


def test_icosphere7_1080p_matches_reference(ref, oracle_lib):
    m, cam = scenes.scene_icosphere_single_view()
    st = check(ref, oracle_lib, m, cam, adv.option(1, 1, 1, 0, True), "icosphere7_1080p")
    assert st.texel_clamps == 0 and st.special_candidates == 0
