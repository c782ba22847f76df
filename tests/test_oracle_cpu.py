"""CPU tests of the oracle's semantics on tiny scenes whose answers follow
from the reference's code by hand (src/renderer/cpu/rasterizer.cc)."""
import numpy as np
import pytest

from ugu_gb300 import scenes

import adversarial as adv


def render(oracle_lib, m, cam, opt, **kw):
    rc, out, st = oracle_lib.render(m, cam, opt, **kw)
    assert rc == 0
    return out, st


def test_uv_sphere_counts(oracle_lib):
    m, cam = scenes.scene_uv_sphere_vertex_color()
    assert (m.num_vertices, m.num_faces) == (1986, 3968)
    out, st = render(oracle_lib, m, cam, adv.option())
    # every covered pixel of a closed sphere seen from outside is a front face
    assert st.special_candidates == 0 and st.texel_clamps == 0
    fid = out["face_id"]
    assert ((fid >= 0) == (out["depth"] > 0)).all()
    assert ((fid > 0) == (out["mask"] == 255)).all()
    # back faces were rasterised into the z-buffer too (rasterizer.cc:198-199)
    assert st.covered > 1.9 * (fid >= 0).sum()


def test_calc_normals_numpy_matches_c(oracle_lib):
    m = scenes.icosphere(3, 1.0, 0.01, seed=3)
    scenes.calc_normals(m)
    fn, n = oracle_lib.calc_normals(m.vertices, m.vertex_indices)
    assert np.array_equal(fn, m.face_normals)
    assert np.array_equal(n, m.normals)


def test_icosphere_sizes():
    for s, (V, F) in [(0, (12, 20)), (2, (162, 320)), (4, (2562, 5120))]:
        m = scenes.icosphere(s, 1.0, 0.0)
        assert (m.num_vertices, m.num_faces) == (V, F)
        assert m.uv.min() >= 0.0099 and m.uv.max() <= 0.9901
        assert m.uv_indices.max() < m.uv.shape[0]


def test_ring_sizes_total():
    sizes = scenes.seeded_sizes(64, 4)
    assert sum(w * h for w, h in sizes) == 54_067_200
    assert sizes == scenes.seeded_sizes(64, 4)


def test_depth_ties_lowest_face_wins(oracle_lib):
    cam = adv.identity_camera()
    m = adv.depth_ties(cam)
    out, _ = render(oracle_lib, m, cam, adv.option(backface_culling=False))
    fid = out["face_id"]
    # faces 1 and 4 repeat face 0 vertex for vertex, face 5 repeats face 3:
    # their depths tie exactly, so the lower id always wins.  Face 2 lists
    # face 0's vertices rotated, which rounds differently and may win.
    ids = set(int(i) for i in np.unique(fid))
    assert not ids & {1, 4, 5}
    assert {0, 3} <= ids


def test_face_zero_keeps_depth_without_mask(oracle_lib):
    cam = adv.identity_camera()
    m = adv.shared_edge_quad(cam)
    out, _ = render(oracle_lib, m, cam, adv.option(backface_culling=False))
    z = out["face_id"] == 0
    assert z.any()
    assert (out["depth"][z] > 0).all()
    assert (out["mask"][z] == 0).all() and (out["color"][z] == 0).all()
    assert (out["normal"][z] == 0).all()


def test_back_face_in_front_clears_with_culling(oracle_lib):
    cam = adv.identity_camera()
    m = adv.back_in_front(cam)
    # the third face is the back face: its normal points away from the camera
    assert m.face_normals[2, 2] > 0 and m.face_normals[1, 2] < 0
    on, _ = render(oracle_lib, m, cam, adv.option(backface_culling=True))
    off, _ = render(oracle_lib, m, cam, adv.option(backface_culling=False))
    cleared = (off["face_id"] == 2) & (on["face_id"] == -1)
    assert cleared.any()
    assert (on["depth"][cleared] == 0).all()
    # with culling on, the front face is NOT revealed behind the back face
    assert not (on["face_id"][off["face_id"] == 2] == 1).any()


def test_near_plane_tiny_and_clamped(oracle_lib):
    cam = adv.identity_camera()
    m = adv.near_plane_and_tiny(cam)
    out, st = render(oracle_lib, m, cam, adv.option(backface_culling=False))
    ids = set(np.unique(out["face_id"]))
    assert 1 not in ids and 2 not in ids and 5 not in ids  # culled / zero area / off screen
    assert {3, 4} <= ids  # partly off screen, bbox clamped


def test_texture_border_linear_addressing(oracle_lib):
    cam = adv.identity_camera()
    m = adv.texture_border(cam)
    out, st = render(oracle_lib, m, cam, adv.option(diffuse_color=1, interp=1))
    assert (out["mask"] == 255).any()
    # uv.x = 1 reads texel (y, cols) == (y + 1, 0) inside the allocation; only
    # reads past the end are clamped
    assert st.texel_clamps >= 0


def test_validation_codes(oracle_lib):
    cam = adv.identity_camera()
    m = adv.shared_edge_quad(cam)
    m2 = m.copy()
    m2.vertex_colors = None
    rc, _, _ = oracle_lib.render(m2, cam, adv.option(diffuse_color=2))
    assert rc == 6
    m3 = m.copy()
    m3.normals = None
    m3.normal_indices = None
    rc, _, _ = oracle_lib.render(m3, cam, adv.option(shading_normal=1))
    assert rc == 8
    rc, _, _ = oracle_lib.render(m, cam, adv.option(), outputs=())
    assert rc == 9


def test_fp64_yardstick_close(oracle_lib):
    m, cam = scenes.scene_uv_sphere_vertex_color()
    opt = adv.option()
    out, _ = render(oracle_lib, m, cam, opt)
    d64, n64, c64 = oracle_lib.interp_f64(m, cam, opt, out["face_id"])
    sel = out["face_id"] >= 0
    rel = np.abs(out["depth"][sel] - d64[sel]) / d64[sel]
    assert rel.max() < 1e-5
    # the FP32 reference itself is ~1e-5 off FP64 at silhouette pixels; this
    # figure is reported, not a parity bound
    s2 = out["face_id"] > 0
    assert np.abs(out["normal"][s2] - n64[s2]).max() < 1e-4
