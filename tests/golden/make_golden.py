"""Regenerates tests/golden/*.npz and tests/golden/ray/*.npz from the
reference itself.

Each fixture holds one scene's inputs (mesh arrays, the camera floats the
reference derived, the options) and the images ugu's own Rasterizer::Render
(golden/) or Raytracer::Render (golden/ray/) produced for it --
src/renderer/cpu/rasterizer.cc, raytracer.cc and friends compiled
unmodified against the Eigen-compatible shim (oracle/_ref).  Run where the
reference checkout exists:  python tests/golden/make_golden.py
"""
import dataclasses
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import adversarial as adv  # noqa: E402
from oracle import ref_build  # noqa: E402
from ugu_gb300 import scenes  # noqa: E402

CASES = [
    ("shared_edge_quad", "vertex_vnormal_cull"), ("shared_edge_quad", "tex_nn_nocull"),
    ("depth_ties", "vertex_fnormal_nocull"), ("back_in_front", "vertex_vnormal_cull"),
    ("back_in_front", "white_lambert_fnormal"), ("near_plane_and_tiny", "tex_bilinear_lambert"),
    ("triangle_soup", "vertex_fnormal_nocull"), ("triangle_soup", "tex_bilinear_lambert"),
    ("triangle_soup", "white_orennayar"), ("shared_vertex_fan", "tex_bilinear_lambert"),
]


RAY_CASES = [
    ("shared_edge_quad", "vertex_vnormal_cull"), ("depth_ties", "vertex_fnormal_nocull"),
    ("back_in_front", "white_lambert_fnormal"), ("near_plane_and_tiny", "tex_bilinear_lambert"),
    ("triangle_soup", "tex_bilinear_lambert"), ("triangle_soup", "white_orennayar"),
    ("shared_vertex_fan", "tex_nn_nocull"),
]


def save(name, m, cam, opt, renderer="raster", folder=HERE):
    fn = ref_build.raytrace if renderer == "ray" else ref_build.render
    rc, out, camf = fn(m, cam, opt)
    assert rc == 0
    cam = dataclasses.replace(cam, **camf)
    arrays = {
        "vertices": m.vertices, "vertex_indices": m.vertex_indices,
        "face_normals": m.face_normals, "normals": m.normals,
        "normal_indices": m.normal_indices, "vertex_colors": m.vertex_colors,
        "uv": m.uv, "uv_indices": m.uv_indices, "material_ids": m.material_ids,
        "texture": m.textures[0] if m.textures else np.zeros((1, 1, 3), np.uint8),
        "cam_int": np.array([cam.width, cam.height], np.int32),
        "cam_f": np.array([cam.fx, cam.fy, cam.cx, cam.cy], np.float32),
        "w2c_R": cam.w2c_R, "w2c_t": cam.w2c_t, "c2w_R": cam.c2w_R,
        "option": np.array([opt.diffuse_color, opt.interp, opt.shading_normal,
                            opt.diffuse_shading, int(opt.backface_culling)], np.int32),
        "sigma": np.array([opt.oren_nayar_sigma], np.float32),
    }
    if renderer == "ray":
        arrays["c2w"] = np.asarray(cam.c2w if cam.c2w is not None else np.eye(4), np.float64)
        arrays["depth_scale"] = np.array([getattr(opt, "depth_scale", 1.0)], np.float32)
    arrays = {k: v for k, v in arrays.items() if v is not None}
    arrays.update({"out_" + k: v for k, v in out.items()})
    np.savez_compressed(os.path.join(folder, name + ".npz"), **arrays)


def main():
    ref_build.build_if_available()
    cam = adv.identity_camera()
    for scene, optname in CASES:
        save(f"{scene}__{optname}", adv.ALL_SMALL[scene](cam), cam, adv.OPTIONS[optname])
    m = scenes.icosphere_textured(4, 64)
    c = scenes.ring_cameras(3, 3.0, [(160, 120)] * 3)[1]
    save("icosphere4_ring_160x120__tex_bilinear", m, c, adv.option(1, 1, 1, 0, True))
    m2, c2 = scenes.scene_uv_sphere_vertex_color()
    c2 = scenes.camera_desc(160, 120, 125.0, 125.0, 80.0, 60.0)
    save("uv_sphere_160x120__vertex_color", m2, c2, adv.option(2, 1, 1, 0, True))

    ray = os.path.join(HERE, "ray")
    os.makedirs(ray, exist_ok=True)
    for scene, optname in RAY_CASES:
        save(f"{scene}__{optname}", adv.ALL_SMALL[scene](cam), cam, adv.OPTIONS[optname],
             "ray", ray)
    save("icosphere4_ring_160x120__tex_bilinear", m, c, adv.option(1, 1, 1, 0, True), "ray", ray)
    o2 = adv.option(2, 1, 1, 1, False)
    o2.depth_scale = 2.5
    save("uv_sphere_160x120__vertex_color_lambert_scaled", m2, c2, o2, "ray", ray)


if __name__ == "__main__":
    main()
