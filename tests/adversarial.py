"""Small hand-built and random scenes that stress the reference's corner
cases: shared edges, exact depth ties, face 0, back faces in front of front
faces, faces straddling z = 0, sub-FLT_MIN areas, off-screen and clamped
bboxes, pixel-centre vertices, texel reads at the texture border."""
from __future__ import annotations

from types import SimpleNamespace as NS

import numpy as np

from ugu_gb300 import scenes

F32 = np.float32


def option(diffuse_color=2, interp=1, shading_normal=1, diffuse_shading=0,
           backface_culling=True, sigma=0.3):
    return NS(diffuse_color=diffuse_color, interp=interp, shading_normal=shading_normal,
              diffuse_shading=diffuse_shading, backface_culling=backface_culling,
              oren_nayar_sigma=sigma, depth_scale=1.0)


def identity_camera(W=64, H=48, f=40.0, cx=None, cy=None):
    return scenes.camera_desc(W, H, f, f, W / 2.0 if cx is None else cx,
                              H / 2.0 if cy is None else cy)


def _finish(v, f, seed=7, tex=16):
    m = scenes.Mesh(vertices=np.ascontiguousarray(v, dtype=F32),
                    vertex_indices=np.ascontiguousarray(f, dtype=np.int32))
    scenes.calc_normals(m)
    scenes.with_vertex_colors(m, seed=seed)
    rng_uv = scenes.uniform01(seed + 1, 2 * m.num_vertices).reshape(-1, 2)
    m.uv = np.ascontiguousarray((0.02 + 0.96 * rng_uv).astype(F32))
    m.uv_indices = m.vertex_indices.copy()
    m.material_ids = np.zeros(m.num_faces, np.int32)
    m.textures = [scenes.random_u8(seed + 2, (tex, tex, 3))]
    m.textures_f32 = [None]
    return m


def unproject(cam, x, y, z):
    """Camera-frame point for pixel (x, y) at depth z (identity pose)."""
    return [(x - cam.cx) * z / cam.fx, (y - cam.cy) * z / cam.fy, z]


def shared_edge_quad(cam):
    """Two triangles of a slanted quad sharing a diagonal, vertices on pixel
    centres, plus face 0 (a small triangle that must keep depth/face_id but
    never get mask/colour)."""
    pts = [unproject(cam, 8, 6, 2.0), unproject(cam, 40, 6, 2.5), unproject(cam, 40, 30, 3.0),
           unproject(cam, 8, 30, 2.2), unproject(cam, 50, 36, 2.0), unproject(cam, 60, 36, 2.0),
           unproject(cam, 50, 44, 2.0)]
    f = [[4, 5, 6], [0, 1, 2], [0, 2, 3]]
    return _finish(pts, f)


def depth_ties(cam):
    """Identical coplanar triangles listed several times (exact depth ties:
    the lowest face id must win) and a nearer copy listed last."""
    a = unproject(cam, 5, 5, 3.0)
    b = unproject(cam, 45, 8, 3.0)
    c = unproject(cam, 20, 40, 3.0)
    d = unproject(cam, 30, 10, 2.0)
    e = unproject(cam, 60, 20, 2.0)
    g = unproject(cam, 40, 45, 2.0)
    v = [a, b, c, d, e, g]
    f = [[0, 1, 2], [0, 1, 2], [1, 2, 0], [3, 4, 5], [0, 1, 2], [3, 4, 5]]
    return _finish(v, f)


def back_in_front(cam):
    """A back-facing triangle in front of a front-facing one: with culling
    the covered pixels clear to depth 0 / face -1."""
    # image axes are x right, y down: (a, c, b) in screen order faces the camera
    front = [unproject(cam, 5, 5, 4.0), unproject(cam, 30, 44, 4.0), unproject(cam, 55, 6, 4.0)]
    back = [unproject(cam, 10, 10, 2.0), unproject(cam, 50, 12, 2.0), unproject(cam, 35, 40, 2.0)]
    filler = [unproject(cam, 0, 0, 5.0), unproject(cam, 2, 0, 5.0), unproject(cam, 0, 2, 5.0)]
    v = filler + front + back
    f = [[0, 1, 2], [3, 4, 5], [6, 7, 8]]
    m = _finish(v, f)
    return m


def near_plane_and_tiny(cam):
    """Faces straddling z = 0 (culled), a face with |area| < FLT_MIN
    (skipped), faces partly off screen (bbox clamped) and fully off screen."""
    v = [
        unproject(cam, 10, 10, 2.0), unproject(cam, 30, 10, 2.0), [0.0, 0.5, -1.0],  # straddle
        unproject(cam, 20, 20, 2.0), unproject(cam, 20, 20, 2.0), unproject(cam, 20, 20, 2.0),  # zero area
        unproject(cam, -20, -10, 3.0), unproject(cam, 30, -5, 3.0), unproject(cam, 10, 30, 3.0),  # clamp
        unproject(cam, 50, 30, 3.0), unproject(cam, 90, 35, 3.0), unproject(cam, 60, 70, 3.0),  # clamp
        unproject(cam, 100, 100, 3.0), unproject(cam, 120, 100, 3.0), unproject(cam, 100, 120, 3.0),
        unproject(cam, 1, 1, 1.0), unproject(cam, 9, 1, 1.0), unproject(cam, 1, 9, 1.0),
    ]
    f = [[15, 16, 17], [0, 1, 2], [3, 4, 5], [6, 7, 8], [9, 10, 11], [12, 13, 14]]
    return _finish(v, f)


def triangle_soup(cam, n_faces=400, seed=11, zmin=1.0, zmax=6.0, spread=1.3):
    """Random overlapping triangles in front of an identity camera, random
    winding (about half are back faces), sizes from sub-pixel to large."""
    u = scenes.uniform01(seed, n_faces * 12).reshape(n_faces, 12)
    verts = []
    for i in range(n_faces):
        cx, cy = (u[i, 0] * spread - spread / 2) * cam.width, (u[i, 1] * spread - spread / 2) * cam.height
        cx += cam.width / 2
        cy += cam.height / 2
        size = 0.5 + (u[i, 2] ** 3) * cam.width * 0.6
        z0 = zmin + u[i, 3] * (zmax - zmin)
        for k in range(3):
            px = cx + (u[i, 4 + 2 * k] - 0.5) * 2 * size
            py = cy + (u[i, 5 + 2 * k] - 0.5) * 2 * size
            z = z0 * (1.0 + 0.2 * (u[i, 10] - 0.5) * (k - 1))
            verts.append(unproject(cam, px, py, z))
    f = np.arange(3 * n_faces, dtype=np.int32).reshape(n_faces, 3)
    return _finish(verts, f, seed=seed)


def shared_vertex_fan(cam, n=24, seed=5):
    """A closed fan of triangles around a centre vertex on a pixel centre:
    every spoke is a shared edge, the centre is shared by all faces."""
    c = unproject(cam, 32, 24, 2.0)
    ring = []
    for k in range(n):
        a = 2 * np.pi * k / n
        ring.append(unproject(cam, 32 + 20 * np.cos(a), 24 + 18 * np.sin(a), 2.0 + 0.3 * np.sin(3 * a)))
    v = [c] + ring
    f = [[0, 1 + k, 1 + (k + 1) % n] for k in range(n)]
    return _finish(v, f, seed=seed)


def texture_border(cam):
    """uv exactly 0 and 1 at the corners: the bilinear fetch reads past the
    last column / row, which the reference addresses linearly."""
    v = [unproject(cam, 2, 2, 2.0), unproject(cam, 60, 2, 2.0), unproject(cam, 60, 45, 2.0),
         unproject(cam, 2, 45, 2.0), unproject(cam, 0, 0, 3.0), unproject(cam, 1, 0, 3.0),
         unproject(cam, 0, 1, 3.0)]
    f = [[4, 6, 5], [0, 2, 1], [0, 3, 2]]  # front-facing (y-down screen)
    m = _finish(v, f)
    m.uv = np.array([[0, 1], [1, 1], [1, 0], [0, 0], [0, 0], [0, 0], [0, 0]], dtype=F32)
    return m


ALL_SMALL = {
    "shared_edge_quad": shared_edge_quad,
    "depth_ties": depth_ties,
    "back_in_front": back_in_front,
    "near_plane_and_tiny": near_plane_and_tiny,
    "triangle_soup": triangle_soup,
    "shared_vertex_fan": shared_vertex_fan,
    "texture_border": texture_border,
}

OPTIONS = {
    "vertex_vnormal_cull": option(2, 1, 1, 0, True),
    "vertex_fnormal_nocull": option(2, 1, 0, 0, False),
    "tex_bilinear_lambert": option(1, 1, 1, 1, True),
    "tex_nn_nocull": option(1, 0, 1, 0, False),
    "white_lambert_fnormal": option(0, 1, 0, 1, True),
    "white_orennayar": option(0, 1, 1, 2, True),
}
