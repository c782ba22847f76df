"""Build and bind oracle/_ref/libugu_ref.so: the reference's own rasterizer
sources compiled unmodified against the Eigen-compatible shim (TEST
INFRASTRUCTURE ONLY).  Only possible where the reference checkout exists
and $UGU_REFERENCE_DIR names it; everything here returns None / skips
elsewhere."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("UGU_REFERENCE_DIR", "")
LIB = os.path.join(HERE, "_ref", "libugu_ref.so")


def available() -> bool:
    return bool(REF) and os.path.exists(os.path.join(REF, "src", "renderer", "cpu",
                                                     "rasterizer.cc"))


def build_if_available() -> str | None:
    if not available():
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={REF}"],
                          stdout=subprocess.DEVNULL)
    return LIB


class RefMesh(C.Structure):
    _fields_ = [("num_vertices", C.c_int), ("vertices", C.c_void_p),
                ("num_faces", C.c_int), ("vertex_indices", C.c_void_p),
                ("face_normals", C.c_void_p),
                ("num_normals", C.c_int), ("normals", C.c_void_p), ("normal_indices", C.c_void_p),
                ("vertex_colors", C.c_void_p),
                ("num_uv", C.c_int), ("uv", C.c_void_p), ("uv_indices", C.c_void_p),
                ("material_ids", C.c_void_p),
                ("num_materials", C.c_int), ("tex_wh", C.c_void_p), ("tex", C.c_void_p)]


class RefOption(C.Structure):
    _fields_ = [("diffuse_color", C.c_int), ("interp", C.c_int), ("shading_normal", C.c_int),
                ("diffuse_shading", C.c_int), ("backface_culling", C.c_int),
                ("oren_nayar_sigma", C.c_float), ("depth_scale", C.c_float)]


_lib = None


def load():
    global _lib
    if _lib is None:
        # make rebuilds only what changed; without the reference checkout an
        # existing build is used as it is
        if build_if_available() is None and not os.path.exists(LIB):
            return None
        lib = C.CDLL(LIB)
        for f in (lib.ref_render, lib.ref_raytrace, lib.ref_render_timed):
            f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                          C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                          C.c_void_p, C.c_void_p, C.c_void_p]
            f.restype = C.c_int
        _lib = lib
    return _lib


def render(mesh, cam, opt):
    """Render with the reference's Rasterizer.  Returns (rc, images, camera
    floats) where the camera floats are the w2c_R / w2c_t / c2w_R the
    reference derived from cam.c2w."""
    return _render(load().ref_render, mesh, cam, opt)


def render_timed(mesh, cam, opt):
    """Render twice on one camera with the reference's Rasterizer.  Returns
    (rc, images, (first call ms, second call ms)): the first call builds the
    camera's ray table, the second finds it built."""
    rc, out, times = _render(load().ref_render_timed, mesh, cam, opt, timed=True)
    return rc, out, (float(times[0]), float(times[1]))


def raytrace(mesh, cam, opt):
    """The same through the reference's Raytracer (naive BVH)."""
    return _render(load().ref_raytrace, mesh, cam, opt)


def _render(fn, mesh, cam, opt, timed=False):
    keep = []

    def a(x, dt):
        if x is None:
            return None
        x = np.ascontiguousarray(x, dtype=dt)
        keep.append(x)
        return x.ctypes.data

    m = RefMesh()
    m.num_vertices, m.vertices = mesh.num_vertices, a(mesh.vertices, np.float32)
    m.num_faces, m.vertex_indices = mesh.num_faces, a(mesh.vertex_indices, np.int32)
    m.face_normals = a(mesh.face_normals, np.float32)
    m.num_normals = 0 if mesh.normals is None else len(mesh.normals)
    m.normals, m.normal_indices = a(mesh.normals, np.float32), a(mesh.normal_indices, np.int32)
    m.vertex_colors = a(mesh.vertex_colors, np.float32)
    m.num_uv = 0 if mesh.uv is None else len(mesh.uv)
    m.uv, m.uv_indices = a(mesh.uv, np.float32), a(mesh.uv_indices, np.int32)
    m.material_ids = a(mesh.material_ids, np.int32)
    texs = list(mesh.textures or [])
    m.num_materials = len(texs)
    wh = np.array([[t.shape[1], t.shape[0]] for t in texs] or [[0, 0]], np.int32)
    m.tex_wh = a(wh, np.int32)
    ptrs = (C.c_void_p * max(1, len(texs)))(*[a(t, np.uint8) for t in texs])
    keep.append(ptrs)
    m.tex = C.addressof(ptrs)
    o = RefOption(int(opt.diffuse_color), int(opt.interp), int(opt.shading_normal),
                  int(opt.diffuse_shading), 1 if opt.backface_culling else 0,
                  float(opt.oren_nayar_sigma), float(getattr(opt, "depth_scale", 1.0)))
    H, W = cam.height, cam.width
    out = {"color": np.zeros((H, W, 3), np.uint8), "depth": np.zeros((H, W), np.float32),
           "normal": np.zeros((H, W, 3), np.float32), "mask": np.zeros((H, W), np.uint8),
           "face_id": np.zeros((H, W), np.int32)}
    c2w = np.ascontiguousarray(cam.c2w if cam.c2w is not None else np.eye(4), np.float64)
    camf = np.zeros(21, np.float32)
    times = np.zeros(2, np.float64)
    rc = fn(C.addressof(m), W, H, cam.fx, cam.fy, cam.cx, cam.cy, c2w.ctypes.data,
                        C.addressof(o), out["color"].ctypes.data, out["depth"].ctypes.data,
                        out["normal"].ctypes.data, out["mask"].ctypes.data,
                        out["face_id"].ctypes.data, (times if timed else camf).ctypes.data)
    if timed:
        return rc, out, times
    return rc, out, {"w2c_R": camf[0:9].reshape(3, 3).copy(), "w2c_t": camf[9:12].copy(),
                     "c2w_R": camf[12:21].reshape(3, 3).copy()}


def bin_packing_2d(rects, x_min, x_max, y_min, y_max):
    """ugu::BinPacking2D (src/discrete/bin_packer_2d.cc), the reference's own
    code, on integer (x, y, width, height) rects: (ok, packed rects, free
    rects), or None without the reference build."""
    lib = load()
    if lib is None:
        return None
    f = lib.ref_bin_packing_2d
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                  C.c_void_p, C.c_int, C.c_void_p]
    r = np.ascontiguousarray(np.asarray(rects, np.int32).reshape(-1, 4))
    n = len(r)
    packed = np.zeros((n, 4), np.int32)
    cap = 4 * n + 8  # each placement turns one free rect into at most two
    free = np.zeros((cap, 4), np.int32)
    n_free = C.c_int(0)
    ok = f(r.ctypes.data, n, x_min, x_max, y_min, y_max, packed.ctypes.data, free.ctypes.data,
           cap, C.byref(n_free))
    return bool(ok), [tuple(int(v) for v in x) for x in packed], \
        [tuple(int(v) for v in x) for x in free[:min(n_free.value, cap)]]


class RefKeyframe(C.Structure):
    _fields_ = [("id", C.c_int), ("width", C.c_int), ("height", C.c_int),
                ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("c2w", C.c_double * 16), ("color", C.c_void_p), ("depth", C.c_void_p),
                ("mask", C.c_void_p)]


class RefVisOption(C.Structure):
    _fields_ = [("backface_culling_angle_rad_th", C.c_float), ("use_mask", C.c_int),
                ("use_depth", C.c_int), ("interp", C.c_int), ("calc_stat_vertex_info", C.c_int),
                ("collect_face_info", C.c_int), ("calc_stat_face_info", C.c_int),
                ("max_viewing_angle", C.c_float),
                ("max_distance_from_camera_to_vertex", C.c_float),
                ("max_depth_difference", C.c_float), ("eps", C.c_float),
                ("invalid_color", C.c_float * 3)]


def visibility(vertices, normals, faces, keyframes, option, facewise):
    """ugu::VisibilityTester::Test(keyframes, info, facewise)
    (src/texturing/visibility_tester.cc), the reference's own code, for
    keyframes = [(id, camera, color, depth or None, mask or None)] and
    option = VisibilityTesterOption fields.  Returns the VisibilityInfo as
    arrays (see ref_visibility.cc), or None without the reference build."""
    lib = load()
    if lib is None:
        return None
    V = np.ascontiguousarray(vertices, np.float32)
    N = np.ascontiguousarray(normals, np.float32)
    F = np.ascontiguousarray(faces, np.int32)
    K, nv, nf = len(keyframes), len(V), len(F)
    keep = []
    kfs = (RefKeyframe * K)()
    for i, (kid, cam, color, depth, mask) in enumerate(keyframes):
        k = kfs[i]
        k.id, k.width, k.height = int(kid), int(cam.width), int(cam.height)
        k.fx, k.fy, k.cx, k.cy = float(cam.fx), float(cam.fy), float(cam.cx), float(cam.cy)
        k.c2w[:] = [float(x) for x in np.asarray(cam.c2w, np.float64).reshape(-1)]
        for name, a, dt in (("color", color, np.uint8), ("depth", depth, np.float32),
                            ("mask", mask, np.uint8)):
            if a is not None:
                a = np.ascontiguousarray(a, dt)
                keep.append(a)
                setattr(k, name, a.ctypes.data)
    o = RefVisOption(float(option.backface_culling_angle_rad_th), int(option.use_mask),
                     int(option.use_depth), int(option.interp),
                     int(option.calc_stat_vertex_info), int(option.collect_face_info),
                     int(option.calc_stat_face_info), float(option.max_viewing_angle),
                     float(option.max_distance_from_camera_to_vertex),
                     float(option.max_depth_difference), float(option.eps),
                     (C.c_float * 3)(0.0, 0.0, 0.0))
    out = {"vcount": np.zeros(nv, np.int32), "vrec_id": np.zeros((nv, K), np.int32),
           "vrec": np.zeros((nv, K, 9), np.float32), "vstat_i": np.zeros((nv, 5), np.int32),
           "vstat": np.zeros((nv, 43), np.float32), "fcount": np.zeros(nf, np.int32),
           "frec_id": np.zeros((nf, K, 2), np.int32), "frec": np.zeros((nf, K, 9), np.float32),
           "fstat_i": np.zeros((nf, 6), np.int32), "fstat": np.zeros((nf, 3), np.float32)}
    f = lib.ref_visibility
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                  C.c_void_p, C.c_int] + [C.c_void_p] * 10
    rc = f(V.ctypes.data, nv, N.ctypes.data, F.ctypes.data, nf, C.addressof(kfs), K,
           C.addressof(o), 1 if facewise else 0,
           *[out[k].ctypes.data for k in ("vcount", "vrec_id", "vrec", "vstat_i", "vstat",
                                          "fcount", "frec_id", "frec", "fstat_i", "fstat")])
    out["rc"] = rc
    return out


def texture_mapping(vertices, normals, faces, keyframes, option, facewise, criteria, uv_type,
                    tex_w, tex_h, padding_kernel=3, uv=None, uv_indices=None):
    """The reference's own VisibilityTester::Test(keyframes, ...) and then
    ugu::TextureMapping (src/texturing/texture_mapper.cc) with the given
    TextureMappingOption fields.  Returns (status, texture H x W x 3 uint8,
    uv N x 2, uv_indices F x 3, material_ids F), or None without the
    reference build; status 0 is success."""
    lib = load()
    if lib is None:
        return None
    V = np.ascontiguousarray(vertices, np.float32)
    N = np.ascontiguousarray(normals, np.float32)
    F = np.ascontiguousarray(faces, np.int32)
    K, nf = len(keyframes), len(F)
    keep = []
    kfs = (RefKeyframe * K)()
    for i, (kid, cam, color, depth, mask) in enumerate(keyframes):
        k = kfs[i]
        k.id, k.width, k.height = int(kid), int(cam.width), int(cam.height)
        k.fx, k.fy, k.cx, k.cy = float(cam.fx), float(cam.fy), float(cam.cx), float(cam.cy)
        k.c2w[:] = [float(x) for x in np.asarray(cam.c2w, np.float64).reshape(-1)]
        for name, a, dt in (("color", color, np.uint8), ("depth", depth, np.float32),
                            ("mask", mask, np.uint8)):
            if a is not None:
                a = np.ascontiguousarray(a, dt)
                keep.append(a)
                setattr(k, name, a.ctypes.data)
    o = RefVisOption(float(option.backface_culling_angle_rad_th), int(option.use_mask),
                     int(option.use_depth), int(option.interp),
                     int(option.calc_stat_vertex_info), int(option.collect_face_info),
                     int(option.calc_stat_face_info), float(option.max_viewing_angle),
                     float(option.max_distance_from_camera_to_vertex),
                     float(option.max_depth_difference), float(option.eps),
                     (C.c_float * 3)(0.0, 0.0, 0.0))
    if uv is not None:
        U = np.ascontiguousarray(uv, np.float32)
        UI = np.ascontiguousarray(uv_indices, np.int32)
        uv_args = (U.ctypes.data, len(U), UI.ctypes.data)
    else:
        uv_args = (None, 0, None)
    f = lib.ref_texture_mapping
    f.restype = C.c_int
    f.argtypes = ([C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                   C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                   C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p,
                   C.c_int, C.c_void_p, C.c_void_p, C.c_void_p])
    tex_cap, uv_cap = 3 * tex_w * tex_h, 3 * nf
    for _ in range(2):  # once more with the sizes a first call reported
        tex = np.zeros(max(tex_cap, 1), np.uint8)
        wh = np.zeros(2, np.int32)
        uv_out = np.zeros((max(uv_cap, 1), 2), np.float32)
        n_uv = C.c_int(0)
        uvi = np.zeros((nf, 3), np.int32)
        mat = np.zeros(nf, np.int32)
        rc = f(V.ctypes.data, len(V), N.ctypes.data, F.ctypes.data, nf, *uv_args,
               C.addressof(kfs), K, C.addressof(o), 1 if facewise else 0, int(criteria),
               int(uv_type), int(tex_w), int(tex_h), int(padding_kernel), tex.ctypes.data,
               tex_cap, wh.ctypes.data, uv_out.ctypes.data, uv_cap, C.byref(n_uv),
               uvi.ctypes.data, mat.ctypes.data)
        if rc != 3:
            break
        tex_cap, uv_cap = 3 * int(wh[0]) * int(wh[1]), int(n_uv.value)
    if rc:
        return rc, None, None, None, None
    w, h = int(wh[0]), int(wh[1])
    return 0, tex[:3 * w * h].reshape(h, w, 3), uv_out[:n_uv.value], uvi, mat


def visualize(depth=None, normal=None, face_id=None, min_d=200.0, max_d=1500.0,
              gl_coord=False):
    """The reference's own Depth2Gray, ConvertTo<uint16_t>, Normal2Color and
    FaceId2RandomColor (src/util/image_util.cc, include/ugu/image_proc.h)
    for the given images; returns a dict like oracle.visualize, or None
    without the reference build."""
    lib = load()
    if lib is None:
        return None
    shp = next(a for a in (depth, normal, face_id) if a is not None).shape
    H, W = shp[0], shp[1]
    d = None if depth is None else np.ascontiguousarray(depth, np.float32)
    n = None if normal is None else np.ascontiguousarray(normal, np.float32)
    f = None if face_id is None else np.ascontiguousarray(face_id, np.int32)
    out = {}
    if d is not None:
        out["vis_depth"] = np.zeros((H, W), np.uint8)
        out["depth_u16"] = np.zeros((H, W), np.uint16)
    if n is not None:
        out["vis_normal"] = np.zeros((H, W, 3), np.uint8)
    if f is not None:
        out["vis_face_id"] = np.zeros((H, W, 3), np.uint8)
    fn = lib.ref_visualize
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 7 + [C.c_float, C.c_float, C.c_int]
    ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
    fn(W, H, ptr(d), ptr(n), ptr(f), ptr(out.get("vis_depth")), ptr(out.get("depth_u16")),
       ptr(out.get("vis_normal")), ptr(out.get("vis_face_id")), float(min_d), float(max_d),
       1 if gl_coord else 0)
    return out
