"""ctypes binding of raster_oracle.c (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "liboracle.so")
SRC = os.path.join(HERE, "raster_oracle.c")
SRC_CC = os.path.join(HERE, "ray_oracle.cc")  # the raytracer's BVH (std::sort order)
SRC_VIS = os.path.join(HERE, "vis_oracle.cc")  # image helpers (std::mt19937, std::round)

# -ffp-contract=off: every float operation rounds once, in source order, on
# x86-64 and on aarch64 alike (GCC contracts to FMA by default on aarch64).
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "raster_oracle.h")
    srcs = (SRC, SRC_CC, SRC_VIS, hdr)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(f) for f in srcs)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    oc, occ, ovis = tmp + ".c.o", tmp + ".cc.o", tmp + ".vis.o"
    subprocess.check_call(["gcc", *CFLAGS, "-c", SRC, "-o", oc])
    subprocess.check_call(["g++", *CXXFLAGS, "-c", SRC_CC, "-o", occ])
    subprocess.check_call(["g++", *CXXFLAGS, "-c", SRC_VIS, "-o", ovis])
    subprocess.check_call(["g++", "-shared", oc, occ, ovis, "-o", tmp, "-lm"])
    for f in (oc, occ, ovis):
        os.remove(f)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("data", C.c_void_p)]


class MeshS(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_int32), ("vertices", C.c_void_p),
        ("num_faces", C.c_int32), ("vertex_indices", C.c_void_p),
        ("num_face_normals", C.c_int32), ("face_normals", C.c_void_p),
        ("num_normals", C.c_int32), ("normals", C.c_void_p),
        ("num_normal_indices", C.c_int32), ("normal_indices", C.c_void_p),
        ("num_vertex_colors", C.c_int32), ("vertex_colors", C.c_void_p),
        ("num_uv", C.c_int32), ("uv", C.c_void_p),
        ("num_uv_indices", C.c_int32), ("uv_indices", C.c_void_p),
        ("num_material_ids", C.c_int32), ("material_ids", C.c_void_p),
        ("num_materials", C.c_int32), ("textures", C.c_void_p),
        ("textures_f32", C.c_void_p),
    ]


class CameraS(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("w2c_R", C.c_float * 9), ("w2c_t", C.c_float * 3), ("c2w_R", C.c_float * 9),
                ("c2w_t", C.c_float * 3)]


class OptionS(C.Structure):
    _fields_ = [("diffuse_color", C.c_int32), ("interp", C.c_int32),
                ("shading_normal", C.c_int32), ("diffuse_shading", C.c_int32),
                ("backface_culling", C.c_int32), ("oren_nayar_sigma", C.c_float)]


class PerturbS(C.Structure):
    _fields_ = [("kind", C.c_int32), ("index", C.c_int64), ("delta", C.c_double)]


PERTURB_TEXEL, PERTURB_VCOLOR, PERTURB_VPOS = 1, 2, 3


class StatsS(C.Structure):
    _fields_ = [("bbox_pixels", C.c_int64), ("covered", C.c_int64),
                ("special_candidates", C.c_int64), ("texel_clamps", C.c_int64)]


@dataclass
class Stats:
    bbox_pixels: int
    covered: int
    special_candidates: int
    texel_clamps: int


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = C.CDLL(LIB_PATH)
        P = C.c_void_p
        lib.oracle_render.argtypes = [P, P, P, P, P, P, P, P, P, P]
        lib.oracle_render.restype = C.c_int
        lib.oracle_ray_w.argtypes = [P, C.c_int32, C.c_int32, P]
        lib.oracle_interp_f64.argtypes = [P, P, P, P, P, P, P]
        lib.oracle_backward_f64.argtypes = [P, P, P, P, P, P, P, P, P]
        lib.oracle_backward_f64.restype = C.c_double
        lib.oracle_calc_normals.argtypes = [C.c_int32, P, C.c_int32, P, P, P]
        lib.oracle_raytrace.argtypes = [P, P, P, C.c_float, P, P, P, P, P, P, P]
        lib.oracle_raytrace.restype = C.c_int
        lib.oracle_visualize.argtypes = [C.c_int32, C.c_int32, P, P, P, P, P, P, P, C.c_float,
                                         C.c_float, C.c_int32]
        lib.oracle_visualize.restype = None
        lib.oracle_texture_mapping.argtypes = [C.c_int32, P, P, C.c_int32, P, P, P, P, P,
                                               C.c_int32, C.c_int32, C.c_int32, P, P]
        lib.oracle_texture_mapping.restype = C.c_int
        lib.oracle_simple_triangles_layout.argtypes = [C.c_int32, P, C.c_int32, C.c_int32, P, P]
        lib.oracle_simple_triangles_layout.restype = C.c_int
        lib.oracle_simple_triangles.argtypes = [C.c_int32, C.c_int32, P, P, P, P, P, C.c_int32,
                                                C.c_int32, P, P, P]
        lib.oracle_simple_triangles.restype = C.c_int
        lib.oracle_simple_tile.argtypes = [C.c_int32, P, P, P, P, C.c_int32, P, P, P, P, P]
        lib.oracle_simple_tile.restype = C.c_int
        lib.oracle_simple_charts.argtypes = [C.c_int32, P, P, P, C.c_int32, P, P, P, C.c_int32,
                                             C.c_int32, P, P, P, P]
        lib.oracle_simple_charts.restype = C.c_int
        lib.oracle_gbuffer.argtypes = [P] * 11
        lib.oracle_gbuffer.restype = C.c_int64
        lib.oracle_test_visibility.argtypes = [P, C.c_int32, P, C.c_int32, P, C.c_int32, P, P,
                                               C.c_int32, P, P, P, P, P, P]
        lib.oracle_test_visibility.restype = None
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class _MeshHandle:
    """Keeps the numpy arrays alive while C holds pointers to them."""

    def __init__(self, mesh):
        self.keep = []

        def arr(a, dt, cols=None):
            if a is None:
                return None, 0
            a = np.ascontiguousarray(a, dtype=dt)
            self.keep.append(a)
            return a, (a.shape[0] if a.ndim else 0)

        s = MeshS()
        v, nv = arr(mesh.vertices, np.float32)
        f, nf = arr(mesh.vertex_indices, np.int32)
        fn, nfn = arr(mesh.face_normals, np.float32)
        n, nn = arr(mesh.normals, np.float32)
        ni, nni = arr(mesh.normal_indices, np.int32)
        vc, nvc = arr(mesh.vertex_colors, np.float32)
        uv, nuv = arr(mesh.uv, np.float32)
        ui, nui = arr(mesh.uv_indices, np.int32)
        mi, nmi = arr(mesh.material_ids, np.int32)
        s.num_vertices, s.vertices = nv, _ptr(v)
        s.num_faces, s.vertex_indices = nf, _ptr(f)
        s.num_face_normals, s.face_normals = nfn, _ptr(fn)
        s.num_normals, s.normals = nn, _ptr(n)
        s.num_normal_indices, s.normal_indices = nni, _ptr(ni)
        s.num_vertex_colors, s.vertex_colors = nvc, _ptr(vc)
        s.num_uv, s.uv = nuv, _ptr(uv)
        s.num_uv_indices, s.uv_indices = nui, _ptr(ui)
        s.num_material_ids, s.material_ids = nmi, _ptr(mi)
        texs = list(mesh.textures or [])
        tf32 = list(mesh.textures_f32 or [])
        nm = max(len(texs), len(tf32))
        tarr = (Texture * max(nm, 1))()
        farr = (C.c_void_p * max(nm, 1))()
        for i in range(nm):
            t8 = texs[i] if i < len(texs) else None
            t32 = tf32[i] if i < len(tf32) else None
            ref = t8 if t8 is not None else t32
            tarr[i].height, tarr[i].width = (ref.shape[0], ref.shape[1]) if ref is not None else (0, 0)
            if t8 is not None:
                t8 = np.ascontiguousarray(t8, dtype=np.uint8)
                self.keep.append(t8)
            tarr[i].data = _ptr(t8)
            if t32 is not None:
                t32 = np.ascontiguousarray(t32, dtype=np.float32)
                self.keep.append(t32)
            farr[i] = _ptr(t32)
        self.keep += [tarr, farr]
        s.num_materials = nm
        s.textures = C.addressof(tarr)
        s.textures_f32 = C.addressof(farr) if any(t is not None for t in tf32) else None
        self.s = s


def camera_struct(cam) -> CameraS:
    c = CameraS()
    c.width, c.height = cam.width, cam.height
    c.fx, c.fy, c.cx, c.cy = cam.fx, cam.fy, cam.cx, cam.cy
    for i, x in enumerate(np.asarray(cam.w2c_R, dtype=np.float32).reshape(-1)):
        c.w2c_R[i] = float(x)
    for i, x in enumerate(np.asarray(cam.w2c_t, dtype=np.float32).reshape(-1)):
        c.w2c_t[i] = float(x)
    for i, x in enumerate(np.asarray(cam.c2w_R, dtype=np.float32).reshape(-1)):
        c.c2w_R[i] = float(x)
    c2w = np.eye(4) if getattr(cam, "c2w", None) is None else np.asarray(cam.c2w, np.float64)
    for i, x in enumerate(c2w[:3, 3].astype(np.float32)):
        c.c2w_t[i] = float(x)
    return c


def option_struct(opt) -> OptionS:
    o = OptionS()
    o.diffuse_color = int(opt.diffuse_color)
    o.interp = int(opt.interp)
    o.shading_normal = int(opt.shading_normal)
    o.diffuse_shading = int(opt.diffuse_shading)
    o.backface_culling = 1 if opt.backface_culling else 0
    o.oren_nayar_sigma = float(opt.oren_nayar_sigma)
    return o


def render(mesh, cam, opt, outputs=("color", "depth", "normal", "mask", "face_id"),
           color_f32=False):
    """Render one view; returns (status, dict of numpy images, Stats)."""
    lib = load()
    H, W = cam.height, cam.width
    out = {}
    if "color" in outputs:
        out["color"] = np.empty((H, W, 3), np.uint8)
    if "depth" in outputs:
        out["depth"] = np.empty((H, W), np.float32)
    if "normal" in outputs:
        out["normal"] = np.empty((H, W, 3), np.float32)
    if "mask" in outputs:
        out["mask"] = np.empty((H, W), np.uint8)
    if "face_id" in outputs:
        out["face_id"] = np.empty((H, W), np.int32)
    if color_f32:
        out["color_f32"] = np.empty((H, W, 3), np.float32)
    mh = _MeshHandle(mesh)
    cs = camera_struct(cam)
    os_ = option_struct(opt)
    st = StatsS()
    rc = lib.oracle_render(C.addressof(mh.s), C.addressof(cs), C.addressof(os_),
                           _ptr(out.get("color")), _ptr(out.get("depth")),
                           _ptr(out.get("normal")), _ptr(out.get("mask")),
                           _ptr(out.get("face_id")), _ptr(out.get("color_f32")),
                           C.addressof(st))
    return rc, out, Stats(st.bbox_pixels, st.covered, st.special_candidates, st.texel_clamps)


def raytrace(mesh, cam, opt, outputs=("color", "depth", "normal", "mask", "face_id"),
             color_f32=False, depth_scale=None, sort_dependent=False):
    """ugu::Raytracer's Render for one view; returns (status, images).  With
    sort_dependent, images["sort_dependent"] marks the pixels whose face the
    reference's std::sort picks among equal distances (more than 16 hits)."""
    lib = load()
    H, W = cam.height, cam.width
    shapes = {"color": ((H, W, 3), np.uint8), "depth": ((H, W), np.float32),
              "normal": ((H, W, 3), np.float32), "mask": ((H, W), np.uint8),
              "face_id": ((H, W), np.int32)}
    out = {k: np.empty(*shapes[k]) for k in outputs}
    if color_f32:
        out["color_f32"] = np.empty((H, W, 3), np.float32)
    if sort_dependent:
        out["sort_dependent"] = np.empty((H, W), np.uint8)
    mh = _MeshHandle(mesh)
    cs = camera_struct(cam)
    os_ = option_struct(opt)
    ds = float(getattr(opt, "depth_scale", 1.0) if depth_scale is None else depth_scale)
    rc = lib.oracle_raytrace(C.addressof(mh.s), C.addressof(cs), C.addressof(os_), ds,
                             _ptr(out.get("color")), _ptr(out.get("depth")),
                             _ptr(out.get("normal")), _ptr(out.get("mask")),
                             _ptr(out.get("face_id")), _ptr(out.get("color_f32")),
                             _ptr(out.get("sort_dependent")))
    return rc, out


def visualize(depth=None, normal=None, face_id=None, min_d=200.0, max_d=1500.0,
              gl_coord=False):
    """Depth2Gray, ConvertTo<uint16_t>, Normal2Color and FaceId2RandomColor
    of ugu's image_util for the given images; returns a dict."""
    lib = load()
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
    lib.oracle_visualize(W, H, _ptr(d), _ptr(n), _ptr(f), _ptr(out.get("vis_depth")),
                         _ptr(out.get("depth_u16")), _ptr(out.get("vis_normal")),
                         _ptr(out.get("vis_face_id")), float(min_d), float(max_d),
                         1 if gl_coord else 0)
    return out


def texture_mapping(uv, uv_indices, kf_colors, face_kf, face_tri, tex_w=1024, tex_h=1024,
                    padding_kernel=3):
    """TextureMapping's texture on the mesh's own uv (kUseOriginalMeshUv):
    face_kf[f] the id of face f's keyframe (-1: none; ids index kf_colors),
    face_tri[f] its projected triangle (3 x 2) in that keyframe.  Returns
    (status, texture H x W x 3 uint8, mask H x W uint8)."""
    lib = load()
    uv = np.ascontiguousarray(uv, np.float32)
    uvi = np.ascontiguousarray(uv_indices, np.int32)
    fk = np.ascontiguousarray(face_kf, np.int32)
    ft = np.ascontiguousarray(face_tri, np.float32)
    cols = [np.ascontiguousarray(c, np.uint8) for c in kf_colors]
    kw = np.array([c.shape[1] for c in cols], np.int32)
    kh = np.array([c.shape[0] for c in cols], np.int32)
    ptrs = (C.c_void_p * max(1, len(cols)))(*[c.ctypes.data for c in cols])
    tex = np.zeros((tex_h, tex_w, 3), np.uint8)
    mask = np.zeros((tex_h, tex_w), np.uint8)
    rc = lib.oracle_texture_mapping(len(fk), uv.ctypes.data, uvi.ctypes.data, len(cols),
                                    kw.ctypes.data, kh.ctypes.data, C.addressof(ptrs),
                                    fk.ctypes.data, ft.ctypes.data, tex_w, tex_h,
                                    padding_kernel, tex.ctypes.data, mask.ctypes.data)
    return rc, tex, mask


def simple_triangles_layout(face_kf, tex_w, tex_h):
    """kGenerateSimpleTriangles' layout: (status, target F x 3 x 2, uv F*3 x 2)."""
    lib = load()
    fk = np.ascontiguousarray(face_kf, np.int32)
    target = np.zeros((len(fk), 3, 2), np.float32)
    uv = np.zeros((3 * len(fk), 2), np.float32)
    rc = lib.oracle_simple_triangles_layout(len(fk), fk.ctypes.data, tex_w, tex_h,
                                            target.ctypes.data, uv.ctypes.data)
    return rc, target, uv


def _kf_arrays(kf_colors):
    cols = [np.ascontiguousarray(c, np.uint8) for c in kf_colors]
    kw = np.array([c.shape[1] for c in cols], np.int32)
    kh = np.array([c.shape[0] for c in cols], np.int32)
    ptrs = (C.c_void_p * max(1, len(cols)))(*[c.ctypes.data for c in cols])
    return cols, kw, kh, ptrs


def simple_triangles(kf_colors, face_kf, face_tri, tex_w, tex_h):
    """TextureMapping with kGenerateSimpleTriangles: (status, texture, mask,
    uv F*3 x 2); face_kf[f] indexes kf_colors (-1: none)."""
    lib = load()
    cols, kw, kh, ptrs = _kf_arrays(kf_colors)
    fk = np.ascontiguousarray(face_kf, np.int32)
    ft = np.ascontiguousarray(face_tri, np.float32)
    tex = np.zeros((tex_h, tex_w, 3), np.uint8)
    mask = np.zeros((tex_h, tex_w), np.uint8)
    uv = np.zeros((3 * len(fk), 2), np.float32)
    rc = lib.oracle_simple_triangles(len(fk), len(cols), kw.ctypes.data, kh.ctypes.data,
                                     C.addressof(ptrs), fk.ctypes.data, ft.ctypes.data, tex_w,
                                     tex_h, tex.ctypes.data, mask.ctypes.data, uv.ctypes.data)
    return rc, tex, mask, uv


def simple_tile(kf_ids, kf_colors, face_kf, face_tri):
    """TextureMapping with kGenerateSimpleTile: (status, texture, uv F*3 x 2)."""
    lib = load()
    cols, kw, kh, ptrs = _kf_arrays(kf_colors)
    ids = np.ascontiguousarray(kf_ids, np.int32)
    fk = np.ascontiguousarray(face_kf, np.int32)
    ft = np.ascontiguousarray(face_tri, np.float32)
    tiles = np.zeros(2, np.int32)
    uv = np.zeros((3 * len(fk), 2), np.float32)
    n = len(cols)
    xt = max(int(np.sqrt(n)), 1) if n else 1
    tex = np.zeros(((n // xt) * (kh[0] if n else 0), xt * (kw[0] if n else 0), 3), np.uint8)
    rc = lib.oracle_simple_tile(n, ids.ctypes.data, kw.ctypes.data, kh.ctypes.data,
                                C.addressof(ptrs), len(fk), fk.ctypes.data, ft.ctypes.data,
                                tiles.ctypes.data, tex.ctypes.data if tex.size else None,
                                uv.ctypes.data)
    return rc, tex, uv


def simple_charts(vertex_indices, kf_colors, face_kf, face_tri, tex_w, tex_h):
    """TextureMapping with kGenerateSimpleCharts: (status, texture, uv,
    uv_indices F x 3); face_kf[f] indexes kf_colors (-1: none)."""
    lib = load()
    cols, kw, kh, ptrs = _kf_arrays(kf_colors)
    vi = np.ascontiguousarray(vertex_indices, np.int32)
    fk = np.ascontiguousarray(face_kf, np.int32)
    ft = np.ascontiguousarray(face_tri, np.float32)
    dims = np.zeros(3, np.int32)
    args = (len(fk), vi.ctypes.data, fk.ctypes.data, ft.ctypes.data, len(cols), kw.ctypes.data,
            kh.ctypes.data, C.addressof(ptrs), int(tex_w), int(tex_h), dims.ctypes.data)
    rc = lib.oracle_simple_charts(*args, None, None, None)
    if rc:
        return rc, None, None, None
    tex = np.zeros((dims[1], dims[0], 3), np.uint8)
    uv = np.zeros((dims[2], 2), np.float32)
    uvi = np.zeros((len(fk), 3), np.int32)
    rc = lib.oracle_simple_charts(*args, tex.ctypes.data, uv.ctypes.data, uvi.ctypes.data)
    return rc, tex, uv, uvi


GBUFFER = ("pos_wld", "pos_cam", "normal_wld", "normal_cam", "bary", "uv")


def gbuffer(mesh, cam, opt, face_id):
    """The G-buffer channels of the faces a render reported; returns
    (number of face ids out of range, dict of images)."""
    lib = load()
    H, W = cam.height, cam.width
    out = {k: np.zeros((H, W, 3), np.float32) for k in GBUFFER}
    out["stencil"] = np.zeros((H, W), np.uint8)
    fid = np.ascontiguousarray(face_id, np.int32)
    mh = _MeshHandle(mesh)
    cs = camera_struct(cam)
    os_ = option_struct(opt)
    bad = lib.oracle_gbuffer(C.addressof(mh.s), C.addressof(cs), C.addressof(os_),
                             fid.ctypes.data, *[out[k].ctypes.data for k in GBUFFER],
                             out["stencil"].ctypes.data)
    return int(bad), out


class KeyframeS(C.Structure):
    _fields_ = [("id", C.c_int32), ("cam", CameraS), ("L", C.c_float * 9),
                ("color", C.c_void_p), ("depth", C.c_void_p), ("mask", C.c_void_p)]


class VisOptionS(C.Structure):
    _fields_ = [("backface_th", C.c_float), ("use_mask", C.c_int32), ("use_depth", C.c_int32),
                ("interp", C.c_int32), ("max_viewing_angle", C.c_float),
                ("max_distance", C.c_float), ("max_depth_difference", C.c_float),
                ("eps", C.c_float)]


def test_visibility(vertices, faces, normals, keyframes, option, facewise):
    """VisibilityTester's per-keyframe test (oracle/ray_oracle.cc) for
    keyframes = [(id, camera, w2c_linear 3x3, color HxWx3 u8, depth or None,
    mask or None)] and option = VisibilityTesterOption fields; returns a dict
    of keyframe-major arrays."""
    lib = load()
    V = np.ascontiguousarray(vertices, np.float32)
    F = np.ascontiguousarray(faces, np.int32)
    N = np.ascontiguousarray(normals, np.float32)
    keep = []
    kfs = (KeyframeS * len(keyframes))()
    for i, (kid, cam, L, color, depth, mask) in enumerate(keyframes):
        kfs[i].id = int(kid)
        kfs[i].cam = camera_struct(cam)
        kfs[i].L[:] = [float(x) for x in np.asarray(L, np.float32).reshape(-1)]
        for name, a, dt in (("color", color, np.uint8), ("depth", depth, np.float32),
                            ("mask", mask, np.uint8)):
            if a is not None:
                a = np.ascontiguousarray(a, dt)
                keep.append(a)
                setattr(kfs[i], name, a.ctypes.data)
    o = VisOptionS(float(option.backface_culling_angle_rad_th), int(option.use_mask),
                   int(option.use_depth), int(option.interp), float(option.max_viewing_angle),
                   float(option.max_distance_from_camera_to_vertex),
                   float(option.max_depth_difference), float(option.eps))
    items = 3 * len(F) if facewise else len(V)
    K = len(keyframes)
    out = {"visible": np.zeros((K, items), np.uint8),
           "projected_pos": np.zeros((K, items, 2), np.float32),
           "viewing_angle": np.zeros((K, items), np.float32),
           "distance": np.zeros((K, items), np.float32),
           "color": np.zeros((K, items, 3), np.float32),
           "intensity": np.zeros((K, items), np.float32)}
    lib.oracle_test_visibility(V.ctypes.data, len(V), F.ctypes.data, len(F), N.ctypes.data, K,
                               C.addressof(kfs), C.addressof(o), 1 if facewise else 0,
                               *[out[k].ctypes.data for k in ("visible", "projected_pos",
                                                              "viewing_angle", "distance",
                                                              "color", "intensity")])
    return out


def ray_w(cam, x: int, y: int) -> np.ndarray:
    lib = load()
    cs = camera_struct(cam)
    o = np.empty(3, np.float32)
    lib.oracle_ray_w(C.addressof(cs), int(x), int(y), o.ctypes.data)
    return o


def interp_f64(mesh, cam, opt, face_id):
    lib = load()
    H, W = cam.height, cam.width
    d = np.empty((H, W), np.float64)
    n = np.empty((H, W, 3), np.float64)
    c = np.empty((H, W, 3), np.float64)
    mh = _MeshHandle(mesh)
    cs = camera_struct(cam)
    os_ = option_struct(opt)
    fid = np.ascontiguousarray(face_id, dtype=np.int32)
    lib.oracle_interp_f64(C.addressof(mh.s), C.addressof(cs), C.addressof(os_),
                          fid.ctypes.data, d.ctypes.data, n.ctypes.data, c.ctypes.data)
    return d, n, c


def backward_f64(mesh, cam, opt, face_id, target, grad_tex=None, grad_vcolor=None,
                 grad_vpos=None, perturb=None) -> float:
    """Accumulates FP64 gradients into the given float64 arrays; returns the
    loss.  perturb = (kind, flat index, delta) moves one parameter in double."""
    lib = load()
    mh = _MeshHandle(mesh)
    cs = camera_struct(cam)
    os_ = option_struct(opt)
    fid = np.ascontiguousarray(face_id, dtype=np.int32)
    tgt = np.ascontiguousarray(target, dtype=np.float32)
    for a in (grad_tex, grad_vcolor, grad_vpos):
        assert a is None or (a.dtype == np.float64 and a.flags.c_contiguous)
    ps = None if perturb is None else PerturbS(int(perturb[0]), int(perturb[1]), float(perturb[2]))
    return lib.oracle_backward_f64(C.addressof(mh.s), C.addressof(cs), C.addressof(os_),
                                   fid.ctypes.data, tgt.ctypes.data, _ptr(grad_tex),
                                   _ptr(grad_vcolor), _ptr(grad_vpos),
                                   None if ps is None else C.addressof(ps))


def calc_normals(vertices, faces):
    lib = load()
    v = np.ascontiguousarray(vertices, np.float32)
    f = np.ascontiguousarray(faces, np.int32)
    fn = np.empty((f.shape[0], 3), np.float32)
    n = np.empty((v.shape[0], 3), np.float32)
    lib.oracle_calc_normals(v.shape[0], v.ctypes.data, f.shape[0], f.ctypes.data,
                            fn.ctypes.data, n.ctypes.data)
    return fn, n
