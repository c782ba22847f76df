"""ctypes binding of include/ugu_gpu.h (libugugpu.so)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_NOT_PREPARED = 2
ERR_NO_FACE_NORMALS = 3
ERR_NO_TEXTURE = 4
ERR_EMPTY_TEXTURE = 5
ERR_NO_VERTEX_COLORS = 6
ERR_NO_FACE_NORMALS_FOR_SHADING = 7
ERR_NO_VERTEX_NORMALS = 8
ERR_NO_OUTPUT = 9
ERR_NO_CAMERA = 10
ERR_INDEX_OUT_OF_RANGE = 11
ERR_CUDA = 12
ERR_OUT_OF_MEMORY = 13
ERR_DEVICE_TIMEOUT = 14
ERR_CAPACITY = 15
ERR_NO_DEVICE = 16
ERR_DEGENERATE_DEPTH = 17

DEVICE_POINTERS = 1
PER_VIEW = 2
ASYNC = 4
TIME_KERNELS = 8
RAYTRACE = 16

P = C.c_void_p


class Option(C.Structure):
    _fields_ = [("diffuse_color", C.c_int32), ("interp", C.c_int32),
                ("shading_normal", C.c_int32), ("diffuse_shading", C.c_int32),
                ("depth_scale", C.c_float), ("backface_culling", C.c_int32),
                ("oren_nayar_sigma", C.c_float)]


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb8", P), ("rgb_f32", P)]


class MeshDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_int32), ("vertices", P),
                ("num_faces", C.c_int32), ("vertex_indices", P),
                ("face_normals", P),
                ("num_normals", C.c_int32), ("normals", P), ("normal_indices", P),
                ("vertex_colors", P),
                ("num_uv", C.c_int32), ("uv", P), ("uv_indices", P),
                ("material_ids", P),
                ("num_materials", C.c_int32), ("materials", P)]


class CameraDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("w2c_R", C.c_float * 9), ("w2c_t", C.c_float * 3), ("c2w_R", C.c_float * 9),
                ("c2w_t", C.c_float * 3)]


class Images(C.Structure):
    _fields_ = [("color", P), ("depth", P), ("normal", P), ("mask", P), ("face_id", P),
                ("color_f32", P)]


class View(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("camera", CameraDesc), ("images", Images)]


PATH_TILED = 0
PATH_GLOBAL = 1


class Tuning(C.Structure):
    _fields_ = [("path", C.c_int32), ("tile_log2", C.c_int32), ("entry_capacity", C.c_int32),
                ("small_bbox_max", C.c_int32), ("group_pixels", C.c_int32),
                ("ctas_per_sm", C.c_int32), ("split_class", C.c_int32),
                ("bin_faces", C.c_int32), ("small_view_pixels", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("launches", C.c_uint64), ("special_candidates", C.c_uint64),
                ("large_face_tiles", C.c_uint64), ("device_bytes", C.c_uint64),
                ("tile_kernel_ms", C.c_double), ("tile_kernel_launches", C.c_uint64)]


EXPORTS = [
    "ugu_gpu_create", "ugu_gpu_destroy", "ugu_gpu_last_error", "ugu_gpu_abi_version",
    "ugu_gpu_set_option", "ugu_gpu_set_mesh", "ugu_gpu_render", "ugu_gpu_render_views",
    "ugu_gpu_plan_create", "ugu_gpu_plan_launch", "ugu_gpu_plan_destroy", "ugu_gpu_backward",
    "ugu_gpu_set_tuning", "ugu_gpu_get_tuning", "ugu_gpu_autotune", "ugu_gpu_get_stats",
    "ugu_gpu_synchronize", "ugu_gpu_set_stream", "ugu_gpu_render_noalloc",
    "ugu_gpu_get_device_mesh", "ugu_gpu_visualize", "ugu_gpu_render_gbuffer",
    "ugu_gpu_test_visibility", "ugu_gpu_texture_mapping", "ugu_gpu_texture_mapping_targets",
    "ugu_gpu_tile_images",
]

NOALLOC_MAX_PIXELS = 2097152
NOALLOC_MAX_MATERIALS = 16


class DeviceTexture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgba8", P), ("rgb_f32", P)]


class DeviceMesh(C.Structure):
    _fields_ = [("num_vertices", C.c_int32), ("num_faces", C.c_int32),
                ("num_normals", C.c_int32), ("num_uv", C.c_int32),
                ("num_materials", C.c_int32), ("vertices4", P), ("vertex_indices4", P),
                ("face_normals4", P), ("normals4", P), ("normal_indices4", P),
                ("vertex_colors4", P), ("uv2", P), ("uv_indices4", P), ("material_ids", P),
                ("materials", P)]

_lib = None


def load(path: str | None = None):
    """Load libugugpu.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIB_PATH
    if not os.path.exists(path):
        _build.build()
    lib = C.CDLL(path)
    lib.ugu_gpu_create.argtypes = [C.c_int32, C.POINTER(P)]
    lib.ugu_gpu_destroy.argtypes = [P]
    lib.ugu_gpu_last_error.argtypes = [P]
    lib.ugu_gpu_last_error.restype = C.c_char_p
    lib.ugu_gpu_abi_version.argtypes = []
    lib.ugu_gpu_set_option.argtypes = [P, C.POINTER(Option)]
    lib.ugu_gpu_set_mesh.argtypes = [P, C.c_int32, C.POINTER(MeshDesc)]
    lib.ugu_gpu_render.argtypes = [P, C.c_int32, C.POINTER(CameraDesc), C.POINTER(Images)]
    lib.ugu_gpu_render_views.argtypes = [P, C.c_int32, P, C.c_uint32]
    lib.ugu_gpu_plan_create.argtypes = [P, C.c_int32, P, C.c_uint32, C.POINTER(P)]
    lib.ugu_gpu_plan_launch.argtypes = [P]
    lib.ugu_gpu_plan_destroy.argtypes = [P]
    lib.ugu_gpu_backward.argtypes = [P, C.c_int32, P, P, P, P, P, P, C.c_uint32]
    lib.ugu_gpu_set_tuning.argtypes = [P, C.POINTER(Tuning)]
    lib.ugu_gpu_get_tuning.argtypes = [P, C.POINTER(Tuning)]
    lib.ugu_gpu_autotune.argtypes = [P, C.c_int32, P, C.POINTER(Tuning)]
    lib.ugu_gpu_get_stats.argtypes = [P, C.POINTER(Stats)]
    lib.ugu_gpu_synchronize.argtypes = [P]
    lib.ugu_gpu_set_stream.argtypes = [P, P]
    lib.ugu_gpu_render_noalloc.argtypes = [C.POINTER(DeviceMesh), C.POINTER(Option),
                                           C.POINTER(CameraDesc), C.POINTER(Images), P]
    lib.ugu_gpu_get_device_mesh.argtypes = [P, C.c_int32, C.POINTER(DeviceMesh)]
    lib.ugu_gpu_visualize.argtypes = [P, C.c_int32, P, C.c_uint32]
    lib.ugu_gpu_render_gbuffer.argtypes = [P, C.c_int32, P, C.c_uint32]
    lib.ugu_gpu_test_visibility.argtypes = [P, C.c_int32, P, C.c_int32, P, P, C.c_int32, P,
                                            C.c_uint32]
    lib.ugu_gpu_texture_mapping.argtypes = [P, C.c_int32, C.c_int32, P, P, P, P, P, P,
                                            C.c_uint32]
    lib.ugu_gpu_texture_mapping_targets.argtypes = [P, C.c_int32, P, C.c_int32, P, P, P, P,
                                                    P, P, C.c_uint32]
    lib.ugu_gpu_tile_images.argtypes = [P, C.c_int32, P, C.c_int32, P, C.c_uint32]
    for name in EXPORTS:
        if name != "ugu_gpu_last_error":
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


class GpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ugu_gpu error {code}: {msg}")
        self.code = code


class Vis(C.Structure):
    """ugu_gpu_vis: the image helpers of one render (include/ugu_gpu.h)."""
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("depth", P), ("normal", P), ("face_id", P),
                ("vis_depth", P), ("depth_u16", P), ("vis_normal", P), ("vis_face_id", P),
                ("min_d", C.c_float), ("max_d", C.c_float), ("gl_coord", C.c_int32)]


GBUFFER = ("pos_wld", "pos_cam", "normal_wld", "normal_cam", "bary", "uv")


class GBufferView(C.Structure):
    """ugu_gpu_gbuffer: G-buffer channels of one rendered view."""
    _fields_ = [("mesh", C.c_int32), ("camera", CameraDesc), ("face_id", P)]
    _fields_ += [(k, P) for k in GBUFFER] + [("stencil", P)]


class KeyframeDesc(C.Structure):
    """ugu_gpu_keyframe."""
    _fields_ = [("id", C.c_int32), ("camera", CameraDesc), ("w2c_linear", C.c_float * 9),
                ("color", P), ("depth", P), ("mask", P)]


class VisibilityOption(C.Structure):
    """ugu_gpu_visibility_option (VisibilityTesterOption)."""
    _fields_ = [("backface_culling_angle_rad_th", C.c_float), ("use_mask", C.c_int32),
                ("use_depth", C.c_int32), ("interp", C.c_int32),
                ("max_viewing_angle", C.c_float),
                ("max_distance_from_camera_to_vertex", C.c_float),
                ("max_depth_difference", C.c_float), ("eps", C.c_float)]


class TextureOption(C.Structure):
    """ugu_gpu_texture_option (TextureMappingOption's texture size and padding)."""
    _fields_ = [("tex_w", C.c_int32), ("tex_h", C.c_int32), ("padding_kernel", C.c_int32)]


class VisibilityOut(C.Structure):
    """ugu_gpu_visibility_out."""
    _fields_ = [("visible", P), ("projected_pos", P), ("viewing_angle", P), ("distance", P),
                ("color", P), ("intensity", P)]


def w2c_linear(cam) -> np.ndarray:
    """camera->w2c().cast<float>()'s linear part: the general 3x3 inverse of
    the c2w rotation block (Affine3d::inverse, camera.h:319), cast."""
    from . import scenes
    c2w = np.eye(4) if getattr(cam, "c2w", None) is None else np.asarray(cam.c2w, np.float64)
    return scenes._inverse3(c2w[:3, :3]).astype(np.float32)


def camera_struct(cam) -> CameraDesc:
    c = CameraDesc()
    c.width, c.height = int(cam.width), int(cam.height)
    c.fx, c.fy, c.cx, c.cy = cam.fx, cam.fy, cam.cx, cam.cy
    c.w2c_R[:] = [float(x) for x in np.asarray(cam.w2c_R, np.float32).reshape(-1)]
    c.w2c_t[:] = [float(x) for x in np.asarray(cam.w2c_t, np.float32).reshape(-1)]
    c.c2w_R[:] = [float(x) for x in np.asarray(cam.c2w_R, np.float32).reshape(-1)]
    # camera.h:322: c2w_t_f_ = c2w_.matrix().block<3, 1>(0, 3).cast<float>()
    c2w = np.eye(4) if getattr(cam, "c2w", None) is None else np.asarray(cam.c2w, np.float64)
    c.c2w_t[:] = [float(x) for x in c2w[:3, 3].astype(np.float32)]
    return c


class MeshUpload:
    """Builds a MeshDesc over contiguous numpy copies kept alive by self."""

    def __init__(self, mesh):
        self.keep = []

        def a(x, dt):
            if x is None:
                return None
            x = np.ascontiguousarray(x, dtype=dt)
            self.keep.append(x)
            return x.ctypes.data

        d = MeshDesc()
        d.num_vertices = mesh.num_vertices
        d.vertices = a(mesh.vertices, np.float32)
        d.num_faces = mesh.num_faces
        d.vertex_indices = a(mesh.vertex_indices, np.int32)
        d.face_normals = a(mesh.face_normals, np.float32)
        d.num_normals = 0 if mesh.normals is None else int(mesh.normals.shape[0])
        d.normals = a(mesh.normals, np.float32)
        d.normal_indices = a(mesh.normal_indices, np.int32)
        d.vertex_colors = a(mesh.vertex_colors, np.float32)
        d.num_uv = 0 if mesh.uv is None else int(mesh.uv.shape[0])
        d.uv = a(mesh.uv, np.float32)
        d.uv_indices = a(mesh.uv_indices, np.int32)
        d.material_ids = a(mesh.material_ids, np.int32)
        texs = list(mesh.textures or [])
        tf32 = list(getattr(mesh, "textures_f32", None) or [])
        n = max(len(texs), len(tf32))
        arr = (Texture * max(n, 1))()
        for i in range(n):
            t8 = texs[i] if i < len(texs) else None
            t32 = tf32[i] if i < len(tf32) else None
            ref = t8 if t8 is not None else t32
            arr[i].height, arr[i].width = (ref.shape[0], ref.shape[1]) if ref is not None else (0, 0)
            arr[i].rgb8 = a(t8, np.uint8)
            arr[i].rgb_f32 = a(t32, np.float32)
        self.keep.append(arr)
        d.num_materials = n
        d.materials = C.addressof(arr) if n else None
        self.desc = d
