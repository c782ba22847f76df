"""Python host side of the GB300 rasterizer.

``Context`` owns one ugu_gpu_context (include/ugu_gpu.h).  ``Rasterizer``
mirrors ugu::Rasterizer (include/ugu/renderer/cpu/rasterizer.h:14-53) --
set_option / set_mesh / PrepareMesh / set_camera / Render / RenderW and the
single-output variants -- with the reference's error behaviour: a failed
precondition logs the reference's message and returns False.
"""
from __future__ import annotations

import ctypes as C
import sys
import weakref
from dataclasses import dataclass

import numpy as np

from . import capi


class DiffuseColor:  # include/ugu/renderer/base.h:11-16
    kNone, kTexture, kVertex = 0, 1, 2


class ColorInterpolation:  # include/ugu/common.h:50-53
    kNn, kBilinear = 0, 1


class ShadingNormal:  # include/ugu/renderer/base.h:18-22
    kFace, kVertex = 0, 1


class DiffuseShading:  # include/ugu/renderer/base.h:24-32
    kNone, kLambertian, kOrenNayar = 0, 1, 2


@dataclass
class RendererCpuOption:
    """include/ugu/renderer/cpu/renderer.h:17-38 (same fields and defaults)."""
    diffuse_color: int = DiffuseColor.kNone
    interp: int = ColorInterpolation.kBilinear
    shading_normal: int = ShadingNormal.kVertex
    diffuse_shading: int = DiffuseShading.kNone
    depth_scale: float = 1.0
    backface_culling: bool = True
    oren_nayar_sigma: float = 0.3

    def CopyTo(self, dst: "RendererCpuOption") -> None:
        """renderer.h:30-37: copies every field except oren_nayar_sigma."""
        dst.diffuse_color = self.diffuse_color
        dst.depth_scale = self.depth_scale
        dst.interp = self.interp
        dst.shading_normal = self.shading_normal
        dst.diffuse_shading = self.diffuse_shading
        dst.backface_culling = self.backface_culling

    def to_struct(self) -> capi.Option:
        o = capi.Option()
        o.diffuse_color = int(self.diffuse_color)
        o.interp = int(self.interp)
        o.shading_normal = int(self.shading_normal)
        o.diffuse_shading = int(self.diffuse_shading)
        o.depth_scale = float(self.depth_scale)
        o.backface_culling = 1 if self.backface_culling else 0
        o.oren_nayar_sigma = float(self.oren_nayar_sigma)
        return o


def LOGE(msg: str) -> None:  # src/log.cc:21-62 error level
    sys.stderr.write(msg if msg.endswith("\n") else msg + "\n")


LOGW = LOGE


class Context:
    """One ugu_gpu_context on a device."""

    def __init__(self, device: int = 0):
        self.lib = capi.load()
        h = C.c_void_p()
        rc = self.lib.ugu_gpu_create(int(device), C.byref(h))
        if rc != capi.OK:
            raise capi.GpuError(rc, self.lib.ugu_gpu_last_error(None).decode())
        self.h = h
        self._uploads = {}
        self._plans = weakref.WeakSet()

    def close(self):
        if getattr(self, "h", None):
            for p in list(getattr(self, "_plans", ())):  # the library frees them with ctx
                p.h = None
            self.lib.ugu_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        return self.lib.ugu_gpu_last_error(self.h).decode()

    def check(self, rc: int):
        if rc != capi.OK:
            raise capi.GpuError(rc, self.last_error())
        return rc

    def set_option(self, opt: RendererCpuOption) -> int:
        s = opt.to_struct()
        return self.lib.ugu_gpu_set_option(self.h, C.byref(s))

    def set_mesh(self, slot: int, mesh) -> int:
        if mesh is None:
            self._uploads.pop(slot, None)
            return self.lib.ugu_gpu_set_mesh(self.h, int(slot), None)
        up = capi.MeshUpload(mesh)
        rc = self.lib.ugu_gpu_set_mesh(self.h, int(slot), C.byref(up.desc))
        return rc

    def render(self, slot: int, cam, images: capi.Images) -> int:
        cs = capi.camera_struct(cam)
        return self.lib.ugu_gpu_render(self.h, int(slot), C.byref(cs), C.byref(images))

    def render_views(self, views, flags: int) -> int:
        arr = (capi.View * len(views))(*views)
        return self.lib.ugu_gpu_render_views(self.h, len(views), C.addressof(arr), int(flags))

    def plan_create(self, views, flags: int):
        arr = (capi.View * len(views))(*views)
        h = C.c_void_p()
        self.check(self.lib.ugu_gpu_plan_create(self.h, len(views), C.addressof(arr), int(flags),
                                                C.byref(h)))
        plan = Plan(self, h)
        self._plans.add(plan)
        return plan

    def synchronize(self) -> int:
        return self.lib.ugu_gpu_synchronize(self.h)

    def set_stream(self, stream_handle: int | None) -> int:
        return self.lib.ugu_gpu_set_stream(self.h, stream_handle)

    def tuning(self) -> capi.Tuning:
        t = capi.Tuning()
        self.check(self.lib.ugu_gpu_get_tuning(self.h, C.byref(t)))
        return t

    def set_tuning(self, t: capi.Tuning) -> int:
        return self.lib.ugu_gpu_set_tuning(self.h, C.byref(t))

    def autotune(self, views) -> capi.Tuning:
        """Times candidate tunings on these views (device pointers) and keeps
        the fastest; returns it."""
        arr = (capi.View * len(views))(*views)
        t = capi.Tuning()
        self.check(self.lib.ugu_gpu_autotune(self.h, len(views), C.addressof(arr), C.byref(t)))
        return t

    def backward(self, views, targets, grad_texels=None, grad_vertex_colors=None,
                 grad_vertices=None, loss=None, flags: int = capi.DEVICE_POINTERS) -> int:
        """ugu_gpu_backward: views carry the forward's face_id images; targets,
        gradients and loss are device pointers (ints) or None."""
        arr = (capi.View * len(views))(*views)
        tg = (C.c_void_p * len(targets))(*targets)
        return self.lib.ugu_gpu_backward(self.h, len(views), C.addressof(arr), C.addressof(tg),
                                         grad_texels, grad_vertex_colors, grad_vertices, loss,
                                         int(flags))

    def device_mesh(self, slot: int):
        """The slot's device arrays (ugu_gpu_get_device_mesh) as a namespace
        with .textures = [DeviceTexture, ...]."""
        d = capi.DeviceMesh()
        self.check(self.lib.ugu_gpu_get_device_mesh(self.h, int(slot), C.byref(d)))
        tex = []
        if d.materials:
            arr = C.cast(d.materials, C.POINTER(capi.DeviceTexture))
            tex = [arr[i] for i in range(d.num_materials)]
        d.textures = tex
        return d

    def test_visibility(self, slot: int, normals, keyframes, option, facewise: bool, out,
                        flags: int = 0) -> int:
        arr = (capi.KeyframeDesc * len(keyframes))(*keyframes)
        n = np.ascontiguousarray(normals, np.float32)
        return self.lib.ugu_gpu_test_visibility(self.h, int(slot), n.ctypes.data, len(keyframes),
                                                C.addressof(arr), C.byref(option),
                                                1 if facewise else 0, C.byref(out), int(flags))

    def render_gbuffer(self, views, flags: int = 0) -> int:
        arr = (capi.GBufferView * len(views))(*views)
        return self.lib.ugu_gpu_render_gbuffer(self.h, len(views), C.addressof(arr), int(flags))

    def visualize(self, items, flags: int = 0) -> int:
        arr = (capi.Vis * len(items))(*items)
        return self.lib.ugu_gpu_visualize(self.h, len(items), C.addressof(arr), int(flags))

    def texture_mapping(self, slot: int, kf_descs, face_kf, face_tri, option,
                        texture: np.ndarray, mask: np.ndarray) -> int:
        """ugu_gpu_texture_mapping with host buffers."""
        arr = (capi.KeyframeDesc * max(1, len(kf_descs)))(*kf_descs)
        fk = np.ascontiguousarray(face_kf, np.int32)
        ft = np.ascontiguousarray(face_tri, np.float32)
        return self.lib.ugu_gpu_texture_mapping(self.h, int(slot), len(kf_descs), C.addressof(arr),
                                                fk.ctypes.data, ft.ctypes.data, C.byref(option),
                                                texture.ctypes.data, mask.ctypes.data, 0)

    def texture_mapping_targets(self, face_target, kf_descs, face_kf, face_tri, option,
                                texture: np.ndarray, mask: np.ndarray) -> int:
        """ugu_gpu_texture_mapping_targets with host buffers: faces drawn into
        the given target triangles (F x 6 texel coordinates)."""
        arr = (capi.KeyframeDesc * max(1, len(kf_descs)))(*kf_descs)
        tg = np.ascontiguousarray(face_target, np.float32)
        fk = np.ascontiguousarray(face_kf, np.int32)
        ft = np.ascontiguousarray(face_tri, np.float32)
        return self.lib.ugu_gpu_texture_mapping_targets(
            self.h, len(fk), tg.ctypes.data, len(kf_descs), C.addressof(arr), fk.ctypes.data,
            ft.ctypes.data, C.byref(option), texture.ctypes.data, mask.ctypes.data, 0)

    def tile_images(self, kf_descs, x_tiles: int, texture: np.ndarray) -> int:
        """ugu_gpu_tile_images with host buffers."""
        arr = (capi.KeyframeDesc * max(1, len(kf_descs)))(*kf_descs)
        return self.lib.ugu_gpu_tile_images(self.h, len(kf_descs), C.addressof(arr), int(x_tiles),
                                            texture.ctypes.data, 0)

    def stats(self) -> capi.Stats:
        s = capi.Stats()
        self.check(self.lib.ugu_gpu_get_stats(self.h, C.byref(s)))
        return s


class Plan:
    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h

    def launch(self) -> int:
        return self.ctx.lib.ugu_gpu_plan_launch(self.h)

    def close(self):
        if self.h:  # None once closed here or with its context
            self.ctx.lib.ugu_gpu_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _out(arg, shape, dtype):
    """None -> skip; True -> allocate; ndarray -> fill in place (reallocated
    when its shape or dtype differ, as ugu::Init does)."""
    if arg is None or arg is False:
        return None
    if isinstance(arg, np.ndarray) and arg.shape == shape and arg.dtype == dtype \
            and arg.flags.c_contiguous:
        return arg
    return np.empty(shape, dtype)


class Rasterizer:
    """ugu::Rasterizer's interface over the GPU (rasterizer.h:14-53)."""

    def __init__(self, option: RendererCpuOption | None = None, device: int = 0):
        self._ctx = Context(device)
        self._option = RendererCpuOption()
        self._mesh = None
        self._mesh_initialized = False
        self._camera = None
        if option is not None:
            self.set_option(option)

    def set_option(self, option: RendererCpuOption) -> None:  # rasterizer.cc:73-75
        option.CopyTo(self._option)

    def set_mesh(self, mesh) -> None:  # rasterizer.cc:77-88
        self._mesh_initialized = False
        self._mesh = mesh
        if mesh.face_normals is None or len(mesh.face_normals) == 0:
            LOGW("face normal is empty. culling and shading may not work\n")
        if mesh.normals is None or len(mesh.normals) == 0:
            LOGW("vertex normal is empty. shading may not work\n")

    def PrepareMesh(self) -> bool:  # rasterizer.cc:90-99
        if self._mesh is None:
            LOGE("mesh has not been set\n")
            return False
        rc = self._ctx.set_mesh(0, self._mesh)
        if rc != capi.OK:
            LOGE(self._ctx.last_error())
            return False
        self._mesh_initialized = True
        return True

    def set_camera(self, camera) -> None:  # rasterizer.cc:101-103
        self._camera = camera

    def Render(self, color=None, depth=None, normal=None, mask=None, face_id=None,
               color_f32=None):
        """rasterizer.cc:105-307.  Returns (ok, {name: image})."""
        if self._camera is None:
            LOGE("camera has not been set\n")
            return False, {}
        if not self._mesh_initialized:
            LOGE("mesh has not been initialized\n")
            return False, {}
        rc = self._ctx.set_option(self._option)
        if rc != capi.OK:
            LOGE(self._ctx.last_error())
            return False, {}
        H, W = self._camera.height, self._camera.width
        outs = {
            "color": _out(color, (H, W, 3), np.uint8),
            "depth": _out(depth, (H, W), np.float32),
            "normal": _out(normal, (H, W, 3), np.float32),
            "mask": _out(mask, (H, W), np.uint8),
            "face_id": _out(face_id, (H, W), np.int32),
            "color_f32": _out(color_f32, (H, W, 3), np.float32),
        }
        im = capi.Images()
        for k, v in outs.items():
            setattr(im, k, None if v is None else v.ctypes.data)
        rc = self._render(im)
        if rc != capi.OK:
            LOGE(self._ctx.last_error())
            return False, {}
        return True, {k: v for k, v in outs.items() if v is not None}

    def _render(self, im: capi.Images) -> int:
        return self._ctx.render(0, self._camera, im)

    def RenderColor(self):
        return self.Render(color=True)

    def RenderDepth(self):
        return self.Render(depth=True)

    def RenderNormal(self):
        return self.Render(normal=True)

    def RenderMask(self):
        return self.Render(mask=True)

    def RenderFaceId(self):
        return self.Render(face_id=True)

    def RenderW(self, color=None, depth=True, normal=None, mask=None, face_id=None):
        """rasterizer.cc:329-344 (raytracer.cc:241-256): float depth converted by ConvertTo
        (image_proc.h:454-...) with scale 1: static_cast<uint16_t>(double)."""
        if depth is None:
            LOGE("depth is nullptr")
            return False, {}
        ok, out = self.Render(color, True, normal, mask, face_id)
        if ok:
            out["depth"] = depth_to_u16(out["depth"])
        return ok, out

    def RenderDepthW(self):
        return self.RenderW(depth=True)

    def RenderGBuffer(self):
        """Extension: ugu::GBuffer's channels (include/ugu/renderer/base.h:
        34-77) for the current camera -- face_id from a render, then the
        G-buffer pass (include/ugu_gpu.h, ugu_gpu_render_gbuffer).  Returns
        (ok, {name: image})."""
        ok, out = self.Render(face_id=True)
        if not ok:
            return False, {}
        H, W = self._camera.height, self._camera.width
        g = {k: np.zeros((H, W, 3), np.float32) for k in capi.GBUFFER}
        g["stencil"] = np.zeros((H, W), np.uint8)
        v = capi.GBufferView()
        v.mesh = 0
        v.camera = capi.camera_struct(self._camera)
        v.face_id = out["face_id"].ctypes.data
        for k, a in g.items():
            setattr(v, k, a.ctypes.data)
        rc = self._ctx.render_gbuffer([v])
        if rc != capi.OK:
            LOGE(self._ctx.last_error())
            return False, {}
        g["face_id"] = out["face_id"]
        return True, g


class Raytracer(Rasterizer):
    """ugu::Raytracer's interface over the GPU (raytracer.h:14-53,
    src/renderer/cpu/raytracer.cc): the same RendererCpu methods; Render
    casts one ray per pixel through the naive BVH (built on the device side
    at the first Render after PrepareMesh) instead of rasterising."""

    def PrepareMesh(self) -> bool:  # raytracer.cc:90-110
        if self._mesh is None:
            LOGE("mesh has not been set\n")
            return False
        if len(self._mesh.vertices) == 0 or len(self._mesh.vertex_indices) == 0:
            LOGE("mesh is empty\n")
            return False
        return super().PrepareMesh()

    def _render(self, im: capi.Images) -> int:
        v = capi.View()
        v.mesh = 0
        v.camera = capi.camera_struct(self._camera)
        v.images = im
        return self._ctx.render_views([v], capi.RAYTRACE)


def _visualize(ctx: Context | None, depth=None, normal=None, face_id=None, min_d=200.0,
               max_d=1500.0, gl_coord=False) -> dict:
    """One ugu_gpu_visualize call on host arrays; returns the outputs."""
    own = ctx is None
    ctx = Context(0) if own else ctx
    try:
        src = next(a for a in (depth, normal, face_id) if a is not None)
        H, W = src.shape[0], src.shape[1]
        keep, out = [], {}
        it = capi.Vis()
        it.width, it.height = W, H
        it.min_d, it.max_d, it.gl_coord = float(min_d), float(max_d), 1 if gl_coord else 0
        for name, a, dt in (("depth", depth, np.float32), ("normal", normal, np.float32),
                            ("face_id", face_id, np.int32)):
            if a is not None:
                a = np.ascontiguousarray(a, dt)
                keep.append(a)
                setattr(it, name, a.ctypes.data)
        if depth is not None:
            out["vis_depth"] = np.zeros((H, W), np.uint8)
            out["depth_u16"] = np.zeros((H, W), np.uint16)
        if normal is not None:
            out["vis_normal"] = np.zeros((H, W, 3), np.uint8)
        if face_id is not None:
            out["vis_face_id"] = np.zeros((H, W, 3), np.uint8)
        for k, v in out.items():
            setattr(it, k, v.ctypes.data)
        ctx.check(ctx.visualize([it]))
        return out
    finally:
        if own:
            ctx.close()


def Depth2Gray(depth, min_d: float = 200.0, max_d: float = 1500.0, ctx=None) -> np.ndarray:
    """src/util/image_util.cc:392-411 on the GPU."""
    return _visualize(ctx, depth=depth, min_d=min_d, max_d=max_d)["vis_depth"]


def Normal2Color(normal, gl_coord: bool = False, ctx=None) -> np.ndarray:
    """src/util/image_util.cc:413-446 (RGB order) on the GPU."""
    return _visualize(ctx, normal=normal, gl_coord=gl_coord)["vis_normal"]


def FaceId2RandomColor(face_id, ctx=None) -> np.ndarray:
    """src/util/image_util.cc:448-487 (RGB order) on the GPU."""
    return _visualize(ctx, face_id=face_id)["vis_face_id"]


def depth_to_u16(depth: np.ndarray) -> np.ndarray:
    """static_cast<uint16_t>(1.0 * double(d)) per pixel: truncation toward
    zero; values outside [0, 65536) keep the low 16 bits of the saturated
    int32 conversion."""
    d = depth.astype(np.float64)
    i = np.where(np.isnan(d), 0, np.clip(np.trunc(d), -2.0 ** 31, 2.0 ** 31 - 1)).astype(np.int64)
    return (i & 0xFFFF).astype(np.uint16)
