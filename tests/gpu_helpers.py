"""Helpers for the GPU tests: render through the C ABI, compare with the oracle."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ugu_gb300 import capi
from ugu_gb300.rasterizer import Context, RendererCpuOption

OUTPUTS = ("color", "depth", "normal", "mask", "face_id", "color_f32")


def to_option(opt) -> RendererCpuOption:
    return RendererCpuOption(diffuse_color=opt.diffuse_color, interp=opt.interp,
                             shading_normal=opt.shading_normal,
                             diffuse_shading=opt.diffuse_shading,
                             backface_culling=bool(opt.backface_culling),
                             oren_nayar_sigma=opt.oren_nayar_sigma,
                             depth_scale=float(getattr(opt, "depth_scale", 1.0)))


def host_images(cam, outputs=OUTPUTS):
    H, W = cam.height, cam.width
    shapes = {"color": ((H, W, 3), np.uint8), "depth": ((H, W), np.float32),
              "normal": ((H, W, 3), np.float32), "mask": ((H, W), np.uint8),
              "face_id": ((H, W), np.int32), "color_f32": ((H, W, 3), np.float32)}
    out = {k: np.full(shapes[k][0], 0x5A, dtype=shapes[k][1]) for k in outputs}
    im = capi.Images()
    for k, v in out.items():
        setattr(im, k, v.ctypes.data)
    return out, im


def gpu_render(ctx: Context, mesh, cam, opt, slot=0, outputs=OUTPUTS, upload=True):
    if upload:
        ctx.check(ctx.set_mesh(slot, mesh))
    ctx.check(ctx.set_option(to_option(opt)))
    out, im = host_images(cam, outputs)
    rc = ctx.render(slot, cam, im)
    return rc, out


def gpu_raytrace(ctx: Context, mesh, cam, opt, slot=0, outputs=OUTPUTS, upload=True):
    """One view through render_views with UGU_GPU_RAYTRACE, host buffers."""
    if upload:
        ctx.check(ctx.set_mesh(slot, mesh))
    ctx.check(ctx.set_option(to_option(opt)))
    out, im = host_images(cam, outputs)
    v = capi.View()
    v.mesh = slot
    v.camera = capi.camera_struct(cam)
    v.images = im
    rc = ctx.render_views([v], capi.RAYTRACE)
    return rc, out


def device_views(torch, cams, slots, outputs=OUTPUTS):
    """Device output tensors for a batch of views and the capi.View list."""
    dev = torch.device("cuda")
    tensors, views = [], []
    for cam, slot in zip(cams, slots):
        H, W = cam.height, cam.width
        t = {}
        if "color" in outputs:
            t["color"] = torch.full((H, W, 3), 0x5A, dtype=torch.uint8, device=dev)
        if "depth" in outputs:
            t["depth"] = torch.full((H, W), 7.0, dtype=torch.float32, device=dev)
        if "normal" in outputs:
            t["normal"] = torch.full((H, W, 3), 7.0, dtype=torch.float32, device=dev)
        if "mask" in outputs:
            t["mask"] = torch.full((H, W), 0x5A, dtype=torch.uint8, device=dev)
        if "face_id" in outputs:
            t["face_id"] = torch.full((H, W), 1234567, dtype=torch.int32, device=dev)
        if "color_f32" in outputs:
            t["color_f32"] = torch.full((H, W, 3), 7.0, dtype=torch.float32, device=dev)
        v = capi.View()
        v.mesh = slot
        v.camera = capi.camera_struct(cam)
        for k, x in t.items():
            setattr(v.images, k, x.data_ptr())
        tensors.append(t)
        views.append(v)
    return tensors, views


def compare(ref: dict, got: dict, name: str = "", color_tol: int = 0):
    """Bit-exact comparison of every output (colour within color_tol LSB)."""
    for k in ref:
        if k not in got:
            continue
        a, b = ref[k], got[k]
        if k == "color" and color_tol:
            d = np.abs(a.astype(np.int32) - b.astype(np.int32))
            assert d.max() <= color_tol, f"{name}: {k} differs by {d.max()} LSB at {np.argwhere(d > color_tol)[:5]}"
            continue
        if k == "color_f32" and color_tol:
            continue
        if a.dtype.kind == "f":
            same = (a.view(np.uint32) == b.view(np.uint32))
        else:
            same = a == b
        if not same.all():
            bad = np.argwhere(~same)
            i = tuple(bad[0])
            raise AssertionError(f"{name}: {k} differs at {len(bad)} elements, first {i}: "
                                 f"ref {a[i]} gpu {b[i]}")
