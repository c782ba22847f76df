"""Small seeded workloads that run each kernel family of libugugpu.so a few
times, for profiling one kernel at a time (for example under
`ncu -k regex:<kernel> -c 3`) and for quick timing.

    python -m ugu_gb300.kernel_cases --case tiled --repeat 3

Cases (the kernels each one launches):
  tiled       k_proj, k_count, k_scan_sum, k_scan_apply, k_place, k_tile:
              a CUDA-graph replay of `views` ring views of icosphere-7
              (2048^2 RGB8 texture, bilinear, vertex normals, culling on)
  global      k_raster, k_tiles, k_resolve: the same views on the global
              z-buffer path
  noalloc     the global path's kernels through ugu_gpu_render_noalloc, one
              1920x1080 view
  visualize   k_vis: Depth2Gray, Normal2Color, FaceId2RandomColor and the
              16-bit depth of the rendered views
  gbuffer     k_gbuffer: the G-buffer channels of the rendered views
  visibility  k_visibility: VisibilityTester over `views` keyframes of
              icosphere-6 at 1280x720
  texmap      k_tm_cover, k_tm_fill, k_tm_pad: TextureMapping on
              the mesh's own uv (2048^2) from those keyframes
  backward    k_proj64, k_backward: the per-pixel L2 gradient of `views`
              640x480 views (float texels)
  raytrace    k_ray: `views` ring views raytraced

`--tuning field=value,...` sets fields of ugu_gpu_tuning before the case
runs (for example the ones a bench line reports), `--autotune` lets
ugu_gpu_autotune choose them on the case's views (tiled and global cases;
with UGU_GPU_TUNING_CACHE set, a second run reuses the first run's choice
without timing anything).

Every case prints one JSON line: the case, its sizes, the tuning and the
milliseconds per call (CUDA events on the context's stream, after one
warm-up call).
Nothing here reads files; meshes, textures and cameras are generated.
"""
import argparse
import ctypes as C
import json

import numpy as np

from . import capi, scenes
from .rasterizer import Context, RendererCpuOption


def _option():
    return RendererCpuOption(diffuse_color=1, interp=1, shading_normal=1, diffuse_shading=0,
                             backface_culling=True)


def _device_views(torch, cams, outputs, slot=0):
    dtypes = {"color": (3, torch.uint8), "depth": (0, torch.float32),
              "normal": (3, torch.float32), "mask": (0, torch.uint8),
              "face_id": (0, torch.int32), "color_f32": (3, torch.float32)}
    tensors, views = [], []
    for cam in cams:
        t = {}
        for k in outputs:
            ch, dt = dtypes[k]
            shape = (cam.height, cam.width, ch) if ch else (cam.height, cam.width)
            t[k] = torch.zeros(shape, dtype=dt, device="cuda")
        v = capi.View()
        v.mesh = slot
        v.camera = capi.camera_struct(cam)
        for k, x in t.items():
            setattr(v.images, k, x.data_ptr())
        tensors.append(t)
        views.append(v)
    return tensors, views


class _Case:
    """A context with a stream of its own and the callable to time."""

    def __init__(self, torch):
        self.torch = torch
        self.ctx = Context(0)
        self.stream = torch.cuda.Stream()
        self.ctx.check(self.ctx.set_stream(self.stream.cuda_stream))
        self.keep = []
        self.info = {}
        self.autotune = False

    def time(self, fn, repeat):
        torch = self.torch
        fn()
        self.ctx.check(self.ctx.synchronize())
        ms = []
        for _ in range(repeat):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(self.stream)
            fn()
            b.record(self.stream)
            self.ctx.check(self.ctx.synchronize())
            b.synchronize()
            ms.append(a.elapsed_time(b))
        return ms


def _ring(c, views):
    m, cams = scenes.scene_ring_batch(views)
    c.ctx.check(c.ctx.set_mesh(0, m))
    c.ctx.check(c.ctx.set_option(_option()))
    c.info.update(views=len(cams), pixels=sum(x.width * x.height for x in cams),
                  faces=m.num_faces)
    return m, cams


def case_tiled(c, views):
    _, cams = _ring(c, views)
    t, v = _device_views(c.torch, cams, ("color", "depth", "normal", "mask", "face_id"))
    if c.autotune:
        c.ctx.autotune(v)
    plan = c.ctx.plan_create(v, capi.DEVICE_POINTERS)
    c.keep += [t, plan]
    return lambda: c.ctx.check(plan.launch())


def case_global(c, views):
    _, cams = _ring(c, views)
    tu = c.ctx.tuning()
    tu.path = capi.PATH_GLOBAL
    tu.tile_log2 = 4
    c.ctx.check(c.ctx.set_tuning(tu))
    t, v = _device_views(c.torch, cams, ("color", "depth", "normal", "mask", "face_id"))
    if c.autotune:
        c.ctx.autotune(v)
    c.keep.append(t)
    return lambda: c.ctx.check(c.ctx.render_views(v, capi.DEVICE_POINTERS))


def case_noalloc(c, views):
    m, cam = scenes.scene_icosphere_single_view()
    c.ctx.check(c.ctx.set_mesh(0, m))
    c.info.update(views=1, pixels=cam.width * cam.height, faces=m.num_faces)
    dm = c.ctx.device_mesh(0)
    o = _option().to_struct()
    cs = capi.camera_struct(cam)
    t, v = _device_views(c.torch, [cam], ("color", "depth", "normal", "mask", "face_id"))
    c.keep += [t, dm, o, cs]
    lib = capi.load()

    def run():
        rc = lib.ugu_gpu_render_noalloc(C.byref(dm), C.byref(o), C.byref(cs),
                                        C.byref(v[0].images), C.c_void_p(c.stream.cuda_stream))
        if rc != capi.OK:
            raise RuntimeError(lib.ugu_gpu_last_error(None))
    return run


def _rendered(c, views, outputs):
    _, cams = _ring(c, views)
    t, v = _device_views(c.torch, cams, outputs)
    c.ctx.check(c.ctx.render_views(v, capi.DEVICE_POINTERS))
    c.keep.append(t)
    return cams, t


def case_visualize(c, views):
    cams, t = _rendered(c, views, ("depth", "normal", "face_id"))
    items = []
    for cam, x in zip(cams, t):
        H, W = cam.height, cam.width
        out = {"vis_depth": c.torch.zeros((H, W, 3), dtype=c.torch.uint8, device="cuda"),
               "depth_u16": c.torch.zeros((H, W), dtype=c.torch.int16, device="cuda"),
               "vis_normal": c.torch.zeros((H, W, 3), dtype=c.torch.uint8, device="cuda"),
               "vis_face_id": c.torch.zeros((H, W, 3), dtype=c.torch.uint8, device="cuda")}
        it = capi.Vis()
        it.width, it.height, it.min_d, it.max_d, it.gl_coord = W, H, 1.0, 5.0, 0
        it.depth, it.normal, it.face_id = (x["depth"].data_ptr(), x["normal"].data_ptr(),
                                           x["face_id"].data_ptr())
        for k, y in out.items():
            setattr(it, k, y.data_ptr())
        c.keep.append(out)
        items.append(it)
    return lambda: c.ctx.check(c.ctx.visualize(items, capi.DEVICE_POINTERS))


def case_gbuffer(c, views):
    cams, t = _rendered(c, views, ("face_id",))
    gv = []
    for cam, x in zip(cams, t):
        H, W = cam.height, cam.width
        out = {k: c.torch.zeros((H, W, 3), device="cuda") for k in capi.GBUFFER}
        out["stencil"] = c.torch.zeros((H, W), dtype=c.torch.uint8, device="cuda")
        v = capi.GBufferView()
        v.mesh = 0
        v.camera = capi.camera_struct(cam)
        v.face_id = x["face_id"].data_ptr()
        for k, y in out.items():
            setattr(v, k, y.data_ptr())
        c.keep.append(out)
        gv.append(v)
    return lambda: c.ctx.check(c.ctx.render_gbuffer(gv, capi.DEVICE_POINTERS))


def _keyframes(c, views, subdiv=6):
    """Keyframes rendered on the GPU (colour, depth, mask) around the mesh."""
    m = scenes.icosphere_textured(subdiv, 2048)
    cams = scenes.ring_cameras(views, 3.0, [(1280, 720)] * views, height=0.4)
    c.ctx.check(c.ctx.set_mesh(0, m))
    c.ctx.check(c.ctx.set_option(_option()))
    frames = []
    for cam in cams:
        H, W = cam.height, cam.width
        out = {"color": np.zeros((H, W, 3), np.uint8), "depth": np.zeros((H, W), np.float32),
               "mask": np.zeros((H, W), np.uint8)}
        im = capi.Images()
        for k, a in out.items():
            setattr(im, k, a.ctypes.data)
        c.ctx.check(c.ctx.render(0, cam, im))
        frames.append((cam, out))
    c.info.update(keyframes=views, pixels=sum(x.width * x.height for x in cams),
                  vertices=m.num_vertices, faces=m.num_faces)
    return m, frames


def _kf_descs(frames, with_w2c=True):
    descs = []
    for k, (cam, im) in enumerate(frames):
        d = capi.KeyframeDesc()
        d.id = k
        d.camera = capi.camera_struct(cam)
        if with_w2c:
            d.w2c_linear[:] = [float(x) for x in capi.w2c_linear(cam).reshape(-1)]
        d.color = im["color"].ctypes.data
        d.depth = im["depth"].ctypes.data
        d.mask = im["mask"].ctypes.data
        descs.append(d)
    return descs


def case_visibility(c, views):
    from .visibility import VisibilityTesterOption
    m, frames = _keyframes(c, views)
    descs = _kf_descs(frames)
    K, n = len(descs), m.num_vertices
    res = {"visible": np.zeros((K, n), np.uint8), "projected_pos": np.zeros((K, n, 2), np.float32),
           "viewing_angle": np.zeros((K, n), np.float32), "distance": np.zeros((K, n), np.float32),
           "color": np.zeros((K, n, 3), np.float32), "intensity": np.zeros((K, n), np.float32)}
    out = capi.VisibilityOut(*[res[k].ctypes.data for k in
                               ("visible", "projected_pos", "viewing_angle", "distance", "color",
                                "intensity")])
    opt = VisibilityTesterOption().to_struct()
    c.keep += [frames, res, out, opt, descs]
    return lambda: c.ctx.check(c.ctx.test_visibility(0, m.normals, descs, opt, False, out))


def case_texmap(c, views):
    m, frames = _keyframes(c, views)
    descs = _kf_descs(frames, with_w2c=False)
    # each face textured from the keyframe it faces most directly, its
    # triangle projected there (the best-keyframe choice is host work)
    F = m.num_faces
    cen = m.vertices[m.vertex_indices].mean(axis=1)
    pos = np.array([np.asarray(cam.c2w)[:3, 3] for cam, _ in frames])
    face_kf = np.argmin(((cen[:, None, :] - pos[None, :, :]) ** 2).sum(-1), axis=1).astype(np.int32)
    face_tri = np.zeros((F, 3, 2), np.float32)
    for k, (cam, _) in enumerate(frames):
        sel = face_kf == k
        pts = m.vertices[m.vertex_indices[sel]].reshape(-1, 3).astype(np.float64)
        pc = pts @ cam.w2c_R.astype(np.float64).T + cam.w2c_t
        u = cam.fx * pc[:, 0] / pc[:, 2] + cam.cx
        v = cam.fy * pc[:, 1] / pc[:, 2] + cam.cy
        face_tri[sel] = np.stack([u, v], -1).reshape(-1, 3, 2).astype(np.float32)
    from .visibility import TextureMappingOption
    opt = TextureMappingOption(tex_w=2048, tex_h=2048)
    o = capi.TextureOption()
    o.tex_w, o.tex_h, o.padding_kernel = opt.tex_w, opt.tex_h, opt.padding_kernel
    tex = np.zeros((opt.tex_h, opt.tex_w, 3), np.uint8)
    mask = np.zeros((opt.tex_h, opt.tex_w), np.uint8)
    c.keep += [frames, descs, face_kf, face_tri, tex, mask, o]
    c.info.update(texture=[opt.tex_w, opt.tex_h])
    return lambda: c.ctx.check(c.ctx.texture_mapping(0, descs, face_kf, face_tri, o, tex, mask))


def case_backward(c, views):
    m, _, cams = scenes.scene_texdescent(views, subdiv=7, tex_size=2048)
    cams = scenes.ring_cameras(views, 3.0, [(640, 480)] * views)
    c.ctx.check(c.ctx.set_mesh(0, m))
    c.ctx.check(c.ctx.set_option(_option()))
    fw, v = _device_views(c.torch, cams, ("face_id", "color_f32"))
    c.ctx.check(c.ctx.render_views(v, capi.DEVICE_POINTERS))
    targets = [c.torch.rand_like(x["color_f32"]) * 255.0 for x in fw]
    gt = c.torch.zeros(m.textures_f32[0].size, dtype=c.torch.float32, device="cuda")
    gp = c.torch.zeros(3 * m.num_vertices, dtype=c.torch.float32, device="cuda")
    loss = c.torch.zeros(len(cams), dtype=c.torch.float32, device="cuda")
    c.keep += [fw, targets, gt, gp, loss]
    c.info.update(views=len(cams), pixels=sum(x.width * x.height for x in cams),
                  faces=m.num_faces)
    return lambda: c.ctx.check(c.ctx.backward(v, [x.data_ptr() for x in targets], gt.data_ptr(),
                                              None, gp.data_ptr(), loss.data_ptr()))


def case_raytrace(c, views):
    _, cams = _ring(c, views)
    t, v = _device_views(c.torch, cams, ("color", "depth", "normal", "mask", "face_id"))
    c.keep.append(t)
    return lambda: c.ctx.check(c.ctx.render_views(v, capi.DEVICE_POINTERS | capi.RAYTRACE))


CASES = {"tiled": (case_tiled, 16), "global": (case_global, 16), "noalloc": (case_noalloc, 1),
         "visualize": (case_visualize, 16), "gbuffer": (case_gbuffer, 16),
         "visibility": (case_visibility, 8), "texmap": (case_texmap, 8),
         "backward": (case_backward, 8), "raytrace": (case_raytrace, 8)}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--case", choices=sorted(CASES), required=True)
    ap.add_argument("--views", type=int, default=0, help="views or keyframes (0: the case's own)")
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--tuning", default="", help="ugu_gpu_tuning fields, e.g. "
                    "tile_log2=5,small_view_pixels=307200,split_class=256")
    ap.add_argument("--autotune", action="store_true")
    a = ap.parse_args(argv)
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("kernel_cases needs a CUDA device")
    fn, default_views = CASES[a.case]
    c = _Case(torch)
    try:
        if a.tuning:
            tu = c.ctx.tuning()
            for kv in a.tuning.split(","):
                k, v = kv.split("=")
                if k not in dict(capi.Tuning._fields_):
                    raise SystemExit(f"unknown tuning field {k}")
                setattr(tu, k, int(v))
            c.ctx.check(c.ctx.set_tuning(tu))
        c.autotune = a.autotune
        step = fn(c, a.views or default_views)
        tu = c.ctx.tuning()
        c.info["tuning"] = {k: getattr(tu, k) for k, _ in capi.Tuning._fields_}
        ms = c.time(step, a.repeat)
        print(json.dumps({"case": a.case, **c.info, "repeat": a.repeat,
                          "ms_per_call": sorted(ms)[len(ms) // 2], "ms": ms}), flush=True)
    finally:
        c.keep.clear()
        c.ctx.close()


if __name__ == "__main__":
    main()
