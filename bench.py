#!/usr/bin/env python
"""Benchmark of the GB300 rasterizer (one JSON line on rank 0).

Workload (the batched-forward configuration): an icosphere subdivided 7 times
(163,842 vertices / 327,680 faces, radial noise sigma 0.01), a 2048x2048 RGB8
texture, seen by 64 cameras on a radius-3 ring at resolutions drawn from
{320x240, 640x480, 1280x720, 1920x1080} (54,067,200 px in total), fx = 0.8 W.
Outputs per view: RGB8 bilinear-textured colour, float depth, float normal,
uint8 mask, int32 face_id.  A step renders all 64 views in one graph-captured
batched launch sequence.

  value    views/s of the batched render, inputs resident in HBM, device
           timed with CUDA events per step, L2 flushed between steps
  e2e      the same views through ugu_gpu_render_views with pinned HOST
           buffers: per step the camera table goes host->device and all
           output images come back device->host inside the timed region
  per_view 64 separate per-view launch sequences (no graph), same outputs

--impl reference times the reference algorithm's CPU implementation (the
oracle restatement, all host threads) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_VIEWS = 64
BYTES_PER_PX = 24  # depth 4 + normal 12 + colour 3 + mask 1 + face_id 4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-per-view", action="store_true")
    ap.add_argument("--views", type=int, default=N_VIEWS)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-backward", action="store_true")
    ap.add_argument("--workload", default="ring64",
                    choices=["ring64", "uvsphere", "single1080", "texdescent256", "raytrace64"],
                    help="ring64 (default): the batched-forward workload; the others "
                         "measure the single-view and large fwd+bwd configurations, and "
                         "the ring64 views through the raytracer")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for n, v in zip(names, r[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(value: float, world: int) -> float:
    """The slowest rank's per-step time (the contract's max over ranks)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_views_per_s(n_views: int, ms_step_max: float, world: int) -> float:
    """Replicas only: every rank renders the whole batch of views, so the
    job renders world * n_views views per (slowest) step."""
    return world * n_views / (ms_step_max / 1e3)


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic():
    """Per-launch DRAM bytes of the tile kernel from an ncu capture, as
    summarised in profiles/k_tile_traffic.txt (null when absent)."""
    p = os.path.join(ROOT, "profiles", "k_tile_traffic.txt")
    try:
        with open(p) as f:
            for line in f:
                if line.strip().startswith("k_tile_dram_bytes_per_launch:"):
                    return int(line.split(":", 1)[1])
    except Exception:
        pass
    return None


def workload(n_views):
    from ugu_gb300 import scenes
    m, cams = scenes.scene_ring_batch(n_views)
    return m, cams


def option():
    from ugu_gb300.rasterizer import RendererCpuOption
    return RendererCpuOption(diffuse_color=1, interp=1, shading_normal=1, diffuse_shading=0,
                             backface_culling=True)


def algorithmic_bytes(m, cams):
    px = sum(c.width * c.height for c in cams)
    V, F = m.num_vertices, m.num_faces
    geometry = V * (12 + 12) + m.uv.shape[0] * 8 + F * (12 + 12 + 12 + 12) + F * 4
    texture = sum(t.size for t in m.textures)
    return px * BYTES_PER_PX + geometry + texture, px


def cpu_oracle_views_per_s(m, cams, threads, max_views=None):
    """Times the oracle port on `threads` host threads over the views."""
    import concurrent.futures as cf

    import oracle
    oracle.build()
    opt = option()
    views = cams if max_views is None else cams[:max_views]

    def one(c):
        rc, _, _ = oracle.render(m, c, opt)
        assert rc == 0
        return c.width * c.height

    t0 = time.perf_counter()
    if threads == 1:
        px = sum(one(c) for c in views)
    else:
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            px = sum(ex.map(one, views))
    dt = time.perf_counter() - t0
    return len(views) / dt, px / dt / 1e9, dt, len(views)


def measure_fwd_bwd(ctx, torch, dev, stream, flush, timed, args, n_views=16, size=(640, 480)):
    import numpy as np

    from ugu_gb300 import capi, scenes
    m = scenes.icosphere_textured(7, 2048, f32=True)
    t = m.copy()
    t.textures = [scenes.random_u8(5, m.textures[0].shape)]
    t.textures_f32 = [t.textures[0].astype(np.float32)]
    r = np.sqrt((t.vertices.astype(np.float64) ** 2).sum(axis=1))
    t.vertices = (t.vertices * (1.0 + 0.005 * scenes.normal(6, t.num_vertices) / r)[:, None]
                  ).astype(np.float32)
    cams = scenes.ring_cameras(n_views, 3.0, [size] * n_views)
    ctx.check(ctx.set_mesh(1, m))
    ctx.check(ctx.set_mesh(2, t))

    def views_for(slot, outs):
        tensors, views = [], []
        for c in cams:
            tt = {k: torch.empty((c.height, c.width) + ((3,) if k == "color_f32" else ()),
                                 dtype=torch.float32 if k == "color_f32" else torch.int32,
                                 device=dev) for k in outs}
            v = capi.View()
            v.mesh = slot
            v.camera = capi.camera_struct(c)
            for k, x in tt.items():
                setattr(v.images, k, x.data_ptr())
            tensors.append(tt)
            views.append(v)
        return tensors, views

    tgt, tviews = views_for(2, ("color_f32",))
    ctx.check(ctx.render_views(tviews, capi.DEVICE_POINTERS))
    fw, fviews = views_for(1, ("face_id", "color_f32"))
    plan = ctx.plan_create(fviews, capi.DEVICE_POINTERS)
    gtex = torch.zeros(m.textures_f32[0].size, dtype=torch.float32, device=dev)
    gpos = torch.zeros(3 * m.num_vertices, dtype=torch.float32, device=dev)
    loss = torch.zeros(n_views, dtype=torch.float32, device=dev)
    tptr = [x["color_f32"].data_ptr() for x in tgt]

    def step():
        ctx.check(plan.launch())
        ctx.check(ctx.backward(fviews, tptr, gtex.data_ptr(), None, gpos.data_ptr(),
                               loss.data_ptr(), capi.DEVICE_POINTERS | capi.ASYNC))

    for _ in range(3):
        step()
    ctx.check(ctx.synchronize())
    ms = timed(step, max(3, args.steps))
    ctx.check(ctx.synchronize())
    plan.close()
    ms_step = sum(ms) / len(ms)
    return {"views_per_s": n_views / (ms_step / 1e3), "ms_per_step": ms_step,
            "workload": f"icosphere7_tex2048_f32_{n_views}x{size[0]}x{size[1]}",
            "grads": "texels + vertex positions"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    m, cams = workload(args.views)
    threads = os.cpu_count() or 1
    import concurrent.futures as cf

    import oracle
    oracle.build()
    opt = option()
    # each step renders a bounded sample of the 64 views (round robin)
    per_step = max(threads, 8)
    order = sorted(range(len(cams)), key=lambda i: i)

    def one(i):
        rc, _, _ = oracle.render(m, cams[i], opt)
        assert rc == 0
        return cams[i].width * cams[i].height

    pos = 0
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for _ in range(args.warmup):
            list(ex.map(one, [order[(pos + k) % len(order)] for k in range(2)]))
        times, views, pix = [], 0, 0
        for _ in range(args.steps):
            sel = [order[(pos + k) % len(order)] for k in range(per_step)]
            pos += per_step
            t0 = time.perf_counter()
            pix += sum(ex.map(one, sel))
            times.append(time.perf_counter() - t0)
            views += len(sel)
    total = sum(times)
    v = views / total
    line = {
        "impl": "reference", "metric": "views/s", "value": v, "unit": "views/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "ring64_icosphere7_tex2048_bilinear", "views": len(cams),
                   "pixels": sum(c.width * c.height for c in cams)},
        "gpix_per_s": pix / total / 1e9,
        "cpu_baseline": {"value": v, "unit": "views/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step} of the 64 views per step, round robin, "
                                   f"{threads} host threads, oracle restatement of "
                                   f"Rasterizer::Render (-O2 -ffp-contract=off)"},
        "e2e": {"value": v, "unit": "views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_single(args, which):
    """One view per step through the C ABI (device outputs, graph replay):
    the UV-sphere vertex-colour view at 640x480 or the textured icosphere-7
    view at 1920x1080; the oracle on one host core beside it."""
    import torch

    from ugu_gb300 import capi, scenes
    from ugu_gb300.rasterizer import Context, RendererCpuOption
    if which == "uvsphere":
        m, cam = scenes.scene_uv_sphere_vertex_color()
        opt = RendererCpuOption(diffuse_color=2, interp=1, shading_normal=1, backface_culling=True)
    else:
        m, cam = scenes.scene_icosphere_single_view()
        opt = option()
    ctx = Context(0)
    ctx.check(ctx.set_mesh(0, m))
    ctx.check(ctx.set_option(opt))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.check(ctx.set_stream(stream.cuda_stream))
    H, W = cam.height, cam.width
    t = {"color": torch.empty((H, W, 3), dtype=torch.uint8, device="cuda"),
         "depth": torch.empty((H, W), dtype=torch.float32, device="cuda"),
         "normal": torch.empty((H, W, 3), dtype=torch.float32, device="cuda"),
         "mask": torch.empty((H, W), dtype=torch.uint8, device="cuda"),
         "face_id": torch.empty((H, W), dtype=torch.int32, device="cuda")}
    v = capi.View()
    v.mesh = 0
    v.camera = capi.camera_struct(cam)
    for k, x in t.items():
        setattr(v.images, k, x.data_ptr())
    tuned = ctx.autotune([v])
    plan = ctx.plan_create([v], capi.DEVICE_POINTERS)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(max(3, args.warmup)):
        ctx.check(plan.launch())
    ctx.check(ctx.synchronize())
    ev = []
    for _ in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.check(plan.launch())
        b.record(stream)
        ev.append((a, b))
    ctx.check(ctx.synchronize())
    ms = sum(a.elapsed_time(b) for a, b in ev) / len(ev)
    import oracle
    oracle.build()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        rc, _, _ = oracle.render(m, cam, opt)
    cpu = reps / (time.perf_counter() - t0)
    print(json.dumps({"metric": "views/s", "value": 1e3 / ms, "unit": "views/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                      "gpix_per_s": W * H / (ms / 1e3) / 1e9,
                      "config": {"workload": which, "pixels": W * H, "faces": m.num_faces,
                                 "tuning": {"path": ["tiled", "global"][tuned.path],
                                            "tile": 1 << tuned.tile_log2}},
                      "cpu_baseline": {"value": cpu, "unit": "views/s", "cores": 1,
                                       "kind": "port"}}), flush=True)


class _DeviceArray:
    """A device buffer as __cuda_array_interface__ (zero-copy for torch)."""

    def __init__(self, ptr, shape, typestr="<f4"):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3}


def run_texdescent(args, n_views=256, iters=20, lr=0.1):
    """The large forward+backward: icosphere-8 (1,310,720 faces, radial noise
    0.01), a 4096^2 float texture, 256 Fibonacci-sphere cameras at distance
    3, 1280x720, fx = 1000; 20 iterations of texture gradient descent
    (texel -= 0.1 * dL/dtexel with L the per-view L2 sum averaged over the
    views), each a batched forward (face_id + float
    colour) and a backward against fixed target images (a second seeded
    texture).  The texels are updated in place in the mesh slot's device
    copy (ugu_gpu_get_device_mesh)."""
    import numpy as np
    import torch

    from ugu_gb300 import capi, scenes
    from ugu_gb300.rasterizer import Context, RendererCpuOption
    t_setup = time.perf_counter()
    m = scenes.icosphere(8, 1.0, 0.01, seed=1)
    scenes.calc_normals(m)
    scenes.with_texture(m, 4096, seed=3, f32=True)
    # float texels in [0, 1], as multi-view texturing optimises them (a step
    # of 0.1 on 0..255 values overshoots and diverges)
    m.textures_f32 = [m.textures_f32[0] / np.float32(255.0)]
    tm = m.copy()
    tm.textures = [scenes.random_u8(5, m.textures[0].shape)]
    tm.textures_f32 = [tm.textures[0].astype(np.float32) / np.float32(255.0)]
    cams = scenes.fibonacci_cameras(n_views, 3.0, 1280, 720, 1000.0)
    ctx = Context(0)
    ctx.check(ctx.set_option(RendererCpuOption(diffuse_color=1, interp=1, shading_normal=1,
                                               backface_culling=True)))
    ctx.check(ctx.set_mesh(0, m))
    ctx.check(ctx.set_mesh(1, tm))
    dev = torch.device("cuda")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.check(ctx.set_stream(stream.cuda_stream))

    def views_for(slot, outs):
        tensors, views = [], []
        for c in cams:
            tt = {k: torch.empty((c.height, c.width) + ((3,) if k == "color_f32" else ()),
                                 dtype=torch.float32 if k == "color_f32" else torch.int32,
                                 device=dev) for k in outs}
            v = capi.View()
            v.mesh = slot
            v.camera = capi.camera_struct(c)
            for k, x in tt.items():
                setattr(v.images, k, x.data_ptr())
            tensors.append(tt)
            views.append(v)
        return tensors, views

    tgt, tviews = views_for(1, ("color_f32",))
    ctx.check(ctx.render_views(tviews, capi.DEVICE_POINTERS))
    dm = ctx.device_mesh(0)
    tex = torch.as_tensor(_DeviceArray(dm.textures[0].rgb_f32, m.textures_f32[0].shape),
                          device=dev)
    grad = torch.zeros_like(tex)
    loss = torch.zeros(n_views, dtype=torch.float32, device=dev)
    fw, fviews = views_for(0, ("face_id", "color_f32"))
    plan = ctx.plan_create(fviews, capi.DEVICE_POINTERS)
    tptr = [x["color_f32"].data_ptr() for x in tgt]
    setup_s = time.perf_counter() - t_setup
    # warm-up iterations run every kernel of a step (the first use of each
    # loads its module) and leave the texels unchanged
    warm = max(3, args.warmup)
    for _ in range(warm):
        ctx.check(plan.launch())
        grad.zero_()
        loss.zero_()
        ctx.check(ctx.backward(fviews, tptr, grad.data_ptr(), None, None, loss.data_ptr(),
                               capi.DEVICE_POINTERS | capi.ASYNC))
        tex.add_(grad, alpha=0.0)
        loss.sum() / n_views
    ctx.check(ctx.synchronize())
    losses = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for it in range(iters):
        ctx.check(plan.launch())
        grad.zero_()
        loss.zero_()
        ctx.check(ctx.backward(fviews, tptr, grad.data_ptr(), None, None, loss.data_ptr(),
                               capi.DEVICE_POINTERS | capi.ASYNC))
        # L = mean over views of the per-pixel L2 sum: dL/dtexel = grad / n_views
        tex.add_(grad, alpha=-lr / n_views)
        losses.append(loss.sum() / n_views)
    e1.record(stream)
    ctx.check(ctx.synchronize())
    ms = e0.elapsed_time(e1)
    losses = [float(x) for x in losses]
    px = sum(c.width * c.height for c in cams)
    plan.close()
    ctx.close()
    print(json.dumps({
        "metric": "views/s (forward+backward)", "value": iters * n_views / (ms / 1e3),
        "unit": "views/s", "n_gpus": 1, "steps": iters, "warmup": warm,
        "ms_per_step": ms / iters, "gpix_per_s": iters * px / (ms / 1e3) / 1e9,
        "config": {"workload": "texdescent256_icosphere8_tex4096_f32_1280x720",
                   "views": n_views, "iterations": iters, "lr": lr, "faces": m.num_faces,
                   "texels": "float32 in [0, 1]"},
        "loss_first": losses[0], "loss_last": losses[-1], "setup_s": setup_s}), flush=True)


def run_raytrace(args):
    """The ring64 views (icosphere-7, 2048^2 texture, 64 views, 54.1 Mpx)
    through the raytracer (UGU_GPU_RAYTRACE: ugu::Raytracer's naive BVH and
    double-precision ray hits), one captured plan replay per step; the
    oracle's raytracer on a bounded sample beside it."""
    import torch

    from ugu_gb300 import build as b
    from ugu_gb300 import capi, scenes
    from ugu_gb300.rasterizer import Context
    b.build()
    m, cams = workload(args.views)
    total_px = sum(c.width * c.height for c in cams)
    ctx = Context(0)
    ctx.check(ctx.set_mesh(0, m))
    ctx.check(ctx.set_option(option()))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.check(ctx.set_stream(stream.cuda_stream))
    outs, views = [], []
    for c in cams:
        H, W = c.height, c.width
        t = {"color": torch.empty((H, W, 3), dtype=torch.uint8, device="cuda"),
             "depth": torch.empty((H, W), dtype=torch.float32, device="cuda"),
             "normal": torch.empty((H, W, 3), dtype=torch.float32, device="cuda"),
             "mask": torch.empty((H, W), dtype=torch.uint8, device="cuda"),
             "face_id": torch.empty((H, W), dtype=torch.int32, device="cuda")}
        v = capi.View()
        v.mesh = 0
        v.camera = capi.camera_struct(c)
        for k, x in t.items():
            setattr(v.images, k, x.data_ptr())
        outs.append(t)
        views.append(v)
    t0 = time.perf_counter()
    plan = ctx.plan_create(views, capi.DEVICE_POINTERS | capi.RAYTRACE)  # builds the BVH
    bvh_s = time.perf_counter() - t0
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(max(3, args.warmup)):
        ctx.check(plan.launch())
    ctx.check(ctx.synchronize())
    ev = []
    sampler = ClockSampler(0)
    sampler.start()
    for _ in range(args.steps):
        flush.zero_()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.check(plan.launch())
        e.record(stream)
        ev.append((a, e))
    ctx.check(ctx.synchronize())
    clocks = sampler.stop()
    ms = sum(a.elapsed_time(e) for a, e in ev) / len(ev)
    plan.close()
    cpu = None
    if not args.no_cpu_baseline:
        import oracle
        oracle.build()
        # bounded sample: the first ring camera at 160x120 (same field of view)
        c0 = cams[0]
        s = 160.0 / c0.width
        cs = scenes.camera_desc(160, int(round(c0.height * s)), c0.fx * s, c0.fy * s,
                                c0.cx * s, c0.cy * s, c0.c2w)
        t0 = time.perf_counter()
        rc, _ = oracle.raytrace(m, cs, option(), outputs=("color", "depth", "normal", "mask",
                                                          "face_id"))
        dt = time.perf_counter() - t0
        px = cs.width * cs.height
        cpu = {"value": px / dt / (total_px / len(cams)), "unit": "views/s", "cores": 1,
               "kind": "port", "sample": f"one {cs.width}x{cs.height} view of the ring "
                                         f"({px} rays), scaled to the mean view's pixels"}
    print(json.dumps({
        "metric": "views/s", "value": len(cams) / (ms / 1e3), "unit": "views/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "dtype": "f32+f64", "data": "synthetic",
        "grays_per_s": total_px / (ms / 1e3) / 1e9,
        "config": {"workload": "raytrace64_icosphere7_tex2048_bilinear", "views": len(cams),
                   "pixels": total_px, "mesh_faces": m.num_faces,
                   "renderer": "raytracer (naive BVH, double-precision hits)",
                   "l2": "flushed (256 MB write) between timed steps",
                   "bvh_build_and_plan_s": bvh_s},
        "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": 1}), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload in ("uvsphere", "single1080"):
        run_single(args, args.workload)
        return
    if args.workload == "texdescent256":
        run_texdescent(args)
        return
    if args.workload == "raytrace64":
        run_raytrace(args)
        return
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)

    from ugu_gb300 import build as b
    from ugu_gb300 import capi
    from ugu_gb300.rasterizer import Context
    b.build()

    m, cams = workload(args.views)
    alg_bytes, total_px = algorithmic_bytes(m, cams)
    ctx = Context(local)
    ctx.check(ctx.set_mesh(0, m))
    ctx.check(ctx.set_option(option()))
    # a dedicated stream: the legacy default stream cannot be graph-captured
    # and does not order against the context's non-blocking stream
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    ctx.check(ctx.set_stream(stream.cuda_stream))

    dev = torch.device("cuda", local)
    outs, views = [], []
    for c in cams:
        H, W = c.height, c.width
        t = {"color": torch.empty((H, W, 3), dtype=torch.uint8, device=dev),
             "depth": torch.empty((H, W), dtype=torch.float32, device=dev),
             "normal": torch.empty((H, W, 3), dtype=torch.float32, device=dev),
             "mask": torch.empty((H, W), dtype=torch.uint8, device=dev),
             "face_id": torch.empty((H, W), dtype=torch.int32, device=dev)}
        v = capi.View()
        v.mesh = 0
        v.camera = capi.camera_struct(c)
        for k, x in t.items():
            setattr(v.images, k, x.data_ptr())
        outs.append(t)
        views.append(v)
    tuned = ctx.autotune(views) if not args.no_autotune else ctx.tuning()
    tuning = {"path": ["tiled", "global"][tuned.path], "tile": 1 << tuned.tile_log2,
              "entry_capacity": tuned.entry_capacity}
    plan = ctx.plan_create(views, capi.DEVICE_POINTERS)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(fn, steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        barrier()
        for s, e in ev:
            flush.zero_()  # L2 flush outside the timed interval
            s.record(stream)
            fn()
            e.record(stream)
        barrier()
        return [s.elapsed_time(e) for s, e in ev]

    def step_plan():
        ctx.check(plan.launch())

    for _ in range(max(3, args.warmup)):
        step_plan()
    ctx.check(ctx.synchronize())

    clocks = ClockSampler(local)
    launches0 = ctx.stats().launches
    clocks.start()
    ms = timed(step_plan, args.steps)
    clk = clocks.stop()
    ctx.check(ctx.synchronize())
    launches = ctx.stats().launches - launches0
    ms_step = max_over_ranks(sum(ms) / len(ms), world)
    views_per_s = replica_views_per_s(len(cams), ms_step, world)

    # the dominant kernel on its own: CUDA events around each tile-kernel
    # launch of a non-graph render of the same views (UGU_GPU_TIME_KERNELS),
    # the L2 flushed before each render
    st0 = ctx.stats()
    for _ in range(max(3, min(args.steps, 10))):
        flush.zero_()
        ctx.check(ctx.render_views(views, capi.DEVICE_POINTERS | capi.TIME_KERNELS))
    st1 = ctx.stats()
    tile_ms = ((st1.tile_kernel_ms - st0.tile_kernel_ms) /
               max(1, st1.tile_kernel_launches - st0.tile_kernel_launches))

    # per-view launch sequences (no graph), same outputs
    per_view = None
    if not args.no_per_view:
        def step_pv():
            ctx.check(ctx.render_views(views, capi.DEVICE_POINTERS | capi.PER_VIEW | capi.ASYNC))
        for _ in range(2):
            step_pv()
        ctx.check(ctx.synchronize())
        pv = timed(step_pv, max(2, min(args.steps, 5)))
        ctx.check(ctx.synchronize())
        per_view = len(cams) / (sum(pv) / len(pv) / 1e3)

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        host, hviews = [], []
        d2h = 0
        for c in cams:
            H, W = c.height, c.width
            t = {"color": torch.empty((H, W, 3), dtype=torch.uint8).pin_memory(),
                 "depth": torch.empty((H, W), dtype=torch.float32).pin_memory(),
                 "normal": torch.empty((H, W, 3), dtype=torch.float32).pin_memory(),
                 "mask": torch.empty((H, W), dtype=torch.uint8).pin_memory(),
                 "face_id": torch.empty((H, W), dtype=torch.int32).pin_memory()}
            v = capi.View()
            v.mesh = 0
            v.camera = capi.camera_struct(c)
            for k, x in t.items():
                setattr(v.images, k, x.data_ptr())
                d2h += x.numel() * x.element_size()
            host.append(t)
            hviews.append(v)
        ctx.check(ctx.render_views(hviews, 0))
        e2e_steps = max(2, min(args.steps, 5))
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ctx.check(ctx.render_views(hviews, 0))
        barrier()
        dt = (time.perf_counter() - t0) / e2e_steps
        h2d = len(cams) * 256  # the per-view descriptor table (DevView, 248 B padded)
        e2e = {"value": world * len(cams) / dt, "unit": "views/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h + 32 * 64}

    # forward + backward: 16 ring views at 640x480 of the same mesh with float
    # texels; a step is one graph-replayed forward (face_id + float colour)
    # and one backward of the per-pixel L2 loss against fixed targets.
    fwd_bwd = None
    if not args.no_backward:
        fwd_bwd = measure_fwd_bwd(ctx, torch, dev, stream, flush, timed, args)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        vps, gps, dt, nv = cpu_oracle_views_per_s(m, cams, threads)
        cpu = {"value": vps, "unit": "views/s", "cores": threads, "kind": "port",
               "sample": f"all {nv} views once on {threads} host threads ({dt:.1f} s wall), "
                         "oracle restatement of Rasterizer::Render (-O2 -ffp-contract=off)"}

    peak, peak_kind = measured_peak_hbm()
    # the tile kernel writes every output byte (24 B/px) and reads the
    # texture and the geometry: the step's algorithmic bytes
    achieved = alg_bytes / (tile_ms / 1e3) / 1e9
    step_achieved = alg_bytes / (ms_step / 1e3) / 1e9
    line = {
        "metric": "views/s", "value": views_per_s, "unit": "views/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "ring64_icosphere7_tex2048_bilinear", "views": len(cams),
                   "pixels": total_px, "mesh_faces": m.num_faces, "mesh_vertices": m.num_vertices,
                   "texture": "2048x2048 RGB8", "outputs": "color,depth,normal,mask,face_id",
                   "l2": "flushed (256 MB write) between timed steps",
                   "launch": "one CUDA-graph replay of the batched render per step",
                   "tuning": tuning},
        "gpix_per_s": world * total_px / (ms_step / 1e3) / 1e9,
        "per_view_views_per_s": per_view,
        "batched_over_per_view": (views_per_s / world / per_view) if per_view else None,
        "fwd_bwd": fwd_bwd,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": committed_traffic(),
                     "peak_source": peak_kind, "kernel": "k_tile",
                     "kernel_ms": tile_ms, "algorithmic_bytes": alg_bytes,
                     "step_achieved": step_achieved, "step_frac": step_achieved / peak},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    plan.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
