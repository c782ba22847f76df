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
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-per-view", action="store_true")
    ap.add_argument("--views", type=int, default=N_VIEWS)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-backward", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the bit-for-bit check of the timed replay against the oracle")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the single-view and texture-descent configurations")
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
        """Starts sampling every 20 ms and returns once the first sample is in
        (at most 3 s), so that the timed region that follows is covered."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.rows and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
            time.sleep(0.005)
        self.first = len(self.rows)

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
        # the rows taken while the timed region ran (the first one, taken
        # before it started, only when nothing later came in)
        rows = self.rows[getattr(self, "first", 0):] or self.rows
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
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


# The sources the tile kernel is compiled from: a committed ncu figure is
# used only while their content hash equals the one it was measured on.
TILE_SOURCES = ("tile.cu", "tilecommon.cuh", "shade.cuh", "span.cuh", "exact.cuh", "internal.cuh")


def tile_source_hash():
    import hashlib
    h = hashlib.sha256()
    for name in TILE_SOURCES:
        with open(os.path.join(ROOT, "ugu_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def committed_tile_profile():
    """Per-launch DRAM bytes and warp instructions of the tile kernel on the
    64-view workload, from the ncu capture summarised in
    profiles/k_tile_traffic.txt, and whether that capture measured the
    current sources (a stale figure is reported as null)."""
    p = os.path.join(ROOT, "profiles", "k_tile_traffic.txt")
    vals = {}
    try:
        with open(p) as f:
            for line in f:
                k, sep, v = line.strip().partition(":")
                if sep and k in ("k_tile_dram_bytes_per_launch", "k_tile_warp_instructions_per_launch",
                                 "tile_sources_sha256_16"):
                    vals[k] = v.strip()
    except Exception:
        return None, None, "absent"
    if vals.get("tile_sources_sha256_16") != tile_source_hash():
        return None, None, "stale (tile kernel sources changed since the capture)"
    tr = vals.get("k_tile_dram_bytes_per_launch")
    ins = vals.get("k_tile_warp_instructions_per_launch")
    return (int(tr) if tr else None), (int(ins) if ins else None), "current"


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


def ring_config(m, cams):
    """The workload's `config`, identical in both arms."""
    return {"workload": "ring64_icosphere7_tex2048_bilinear", "views": len(cams),
            "pixels": sum(c.width * c.height for c in cams), "mesh_faces": m.num_faces,
            "mesh_vertices": m.num_vertices, "texture": "2048x2048 RGB8",
            "outputs": "color,depth,normal,mask,face_id",
            "l2": "outputs (1.30 GB) exceed L2; the GPU arm also flushes L2 (256 MB write) "
                  "between timed steps"}


OUT_KEYS = ("color", "depth", "normal", "mask", "face_id")


def oracle_all_views(m, cams, threads, keep=False):
    """Renders every view once with the oracle port on `threads` host
    threads, largest views first; returns (seconds, outputs or None)."""
    import concurrent.futures as cf

    import oracle
    oracle.build()
    opt = option()
    order = sorted(range(len(cams)), key=lambda i: -cams[i].width * cams[i].height)
    res = [None] * len(cams)

    def one(i):
        rc, out, _ = oracle.render(m, cams[i], opt)
        assert rc == 0
        if keep:
            res[i] = {k: out[k] for k in OUT_KEYS}

    t0 = time.perf_counter()
    if threads == 1:
        for i in order:
            one(i)
    else:
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(one, order))
    return time.perf_counter() - t0, (res if keep else None)


def fp64_errors(m, cams, outs, threads):
    """The largest error of the GPU's float outputs against an FP64
    recomputation of the interpolation at the GPU's own face ids (the
    oracle's interp_f64), over all views: depth relative, camera-frame
    normal absolute, and the 8-bit colour's distance from the FP64 colour
    (truncation included)."""
    import concurrent.futures as cf

    import numpy as np

    import oracle
    opt = option()

    def one(i):
        o = outs[i]
        d64, n64, c64 = oracle.interp_f64(m, cams[i], opt, o["face_id"])
        vis, shaded = o["face_id"] >= 0, o["face_id"] > 0
        dr = float(np.max(np.abs(o["depth"][vis] - d64[vis]) / d64[vis])) if vis.any() else 0.0
        na = float(np.max(np.abs(o["normal"][shaded] - n64[shaded]))) if shaded.any() else 0.0
        ca = (float(np.max(np.abs(o["color"][shaded].astype(np.float64) - c64[shaded])))
              if shaded.any() else 0.0)
        return dr, na, ca

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        errs = list(ex.map(one, range(len(cams))))
    return {"views": len(cams), "depth_max_rel": max(e[0] for e in errs),
            "normal_max_abs": max(e[1] for e in errs),
            "color_u8_max_abs": max(e[2] for e in errs),
            "against": "FP64 recomputation of the interpolation at the GPU's face ids"}


def tuning_record(tuned, autotuned):
    """The bench line's record of a ugu_gpu_tuning."""
    return {"path": ["tiled", "global"][tuned.path], "tile": 1 << tuned.tile_log2,
            "ctas_per_sm": tuned.ctas_per_sm or "occupancy limit",
            "split_class": tuned.split_class, "bin_faces_per_thread": tuned.bin_faces,
            "small_view_pixels_on_16px_tiles": tuned.small_view_pixels,
            "small_bbox_max": tuned.small_bbox_max, "group_pixels": tuned.group_pixels,
            "chosen_by": "ugu_gpu_autotune (coordinate search, timed on these views)"
            if autotuned else "defaults"}


def view_digest(outs):
    import hashlib
    h = hashlib.blake2b(digest_size=16)
    for k in OUT_KEYS:
        h.update(outs[k].tobytes())
    return h.hexdigest()


def mismatched_pixels(ref, got):
    """Pixels where any output differs from the oracle's bits."""
    import numpy as np
    bad = None
    for k in OUT_KEYS:
        a, b = ref[k], got[k]
        if a.dtype.kind == "f":
            a, b = a.view(np.uint32), b.view(np.uint32)
        d = a != b
        if d.ndim == 3:
            d = d.any(axis=2)
        bad = d if bad is None else (bad | d)
    return int(bad.sum())


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
    tuned = ctx.autotune(fviews) if not args.no_autotune else ctx.tuning()
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
            "grads": "texels + vertex positions",
            "tuning": tuning_record(tuned, not args.no_autotune)}


def run_reference(args):
    """The reference arm: the oracle restatement of Rasterizer::Render (the
    reference's own build does not travel to the Arm machine), every one of the
    workload's views rendered in each step, on all host threads, largest
    views first."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    m, cams = workload(args.views)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle_all_views(m, cams, threads)
    times = [oracle_all_views(m, cams, threads)[0] for _ in range(args.steps)]
    total = sum(times)
    v = len(cams) * args.steps / total
    px = sum(c.width * c.height for c in cams)
    line = {
        "impl": "reference", "metric": "views/s", "value": v, "unit": "views/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": ring_config(m, cams),
        "gpix_per_s": px * args.steps / total / 1e9,
        "cpu_baseline": {"value": v, "unit": "views/s", "cores": threads, "kind": "port",
                         "sample": f"all {len(cams)} views per step, largest first, on "
                                   f"{threads} host threads; oracle restatement of "
                                   f"Rasterizer::Render (-O2 -ffp-contract=off)"},
        "e2e": {"value": v, "unit": "views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def measure_single(which, steps, warmup, cpu=True):
    """One view per step through the C ABI with device outputs: the UV-sphere
    vertex-colour view at 640x480 (uvsphere) or the textured icosphere-7 view
    at 1920x1080 (single1080), as one graph replay per step and as one direct
    render call per step; the oracle on one host core beside it."""
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

    def timed(fn):
        for _ in range(max(3, warmup)):
            fn()
        ctx.check(ctx.synchronize())
        # a timed region of at least 0.3 s (one step here takes well under a
        # millisecond), so that the clock sampler sees it
        t0 = time.perf_counter()
        fn()
        ctx.check(ctx.synchronize())
        n = max(steps, int(0.3 / max(time.perf_counter() - t0, 1e-5)))
        ev = []
        for _ in range(n):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            ev.append((a, b))
        ctx.check(ctx.synchronize())
        return sum(a.elapsed_time(b) for a, b in ev) / len(ev), n

    sampler = ClockSampler(0)
    sampler.start()
    ms, n_steps = timed(lambda: ctx.check(plan.launch()))
    ctx.check(ctx.synchronize())
    replay = {k: x.cpu().numpy() for k, x in t.items()}
    ms_direct, _ = timed(lambda: ctx.check(ctx.render_views([v], capi.DEVICE_POINTERS | capi.ASYNC)))
    clocks = sampler.stop()
    ctx.check(ctx.synchronize())  # reports any asynchronous render that overflowed
    direct_same = view_digest({k: x.cpu().numpy() for k, x in t.items()}) == view_digest(replay)
    plan.close()
    ctx.close()
    cpu_line = None
    if cpu:
        import oracle
        oracle.build()
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            rc, _, _ = oracle.render(m, cam, opt)
            assert rc == 0
        cpu_line = {"value": reps / (time.perf_counter() - t0), "unit": "views/s", "cores": 1,
                    "kind": "port", "sample": f"{reps} renders of the view on one host core"}
    return {"metric": "views/s", "value": 1e3 / ms, "unit": "views/s", "n_gpus": 1,
            "steps": n_steps, "warmup": max(3, warmup), "ms_per_step": ms,
            "gpix_per_s": W * H / (ms / 1e3) / 1e9,
            "direct_call": {"views_per_s": 1e3 / ms_direct, "ms_per_step": ms_direct,
                            "gpix_per_s": W * H / (ms_direct / 1e3) / 1e9,
                            "same_images_as_replay": direct_same},
            "config": {"workload": which, "pixels": W * H, "faces": m.num_faces,
                       "launch": "one CUDA-graph replay of the one-view render per step "
                                 "(direct_call: one ugu_gpu_render_views call per step)",
                       "l2": "flushed (256 MB write) between timed steps",
                       "tuning": {"path": ["tiled", "global"][tuned.path],
                                  "tile": 1 << tuned.tile_log2}},
            "cpu_baseline": cpu_line, "clocks": clocks}


def run_single(args, which):
    print(json.dumps(measure_single(which, args.steps, args.warmup)), flush=True)


class _DeviceArray:
    """A device buffer as __cuda_array_interface__ (zero-copy for torch)."""

    def __init__(self, ptr, shape, typestr="<f4"):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3}


def measure_texdescent(warmup, n_views=256, iters=20, lr=0.1, autotune=True):
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
    m, tm, cams = scenes.scene_texdescent(n_views)
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
    tuned = ctx.autotune(fviews) if autotune else ctx.tuning()
    plan = ctx.plan_create(fviews, capi.DEVICE_POINTERS)
    tptr = [x["color_f32"].data_ptr() for x in tgt]
    setup_s = time.perf_counter() - t_setup
    # warm-up iterations run every kernel of a step (the first use of each
    # loads its module) and leave the texels unchanged
    warm = max(3, warmup)
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
    sampler = ClockSampler(0)
    sampler.start()
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
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    # the loss after the last update (one more forward + backward, untimed)
    ctx.check(plan.launch())
    loss.zero_()
    ctx.check(ctx.backward(fviews, tptr, grad.data_ptr(), None, None, loss.data_ptr(),
                           capi.DEVICE_POINTERS | capi.ASYNC))
    losses = [float(x) for x in losses] + [float(loss.sum() / n_views)]
    px = sum(c.width * c.height for c in cams)
    plan.close()
    ctx.close()
    return {
        "metric": "views/s (forward+backward)", "value": iters * n_views / (ms / 1e3),
        "unit": "views/s", "n_gpus": 1, "steps": iters, "warmup": warm,
        "ms_per_step": ms / iters, "gpix_per_s": iters * px / (ms / 1e3) / 1e9,
        "config": {"workload": "texdescent256_icosphere8_tex4096_f32_1280x720",
                   "views": n_views, "iterations": iters, "lr": lr, "faces": m.num_faces,
                   "texels": "float32 in [0, 1]",
                   "step": "one graph-replayed forward (face_id + float colour), one "
                           "backward (texel gradient), one texel update per iteration"},
        "loss_iter0": losses[0], "loss_iter20": losses[iters], "loss_curve": losses,
        "setup_s": setup_s, "clocks": clocks, "tuning": tuning_record(tuned, autotune)}


def run_texdescent(args):
    print(json.dumps(measure_texdescent(args.warmup, autotune=not args.no_autotune)), flush=True)


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
    tuning = tuning_record(tuned, not args.no_autotune)
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
    # the last timed replay's images, kept for the parity check below
    replay = [{k: x.cpu().numpy() for k, x in t.items()} for t in outs]

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
    same_as_replay = {}
    if not args.no_per_view:
        def step_pv():
            ctx.check(ctx.render_views(views, capi.DEVICE_POINTERS | capi.PER_VIEW | capi.ASYNC))
        for _ in range(2):
            step_pv()
        ctx.check(ctx.synchronize())
        pv = timed(step_pv, max(2, min(args.steps, 5)))
        ctx.check(ctx.synchronize())
        per_view = len(cams) / (sum(pv) / len(pv) / 1e3)
        same_as_replay["per_view"] = all(
            view_digest({k: x.cpu().numpy() for k, x in t.items()}) == view_digest(r)
            for t, r in zip(outs, replay))

    # end to end through the C ABI with pinned host buffers: as a batch
    # renderer's caller holds them, one pinned buffer per output for all the
    # views, each view a slice of it (the library then copies each output of
    # a view group with one call); and, for comparison, one pinned buffer
    # per output and view
    e2e = None
    if not args.no_e2e:
        shapes = {"color": ((3,), torch.uint8), "depth": ((), torch.float32),
                  "normal": ((3,), torch.float32), "mask": ((), torch.uint8),
                  "face_id": ((), torch.int32)}

        def e2e_run(sliced):
            host, hviews = [], []
            d2h = 0
            flat = {}
            if sliced:
                for k, (ch, dt) in shapes.items():
                    n = sum(c.height * c.width * (ch[0] if ch else 1) for c in cams)
                    flat[k] = torch.empty(n, dtype=dt).pin_memory()
            at = {k: 0 for k in shapes}
            for c in cams:
                H, W = c.height, c.width
                t = {}
                for k, (ch, dt) in shapes.items():
                    if sliced:
                        n = H * W * (ch[0] if ch else 1)
                        t[k] = flat[k][at[k]:at[k] + n].view((H, W) + ch)
                        at[k] += n
                    else:
                        t[k] = torch.empty((H, W) + ch, dtype=dt).pin_memory()
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
            same = all(view_digest({k: x.numpy() for k, x in t.items()}) == view_digest(r)
                       for t, r in zip(host, replay))
            return world * len(cams) / dt, d2h, same

        value, d2h, same = e2e_run(True)
        per_view_value, _, same_pv = e2e_run(False)
        h2d = len(cams) * 256  # the per-view descriptor table (DevView, 248 B padded)
        e2e = {"value": value, "unit": "views/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h + 32 * 64,
               "host_buffers": "one pinned buffer per output for all views, a slice per view",
               "per_view_buffers": {"value": per_view_value, "unit": "views/s",
                                    "host_buffers": "one pinned buffer per output and view"}}
        same_as_replay["e2e_host_buffers"] = same and same_pv

    # forward + backward: 16 ring views at 640x480 of the same mesh with float
    # texels; a step is one graph-replayed forward (face_id + float colour)
    # and one backward of the per-pixel L2 loss against fixed targets.
    fwd_bwd = None
    if not args.no_backward:
        fwd_bwd = measure_fwd_bwd(ctx, torch, dev, stream, flush, timed, args)
    plan.close()
    ctx.close()

    # the oracle on all host threads over the same views: the CPU baseline,
    # and the bit-for-bit check of the timed replay's images
    cpu = None
    parity = None
    if rank == 0 and not (args.no_cpu_baseline and args.no_parity):
        threads = os.cpu_count() or 1
        dt, ref = oracle_all_views(m, cams, threads, keep=not args.no_parity)
        if not args.no_cpu_baseline:
            cpu = {"value": len(cams) / dt, "unit": "views/s", "cores": threads, "kind": "port",
                   "sample": f"all {len(cams)} views once, largest first, on {threads} host "
                             f"threads ({dt:.2f} s wall); oracle restatement of "
                             "Rasterizer::Render (-O2 -ffp-contract=off)"}
            # one core, the views in turn, as the reference's serial loops run
            dt1, _ = oracle_all_views(m, cams, 1)
            cpu["single_core"] = {"value": len(cams) / dt1, "unit": "views/s", "cores": 1,
                                  "sample": f"all {len(cams)} views serially ({dt1:.2f} s)"}
        if ref is not None:
            bad = [mismatched_pixels(r, g) for r, g in zip(ref, replay)]
            parity = {"views": len(cams), "mismatched_px": int(sum(bad)),
                      "mismatched_views": int(sum(b > 0 for b in bad)),
                      "outputs": list(OUT_KEYS), "against": "oracle, bit for bit",
                      "checked": "the last timed graph replay",
                      "identical_to_replay": same_as_replay}
            del ref
            parity["fp64_error"] = fp64_errors(m, cams, replay, threads)
    del replay

    peak, peak_kind = measured_peak_hbm()
    traffic, warp_inst, prof_state = committed_tile_profile()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    # the tile kernel writes every output byte (24 B/px) and reads the
    # texture and the geometry: the step's algorithmic bytes
    achieved = alg_bytes / (tile_ms / 1e3) / 1e9
    step_achieved = alg_bytes / (ms_step / 1e3) / 1e9
    # issue-side ceiling: warp instructions over what the SMs' 4 schedulers
    # can issue in the kernel's time at the sampled SM clock
    issue_frac = None
    if warp_inst and clk.get("sm_mhz"):
        issue_frac = warp_inst / (sms * 4 * clk["sm_mhz"] * 1e6 * tile_ms / 1e3)
    config = ring_config(m, cams)
    line = {
        "metric": "views/s", "value": views_per_s, "unit": "views/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": config,
        "launch": "one CUDA-graph replay of the batched render per step",
        "tuning": tuning,
        "gpix_per_s": world * total_px / (ms_step / 1e3) / 1e9,
        "per_view_views_per_s": per_view,
        "batched_over_per_view": (views_per_s / world / per_view) if per_view else None,
        "fwd_bwd": fwd_bwd,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": f"profiles/k_tile_traffic.txt ({prof_state})",
                     "peak_source": peak_kind, "kernel": "k_tile",
                     "kernel_ms": tile_ms, "algorithmic_bytes": alg_bytes,
                     "step_achieved": step_achieved, "step_frac": step_achieved / peak,
                     "warp_instructions": warp_inst, "issue_frac": issue_frac},
        "parity": parity,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if rank == 0 and not args.no_extras:
        # the other configurations, each with its own clock record: the
        # single-view forwards (UV sphere 640x480, textured icosphere-7
        # 1920x1080) and the large forward+backward texture descent
        line["extra"] = {
            "c1_uvsphere_640x480": measure_single("uvsphere", args.steps, args.warmup),
            "c2_icosphere7_1920x1080": measure_single("single1080", args.steps, args.warmup),
            "c5_texdescent256": measure_texdescent(args.warmup, autotune=not args.no_autotune),
        }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
