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


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic():
    """Per-launch DRAM bytes of the batched render from an ncu capture, as
    summarised in profiles/traffic.json (null when absent)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get("batched_forward_dram_bytes_per_launch")
    except Exception:
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


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
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
              "bin_capacity": tuned.bin_capacity}
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
    ms_step = sum(ms) / len(ms)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms_step], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    views_per_s = world * len(cams) / (ms_step / 1e3)

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

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        vps, gps, dt, nv = cpu_oracle_views_per_s(m, cams, threads)
        cpu = {"value": vps, "unit": "views/s", "cores": threads, "kind": "port",
               "sample": f"all {nv} views once on {threads} host threads ({dt:.1f} s wall), "
                         "oracle restatement of Rasterizer::Render (-O2 -ffp-contract=off)"}

    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
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
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": committed_traffic(),
                     "peak_source": peak_kind,
                     "scope": "batched forward graph replay (all kernels of one step)"},
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
