"""Single-core CPU timings of the reference's own Rasterizer::Render
(oracle/_ref, compiled from the reference checkout) and of the oracle
restatement, on the rasterizer workloads: TEST INFRASTRUCTURE ONLY, for the
CPU baseline figures.  Each view is rendered twice on one camera, so that the
first call includes building the camera's lazy ray table
(PinholeCamera::InitRayTable, camera.h:100-101) and the second does not.

    UGU_REFERENCE_DIR=<checkout> python -m oracle.ref_timing [--views N]

Prints one JSON line per workload: views/s on one core for the reference
with a cold and a warm ray table, and for the oracle restatement (which has
no ray table), plus the machine.
"""
import argparse
import json
import os
import platform
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle, ref_build  # noqa: E402
from ugu_gb300 import scenes  # noqa: E402
from ugu_gb300.rasterizer import RendererCpuOption  # noqa: E402


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def workloads(n_ring):
    vc = RendererCpuOption(diffuse_color=2, interp=1, shading_normal=1, diffuse_shading=0,
                           backface_culling=True)
    tex = RendererCpuOption(diffuse_color=1, interp=1, shading_normal=1, diffuse_shading=0,
                            backface_culling=True)
    m1, c1 = scenes.scene_uv_sphere_vertex_color()
    m2, c2 = scenes.scene_icosphere_single_view()
    m3, c3 = scenes.scene_ring_batch(64)
    return [("uvsphere 640x480, vertex colour", m1, [c1], vc),
            ("icosphere-7 1920x1080, 2048^2 texture", m2, [c2], tex),
            (f"ring: {n_ring} of the 64 ring views, icosphere-7, 2048^2 texture", m3,
             c3[:n_ring], tex)]


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--views", type=int, default=64, help="ring views timed (of 64)")
    a = ap.parse_args(argv)
    if ref_build.load() is None:
        raise SystemExit("the reference build is not available (set UGU_REFERENCE_DIR)")
    for name, m, cams, opt in workloads(a.views):
        cold = warm = port = 0.0
        px = 0
        for cam in cams:
            rc, _, (t_cold, t_warm) = ref_build.render_timed(m, cam, opt)
            assert rc == 0, rc
            cold += t_cold / 1e3
            warm += t_warm / 1e3
            t0 = time.perf_counter()
            rc, _, _ = oracle.render(m, cam, opt)
            port += time.perf_counter() - t0
            assert rc == 0, rc
            px += cam.width * cam.height
        n = len(cams)
        print(json.dumps({"workload": name, "views": n, "pixels": px,
                          "reference_cold_views_per_s": n / cold,
                          "reference_warm_views_per_s": n / warm,
                          "oracle_views_per_s": n / port,
                          "ray_table_ms_per_view": 1e3 * (cold - warm) / n,
                          "cores": 1, "cpu": cpu_model(), "machine": platform.machine()}),
              flush=True)


if __name__ == "__main__":
    main()
