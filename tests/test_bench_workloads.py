"""The benchmarked configurations themselves against the oracle, bit for bit.

* The batched forward that bench.py times: the icosphere-7 mesh (2048^2 RGB8
  texture, bilinear, vertex normals, culling on) from the 64 ring cameras at
  their seeded resolutions (54,067,200 px), rendered through a captured plan
  on the tuning the autotuner picks, then through per-view launches and into
  host buffers.  Every output of every view is compared with the oracle
  (rasterizer.cc:105-307 restated), run on all host threads.
* The large forward+backward configuration's forward: the icosphere-8 mesh
  (1,310,720 faces) with its 4096^2 float32 texture, 8 of its 256
  Fibonacci-sphere cameras at 1280x720, fx = 1000, through the float-texel
  path (float colour beside the 8-bit one).
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

from gpu_helpers import compare, device_views, host_images, to_option
from ugu_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def bench_option():
    from ugu_gb300.rasterizer import RendererCpuOption
    return RendererCpuOption(diffuse_color=1, interp=1, shading_normal=1, diffuse_shading=0,
                             backface_culling=True)


def oracle_check_all(oracle_lib, m, cams, opt, got, color_f32=False):
    """Renders every view with the oracle on all host threads and compares
    it with `got[i]` (host arrays) bit for bit; returns the oracle's total of
    texel clamp events."""
    threads = os.cpu_count() or 1
    order = sorted(range(len(cams)), key=lambda i: -cams[i].width * cams[i].height)

    def one(i):
        rc, ref, st = oracle_lib.render(m, cams[i], opt, color_f32=color_f32)
        assert rc == 0
        compare(ref, got[i], f"view {i} ({cams[i].width}x{cams[i].height})")
        return st.texel_clamps

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return sum(ex.map(one, order))


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def test_ring64_benchmark_batch_bit_exact(gpu_lib, oracle_lib, torch_cuda):
    torch = torch_cuda
    from ugu_gb300.rasterizer import Context
    m, cams = scenes.scene_ring_batch(64)
    assert sum(c.width * c.height for c in cams) == 54_067_200
    opt = bench_option()
    ctx = Context(0)
    try:
        ctx.check(ctx.set_mesh(0, m))
        ctx.check(ctx.set_option(opt))
        tensors, views = device_views(torch, cams, [0] * len(cams),
                                      outputs=("color", "depth", "normal", "mask", "face_id"))
        tuned = ctx.autotune(views)
        plan = ctx.plan_create(views, capi.DEVICE_POINTERS)
        try:
            for _ in range(2):  # a second replay over the first one's images
                ctx.check(plan.launch())
            ctx.check(ctx.synchronize())
        finally:
            plan.close()
        replay = [{k: x.cpu().numpy() for k, x in t.items()} for t in tensors]
        clamps = oracle_check_all(oracle_lib, m, cams, opt, replay)
        assert clamps == 0
        assert tuned.path in (capi.PATH_TILED, capi.PATH_GLOBAL)

        # the same views as per-view launch sequences, then into host buffers
        for t in tensors:
            for x in t.values():
                x.fill_(3)
        ctx.check(ctx.render_views(views, capi.DEVICE_POINTERS | capi.PER_VIEW))
        for i, t in enumerate(tensors):
            for k, x in t.items():
                assert np.array_equal(x.cpu().numpy(), replay[i][k]), (i, k, "per-view")
        hviews, hosts = [], []
        for c in cams:
            h, im = host_images(c, ("color", "depth", "normal", "mask", "face_id"))
            v = capi.View()
            v.mesh = 0
            v.camera = capi.camera_struct(c)
            v.images = im
            hosts.append(h)
            hviews.append(v)
        ctx.check(ctx.render_views(hviews, 0))
        for i, h in enumerate(hosts):
            for k, x in h.items():
                assert np.array_equal(x, replay[i][k]), (i, k, "host buffers")
    finally:
        ctx.close()


def test_texdescent_views_float_texels_bit_exact(gpu_lib, oracle_lib, torch_cuda):
    torch = torch_cuda
    from ugu_gb300.rasterizer import Context, RendererCpuOption
    m, _, cams = scenes.scene_texdescent(256)
    assert m.num_faces == 1_310_720 and m.textures_f32[0].shape == (4096, 4096, 3)
    sel = [cams[i] for i in range(0, 256, 32)]
    opt = RendererCpuOption(diffuse_color=1, interp=1, shading_normal=1, diffuse_shading=0,
                            backface_culling=True)
    ctx = Context(0)
    try:
        ctx.check(ctx.set_mesh(0, m))
        ctx.check(ctx.set_option(opt))
        tensors, views = device_views(torch, sel, [0] * len(sel))
        plan = ctx.plan_create(views, capi.DEVICE_POINTERS)
        try:
            ctx.check(plan.launch())
            ctx.check(ctx.synchronize())
        finally:
            plan.close()
        got = [{k: x.cpu().numpy() for k, x in t.items()} for t in tensors]
        clamps = oracle_check_all(oracle_lib, m, sel, opt, got, color_f32=True)
        assert clamps == 0
        assert all((g["mask"] == 255).sum() > 100_000 for g in got)
    finally:
        ctx.close()
