"""GPU vs oracle parity through the C ABI (libugugpu.so).

face_id, mask, depth, normal and colour are compared bit for bit; only the
Oren-Nayar shader (acos/sin/tan from two different math libraries) is
allowed 1 LSB of 8-bit colour."""
import numpy as np
import pytest

import adversarial as adv
from gpu_helpers import compare, device_views, gpu_render
from ugu_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    from ugu_gb300.rasterizer import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def oracle_render(oracle_lib, m, cam, opt):
    rc, ref, st = oracle_lib.render(m, cam, opt, color_f32=True)
    assert rc == 0
    return ref, st


@pytest.mark.parametrize("optname", list(adv.OPTIONS))
@pytest.mark.parametrize("scene", list(adv.ALL_SMALL))
def test_small_scenes(ctx, oracle_lib, scene, optname):
    cam = adv.identity_camera()
    m = adv.ALL_SMALL[scene](cam)
    opt = adv.OPTIONS[optname]
    ref, _ = oracle_render(oracle_lib, m, cam, opt)
    rc, got = gpu_render(ctx, m, cam, opt)
    assert rc == 0, ctx.last_error()
    compare(ref, got, f"{scene}/{optname}", color_tol=1 if opt.diffuse_shading == 2 else 0)


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5, 6])
def test_triangle_soup_seeds(ctx, oracle_lib, seed):
    cam = adv.identity_camera(W=160, H=120, f=100.0)
    m = adv.triangle_soup(cam, n_faces=3000, seed=seed)
    for opt in (adv.option(2, 1, 1, 0, True), adv.option(1, 1, 0, 1, False)):
        ref, _ = oracle_render(oracle_lib, m, cam, opt)
        rc, got = gpu_render(ctx, m, cam, opt)
        assert rc == 0, ctx.last_error()
        compare(ref, got, f"soup{seed}")


def span_scene(cam, n=2500, seed=31):
    """Faces of the shapes the tiled path's row spans must handle, placed in
    screen space and lifted to camera depths 1.5 .. 6: small faces, slivers
    (one vertex 1e-6 .. 1 pixel off a long edge), vertices on integer and
    half-integer pixel lines, faces of 9 to 16 rows, near-collinear faces
    around the spans' area threshold, and nearly horizontal or vertical
    edges."""
    rng = np.random.default_rng(seed)
    W, H = cam.width, cam.height
    verts, faces = [], []
    for i in range(n):
        kind = i % 6
        cx, cy = rng.uniform(-4, W + 4), rng.uniform(-4, H + 4)
        if kind == 0:
            s = 0.3 + 12 * rng.uniform() ** 2
            p = np.stack([cx + s * (rng.uniform(size=3) - 0.5), cy + s * (rng.uniform(size=3) - 0.5)], 1)
        elif kind == 1:
            ln, ang = 1 + 40 * rng.uniform(), 2 * np.pi * rng.uniform()
            dx, dy = ln * np.cos(ang), ln * np.sin(ang)
            t, off = rng.uniform(), 10 ** rng.uniform(-6, 0) * rng.choice([-1, 1])
            p = np.array([[cx, cy], [cx + dx, cy + dy],
                          [cx + t * dx - off * dy / ln, cy + t * dy + off * dx / ln]])
        elif kind == 2:
            p = np.stack([np.floor(cx) + 0.5 * rng.integers(0, 13, 3) - 3,
                          np.floor(cy) + 0.5 * rng.integers(0, 13, 3) - 3], 1)
        elif kind == 3:
            p = np.stack([cx + rng.uniform(-12, 12, 3), cy + rng.uniform(-8.5, 8.5, 3)], 1)
        elif kind == 4:
            dx, dy, t = rng.uniform(-12, 12), rng.uniform(-6, 6), rng.uniform()
            p = np.array([[cx, cy], [cx + dx, cy + dy], [cx + t * dx, cy + t * dy]], np.float32)
            p[2] = np.nextafter(p[2], p[2] + rng.choice([-1, 1]) * 1e3)
        else:
            p = np.array([[cx, cy], [cx + rng.uniform(-10, 10), cy + rng.uniform(-1e-4, 1e-4)],
                          [cx + rng.uniform(-1e-4, 1e-4), cy + rng.uniform(-6, 6)]])
            if rng.uniform() < 0.5:
                p = p[:, ::-1].copy()
        z = rng.uniform(1.5, 6.0)
        k = len(verts)
        verts += [adv.unproject(cam, float(x), float(y), z) for x, y in p]
        faces.append([k, k + 1, k + 2])
    return adv._finish(np.array(verts, np.float32), np.array(faces, np.int32))


@pytest.mark.parametrize("seed", [31, 32])
def test_span_shapes_tiled(ctx, oracle_lib, seed):
    """The tiled path with its row spans against the oracle on faces shaped
    to stress the spans' bound and encoding (slivers, pixel-line vertices,
    9-16-row faces, near-threshold areas): every output bit for bit."""
    cam = adv.identity_camera(W=256, H=192, f=160.0)
    m = span_scene(cam, seed=seed)
    for opt in (adv.option(1, 1, 1, 0, True), adv.option(2, 0, 0, 1, False)):
        ref, _ = oracle_render(oracle_lib, m, cam, opt)
        rc, got = gpu_render(ctx, m, cam, opt)
        assert rc == 0, ctx.last_error()
        compare(ref, got, f"spans{seed}")


def test_uv_sphere_vertex_color_640x480(ctx, oracle_lib):
    m, cam = scenes.scene_uv_sphere_vertex_color()
    opt = adv.option(2, 1, 1, 0, True)
    ref, st = oracle_render(oracle_lib, m, cam, opt)
    rc, got = gpu_render(ctx, m, cam, opt)
    assert rc == 0, ctx.last_error()
    compare(ref, got, "uv_sphere")
    assert (got["mask"] == 255).sum() > 90000


def test_icosphere7_textured_1080p(ctx, oracle_lib):
    m, cam = scenes.scene_icosphere_single_view()
    opt = adv.option(1, 1, 1, 0, True)
    ref, st = oracle_render(oracle_lib, m, cam, opt)
    assert st.texel_clamps == 0
    rc, got = gpu_render(ctx, m, cam, opt)
    assert rc == 0, ctx.last_error()
    compare(ref, got, "icosphere7")


TUNINGS = [  # (path, tile_log2, entry_capacity, small_bbox_max, group_pixels, ctas_per_sm,
             #  split_class, bin_faces[, small_view_pixels])
    (capi.PATH_TILED, 5, 0, 256, 1 << 22, 0, 64, 2),
    (capi.PATH_TILED, 4, 0, 256, 1 << 22, 0, 64, 2),
    (capi.PATH_TILED, 5, 16, 256, 1 << 22, 0, 64, 2),   # entries overflow: the render is retried
    (capi.PATH_TILED, 4, 1, 256, 1 << 22, 0, 64, 2),
    (capi.PATH_TILED, 5, 0, 256, 1 << 22, 6, 1, 1),     # the autotuner's other candidates
    (capi.PATH_TILED, 5, 0, 256, 1 << 22, 7, 256, 4),
    (capi.PATH_TILED, 4, 0, 256, 1 << 22, 0, 4096, 4),
    (capi.PATH_TILED, 5, 0, 256, 1 << 22, 0, 64, 2, 200 * 150),  # small views: 16-px tiles
    (capi.PATH_TILED, 5, 0, 256, 1 << 22, 0, 64, 2, 100 * 100),
    (capi.PATH_GLOBAL, 3, 2048, 0, 1 << 22, 0, 0, 0),  # every face split into tile items
    (capi.PATH_GLOBAL, 4, 2048, 0, 1 << 22, 0, 0, 0),
    (capi.PATH_GLOBAL, 5, 2048, 16, 1 << 22, 0, 0, 0),
    (capi.PATH_GLOBAL, 6, 2048, 1 << 20, 1 << 22, 0, 0, 0),
]


def with_tuning(ctx, tup):
    return capi.Tuning(*tup)


@pytest.mark.parametrize("tup", TUNINGS,
                         ids=[f"p{t[0]}_t{t[1]}_c{t[2]}_s{t[3]}_k{t[5]}_sc{t[6]}_a{t[7]}"
                              f"_v{t[8] if len(t) > 8 else 0}" for t in TUNINGS])
def test_tuning_does_not_change_results(ctx, oracle_lib, tup):
    cam = adv.identity_camera(W=200, H=150, f=120.0)
    m = adv.triangle_soup(cam, n_faces=800, seed=9)
    t0 = ctx.tuning()
    for opt in (adv.option(2, 1, 1, 0, False), adv.option(1, 1, 0, 1, True)):
        ref, _ = oracle_render(oracle_lib, m, cam, opt)
        ctx.check(ctx.set_tuning(with_tuning(ctx, tup)))
        try:
            rc, got = gpu_render(ctx, m, cam, opt)
        finally:
            ctx.check(ctx.set_tuning(t0))
        assert rc == 0, ctx.last_error()
        compare(ref, got, f"tuning {tup}")


def _ring(subdiv, n, seed=4):
    m = scenes.icosphere_textured(subdiv, 256)
    sizes = scenes.seeded_sizes(n, seed, [(160, 120), (320, 240), (400, 300), (240, 320)])
    cams = scenes.ring_cameras(n, 3.0, sizes)
    return m, cams


@pytest.mark.parametrize("path", [capi.PATH_TILED, capi.PATH_GLOBAL])
@pytest.mark.parametrize("flags", [0, capi.PER_VIEW])
def test_batched_views_two_meshes(ctx, oracle_lib, torch_cuda, flags, path):
    torch = torch_cuda
    m0, cams = _ring(5, 8)
    m1, cam1 = scenes.scene_uv_sphere_vertex_color()
    m1 = m1.copy()
    m1.uv, m1.uv_indices = m0.uv[: 1], np.zeros_like(m1.vertex_indices)
    m1.material_ids = np.zeros(m1.num_faces, np.int32)
    m1.textures = m0.textures
    m1.textures_f32 = [None]
    ctx.check(ctx.set_mesh(0, m0))
    ctx.check(ctx.set_mesh(1, m1))
    opt = adv.option(1, 1, 1, 1, True)
    from gpu_helpers import to_option
    ctx.check(ctx.set_option(to_option(opt)))
    all_cams = cams + [cam1]
    slots = [0] * len(cams) + [1]
    meshes = [m0] * len(cams) + [m1]
    t = ctx.tuning()
    # several view groups on the global path; 16x16 tiles on the tiled one
    ctx.check(ctx.set_tuning(capi.Tuning(path, 4, 1024, 256, 100_000, 0, 64, 2)))
    try:
        tensors, views = device_views(torch, all_cams, slots)
        rc = ctx.render_views(views, capi.DEVICE_POINTERS | flags)
        assert rc == 0, ctx.last_error()
        torch.cuda.synchronize()
    finally:
        ctx.check(ctx.set_tuning(t))
    for i, (cam, mesh) in enumerate(zip(all_cams, meshes)):
        ref, _ = oracle_render(oracle_lib, mesh, cam, opt)
        got = {k: v.cpu().numpy() for k, v in tensors[i].items()}
        compare(ref, got, f"view{i}")


def test_host_outputs_span_copy_chunks(ctx, torch_cuda):
    """Host-buffer renders are cut into chunks of at most 4M pixels whose
    copies overlap the next chunk's kernels: a batch of 8.3M pixels (three
    chunks) into host buffers equals the same batch into device buffers,
    including a view that asks for colour without face ids."""
    torch = torch_cuda
    m = scenes.icosphere_textured(5, 256)
    cams = scenes.ring_cameras(5, 3.0, [(1920, 1080), (640, 480), (1920, 1080), (1920, 1080),
                                        (1280, 720)])
    ctx.check(ctx.set_mesh(0, m))
    from gpu_helpers import to_option
    ctx.check(ctx.set_option(to_option(adv.option(1, 1, 1, 0, True))))
    outs = [gpu_helpers_outputs(k) for k in range(len(cams))]
    want, dviews = [], []
    for cam, o in zip(cams, outs):
        t, v = device_views(torch, [cam], [0], outputs=o)
        want += t
        dviews += v
    ctx.check(ctx.render_views(dviews, capi.DEVICE_POINTERS))
    torch.cuda.synchronize()
    from gpu_helpers import host_images
    got, hviews = [], []
    for cam, o in zip(cams, outs):
        h, im = host_images(cam, o)
        v = capi.View()
        v.mesh = 0
        v.camera = capi.camera_struct(cam)
        v.images = im
        got.append(h)
        hviews.append(v)
    ctx.check(ctx.render_views(hviews, 0))
    for i in range(len(cams)):
        for k, t in want[i].items():
            assert np.array_equal(t.cpu().numpy(), got[i][k]), (i, k)


def test_host_outputs_in_one_buffer_per_output(ctx, torch_cuda):
    """Host buffers that are slices of one buffer per output, view after
    view, are copied back a run of views at a time: the same batch of three
    copy chunks equals the device-buffer render, with a view in the middle
    that asks for fewer outputs (it breaks the runs of the others) and a
    view whose slices are out of order (never merged)."""
    torch = torch_cuda
    m = scenes.icosphere_textured(5, 256)
    cams = scenes.ring_cameras(6, 3.0, [(1920, 1080), (640, 480), (1920, 1080), (1920, 1080),
                                        (1280, 720), (320, 240)])
    ctx.check(ctx.set_mesh(0, m))
    from gpu_helpers import to_option
    ctx.check(ctx.set_option(to_option(adv.option(1, 1, 1, 0, True))))
    outs = [gpu_helpers_outputs(k) for k in range(len(cams))]
    want, dviews = [], []
    for cam, o in zip(cams, outs):
        t, v = device_views(torch, [cam], [0], outputs=o)
        want += t
        dviews += v
    ctx.check(ctx.render_views(dviews, capi.DEVICE_POINTERS))
    torch.cuda.synchronize()
    spec = {"color": ((3,), np.uint8), "depth": ((), np.float32), "normal": ((3,), np.float32),
            "mask": ((), np.uint8), "face_id": ((), np.int32)}
    order = [0, 1, 2, 3, 5, 4]  # the last two views' slices swapped
    flat = {k: np.zeros(sum(c.width * c.height * (ch[0] if ch else 1) for c in cams), dt)
            for k, (ch, dt) in spec.items()}
    at = {k: 0 for k in spec}
    sl = [dict() for _ in cams]
    for i in order:
        c = cams[i]
        for k, (ch, dt) in spec.items():
            n = c.width * c.height * (ch[0] if ch else 1)
            if k in outs[i]:
                sl[i][k] = flat[k][at[k]:at[k] + n].reshape((c.height, c.width) + ch)
            at[k] += n
    hviews = []
    for i, cam in enumerate(cams):
        v = capi.View()
        v.mesh = 0
        v.camera = capi.camera_struct(cam)
        for k, a in sl[i].items():
            setattr(v.images, k, a.ctypes.data)
        hviews.append(v)
    ctx.check(ctx.render_views(hviews, 0))
    for i in range(len(cams)):
        for k, t in want[i].items():
            assert np.array_equal(t.cpu().numpy(), sl[i][k]), (i, k)


def gpu_helpers_outputs(k):
    full = ("color", "depth", "normal", "mask", "face_id")
    return ("color", "normal") if k == 3 else full


def test_graph_plan_replays(ctx, oracle_lib, torch_cuda):
    torch = torch_cuda
    m, cams = _ring(4, 6)
    ctx.check(ctx.set_mesh(0, m))
    opt = adv.option(1, 1, 1, 0, True)
    from gpu_helpers import to_option
    ctx.check(ctx.set_option(to_option(opt)))
    tensors, views = device_views(torch, cams, [0] * len(cams))
    plan = ctx.plan_create(views, capi.DEVICE_POINTERS)
    try:
        for rep in range(3):
            for t in tensors:
                for x in t.values():
                    x.fill_(3)
            ctx.check(plan.launch())
            ctx.check(ctx.synchronize())
            for i, cam in enumerate(cams):
                ref, _ = oracle_render(oracle_lib, m, cam, opt)
                compare(ref, {k: v.cpu().numpy() for k, v in tensors[i].items()}, f"rep{rep}/view{i}")
    finally:
        plan.close()


def test_validation_errors(ctx):
    cam = adv.identity_camera()
    m = adv.shared_edge_quad(cam)
    m2 = m.copy()
    m2.vertex_colors = None
    rc, _ = gpu_render(ctx, m2, cam, adv.option(diffuse_color=2))
    assert rc == capi.ERR_NO_VERTEX_COLORS
    m3 = m.copy()
    m3.vertex_indices = m3.vertex_indices.copy()
    m3.vertex_indices[1, 1] = 10_000
    assert ctx.set_mesh(0, m3) == capi.ERR_INDEX_OUT_OF_RANGE
    rc, _ = gpu_render(ctx, m, cam, adv.option(), outputs=())
    assert rc == capi.ERR_NO_OUTPUT
    # an empty slot is "mesh has not been initialized"
    ctx.check(ctx.set_mesh(3, None))
    rc, _ = gpu_render(ctx, m, cam, adv.option(), slot=3, upload=False)
    assert rc == capi.ERR_NOT_PREPARED


def test_python_rasterizer_mirror(gpu_lib, oracle_lib):
    from ugu_gb300.rasterizer import Rasterizer, RendererCpuOption, DiffuseColor
    m, cam = scenes.scene_uv_sphere_vertex_color()
    r = Rasterizer(RendererCpuOption(diffuse_color=DiffuseColor.kVertex, oren_nayar_sigma=0.9))
    ok, _ = r.Render(color=True)
    assert not ok  # no camera yet
    r.set_camera(cam)
    ok, _ = r.Render(color=True)
    assert not ok  # mesh not prepared
    r.set_mesh(m)
    assert r.PrepareMesh()
    ok, out = r.Render(color=True, depth=True, normal=True, mask=True, face_id=True)
    assert ok
    ref, _ = oracle_render(oracle_lib, m, cam, adv.option(2, 1, 1, 0, True))
    compare(ref, out, "mirror")
    ok, outw = r.RenderW(depth=True)
    assert ok and outw["depth"].dtype == np.uint16
    assert np.array_equal(outw["depth"], np.trunc(ref["depth"]).astype(np.uint16))


@pytest.mark.parametrize("path", [capi.PATH_TILED, capi.PATH_GLOBAL])
def test_mesh_without_faces(ctx, oracle_lib, path):
    """Vertices but no faces: the reference's checks pass (culling off,
    vertex normals and colours present) and it renders empty images; so do
    both paths here (no zero-block launch)."""
    cam = adv.identity_camera()
    m = adv.shared_edge_quad(cam)
    m.vertex_indices = np.zeros((0, 3), np.int32)
    m.face_normals = np.zeros((0, 3), np.float32)
    m.normal_indices = np.zeros((0, 3), np.int32)
    m.uv_indices = np.zeros((0, 3), np.int32)
    m.material_ids = np.zeros(0, np.int32)
    opt = adv.option(2, 1, 1, 0, False)
    ref, _ = oracle_render(oracle_lib, m, cam, opt)
    assert (ref["face_id"] == -1).all()
    t0 = ctx.tuning()
    ctx.check(ctx.set_tuning(capi.Tuning(path, 4, 0 if path == capi.PATH_TILED else 2048, 256,
                                         1 << 22, 0, 64, 2)))
    try:
        for _ in range(2):
            rc, got = gpu_render(ctx, m, cam, opt)
            assert rc == 0, ctx.last_error()
            compare(ref, got, "no faces")
    finally:
        ctx.check(ctx.set_tuning(t0))


def test_async_render_sizes_first_and_matches_oracle(gpu_lib, oracle_lib, torch_cuda):
    """A fresh context's first UGU_GPU_ASYNC render of the 1920x1080
    icosphere-7 view on 16x16 tiles needs more (face, tile) entries than the
    default lists hold: it sizes them first, so the images are exact and the
    next synchronize reports nothing."""
    torch = torch_cuda
    from gpu_helpers import to_option
    from ugu_gb300.rasterizer import Context
    m, cam = scenes.scene_icosphere_single_view()
    opt = adv.option(1, 1, 1, 0, True)
    c = Context(0)
    try:
        t = c.tuning()
        t.path, t.tile_log2 = capi.PATH_TILED, 4
        c.check(c.set_tuning(t))
        c.check(c.set_mesh(0, m))
        c.check(c.set_option(to_option(opt)))
        tensors, views = device_views(torch, [cam], [0])
        ref, _ = oracle_render(oracle_lib, m, cam, opt)
        for _ in range(2):
            c.check(c.render_views(views, capi.DEVICE_POINTERS | capi.ASYNC))
            assert c.synchronize() == 0, c.last_error()
            compare(ref, {k: v.cpu().numpy() for k, v in tensors[0].items()}, "async")
            for x in tensors[0].values():
                x.fill_(3)
    finally:
        c.close()


def test_async_overflow_is_reported_at_synchronize(gpu_lib, torch_cuda):
    """The global path keeps a fixed list of (face, tile) items: 200 faces
    over a whole 1920x1080 image in 8x8 tiles need 6.5 M of them.  An
    asynchronous render cannot retry, so ugu_gpu_synchronize reports the
    overflow (its images are not valid); a synchronous render, which grows
    the list and retries, then succeeds."""
    torch = torch_cuda
    from gpu_helpers import to_option
    from ugu_gb300.rasterizer import Context
    cam = adv.identity_camera(W=1920, H=1080, f=1000.0)
    verts, faces = [], []
    for k in range(200):
        z = 2.0 + 0.001 * k
        b = len(verts)
        verts += [adv.unproject(cam, -3000.0, -3000.0, z), adv.unproject(cam, 6000.0, -3000.0, z),
                  adv.unproject(cam, -3000.0, 6000.0, z)]
        faces.append([b, b + 1, b + 2])
    m = adv._finish(np.array(verts, np.float32), np.array(faces, np.int32))
    c = Context(0)
    try:
        c.check(c.set_tuning(capi.Tuning(capi.PATH_GLOBAL, 3, 0, 0, 1 << 22, 0, 64, 2)))
        c.check(c.set_mesh(0, m))
        c.check(c.set_option(to_option(adv.option(2, 1, 1, 0, False))))
        tensors, views = device_views(torch, [cam], [0], outputs=("face_id",))
        c.check(c.render_views(views, capi.DEVICE_POINTERS | capi.ASYNC))
        assert c.synchronize() == capi.ERR_CAPACITY
        assert c.synchronize() == 0  # reported once
        c.check(c.render_views(views, capi.DEVICE_POINTERS))
        assert (tensors[0]["face_id"].cpu().numpy() == 0).all()
        assert c.synchronize() == 0
    finally:
        c.close()


def test_autotune_caches_per_workload(gpu_lib, oracle_lib, torch_cuda, tmp_path, monkeypatch):
    """ugu_gpu_autotune picks among path, tile size, blocks per SM and the
    draw and binning thresholds; its choice renders exactly what the oracle
    renders, a second call on the same workload shape returns the cached
    choice, and the choice is appended to UGU_GPU_TUNING_CACHE and read back
    by a new context."""
    torch = torch_cuda
    from gpu_helpers import to_option
    from ugu_gb300.rasterizer import Context
    cache = tmp_path / "tuning.txt"
    monkeypatch.setenv("UGU_GPU_TUNING_CACHE", str(cache))
    m, cams = _ring(5, 6)
    opt = adv.option(1, 1, 1, 0, True)
    fields = [f for f, _ in capi.Tuning._fields_]
    chosen = []
    for _ in range(2):
        c = Context(0)
        try:
            c.check(c.set_mesh(0, m))
            c.check(c.set_option(to_option(opt)))
            tensors, views = device_views(torch, cams, [0] * len(cams))
            t1 = c.autotune(views)
            t2 = c.autotune(views)  # cached
            assert [getattr(t1, f) for f in fields] == [getattr(t2, f) for f in fields]
            chosen.append([getattr(t1, f) for f in fields])
            c.check(c.render_views(views, capi.DEVICE_POINTERS))
            for i, cam in enumerate(cams):
                ref, _ = oracle_render(oracle_lib, m, cam, opt)
                compare(ref, {k: v.cpu().numpy() for k, v in tensors[i].items()}, f"view{i}")
        finally:
            c.close()
    assert chosen[0] == chosen[1]
    lines = cache.read_text().split("\n")
    assert len([x for x in lines if x.strip()]) == 1  # the second context read it back


def test_views_on_two_tile_sizes(ctx, oracle_lib, torch_cuda):
    """One batch whose small views use 16-pixel tiles and whose larger ones
    use 32-pixel tiles (small_view_pixels): every view bit for bit."""
    torch = torch_cuda
    from gpu_helpers import to_option
    m0, cams = _ring(5, 8)
    opt = adv.option(1, 1, 1, 0, True)
    ctx.check(ctx.set_mesh(0, m0))
    ctx.check(ctx.set_option(to_option(opt)))
    t0 = ctx.tuning()
    ctx.check(ctx.set_tuning(capi.Tuning(capi.PATH_TILED, 5, 0, 256, 1 << 22, 0, 64, 2, 320 * 240)))
    try:
        assert len({c.width * c.height <= 320 * 240 for c in cams}) == 2
        tensors, views = device_views(torch, cams, [0] * len(cams))
        for flags in (capi.DEVICE_POINTERS, capi.DEVICE_POINTERS | capi.PER_VIEW):
            for t in tensors:
                for x in t.values():
                    x.fill_(3)
            ctx.check(ctx.render_views(views, flags))
            torch.cuda.synchronize()
            for i, cam in enumerate(cams):
                ref, _ = oracle_render(oracle_lib, m0, cam, opt)
                compare(ref, {k: v.cpu().numpy() for k, v in tensors[i].items()}, f"view{i}")
    finally:
        ctx.check(ctx.set_tuning(t0))


@pytest.mark.parametrize("sizes", [[(1024, 1024)], [(1024, 1024), (16, 16)],
                                   [(16, 16), (2048, 1024), (24, 8)]],
                         ids=["4096_tiles", "4097_tiles", "8195_tiles"])
def test_tile_scan_chunk_boundaries(ctx, oracle_lib, torch_cuda, sizes):
    """The tile-count scan runs one block per chunk of 4,096 tiles: batches
    of exactly one chunk, one chunk and one tile, and two chunks and three
    tiles (16-pixel tiles throughout) render every view as the oracle does."""
    torch = torch_cuda
    m = scenes.icosphere_textured(4, 128)
    cams = scenes.ring_cameras(len(sizes), 3.0, sizes)
    ctx.check(ctx.set_mesh(0, m))
    opt = adv.option(1, 1, 1, 0, True)
    from gpu_helpers import to_option
    ctx.check(ctx.set_option(to_option(opt)))
    t0 = ctx.tuning()
    ctx.check(ctx.set_tuning(capi.Tuning(capi.PATH_TILED, 4, 0, 256, 1 << 22, 0, 64, 2, 0)))
    try:
        tensors, views = device_views(torch, cams, [0] * len(cams))
        ctx.check(ctx.render_views(views, capi.DEVICE_POINTERS))
        torch.cuda.synchronize()
    finally:
        ctx.check(ctx.set_tuning(t0))
    for i, cam in enumerate(cams):
        ref, _ = oracle_render(oracle_lib, m, cam, opt)
        got = {k: v.cpu().numpy() for k, v in tensors[i].items()}
        compare(ref, got, f"view {i} {sizes[i]}")
