"""The raytracer (ugu::Raytracer, src/renderer/cpu/raytracer.cc) through
UGU_GPU_RAYTRACE.

CPU: the oracle's restatement (oracle/ray_oracle.cc + oracle_raytrace)
reproduces the reference's own Raytracer bit for bit -- on the committed
fixtures everywhere, and live against oracle/_ref where the reference
checkout exists.  GPU: the CUDA path reproduces the oracle bit for bit on the
same scenes, on batched views, through plans, and on the cases that stress
its pruning (axis-aligned planes hit by axis-parallel rays, rays along a
box face, a camera inside the geometry, odd face counts that duplicate
faces into both children of a BVH node, faces below the determinant
threshold), except on pixels whose face the reference's std::sort picks
among equal distances (more than 16 hits on the ray), which are counted."""
import dataclasses
import glob
import os

import numpy as np
import pytest

import adversarial as adv
from ugu_gb300 import capi, scenes

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "ray", "*.npz")))
OUTS = ("color", "depth", "normal", "mask", "face_id")


def load(path):
    z = np.load(path)
    g = lambda k: z[k] if k in z.files else None  # noqa: E731
    m = scenes.Mesh(vertices=z["vertices"], vertex_indices=z["vertex_indices"],
                    face_normals=g("face_normals"), normals=g("normals"),
                    normal_indices=g("normal_indices"), vertex_colors=g("vertex_colors"),
                    uv=g("uv"), uv_indices=g("uv_indices"), material_ids=g("material_ids"),
                    textures=[z["texture"]], textures_f32=[None])
    W, H = (int(x) for x in z["cam_int"])
    fx, fy, cx, cy = (float(x) for x in z["cam_f"])
    cam = scenes.Camera(W, H, fx, fy, cx, cy, z["w2c_R"], z["w2c_t"], z["c2w_R"], z["c2w"])
    o = z["option"]
    opt = adv.option(int(o[0]), int(o[1]), int(o[2]), int(o[3]), bool(o[4]),
                     float(z["sigma"][0]))
    opt.depth_scale = float(z["depth_scale"][0])
    return m, cam, opt, {k: z["out_" + k] for k in OUTS}


def same(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                          np.ascontiguousarray(b).view(np.uint8))


def outside_sort_dependent(oracle_lib, m, cam, opt, ref, got, limit=4):
    """The pixels whose face the reference's std::sort picks among equal
    distances (a ray with more than 16 hits, several at the smallest t:
    beyond 16 elements std::sort does not keep collection order) are
    excluded: the GPU reports the first such face in collection order.
    Returns copies of ref with those pixels taken from got."""
    rc, o = oracle_lib.raytrace(m, cam, opt, outputs=("face_id",), sort_dependent=True)
    sd = o["sort_dependent"].astype(bool)
    assert sd.sum() <= limit, f"{int(sd.sum())} sort-dependent pixels"
    out = {}
    for k, v in ref.items():
        v = v.copy()
        if k in got:
            v[sd] = got[k][sd]
        out[k] = v
    return out


# --- scenes ------------------------------------------------------------------

def axis_plane(cam, n=9):
    """A planar grid at z = 3 exactly, seen head-on by the identity camera:
    flat BVH boxes, and the centre pixel's ray has x and y components 0."""
    xs = np.linspace(-2.0, 2.0, n, dtype=np.float32)
    v = np.array([[x, y, 3.0] for y in xs for x in xs], np.float32)
    f = []
    for j in range(n - 1):
        for i in range(n - 1):
            a = j * n + i
            f += [[a, a + n, a + 1], [a + 1, a + n, a + n + 1]]
    return adv._finish(v, np.array(f, np.int32))


def inside_sphere(cam):
    """The camera at the centre of an icosphere of radius 4: every ray
    starts inside every box on its way out."""
    m = scenes.icosphere(3, 4.0, 0.0, seed=1)
    return adv._finish(m.vertices, m.vertex_indices)


def single_face(cam):
    v = np.array([[-1, -1, 3], [1, -1, 3], [0, 1, 3]], np.float32)
    return adv._finish(v, np.array([[0, 1, 2]], np.int32))


def odd_soup(cam):
    """41 faces: every split of an odd count puts its middle face in both
    children."""
    return adv.triangle_soup(cam, n_faces=41, seed=3)


def grazing(cam):
    """Thin slivers nearly along the rays: many faces fall below the
    determinant threshold 1e-8 of the double test, some just above it."""
    rng = np.random.default_rng(9)
    v, f = [], []
    for i in range(300):
        c = rng.uniform([-1.5, -1.0, 2.0], [1.5, 1.0, 5.0])
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        w = 10.0 ** rng.uniform(-6, -2)
        ray = c / np.linalg.norm(c)
        side = np.cross(ray, d)
        side /= np.linalg.norm(side) + 1e-30
        k = len(v)
        v += [c, c + 0.3 * ray, c + w * side]
        f.append([k, k + 1, k + 2])
    return adv._finish(np.array(v, np.float32), np.array(f, np.int32))


EDGE_SCENES = {"axis_plane": axis_plane, "inside_sphere": inside_sphere,
               "single_face": single_face, "odd_soup": odd_soup, "grazing": grazing}
EDGE_OPTIONS = {"vertex_vnormal_nocull": adv.option(2, 1, 1, 0, False),
                "tex_bilinear_lambert_cull": adv.option(1, 1, 1, 1, True)}


# --- CPU ---------------------------------------------------------------------

def test_sort_dependent_pixels_are_marked(oracle_lib):
    """The ray through the centre of a 24-face fan hits all 24 faces at the
    same distance: the reference's std::sort decides the face there."""
    cam = adv.identity_camera()
    m = adv.shared_vertex_fan(cam)
    rc, o = oracle_lib.raytrace(m, cam, adv.option(2, 1, 1, 0, False), outputs=("face_id",),
                                sort_dependent=True)
    assert rc == 0 and 1 <= int(o["sort_dependent"].sum()) <= 4


def test_ray_fixtures_present():
    assert len(FIXTURES) >= 8


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_oracle_reproduces_reference_raytracer_fixture(oracle_lib, path):
    m, cam, opt, ref = load(path)
    rc, out = oracle_lib.raytrace(m, cam, opt)
    assert rc == 0
    for k in OUTS:
        assert same(ref[k], out[k]), k


def _ref():
    rb = pytest.importorskip("oracle.ref_build")
    if not rb.available():
        pytest.skip("reference sources not present")
    rb.build_if_available()
    return rb


@pytest.mark.parametrize("scene", list(EDGE_SCENES))
def test_oracle_matches_reference_raytracer_on_edge_scenes(oracle_lib, scene):
    rb = _ref()
    cam = adv.identity_camera()
    m = EDGE_SCENES[scene](cam)
    for name, opt in EDGE_OPTIONS.items():
        rc, a, _ = rb.raytrace(m, cam, opt)
        rc2, b = oracle_lib.raytrace(m, cam, opt)
        assert rc == rc2 == 0
        for k in a:
            assert same(a[k], b[k]), f"{scene}/{name}: {k}"


def test_oracle_matches_reference_raytracer_on_soups_and_rings(oracle_lib):
    rb = _ref()
    for seed in (1, 2):
        cam = adv.identity_camera(W=120, H=90, f=80.0)
        m = adv.triangle_soup(cam, n_faces=1500, seed=seed)
        for opt in (adv.option(2, 1, 1, 1, False), adv.option(1, 0, 0, 2, True)):
            rc, a, _ = rb.raytrace(m, cam, opt)
            rc2, b = oracle_lib.raytrace(m, cam, opt)
            for k in a:
                assert same(a[k], b[k]), f"soup{seed}: {k}"
    m = scenes.icosphere_textured(5, 256)
    sizes = scenes.seeded_sizes(3, 4, [(160, 120), (200, 150), (120, 160)])
    for cam in scenes.ring_cameras(3, 3.0, sizes):
        opt = adv.option(1, 1, 1, 0, True)
        rc, a, _ = rb.raytrace(m, cam, opt)
        rc2, b = oracle_lib.raytrace(m, cam, opt)
        for k in a:
            assert same(a[k], b[k]), f"ring: {k}"


# --- GPU ---------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_gpu_raytracer_reproduces_reference_fixture(gpu_lib, oracle_lib, path):
    from gpu_helpers import compare, gpu_raytrace
    from ugu_gb300.rasterizer import Context
    m, cam, opt, ref = load(path)
    ctx = Context(0)
    try:
        rc, got = gpu_raytrace(ctx, m, cam, opt, outputs=OUTS)
        assert rc == 0, ctx.last_error()
    finally:
        ctx.close()
    ref = outside_sort_dependent(oracle_lib, m, cam, opt, ref, got)
    tol = 1 if opt.diffuse_shading == 2 else 0  # Oren-Nayar's acos/sin/tan
    compare(ref, got, os.path.basename(path), color_tol=tol)


@pytest.mark.gpu
@pytest.mark.parametrize("optname", list(adv.OPTIONS))
@pytest.mark.parametrize("scene", [s for s in adv.ALL_SMALL if s != "texture_border"]
                         + list(EDGE_SCENES))
def test_gpu_raytracer_matches_oracle(gpu_lib, oracle_lib, scene, optname):
    from gpu_helpers import compare, gpu_raytrace
    from ugu_gb300.rasterizer import Context
    cam = adv.identity_camera()
    m = (EDGE_SCENES.get(scene) or adv.ALL_SMALL[scene])(cam)
    opt = adv.OPTIONS[optname]
    rc, ref = oracle_lib.raytrace(m, cam, opt, color_f32=True)
    assert rc == 0
    ctx = Context(0)
    try:
        rc, got = gpu_raytrace(ctx, m, cam, opt)
        assert rc == 0, ctx.last_error()
    finally:
        ctx.close()
    ref = outside_sort_dependent(oracle_lib, m, cam, opt, ref, got)
    compare(ref, got, f"{scene}/{optname}", color_tol=1 if opt.diffuse_shading == 2 else 0)


@pytest.mark.gpu
def test_gpu_raytracer_batched_views_device_and_host(gpu_lib, oracle_lib):
    """Eight ring views of two meshes and three sizes in one call, device
    pointers, then the same views into host buffers; depth scaled."""
    import torch
    from gpu_helpers import compare, device_views, host_images, to_option
    from ugu_gb300.rasterizer import Context
    m1 = scenes.icosphere_textured(5, 256)
    m2 = scenes.icosphere_textured(3, 64, seed=4)
    sizes = scenes.seeded_sizes(8, 4, [(160, 120), (200, 150), (120, 160)])
    cams = scenes.ring_cameras(8, 3.0, sizes)
    slots = [0, 1] * 4
    opt = adv.option(1, 1, 1, 1, True)
    opt.depth_scale = 0.75
    ctx = Context(0)
    try:
        ctx.check(ctx.set_mesh(0, m1))
        ctx.check(ctx.set_mesh(1, m2))
        ctx.check(ctx.set_option(to_option(opt)))
        tens, views = device_views(torch, cams, slots)
        ctx.check(ctx.render_views(views, capi.DEVICE_POINTERS | capi.RAYTRACE))
        hosts = []
        hviews = []
        for cam, s in zip(cams, slots):
            out, im = host_images(cam)
            v = capi.View()
            v.mesh = s
            v.camera = capi.camera_struct(cam)
            v.images = im
            hosts.append(out)
            hviews.append(v)
        ctx.check(ctx.render_views(hviews, capi.RAYTRACE))
        for i, (cam, s) in enumerate(zip(cams, slots)):
            rc, ref = oracle_lib.raytrace((m1, m2)[s], cam, opt, color_f32=True)
            assert rc == 0
            got = {k: v.cpu().numpy() for k, v in tens[i].items()}
            compare(outside_sort_dependent(oracle_lib, (m1, m2)[s], cam, opt, ref, got), got,
                    f"device view {i}")
            compare(outside_sort_dependent(oracle_lib, (m1, m2)[s], cam, opt, ref, hosts[i]),
                    hosts[i], f"host view {i}")
    finally:
        ctx.close()


@pytest.mark.gpu
def test_gpu_raytracer_plan_replays(gpu_lib, oracle_lib):
    import torch
    from gpu_helpers import compare, device_views, to_option
    from ugu_gb300.rasterizer import Context
    m = scenes.icosphere_textured(4, 128)
    cams = scenes.ring_cameras(4, 3.0, [(160, 120)] * 4)
    opt = adv.option(1, 0, 0, 0, True)
    ctx = Context(0)
    try:
        ctx.check(ctx.set_mesh(0, m))
        ctx.check(ctx.set_option(to_option(opt)))
        tens, views = device_views(torch, cams, [0] * 4)
        plan = ctx.plan_create(views, capi.DEVICE_POINTERS | capi.RAYTRACE)
        for _ in range(3):
            for t in tens:
                for x in t.values():
                    x.fill_(7)
            ctx.check(plan.launch())
            ctx.check(ctx.synchronize())
        for i, cam in enumerate(cams):
            rc, ref = oracle_lib.raytrace(m, cam, opt, color_f32=True)
            got = {k: v.cpu().numpy() for k, v in tens[i].items()}
            compare(outside_sort_dependent(oracle_lib, m, cam, opt, ref, got), got,
                    f"plan view {i}")
    finally:
        ctx.close()  # destroys the plan with it


@pytest.mark.gpu
def test_gpu_raytracer_errors(gpu_lib):
    """ValidateAndInitBeforeRender's failures come back as status codes."""
    from gpu_helpers import gpu_raytrace
    from ugu_gb300.rasterizer import Context
    cam = adv.identity_camera()
    m = single_face(cam)
    ctx = Context(0)
    try:
        m2 = dataclasses.replace(m, face_normals=None)
        rc, _ = gpu_raytrace(ctx, m2, cam, adv.option(0, 1, 0, 0, True))
        assert rc == capi.ERR_NO_FACE_NORMALS, ctx.last_error()
    finally:
        ctx.close()
