"""ugu_gpu_render_noalloc, the entry point for callers that cannot allocate
device memory (a plug-in given only finished buffers, code under another
allocator's fixed budget, a frame loop that cannot take cudaMalloc's implicit
synchronisation).  It must produce exactly what the regular entry point
produces for the same view, and what the oracle produces, on two calls in a
row (the second call reuses the static scratch the first one left behind).

Collected last on purpose: if it fails, a run that stops at the first
failure has already run every other test.  It creates everything it uses, so
it passes alone in a fresh process as well as after the other tests."""
import ctypes as C

import numpy as np
import pytest

import adversarial as adv
from gpu_helpers import compare, device_views, to_option
from ugu_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def _four(a, dtype):
    a = np.asarray(a)
    out = np.zeros((a.shape[0], 4), dtype)
    out[:, :3] = a
    return out


def _device_mesh(torch, m):
    """The mesh in the 4-wide device layout the entry point documents."""
    keep = []

    def dev(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
        keep.append(t)
        return t.data_ptr()

    d = capi.DeviceMesh()
    d.num_vertices, d.num_faces = m.num_vertices, m.num_faces
    d.num_normals, d.num_uv = len(m.normals), len(m.uv)
    d.vertices4 = dev(_four(m.vertices, np.float32))
    d.vertex_indices4 = dev(_four(m.vertex_indices, np.int32))
    d.face_normals4 = dev(_four(m.face_normals, np.float32))
    d.normals4 = dev(_four(m.normals, np.float32))
    d.normal_indices4 = dev(_four(m.normal_indices, np.int32))
    d.vertex_colors4 = dev(_four(m.vertex_colors, np.float32))
    d.uv2 = dev(m.uv.astype(np.float32))
    d.uv_indices4 = dev(_four(m.uv_indices, np.int32))
    d.material_ids = dev(m.material_ids.astype(np.int32))
    t = m.textures[0].astype(np.uint32)
    rgba = (t[..., 0] | (t[..., 1] << 8) | (t[..., 2] << 16)).astype(np.uint32)
    tex = (capi.DeviceTexture * 1)()
    tex[0].width, tex[0].height = t.shape[1], t.shape[0]
    tex[0].rgba8 = dev(rgba.view(np.int32))
    tex[0].rgb_f32 = None
    keep.append(tex)
    d.num_materials = 1
    d.materials = C.addressof(tex)
    return d, keep


def test_noalloc_matches_regular_entry_point_twice(gpu_lib, oracle_lib):
    torch = pytest.importorskip("torch")
    from ugu_gb300.rasterizer import Context
    m = scenes.icosphere_textured(5, 256)
    cams = scenes.ring_cameras(4, 3.0, [(640, 480), (320, 240), (400, 300), (1920, 1080)])
    cams = [cams[0], cams[3]]  # two calls, the second one larger
    ctx = Context(0)
    try:
        for opt in (adv.option(1, 1, 1, 1, True), adv.option(2, 1, 0, 0, False)):
            ctx.check(ctx.set_mesh(0, m))
            ctx.check(ctx.set_option(to_option(opt)))
            want, views = device_views(torch, cams, [0, 0])
            ctx.check(ctx.render_views(views, capi.DEVICE_POINTERS))
            torch.cuda.synchronize()
            dmesh, keep = _device_mesh(torch, m)
            o = to_option(opt).to_struct()
            got, gviews = device_views(torch, cams, [0, 0])
            for i, cam in enumerate(cams):
                cs = capi.camera_struct(cam)
                rc = gpu_lib.ugu_gpu_render_noalloc(C.byref(dmesh), C.byref(o), C.byref(cs),
                                                    C.byref(gviews[i].images), None)
                assert rc == 0, gpu_lib.ugu_gpu_last_error(None)
                ref = {k: v.cpu().numpy() for k, v in want[i].items()}
                out = {k: v.cpu().numpy() for k, v in got[i].items()}
                compare(ref, out, f"noalloc view {i}")
                rc, orc, _ = oracle_lib.render(m, cam, opt, color_f32=True)
                assert rc == 0
                compare(orc, out, f"noalloc view {i} vs oracle")
            del keep
    finally:
        ctx.close()


def test_noalloc_rejects_oversized_images(gpu_lib):
    torch = pytest.importorskip("torch")
    m = scenes.icosphere_textured(2, 16)
    dmesh, keep = _device_mesh(torch, m)
    o = to_option(adv.option(1, 1, 1, 0, True)).to_struct()
    cam = scenes.camera_desc(2048, 1025, 1000.0, 1000.0, 1024.0, 512.0)  # 1 row too many
    im = capi.Images()
    fid = torch.empty((1025, 2048), dtype=torch.int32, device="cuda")
    im.face_id = fid.data_ptr()
    rc = gpu_lib.ugu_gpu_render_noalloc(C.byref(dmesh), C.byref(o),
                                        C.byref(capi.camera_struct(cam)), C.byref(im), None)
    assert rc == capi.ERR_CAPACITY
    assert b"UGU_GPU_NOALLOC_MAX_PIXELS" in gpu_lib.ugu_gpu_last_error(None)


def test_noalloc_mesh_without_faces(gpu_lib, oracle_lib):
    """A mesh with vertices but no faces renders empty images, as the
    reference does when its checks pass (culling off, vertex normals and
    colours present); no face normals are needed then."""
    torch = pytest.importorskip("torch")
    cam = adv.identity_camera()
    m = adv.shared_edge_quad(cam)
    m.vertex_indices = np.zeros((0, 3), np.int32)
    m.face_normals = np.zeros((0, 3), np.float32)
    m.normal_indices = np.zeros((0, 3), np.int32)
    m.uv_indices = np.zeros((0, 3), np.int32)
    m.material_ids = np.zeros(0, np.int32)
    opt = adv.option(2, 1, 1, 0, False)
    rc, ref, _ = oracle_lib.render(m, cam, opt, color_f32=True)
    assert rc == 0 and (ref["face_id"] == -1).all()
    dmesh, keep = _device_mesh(torch, m)
    dmesh.face_normals4 = None
    dmesh.normal_indices4 = None
    o = to_option(opt).to_struct()
    got, gviews = device_views(torch, [cam, cam], [0, 0])
    for i in range(2):
        rc = gpu_lib.ugu_gpu_render_noalloc(C.byref(dmesh), C.byref(o),
                                            C.byref(capi.camera_struct(cam)),
                                            C.byref(gviews[i].images), None)
        assert rc == 0, gpu_lib.ugu_gpu_last_error(None)
        compare(ref, {k: v.cpu().numpy() for k, v in got[i].items()}, f"no faces, call {i}")


def test_noalloc_reports_item_overflow(gpu_lib):
    """Forty faces that each cover the whole 1920x1080 image need 326,400
    (face, 16x16 tile) items, more than UGU_GPU_NOALLOC_MAX_ITEMS: the call
    reports UGU_GPU_ERR_CAPACITY (its images are then not valid), and the
    next call in range succeeds."""
    torch = pytest.importorskip("torch")
    cam = adv.identity_camera(W=1920, H=1080, f=1000.0)
    verts, faces = [], []
    for k in range(40):
        z = 2.0 + 0.01 * k
        base = len(verts)
        verts += [adv.unproject(cam, -3000.0, -3000.0, z), adv.unproject(cam, 6000.0, -3000.0, z),
                  adv.unproject(cam, -3000.0, 6000.0, z)]
        faces.append([base, base + 1, base + 2])
    m = adv._finish(np.array(verts, np.float32), np.array(faces, np.int32))
    dmesh, keep = _device_mesh(torch, m)
    o = to_option(adv.option(2, 1, 1, 0, False)).to_struct()
    got, gviews = device_views(torch, [cam], [0], outputs=("face_id",))
    rc = gpu_lib.ugu_gpu_render_noalloc(C.byref(dmesh), C.byref(o),
                                        C.byref(capi.camera_struct(cam)),
                                        C.byref(gviews[0].images), None)
    assert rc == capi.ERR_CAPACITY
    assert b"large-face tile items" in gpu_lib.ugu_gpu_last_error(None)
    small = adv.identity_camera()
    got, gviews = device_views(torch, [small], [0], outputs=("face_id",))
    rc = gpu_lib.ugu_gpu_render_noalloc(C.byref(dmesh), C.byref(o),
                                        C.byref(capi.camera_struct(small)),
                                        C.byref(gviews[0].images), None)
    assert rc == 0, gpu_lib.ugu_gpu_last_error(None)
    assert (got[0]["face_id"].cpu().numpy() == 0).all()  # face 0 is nearest everywhere
