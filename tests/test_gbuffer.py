"""G-buffer channels (ugu::GBuffer's layout, include/ugu/renderer/base.h:
34-77, as RendererGl reads it back) from a render's face ids.

CPU: the oracle's channels are consistent with the render itself -- the
camera-frame position's z is the rendered depth (to float rounding), the
barycentrics sum to one, the world normals are unit length, face ids out
of range are counted.  GPU: the device pass reproduces the oracle bit for
bit, with device and host buffers, vertex and face normals, meshes with
and without texture coordinates, and reports bad face ids."""
import numpy as np
import pytest

import adversarial as adv
from ugu_gb300 import capi, scenes
from ugu_gb300.rasterizer import RendererCpuOption

KEYS = capi.GBUFFER + ("stencil",)


def scene(kind):
    if kind == "icosphere_ring":
        m = scenes.icosphere_textured(4, 64)
        cam = scenes.ring_cameras(3, 3.0, [(160, 120)] * 3)[1]
    elif kind == "soup":
        cam = adv.identity_camera(W=120, H=90, f=80.0)
        m = adv.triangle_soup(cam, n_faces=800, seed=2)
    else:  # UV sphere, vertex colours, no texture coordinates
        m, _ = scenes.scene_uv_sphere_vertex_color()
        cam = scenes.camera_desc(160, 120, 125.0, 125.0, 80.0, 60.0)
    return m, cam


@pytest.mark.parametrize("kind", ["icosphere_ring", "soup", "uv_sphere"])
def test_oracle_gbuffer_consistent_with_render(oracle_lib, kind):
    m, cam = scene(kind)
    opt = RendererCpuOption(diffuse_color=2, shading_normal=1, backface_culling=False)
    rc, out, _ = oracle_lib.render(m, cam, opt)
    assert rc == 0
    bad, g = oracle_lib.gbuffer(m, cam, opt, out["face_id"])
    assert bad == 0
    cov = out["face_id"] >= 0
    assert np.array_equal(g["stencil"] == 255, cov)
    rel = np.abs(g["pos_cam"][..., 2][cov] - out["depth"][cov]) / out["depth"][cov]
    assert rel.max() < 1e-5
    assert np.abs(g["bary"][cov].sum(-1) - 1).max() < 1e-6
    assert np.abs(np.linalg.norm(g["normal_wld"][cov], axis=-1) - 1).max() < 1e-5
    for k in capi.GBUFFER:
        assert not g[k][~cov].any(), k
    fid = out["face_id"].copy()
    fid[0, 0] = m.num_faces
    bad, _ = oracle_lib.gbuffer(m, cam, opt, fid)
    assert bad == 1


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["icosphere_ring", "soup", "uv_sphere"])
@pytest.mark.parametrize("sn", [0, 1])
def test_gpu_gbuffer_matches_oracle(gpu_lib, oracle_lib, kind, sn):
    import torch
    from gpu_helpers import gpu_render, to_option
    from ugu_gb300.rasterizer import Context
    m, cam = scene(kind)
    opt = adv.option(2, 1, sn, 0, True)
    ctx = Context(0)
    try:
        rc, out = gpu_render(ctx, m, cam, opt, outputs=("face_id",))
        assert rc == 0, ctx.last_error()
        bad, ref = oracle_lib.gbuffer(m, cam, opt, out["face_id"])
        H, W = cam.height, cam.width
        # host buffers
        got = {k: np.full((H, W, 3), 7.0, np.float32) for k in capi.GBUFFER}
        got["stencil"] = np.full((H, W), 7, np.uint8)
        v = capi.GBufferView()
        v.mesh = 0
        v.camera = capi.camera_struct(cam)
        v.face_id = out["face_id"].ctypes.data
        for k, a in got.items():
            setattr(v, k, a.ctypes.data)
        ctx.check(ctx.render_gbuffer([v]))
        for k in KEYS:
            assert np.array_equal(ref[k].view(np.uint8), got[k].view(np.uint8)), k
        # device buffers
        fid_d = torch.from_numpy(out["face_id"]).cuda()
        dg = {k: torch.full((H, W, 3), 7.0, device="cuda") for k in capi.GBUFFER}
        dg["stencil"] = torch.full((H, W), 7, dtype=torch.uint8, device="cuda")
        v2 = capi.GBufferView()
        v2.mesh = 0
        v2.camera = capi.camera_struct(cam)
        v2.face_id = fid_d.data_ptr()
        for k, t in dg.items():
            setattr(v2, k, t.data_ptr())
        ctx.check(ctx.render_gbuffer([v2], capi.DEVICE_POINTERS))
        for k in KEYS:
            a = dg[k].cpu().numpy()
            assert np.array_equal(ref[k].view(np.uint8), a.view(np.uint8)), (k, "device")
        # a face id out of range is reported
        fid = out["face_id"].copy()
        fid[0, 0] = m.num_faces + 5
        v.face_id = fid.ctypes.data
        assert ctx.render_gbuffer([v]) == capi.ERR_INDEX_OUT_OF_RANGE
    finally:
        ctx.close()
