"""The image helpers after a render (ugu's image_util Depth2Gray,
Normal2Color, FaceId2RandomColor, ConvertTo to 16 bits) and the host
writers (WriteFaceIdAsText, netpbm, PFM).

CPU: the oracle's restatement on known answers -- std::mt19937 is the
standard generator, so its first draw for seed 5489 is 3499211612 (92 mod
256); Normal2Color rounds halves away from zero.  GPU: the device pass
reproduces the oracle bit for bit on random and edge inputs, with device
and host buffers."""
import os

import numpy as np
import pytest

from ugu_gb300 import capi, imageio, scenes


def edge_inputs(H=37, W=53, seed=3):
    rng = np.random.default_rng(seed)
    depth = rng.uniform(0, 2000, (H, W)).astype(np.float32)
    depth[0, :6] = [0, 200, 1500, 199.99, 1500.01, 70000.5]
    normal = rng.uniform(-1, 1, (H, W, 3)).astype(np.float32)
    # exact halves of the rounding: (n + 1) * 0.5 * 255 = k + 0.5, -n * 127 = k + 0.5
    normal[1, 0] = [1.0 / 255.0 * 2 - 1.0, 0.0, 0.5 / 127.0]
    normal[1, 1] = [-1.0, 1.0, -1.0]
    face_id = rng.integers(-3, 2_000_000, (H, W)).astype(np.int32)
    face_id[2, :4] = [-1, 0, 5489, 2147483647]
    return depth, normal, face_id


def test_oracle_known_answers(oracle_lib):
    o = oracle_lib.visualize(depth=np.array([[100, 200, 850, 1500, 2000]], np.float32),
                             face_id=np.array([[-1, 5489]], np.int32).repeat(3, 1)[:, :5])
    assert o["vis_depth"].tolist() == [[0, 0, 127, 255, 255]]
    assert o["depth_u16"].tolist() == [[100, 200, 850, 1500, 2000]]
    o = oracle_lib.visualize(face_id=np.array([[-1, 5489]], np.int32))
    assert o["vis_face_id"][0, 0].tolist() == [0, 0, 0]
    assert o["vis_face_id"][0, 1, 0] == 3499211612 % 256
    o = oracle_lib.visualize(normal=np.array([[[0.0, 0.0, 0.0]]], np.float32))
    assert o["vis_normal"].tolist() == [[[128, 128, 128]]]  # 127.5 rounds up


def test_writers_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    g = rng.integers(0, 256, (5, 7), dtype=np.uint8)
    c = rng.integers(0, 256, (5, 7, 3), dtype=np.uint8)
    w = rng.integers(0, 65536, (5, 7), dtype=np.uint16)
    f1 = rng.normal(size=(5, 7)).astype(np.float32)
    f3 = rng.normal(size=(5, 7, 3)).astype(np.float32)
    for name, img in (("g.pgm", g), ("c.ppm", c), ("w.pgm", w)):
        imageio.write_pnm(str(tmp_path / name), img)
        assert np.array_equal(imageio.read_pnm(str(tmp_path / name)), img)
    for name, img in (("f1.pfm", f1), ("f3.pfm", f3)):
        imageio.write_pfm(str(tmp_path / name), img)
        assert np.array_equal(imageio.read_pfm(str(tmp_path / name)), img)
    fid = rng.integers(-1, 1000, (4, 3)).astype(np.int32)
    imageio.WriteFaceIdAsText(fid, str(tmp_path / "fid.txt"))
    lines = (tmp_path / "fid.txt").read_text().splitlines()
    assert [int(x) for x in lines] == fid.reshape(-1).tolist()


@pytest.mark.gpu
def test_gpu_visualize_matches_oracle_host_and_device(gpu_lib, oracle_lib):
    import torch
    from ugu_gb300.rasterizer import Context
    depth, normal, face_id = edge_inputs()
    H, W = depth.shape
    ctx = Context(0)
    try:
        for gl in (False, True):
            ref = oracle_lib.visualize(depth, normal, face_id, 150.0, 1800.0, gl)
            # host buffers
            out = {k: np.full_like(v, 0x5A) for k, v in ref.items()}
            it = capi.Vis()
            it.width, it.height, it.min_d, it.max_d, it.gl_coord = W, H, 150.0, 1800.0, int(gl)
            it.depth, it.normal, it.face_id = depth.ctypes.data, normal.ctypes.data, face_id.ctypes.data
            for k, v in out.items():
                setattr(it, k, v.ctypes.data)
            ctx.check(ctx.visualize([it]))
            for k in ref:
                assert np.array_equal(ref[k], out[k]), (k, gl)
            # device buffers
            dev = {k: torch.from_numpy(v).cuda() for k, v in
                   (("depth", depth), ("normal", normal), ("face_id", face_id))}
            dout = {k: torch.full(v.shape, 0x5A, dtype=torch.from_numpy(v).dtype, device="cuda")
                    for k, v in ref.items()}
            it2 = capi.Vis()
            it2.width, it2.height, it2.min_d, it2.max_d, it2.gl_coord = W, H, 150.0, 1800.0, int(gl)
            for k, t in dev.items():
                setattr(it2, k, t.data_ptr())
            for k, t in dout.items():
                setattr(it2, k, t.data_ptr())
            ctx.check(ctx.visualize([it2], capi.DEVICE_POINTERS))
            for k in ref:
                assert np.array_equal(ref[k], dout[k].cpu().numpy()), (k, gl, "device")
    finally:
        ctx.close()


@pytest.mark.gpu
def test_gpu_visualize_a_render(gpu_lib, oracle_lib):
    """The ex02 flow: render, then the three helpers on its outputs."""
    from ugu_gb300.rasterizer import (Depth2Gray, FaceId2RandomColor, Normal2Color, Rasterizer,
                                      RendererCpuOption)
    m = scenes.icosphere_textured(4, 64)
    cam = scenes.ring_cameras(3, 3.0, [(160, 120)] * 3)[1]
    r = Rasterizer(RendererCpuOption(diffuse_color=1, interp=1, shading_normal=1))
    r.set_mesh(m)
    assert r.PrepareMesh()
    r.set_camera(cam)
    ok, out = r.Render(depth=True, normal=True, face_id=True)
    assert ok
    ref = oracle_lib.visualize(out["depth"], out["normal"], out["face_id"], 1.0, 4.0)
    assert np.array_equal(Depth2Gray(out["depth"], 1.0, 4.0), ref["vis_depth"])
    assert np.array_equal(Normal2Color(out["normal"]), ref["vis_normal"])
    assert np.array_equal(FaceId2RandomColor(out["face_id"]), ref["vis_face_id"])


@pytest.mark.parametrize("gl_coord", [False, True])
def test_visualize_pinned_to_the_reference(oracle_lib, gl_coord):
    """The oracle's image helpers against the reference's own
    (src/util/image_util.cc and image_proc.h's ConvertTo, built into
    oracle/_ref), bit for bit, on the edge inputs wherever the reference's
    float-to-integer casts are defined (depths below 65536, normals in
    [-1, 1]).  Runs where the reference checkout is present."""
    ref_build = pytest.importorskip("oracle.ref_build")
    if not ref_build.available():
        pytest.skip("reference sources not present")
    depth, normal, face_id = edge_inputs()
    depth[0, 5] = 60000.5  # the cast to 16 bits stays defined
    for kw in ({"min_d": 200.0, "max_d": 1500.0}, {"min_d": 0.5, "max_d": 70000.0}):
        want = ref_build.visualize(depth, normal, face_id, gl_coord=gl_coord, **kw)
        got = oracle_lib.visualize(depth, normal, face_id, gl_coord=gl_coord, **kw)
        for k in want:
            assert np.array_equal(want[k], got[k]), (k, kw)
