"""Golden fixtures: images produced by ugu's own Rasterizer::Render
(tests/golden/make_golden.py), with the inputs that produced them.  The
oracle must reproduce them bit for bit on any host; the GPU path must too
(Oren-Nayar colour within 1 LSB)."""
import glob
import os
from types import SimpleNamespace as NS

import numpy as np
import pytest

from ugu_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
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
    cam = scenes.Camera(W, H, fx, fy, cx, cy, z["w2c_R"], z["w2c_t"], z["c2w_R"])
    o = z["option"]
    opt = NS(diffuse_color=int(o[0]), interp=int(o[1]), shading_normal=int(o[2]),
             diffuse_shading=int(o[3]), backface_culling=bool(o[4]),
             oren_nayar_sigma=float(z["sigma"][0]), depth_scale=1.0)
    ref = {k: z["out_" + k] for k in OUTS}
    return m, cam, opt, ref


def test_fixtures_present():
    assert len(FIXTURES) >= 10


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_oracle_reproduces_reference_fixture(oracle_lib, path):
    m, cam, opt, ref = load(path)
    rc, out, _ = oracle_lib.render(m, cam, opt)
    assert rc == 0
    for k in OUTS:
        assert np.array_equal(ref[k].view(np.uint8), out[k].view(np.uint8)), k


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_gpu_reproduces_reference_fixture(gpu_lib, path):
    from gpu_helpers import compare, gpu_render
    from ugu_gb300.rasterizer import Context
    m, cam, opt, ref = load(path)
    ctx = Context(0)
    try:
        rc, got = gpu_render(ctx, m, cam, opt, outputs=OUTS)
        assert rc == 0, ctx.last_error()
    finally:
        ctx.close()
    compare(ref, got, os.path.basename(path), color_tol=1 if opt.diffuse_shading == 2 else 0)
