"""Harder scenes for the raytracer's exactness (UGU_GPU_RAYTRACE): ties in
ray distance decided by the reference's traversal order, rays parallel to
and along box faces and edges, coordinates far from the origin (the float
error bounds' magnitudes), and triangles around the double test's
determinant threshold.  CPU: the oracle against the reference's own
raytracer where the checkout exists.  GPU: the CUDA path against the
oracle, bit for bit outside the documented sort-dependent pixels."""
import numpy as np
import pytest

import adversarial as adv
from ugu_gb300 import scenes

F32 = np.float32


def cube(cam):
    """An axis-aligned unit cube at z = 3 (two triangles per side)."""
    c = np.array([[x, y, z] for z in (2.5, 3.5) for y in (-0.5, 0.5) for x in (-0.5, 0.5)], F32)
    f = [[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1],
         [2, 3, 7], [2, 7, 6], [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]]
    return adv._finish(c, np.array(f, np.int32))


def duplicated_soup(cam):
    """Every triangle twice (and a third copy with its winding reversed):
    each hit ties exactly, and the reported face is the first in the
    reference's depth-first order."""
    m = adv.triangle_soup(cam, n_faces=40, seed=21)
    f = m.vertex_indices
    ff = np.concatenate([f, f, f[:, ::-1]], 0)
    return adv._finish(m.vertices, ff)


def far_offset(cam):
    """A soup 1000 units off the axis, seen by a camera moved there too."""
    m = adv.triangle_soup(cam, n_faces=300, seed=22)
    v = m.vertices.astype(np.float64) + np.array([1000.0, -700.0, 500.0])
    return adv._finish(v.astype(F32), m.vertex_indices)


def micro(cam):
    """Triangles with edges from 1e-5 to 1e-3 centred on pixel rays
    ((x - cx) / fx, (y - cy) / fy, 1) of the identity camera, randomly
    oriented: |det| lies around the double test's 1e-8 threshold."""
    rng = np.random.default_rng(23)
    v, f = [], []
    for i in range(1200):
        x, y = rng.integers(0, cam.width), rng.integers(0, cam.height)
        d = np.array([(x - cam.cx) / cam.fx, (y - cam.cy) / cam.fy, 1.0])
        c = rng.uniform(2.0, 4.0) * d / np.linalg.norm(d)
        e = 10 ** rng.uniform(-5, -3) * rng.normal(size=(3, 3))
        k = len(v)
        v += list(c + e - e.mean(0))
        f.append([k, k + 1, k + 2])
    return adv._finish(np.array(v, F32), np.array(f, np.int32))


def camera_for(name):
    if name == "far_offset":
        c2w = np.eye(4)
        c2w[:3, 3] = [1000.0, -700.0, 500.0]
        return scenes.camera_desc(80, 60, 50.0, 50.0, 40.0, 30.0, c2w)
    if name == "cube_corner":
        c2w = scenes.look_at_c2w((2.0, 1.5, 0.5), (0.0, 0.0, 3.0), (0.0, -1.0, 0.0))
        return scenes.camera_desc(80, 60, 50.0, 50.0, 40.0, 30.0, c2w)
    return adv.identity_camera(W=80, H=60, f=50.0)


SCENES = {"cube": cube, "cube_corner": cube, "duplicated_soup": duplicated_soup,
          "far_offset": far_offset, "micro": micro}
OPTS = [adv.option(2, 1, 1, 0, False), adv.option(1, 1, 0, 1, True)]


def same(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                          np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("name", list(SCENES))
def test_oracle_matches_reference_on_hard_scenes(oracle_lib, name):
    rb = pytest.importorskip("oracle.ref_build")
    if not rb.available():
        pytest.skip("reference sources not present")
    rb.build_if_available()
    cam = camera_for(name)
    m = SCENES[name](cam)
    for opt in OPTS:
        rc, a, _ = rb.raytrace(m, cam, opt)
        rc2, b = oracle_lib.raytrace(m, cam, opt)
        assert rc == rc2 == 0
        for k in a:
            assert same(a[k], b[k]), f"{name}: {k}"


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(SCENES))
def test_gpu_matches_oracle_on_hard_scenes(gpu_lib, oracle_lib, name):
    from gpu_helpers import compare, gpu_raytrace
    from test_raytrace import outside_sort_dependent
    from ugu_gb300.rasterizer import Context
    cam = camera_for(name)
    m = SCENES[name](cam)
    ctx = Context(0)
    try:
        for opt in OPTS:
            rc, ref = oracle_lib.raytrace(m, cam, opt, color_f32=True)
            assert rc == 0
            rc, got = gpu_raytrace(ctx, m, cam, opt)
            assert rc == 0, ctx.last_error()
            ref = outside_sort_dependent(oracle_lib, m, cam, opt, ref, got)
            compare(ref, got, name)
    finally:
        ctx.close()
