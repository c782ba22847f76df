"""The C++ drop-in ugu::RasterizerGpu (ugu_gb300/host) against the reference's
own ugu::Rasterizer, both driven through the ugu::RendererCpu interface.

The drop-in needs ugu's headers, so it is built here from the reference
checkout (skipped elsewhere).  Linked against a test double of the C ABI that
runs the oracle, it must produce byte-identical images to the reference:
that checks its marshalling of ugu::Mesh / PinholeCamera / RendererCpuOption
into include/ugu_gpu.h and the outputs back.  Linked against the real
libugugpu.so without a GPU, every render must fail cleanly (false + LOGE)."""
import ctypes as C
import dataclasses
import os
import subprocess

import numpy as np
import pytest

import adversarial as adv
from ugu_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ref_build = pytest.importorskip("oracle.ref_build")
if not ref_build.available():
    pytest.skip("reference sources not present", allow_module_level=True)
REF = ref_build.REF
OUT = os.path.join(ROOT, "oracle", "_ref")


def _build(name, backend):
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, name)
    srcs = [f"{REF}/src/renderer/cpu/rasterizer.cc", f"{REF}/src/renderer/cpu/raytracer.cc",
            f"{REF}/src/renderer/cpu/util_private.cc",
            f"{REF}/src/log.cc", f"{REF}/src/image.cc", f"{REF}/src/util/thread_util.cc",
            f"{REF}/src/common.cc", os.path.join(ROOT, "oracle/ref/mesh_min.cc"),
            os.path.join(ROOT, "oracle/ref/geom_min.cc"),
            os.path.join(ROOT, "ugu_gb300/host/rasterizer_gpu.cc"),
            os.path.join(ROOT, "tests/cpp/drop_in_check.cc")]
    inc = ["-I", os.path.join(ROOT, "oracle/ref/override"),
           "-I", os.path.join(ROOT, "oracle/ref/eigen_shim"), "-I", f"{REF}/include",
           "-I", f"{REF}/src", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "ugu_gb300/host"), "-I", os.path.join(ROOT, "oracle")]
    extra = []
    if backend == "fake":
        obj = os.path.join(OUT, "raster_oracle_dropin.o")
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-c",
                               os.path.join(ROOT, "oracle/raster_oracle.c"), "-o", obj])
        srcs.append(os.path.join(ROOT, "tests/cpp/fake_ugu_gpu.cc"))
        srcs.append(os.path.join(ROOT, "oracle/ray_oracle.cc"))
        extra = [obj, "-lm"]
    else:
        from ugu_gb300 import build
        build.build()
        extra = [build.LIB_PATH, "-Wl,-rpath," + os.path.dirname(build.LIB_PATH)]
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                           "-w", *inc, *srcs, *extra, "-o", lib, "-lpthread"])
    return C.CDLL(lib)


@pytest.fixture(scope="module")
def fake_lib():
    return _build("libdropin_fake.so", "fake")


def run(lib, m, cam, opt, ray=False):
    f = lambda a, dt: np.ascontiguousarray(a, dt)  # noqa: E731
    arrs = [f(m.vertices, np.float32), f(m.vertex_indices, np.int32),
            f(m.face_normals, np.float32), f(m.normals, np.float32),
            f(m.vertex_colors, np.float32), f(m.uv, np.float32), f(m.uv_indices, np.int32),
            f(m.textures[0], np.uint8)]
    c2w = np.ascontiguousarray(cam.c2w if cam.c2w is not None else np.eye(4), np.float64)
    out = np.zeros(6, np.int64)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    fn = lib.drop_in_check_ray if ray else lib.drop_in_check
    fn.restype = C.c_int
    extra = (C.c_float(getattr(opt, "depth_scale", 1.0)),) if ray else ()
    rc = fn(
        C.c_int(m.num_vertices), P(arrs[0]), C.c_int(m.num_faces), P(arrs[1]), P(arrs[2]),
        P(arrs[3]), P(arrs[4]), C.c_int(len(m.uv)), P(arrs[5]), P(arrs[6]),
        C.c_int(m.textures[0].shape[1]), C.c_int(m.textures[0].shape[0]), P(arrs[7]),
        C.c_int(cam.width), C.c_int(cam.height), C.c_float(cam.fx), C.c_float(cam.fy),
        C.c_float(cam.cx), C.c_float(cam.cy), P(c2w), C.c_int(opt.diffuse_color),
        C.c_int(opt.interp), C.c_int(opt.shading_normal), C.c_int(opt.diffuse_shading),
        C.c_int(int(opt.backface_culling)), *extra, P(out))
    return rc, out


@pytest.mark.parametrize("optname", list(adv.OPTIONS))
def test_drop_in_matches_reference_ring_view(fake_lib, optname):
    m = scenes.icosphere_textured(4, 64)
    cam = scenes.ring_cameras(5, 3.0, [(120, 90)] * 5)[2]
    rc, diffs = run(fake_lib, m, cam, adv.OPTIONS[optname])
    assert rc == 0
    assert diffs.tolist() == [0] * 6, dict(zip(["color", "depth", "normal", "mask", "face_id",
                                                "depthW"], diffs.tolist()))


def test_drop_in_matches_reference_soup(fake_lib):
    cam = adv.identity_camera(W=96, H=72, f=60.0)
    cam.c2w = np.eye(4)
    m = adv.triangle_soup(cam, n_faces=600, seed=4)
    rc, diffs = run(fake_lib, m, cam, adv.option(1, 1, 0, 1, False))
    assert rc == 0 and diffs.tolist() == [0] * 6


@pytest.mark.parametrize("optname", ["vertex_vnormal_cull", "tex_bilinear_lambert",
                                     "white_orennayar"])
def test_raytracer_drop_in_matches_reference_ring_view(fake_lib, optname):
    m = scenes.icosphere_textured(4, 64)
    cam = scenes.ring_cameras(5, 3.0, [(120, 90)] * 5)[3]
    opt = dataclasses.replace(adv.OPTIONS[optname]) if dataclasses.is_dataclass(
        adv.OPTIONS[optname]) else type(adv.OPTIONS[optname])(**vars(adv.OPTIONS[optname]))
    opt.depth_scale = 1.5
    rc, diffs = run(fake_lib, m, cam, opt, ray=True)
    assert rc == 0
    assert diffs.tolist() == [0] * 6, dict(zip(["color", "depth", "normal", "mask", "face_id",
                                                "depthW"], diffs.tolist()))


def test_drop_in_error_paths(fake_lib):
    fake_lib.drop_in_errors.restype = C.c_int
    assert fake_lib.drop_in_errors() == 0


def test_drop_in_links_real_library_and_fails_cleanly_without_gpu():
    from conftest import HAS_GPU
    lib = _build("libdropin_real.so", "real")
    lib.drop_in_errors.restype = C.c_int
    assert lib.drop_in_errors() == 0
    if HAS_GPU:
        pytest.skip("a GPU is present: the no-device path is not reachable")
    m = scenes.icosphere_textured(2, 16)
    cam = scenes.ring_cameras(1, 3.0, [(32, 24)])[0]
    rc, _ = run(lib, m, cam, adv.option(1, 1, 1, 0, True))
    assert rc == 101  # the second renderer's PrepareMesh() returns false: no CUDA device
