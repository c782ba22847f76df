"""CPU-only checks of the C ABI library: it builds for sm_103a, loads, exports
every function include/ugu_gpu.h declares, and fails cleanly without a GPU."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "ugu_gpu.h")).read()
    return sorted(set(re.findall(r"UGU_GPU_API\s+[\w\s\*]*?\b(ugu_gpu_\w+)\s*\(", src)))


def test_header_declares_the_abi():
    names = declared_functions()
    assert "ugu_gpu_render" in names and "ugu_gpu_backward" in names
    assert len(names) >= 18


def test_library_exports_every_declared_symbol(gpu_lib):
    from ugu_gb300 import build
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(ugu_gpu_\w+)\b", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert hasattr(gpu_lib, n)


def test_binding_lists_every_symbol():
    from ugu_gb300 import capi
    assert sorted(capi.EXPORTS) == declared_functions()


def test_abi_version(gpu_lib):
    assert gpu_lib.ugu_gpu_abi_version() == 4


def test_create_without_gpu_fails_cleanly(gpu_lib):
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = gpu_lib.ugu_gpu_create(0, C.byref(h))
    assert rc == 16  # UGU_GPU_ERR_NO_DEVICE
    assert not h.value
    assert b"CUDA" in gpu_lib.ugu_gpu_last_error(None) or gpu_lib.ugu_gpu_last_error(None)


def test_null_arguments_are_rejected(gpu_lib):
    assert gpu_lib.ugu_gpu_render(None, 0, None, None) == 1
    assert gpu_lib.ugu_gpu_set_mesh(None, 0, None) == 1
    assert gpu_lib.ugu_gpu_destroy(None) == 0


def test_python_mirror_without_gpu_raises():
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    from ugu_gb300 import capi
    from ugu_gb300.rasterizer import Context
    with pytest.raises(capi.GpuError) as e:
        Context(0)
    assert e.value.code == capi.ERR_NO_DEVICE


def test_kernel_cases_lists_every_kernel_family():
    """The profiling cases cover every kernel family of the library, and
    without a device the runner stops with a message instead of running."""
    import pytest as _pytest
    from ugu_gb300 import kernel_cases
    assert set(kernel_cases.CASES) == {"tiled", "global", "noalloc", "visualize", "gbuffer",
                                       "visibility", "texmap", "backward", "raytrace"}
    torch = _pytest.importorskip("torch")
    if not torch.cuda.is_available():
        with _pytest.raises(SystemExit):
            kernel_cases.main(["--case", "tiled", "--repeat", "1"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["tiled", "global", "noalloc", "visualize", "gbuffer",
                                  "visibility", "texmap", "backward", "raytrace"])
def test_kernel_cases_run_on_the_gpu(case, capsys):
    """Every profiling case runs once on the device and reports its timing."""
    import json
    from ugu_gb300 import kernel_cases
    views = {"tiled": 2, "global": 2, "visualize": 2, "gbuffer": 2, "visibility": 2,
             "texmap": 2, "backward": 2, "raytrace": 1}.get(case, 0)
    kernel_cases.main(["--case", case, "--repeat", "1", "--views", str(views)])
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["case"] == case and line["ms_per_call"] > 0.0
