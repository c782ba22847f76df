"""The tiled rasterizer's candidate pixels (ugu_gb300/csrc/span.cuh) on the
host: every pixel the exact coverage test of rasterizer.cc:201-207 finds
covered, with either back-face sign, lies in the face's row spans, and the
spans decode one-to-one.  tests/cpp/span_check.cc runs the header's own code
under -ffp-contract=off, so its float arithmetic is the kernel's."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def span_check(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("span") / "span_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "ugu_gb300", "csrc"),
                    os.path.join(HERE, "cpp", "span_check.cc"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_spans_contain_every_covered_pixel(span_check, seed):
    r = subprocess.run([span_check, "300000", str(seed)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    ok, faces, box, cand, cov, span_faces, span_box, span_cand = r.stdout.split()
    assert ok == "ok"
    # the check exercised spans, and they are much tighter than the boxes
    assert int(span_faces) > 100000
    assert int(span_cand) < int(span_box) // 4
    assert int(cov) <= int(span_cand)
