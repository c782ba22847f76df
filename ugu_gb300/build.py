"""Build libugugpu.so (the CUDA kernels + C ABI) for sm_103a with nvcc.

The translation units compile in parallel; the library lands in
ugu_gb300/_lib/.  Only nvcc and a host C++ compiler are needed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libugugpu.so")
NVCC = os.environ.get("NVCC", "nvcc")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: belt and braces -- the parity-critical arithmetic already
# uses explicitly rounded intrinsics that are never contracted.
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fvisibility=hidden", "-I" + os.path.join(ROOT, "include")]

SOURCES = ["capi.cu", "raster.cu", "tile.cu", "bin.cu", "backward.cu", "noalloc.cu", "ray.cu", "bvh.cu",
           "vis.cu", "texmap.cu"]


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "ugu_gpu.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _deps():
        return LIB_PATH
    objs = []

    def compile_one(src):
        obj = os.path.join(LIB_DIR, src.replace(".cu", ".o"))
        cmd = [NVCC, *GENCODE, *NVFLAGS, *extra_flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(_sources()), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = [NVCC, *GENCODE, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
