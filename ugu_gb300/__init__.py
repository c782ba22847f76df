"""GB300-native rasterizer with the interface of ugu's CPU rasterizer.

The product is libugugpu.so (ugu_gb300/csrc, C ABI in include/ugu_gpu.h):
hand-written sm_103a CUDA kernels behind a plain C ABI.  This package holds
its build recipe, the ctypes binding, a Python mirror of ugu::Rasterizer and
the seeded scene generators.  There is no CPU fallback: without the library
or a GPU every render returns an error.
"""
from .rasterizer import (  # noqa: F401
    ColorInterpolation, Context, DiffuseColor, DiffuseShading, Rasterizer,
    RendererCpuOption, ShadingNormal,
)
from . import capi, scenes  # noqa: F401
