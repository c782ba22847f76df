"""The oracle: CPU restatement of ugu's rasterizer (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package.  See raster_oracle.c for the reference lines each part restates.
"""
from .oracle import (  # noqa: F401
    build, load, render, raytrace, visualize, gbuffer, test_visibility, texture_mapping, ray_w,
    interp_f64, backward_f64, calc_normals, Stats, simple_triangles_layout, simple_triangles,
    simple_tile, simple_charts,
)
