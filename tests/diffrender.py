"""Scenes for the differentiable path: a mesh with float texels and vertex
colours, and target images rendered from the same mesh with a second seeded
texture and per-vertex position noise."""
from __future__ import annotations

import numpy as np

from ugu_gb300 import scenes


def mesh_and_target_mesh(subdiv=5, tex=256, noise=0.005, seed=1):
    m = scenes.icosphere_textured(subdiv, tex, seed=seed, f32=True, vcolor_seed=2)
    t = m.copy()
    t.textures = [scenes.random_u8(5, m.textures[0].shape)]
    t.textures_f32 = [t.textures[0].astype(np.float32)]
    r = np.sqrt((t.vertices.astype(np.float64) ** 2).sum(axis=1))
    d = 1.0 + noise * scenes.normal(6, t.num_vertices) / np.maximum(r, 1e-9)
    t.vertices = (t.vertices.astype(np.float64) * d[:, None]).astype(np.float32)
    t.vertex_colors = (scenes.uniform01(7, 3 * t.num_vertices).reshape(-1, 3) * 255).astype(np.float32)
    return m, t


def seeded_params(m, n=256, seed=7):
    """n (kind, flat index) pairs: texels seen through the views, vertex
    colours, vertex positions, in roughly equal shares."""
    u = scenes.splitmix64(seed, 3 * n)
    out = []
    for i in range(n):
        kind = 1 + i % 3
        if kind == 1:
            size = m.textures_f32[0].size
        else:
            size = 3 * m.num_vertices
        out.append((kind, int(u[i] % np.uint64(size))))
    return out
