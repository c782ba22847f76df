"""Seeded synthetic scenes: meshes, textures and pinhole cameras.

These stand in for the meshes ugu's examples load from disk (the bunny of
examples/ex02_renderer.cc is a network download).  Everything is generated from
integer seeds with a portable RNG (splitmix64), so a scene is the same on any
host.  Float32 arithmetic that feeds the rasterizer is written out element by
element in the order ugu's C++ evaluates it.

* ``uv_sphere``      -- ugu::MakeUvSphere (src/util/geom_util.cc:643-714) with
                        Mesh::Scale / Mesh::Translate (src/mesh.cc:223-228, 267-275).
* ``calc_normals``   -- Mesh::CalcFaceNormal / Mesh::CalcNormal (src/mesh.cc:297-349).
* ``icosphere``      -- subdivided icosahedron with radial noise and spherical
                        UVs (no reference counterpart; the reference has no
                        icosphere generator).
* ``look_at_c2w``    -- the look-at rotation of ugu::c2w (src/util/camera_util.cc:19-34).
* ``camera_desc``    -- the float camera parameters Rasterizer::Impl::Render reads
                        (rasterizer.cc:118-119, camera.h:317-331, 380-387, 438-448).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

F32 = np.float32


# --------------------------------------------------------------------------
# Portable RNG
# --------------------------------------------------------------------------

_M64 = (1 << 64) - 1


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n successive splitmix64 outputs for a seed, as uint64."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed & _M64) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int) -> np.ndarray:
    """float64 uniforms in [0, 1) with 53 random bits."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def normal(seed: int, n: int) -> np.ndarray:
    """Standard normals by the Box-Muller transform (float64)."""
    m = (n + 1) // 2
    u = uniform01(seed, 2 * m)
    u1 = 1.0 - u[0::2]  # (0, 1]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2.0 * math.pi * u2), r * np.sin(2.0 * math.pi * u2)])
    return z[:n]


def random_u8(seed: int, shape) -> np.ndarray:
    n = int(np.prod(shape))
    return (splitmix64(seed, n) >> np.uint64(56)).astype(np.uint8).reshape(shape)


# --------------------------------------------------------------------------
# Mesh container (ugu::Mesh's SoA fields, include/ugu/mesh.h:83-98)
# --------------------------------------------------------------------------


@dataclass
class Mesh:
    vertices: np.ndarray                      # V x 3 float32
    vertex_indices: np.ndarray                # F x 3 int32
    face_normals: np.ndarray | None = None    # F x 3 float32
    normals: np.ndarray | None = None         # N x 3 float32
    normal_indices: np.ndarray | None = None  # F x 3 int32
    vertex_colors: np.ndarray | None = None   # V x 3 float32
    uv: np.ndarray | None = None              # T x 2 float32
    uv_indices: np.ndarray | None = None      # F x 3 int32
    material_ids: np.ndarray | None = None    # F int32
    textures: list = field(default_factory=list)      # per material: H x W x 3 uint8
    textures_f32: list = field(default_factory=list)  # per material: H x W x 3 float32 (or None)

    @property
    def num_vertices(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def num_faces(self) -> int:
        return int(self.vertex_indices.shape[0])

    def copy(self) -> "Mesh":
        c = lambda a: None if a is None else a.copy()  # noqa: E731
        return Mesh(c(self.vertices), c(self.vertex_indices), c(self.face_normals),
                    c(self.normals), c(self.normal_indices), c(self.vertex_colors),
                    c(self.uv), c(self.uv_indices), c(self.material_ids),
                    [t.copy() for t in self.textures],
                    [None if t is None else t.copy() for t in self.textures_f32])


def _normalize_rows_f32(v: np.ndarray) -> np.ndarray:
    """Eigen normalize()/normalized() on float32 rows: divide by sqrt of
    x*x + (y*y + z*z) when that is > 0."""
    v = v.astype(F32, copy=True)
    n2 = v[:, 0] * v[:, 0] + (v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    ok = n2 > F32(0)
    s = np.sqrt(n2[ok])
    v[ok, 0] = v[ok, 0] / s
    v[ok, 1] = v[ok, 1] / s
    v[ok, 2] = v[ok, 2] / s
    return v


def calc_face_normals(vertices: np.ndarray, faces: np.ndarray) -> np.ndarray:
    """Mesh::CalcFaceNormal (src/mesh.cc:339-349)."""
    a = vertices[faces[:, 0]]
    b = vertices[faces[:, 1]]
    c = vertices[faces[:, 2]]
    e1 = _normalize_rows_f32(b - a)
    e2 = _normalize_rows_f32(c - a)
    n = np.empty_like(e1)
    n[:, 0] = e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1]
    n[:, 1] = e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2]
    n[:, 2] = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    return _normalize_rows_f32(n)


def calc_normals(mesh: Mesh) -> Mesh:
    """Mesh::CalcNormal (src/mesh.cc:297-337): face normals, then per vertex
    the incident face normals summed in face order, divided by the count and
    normalised; normal_indices = vertex_indices."""
    V, F = mesh.num_vertices, mesh.num_faces
    fn = calc_face_normals(mesh.vertices, mesh.vertex_indices)
    corner_v = mesh.vertex_indices.reshape(-1).astype(np.int64)
    corner_f = np.repeat(np.arange(F, dtype=np.int64), 3)
    order = np.argsort(corner_v, kind="stable")  # keeps face order per vertex
    sv = corner_v[order]
    sf = corner_f[order]
    counts = np.bincount(corner_v, minlength=V)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    rank = np.arange(sv.shape[0]) - starts[sv]
    acc = np.zeros((V, 3), dtype=F32)
    for k in range(int(counts.max()) if V else 0):
        sel = rank == k
        acc[sv[sel]] = acc[sv[sel]] + fn[sf[sel]]
    nrm = np.zeros((V, 3), dtype=F32)
    ok = counts > 0
    c = counts[ok].astype(F32)
    nrm[ok] = acc[ok] / c[:, None]
    nrm[ok] = _normalize_rows_f32(nrm[ok])
    mesh.face_normals = fn
    mesh.normals = nrm
    mesh.normal_indices = mesh.vertex_indices.copy()
    return mesh


# --------------------------------------------------------------------------
# Meshes
# --------------------------------------------------------------------------


def uv_sphere(n_stacks: int = 32, n_slices: int = 64, center=(0.0, 0.0, 3.0),
              r: float = 1.0) -> Mesh:
    """MakeUvSphere(center, r, n_stacks, n_slices) (geom_util.cc:643-714).

    The reference pushes one uv per ring vertex only and reuses the vertex
    indices as uv indices; the rasterizer's vertex-colour path never reads
    them, so they are omitted here."""
    verts = [(0.0, 1.0, 0.0)]
    for i in range(n_stacks - 1):
        phi = math.pi * float(i + 1) / float(n_stacks)
        for j in range(n_slices):
            theta = 2.0 * math.pi * float(j) / float(n_slices)
            verts.append((math.sin(phi) * math.cos(theta), math.cos(phi),
                          math.sin(phi) * math.sin(theta)))
    v1 = len(verts)
    verts.append((0.0, -1.0, 0.0))
    faces = []
    for i in range(n_slices):
        i0 = i + 1
        i1 = (i + 1) % n_slices + 1
        faces.append((0, i1, i0))
        i0 = i + n_slices * (n_stacks - 2) + 1
        i1 = (i + 1) % n_slices + n_slices * (n_stacks - 2) + 1
        faces.append((v1, i0, i1))
    for j in range(n_stacks - 2):
        j0 = j * n_slices + 1
        j1 = (j + 1) * n_slices + 1
        for i in range(n_slices):
            i0 = j0 + i
            i1 = j0 + (i + 1) % n_slices
            i2 = j1 + (i + 1) % n_slices
            i3 = j1 + i
            faces.append((i0, i1, i2))
            faces.append((i0, i2, i3))
    v = np.array(verts, dtype=np.float64).astype(F32)
    # Mesh::Scale then Mesh::Translate (float32, per component).
    v = v * F32(r)
    v = v + np.asarray(center, dtype=F32)[None, :]
    m = Mesh(vertices=np.ascontiguousarray(v, dtype=F32),
             vertex_indices=np.array(faces, dtype=np.int32))
    return m


_ICO_T = (1.0 + math.sqrt(5.0)) / 2.0


def _icosahedron():
    t = _ICO_T
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]],
                 dtype=np.int64)
    v = v / np.sqrt((v * v).sum(axis=1))[:, None]
    return v, f


def icosphere(subdiv: int, radius: float = 1.0, noise_sigma: float = 0.0,
              seed: int = 1, center=(0.0, 0.0, 0.0), uv_margin: float = 0.01) -> Mesh:
    """Icosahedron subdivided ``subdiv`` times (V = 10*4^n + 2, F = 20*4^n),
    every vertex displaced radially by N(0, noise_sigma) from ``seed``, with
    spherical UVs (u from longitude, v from latitude) and seam vertices
    duplicated in uv space.  UVs are mapped into [margin, 1 - margin] so that
    bilinear fetches never reach the texture's last row or column."""
    v, f = _icosahedron()
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid = mid / np.sqrt((mid * mid).sum(axis=1))[:, None]
        base = v.shape[0]
        v = np.concatenate([v, mid], axis=0)
        F = f.shape[0]
        m01 = base + inv[0:F]
        m12 = base + inv[F:2 * F]
        m20 = base + inv[2 * F:3 * F]
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], axis=1),
            np.stack([f[:, 1], m12, m01], axis=1),
            np.stack([f[:, 2], m20, m12], axis=1),
            np.stack([m01, m12, m20], axis=1)], axis=0)
    rad = np.full(v.shape[0], radius, dtype=np.float64)
    if noise_sigma > 0.0:
        rad = rad + noise_sigma * normal(seed, v.shape[0])
    pos = v * rad[:, None] + np.asarray(center, dtype=np.float64)[None, :]
    # spherical uv per corner; fix the longitude wrap per face
    lon = np.arctan2(v[:, 2], v[:, 0]) / (2.0 * math.pi) + 0.5  # [0, 1]
    lat = np.arcsin(np.clip(v[:, 1], -1.0, 1.0)) / math.pi + 0.5
    cu = lon[f]
    wrap = (cu.max(axis=1) - cu.min(axis=1)) > 0.5
    shift = wrap[:, None] & (cu < 0.5)
    key = f * 2 + shift.astype(np.int64)
    uniq, uv_idx = np.unique(key.reshape(-1), return_inverse=True)
    uvert = uniq // 2
    ushift = uniq % 2
    uu = (lon[uvert] + ushift) / 1.5  # wrapped duplicates lie in [1, 1.5)
    uv = np.stack([uv_margin + (1.0 - 2.0 * uv_margin) * uu,
                   uv_margin + (1.0 - 2.0 * uv_margin) * lat[uvert]], axis=1)
    m = Mesh(vertices=np.ascontiguousarray(pos.astype(F32)),
             vertex_indices=np.ascontiguousarray(f.astype(np.int32)),
             uv=np.ascontiguousarray(uv.astype(F32)),
             uv_indices=np.ascontiguousarray(uv_idx.reshape(-1, 3).astype(np.int32)),
             material_ids=np.zeros(f.shape[0], dtype=np.int32))
    return m


def with_vertex_colors(mesh: Mesh, seed: int, scale: float = 255.0) -> Mesh:
    """Per-vertex RGB uniform in [0, 1) from ``seed``, times ``scale``.  The
    reference truncates colours to u8 (pixel_shader.h:252-255), so the u8 path
    is fed 255 * U[0, 1)."""
    c = uniform01(seed, 3 * mesh.num_vertices).reshape(-1, 3)
    mesh.vertex_colors = np.ascontiguousarray((c * scale).astype(F32))
    return mesh


def with_texture(mesh: Mesh, size: int, seed: int, f32: bool = False) -> Mesh:
    tex = random_u8(seed, (size, size, 3))
    mesh.textures = [tex]
    mesh.textures_f32 = [tex.astype(F32)] if f32 else [None]
    if mesh.material_ids is None:
        mesh.material_ids = np.zeros(mesh.num_faces, dtype=np.int32)
    return mesh


# --------------------------------------------------------------------------
# Cameras
# --------------------------------------------------------------------------


@dataclass
class Camera:
    """The float parameters ugu's Rasterizer reads from a PinholeCamera."""
    width: int
    height: int
    fx: float
    fy: float
    cx: float
    cy: float
    w2c_R: np.ndarray  # 3x3 float32, row-major
    w2c_t: np.ndarray  # 3 float32
    c2w_R: np.ndarray  # 3x3 float32
    c2w: np.ndarray | None = None  # the 4x4 double pose these came from

    @property
    def pixels(self) -> int:
        return self.width * self.height


def _normalized64(v):
    n2 = v[0] * v[0] + (v[1] * v[1] + v[2] * v[2])
    return v / math.sqrt(n2) if n2 > 0.0 else v


def _cross64(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]])


def look_at_c2w(position, target, up) -> np.ndarray:
    """4x4 camera-to-world pose with the rotation of ugu::c2w
    (camera_util.cc:19-34): z = normalize(target - position),
    x = normalize(z x up), y = normalize(z x x) (OpenCV axes)."""
    p = np.asarray(position, dtype=np.float64)
    z = _normalized64(np.asarray(target, dtype=np.float64) - p)
    x = _normalized64(_cross64(z, np.asarray(up, dtype=np.float64)))
    y = _normalized64(_cross64(z, x))
    T = np.eye(4)
    T[:3, 0], T[:3, 1], T[:3, 2], T[:3, 3] = x, y, z, p
    return T


def _inverse3(m):
    """Cofactor inverse of a 3x3 double matrix."""
    c00 = m[1, 1] * m[2, 2] - m[1, 2] * m[2, 1]
    c10 = m[1, 2] * m[2, 0] - m[1, 0] * m[2, 2]
    c20 = m[1, 0] * m[2, 1] - m[1, 1] * m[2, 0]
    # expansion along column 0, as Eigen's 3x3 inverse computes it
    d10 = m[2, 1] * m[0, 2] - m[2, 2] * m[0, 1]
    d20 = m[0, 1] * m[1, 2] - m[0, 2] * m[1, 1]
    det = c00 * m[0, 0] + (d10 * m[1, 0] + d20 * m[2, 0])
    inv = np.empty((3, 3))
    invdet = 1.0 / det
    inv[0, 0], inv[0, 1], inv[0, 2] = c00 * invdet, (m[0, 2] * m[2, 1] - m[0, 1] * m[2, 2]) * invdet, (m[0, 1] * m[1, 2] - m[0, 2] * m[1, 1]) * invdet
    inv[1, 0], inv[1, 1], inv[1, 2] = c10 * invdet, (m[0, 0] * m[2, 2] - m[0, 2] * m[2, 0]) * invdet, (m[0, 2] * m[1, 0] - m[0, 0] * m[1, 2]) * invdet
    inv[2, 0], inv[2, 1], inv[2, 2] = c20 * invdet, (m[0, 1] * m[2, 0] - m[0, 0] * m[2, 1]) * invdet, (m[0, 0] * m[1, 1] - m[0, 1] * m[1, 0]) * invdet
    return inv


def _polar_rotation(m):
    """Orthogonal factor of the polar decomposition (Transform::rotation()),
    by Newton's iteration X <- (X + X^-T) / 2; exact for an orthonormal
    input such as the identity."""
    x = m.copy()
    for _ in range(32):
        nx = 0.5 * (x + _inverse3(x).T)
        if np.array_equal(nx, x):
            break
        x = nx
    return x


def camera_desc(width: int, height: int, fx: float, fy: float, cx: float, cy: float,
                c2w: np.ndarray | None = None) -> Camera:
    """PinholeCamera(width, height, c2w, principal_point, focal_length)
    (camera.h:301-331) reduced to the floats Render reads:
    w2c = c2w^-1 in double; w2c_R = w2c.rotation() cast to float
    (rasterizer.cc:118); w2c_t = w2c.translation() cast to float (:119);
    c2w_R = c2w block<3,3> cast to float (camera.h:321)."""
    if c2w is None:
        c2w = np.eye(4)
    R = np.asarray(c2w, dtype=np.float64)[:3, :3]
    t = np.asarray(c2w, dtype=np.float64)[:3, 3]
    Ri = _inverse3(R)
    # -(L^-1 t), each row summed a0 + (a1 + a2) like Eigen's matrix product
    ti = np.array([-(Ri[i, 0] * t[0] + (Ri[i, 1] * t[1] + Ri[i, 2] * t[2])) for i in range(3)])
    if np.array_equal(R, np.eye(3)):
        rot = np.eye(3)
    else:
        rot = _polar_rotation(Ri)
    return Camera(int(width), int(height), float(F32(fx)), float(F32(fy)),
                  float(F32(cx)), float(F32(cy)),
                  np.ascontiguousarray(rot.astype(F32)),
                  np.ascontiguousarray(ti.astype(F32)),
                  np.ascontiguousarray(R.astype(F32)),
                  np.array(c2w, dtype=np.float64))


def ring_cameras(n: int, radius: float, sizes, focal_scale: float = 0.8,
                 height: float = 0.0, target=(0.0, 0.0, 0.0)) -> list:
    """n cameras on a horizontal ring around ``target``, looking at it.
    ``sizes`` is a list of (W, H) per camera; fx = fy = focal_scale * W and
    the principal point is the image centre (W/2, H/2)."""
    cams = []
    for i in range(n):
        a = 2.0 * math.pi * i / n
        pos = (target[0] + radius * math.cos(a), target[1] + height, target[2] + radius * math.sin(a))
        c2w = look_at_c2w(pos, target, (0.0, -1.0, 0.0))
        W, H = sizes[i]
        f = focal_scale * W
        cams.append(camera_desc(W, H, f, f, W / 2.0, H / 2.0, c2w))
    return cams


def fibonacci_cameras(n: int, radius: float, width: int, height: int, focal: float,
                      target=(0.0, 0.0, 0.0)) -> list:
    """n cameras on a Fibonacci sphere of the given radius, looking at the
    centre; the up vector switches from -y to +z near the poles."""
    cams = []
    ga = math.pi * (3.0 - math.sqrt(5.0))
    for i in range(n):
        y = 1.0 - 2.0 * (i + 0.5) / n
        r = math.sqrt(max(0.0, 1.0 - y * y))
        th = ga * i
        pos = (target[0] + radius * r * math.cos(th), target[1] + radius * y,
               target[2] + radius * r * math.sin(th))
        up = (0.0, -1.0, 0.0) if abs(y) < 0.9 else (0.0, 0.0, 1.0)
        c2w = look_at_c2w(pos, target, up)
        cams.append(camera_desc(width, height, focal, focal, width / 2.0, height / 2.0, c2w))
    return cams


RING_SIZES = [(320, 240), (640, 480), (1280, 720), (1920, 1080)]


def seeded_sizes(n: int, seed: int, choices=RING_SIZES) -> list:
    """Per-camera resolutions drawn by ``seed`` from ``choices``: a seeded
    shuffle of n // len(choices) copies of each (so 64 ring views total
    exactly 54,067,200 px, the expected mean of a uniform draw), with any
    remainder drawn uniformly."""
    k = len(choices)
    base = [choices[i % k] for i in range((n // k) * k)]
    extra = splitmix64(seed ^ 0x5EED, n - len(base)) % np.uint64(k)
    pool = base + [choices[int(e)] for e in extra]
    order = np.argsort(splitmix64(seed, n), kind="stable")
    return [pool[int(i)] for i in order]


# --------------------------------------------------------------------------
# Benchmark / test workloads (sizes of the reference's configs)
# --------------------------------------------------------------------------


def scene_uv_sphere_vertex_color():
    """UV sphere r=1 at (0,0,3), 32 stacks x 64 slices (1986 V / 3968 F),
    vertex colours 255 * U[0,1) (seed 2), camera at the origin looking down +z,
    640x480, fx=fy=500, cx=320, cy=240."""
    m = calc_normals(uv_sphere(32, 64, (0.0, 0.0, 3.0), 1.0))
    with_vertex_colors(m, seed=2)
    cam = camera_desc(640, 480, 500.0, 500.0, 320.0, 240.0)
    return m, cam


def icosphere_textured(subdiv: int = 7, tex_size: int = 2048, seed: int = 1,
                       noise: float = 0.01, f32: bool = False, vcolor_seed: int | None = 2):
    m = icosphere(subdiv, 1.0, noise, seed=seed)
    calc_normals(m)
    with_texture(m, tex_size, seed=3, f32=f32)
    if vcolor_seed is not None:
        with_vertex_colors(m, seed=vcolor_seed)
    return m


def scene_icosphere_single_view(subdiv: int = 7, tex_size: int = 2048):
    """Icosphere-7 (163842 V / 327680 F), noise N(0, 0.01), 2048^2 RGB8
    texture, 1920x1080, fx=fy=1500, principal point (960, 540), distance 3."""
    m = icosphere_textured(subdiv, tex_size)
    c2w = look_at_c2w((0.0, 0.0, -3.0), (0.0, 0.0, 0.0), (0.0, -1.0, 0.0))
    cam = camera_desc(1920, 1080, 1500.0, 1500.0, 960.0, 540.0, c2w)
    return m, cam


def scene_ring_batch(n_views: int = 64, subdiv: int = 7, tex_size: int = 2048, seed: int = 4):
    """The single-view mesh seen from n cameras on a radius-3 ring with
    resolutions drawn (seed 4) from 320x240 .. 1920x1080, fx = 0.8 * W."""
    m = icosphere_textured(subdiv, tex_size)
    cams = ring_cameras(n_views, 3.0, seeded_sizes(n_views, seed))
    return m, cams


def scene_texdescent(n_views: int = 256, subdiv: int = 8, tex_size: int = 4096):
    """The large forward+backward configuration: an icosphere subdivided 8
    times (655,362 vertices / 1,310,720 faces, radial noise sigma 0.01, seed
    1), a tex_size^2 float32 texture with texels in [0, 1] (seed 3), the
    target mesh with a second texture (seed 5), and n cameras on a
    Fibonacci sphere at distance 3, 1280x720, fx = 1000.  Returns (mesh,
    target mesh, cameras)."""
    m = icosphere(subdiv, 1.0, 0.01, seed=1)
    calc_normals(m)
    with_texture(m, tex_size, seed=3, f32=True)
    # float texels in [0, 1], as multi-view texturing optimises them
    m.textures_f32 = [m.textures_f32[0] / np.float32(255.0)]
    tm = m.copy()
    tm.textures = [random_u8(5, m.textures[0].shape)]
    tm.textures_f32 = [tm.textures[0].astype(np.float32) / np.float32(255.0)]
    cams = fibonacci_cameras(n_views, 3.0, 1280, 720, 1000.0)
    return m, tm, cams
