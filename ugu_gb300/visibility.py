"""ugu::VisibilityTester over the GPU (include/ugu/texturing/visibility_tester.h,
src/texturing/visibility_tester.cc).

The per-keyframe test of every vertex (TestVertex, :416-529), or of every
face corner (TestFacewiseVertices, :606-668), runs on the device for all
keyframes in one launch (ugu_gpu_test_visibility): one ray cast each through
the tester's naive BVH.  This module assembles the results into
VisibilityInfo the way the reference does on the host -- per vertex the
keyframes it is visible from, per face the keyframes all three of its
vertices (corners) are visible from, with the averaged viewing angle and
distance and the projected triangle's area (TestFaces, :551-604) -- and
computes the simple statistics of CalcStat (mean colour, distance and
viewing angle; the minimum-viewing-angle and minimum-distance keyframes;
FaceInfo's max-area, min-viewing-angle and min-distance keyframes).
Medians, weighted medians and modes of CalcStat are not reproduced.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .rasterizer import Context

F32 = np.float32


@dataclass
class VisibilityTesterOption:
    """VisibilityTesterOption (visibility_tester.h:38-58), same defaults."""
    backface_culling_angle_rad_th: float = float(F32(math.radians(90.0)))
    use_mask: bool = True
    use_depth: bool = True
    interp: int = 1  # ColorInterpolation::kBilinear
    calc_stat_vertex_info: bool = True
    collect_face_info: bool = True
    calc_stat_face_info: bool = True
    max_viewing_angle: float = float(F32(math.radians(90.0)))
    max_distance_from_camera_to_vertex: float = float(np.finfo(np.float32).max)
    max_depth_difference: float = float(np.finfo(np.float32).max)
    eps: float = 0.1

    def to_struct(self) -> capi.VisibilityOption:
        return capi.VisibilityOption(self.backface_culling_angle_rad_th, int(self.use_mask),
                                     int(self.use_depth), int(self.interp),
                                     self.max_viewing_angle,
                                     self.max_distance_from_camera_to_vertex,
                                     self.max_depth_difference, self.eps)


@dataclass
class Keyframe:
    """ugu::Keyframe (visibility_tester.h:196-212): id, camera, images."""
    id: int
    camera: object
    color: np.ndarray                  # H x W x 3 uint8
    depth: np.ndarray | None = None    # H x W float32
    mask: np.ndarray | None = None     # H x W uint8


@dataclass
class VertexInfoPerKeyframe:
    kf_id: int
    color: np.ndarray
    intensity: float
    projected_pos: np.ndarray
    viewing_angle: float
    distance: float


@dataclass
class FaceInfoPerKeyframe:
    kf_id: int
    face_id: int
    area: float
    viewing_angle: float
    distance: float
    projected_tri: np.ndarray


@dataclass
class VertexInfo:
    visible_keyframes: list = field(default_factory=list)
    mean_color: np.ndarray | None = None
    mean_distance: float = -1.0
    mean_viewing_angle: float = -1.0
    min_viewing_angle_index: int = -1
    min_viewing_angle_id: int = -1
    min_viewing_angle_color: np.ndarray | None = None
    min_distance_index: int = -1
    min_distance_id: int = -1
    min_distance_color: np.ndarray | None = None

    def VisibleFrom(self, kf_id: int) -> int:  # visibility_tester.cc:178-194
        for i, v in enumerate(self.visible_keyframes):
            if v.kf_id == kf_id:
                return i
        return -1

    def CalcStat(self):  # the mean / min parts of :68-176
        if not self.visible_keyframes:
            return
        cols = np.array([v.color for v in self.visible_keyframes], np.float32)
        self.mean_color = cols.sum(0, dtype=np.float32) / F32(len(cols))
        self.mean_distance = float(sum(v.distance for v in self.visible_keyframes)
                                   / len(self.visible_keyframes))
        self.mean_viewing_angle = float(sum(v.viewing_angle for v in self.visible_keyframes)
                                        / len(self.visible_keyframes))
        va = [v.viewing_angle for v in self.visible_keyframes]
        di = [v.distance for v in self.visible_keyframes]
        self.min_viewing_angle_index = int(np.argmin(va))
        self.min_viewing_angle_id = self.visible_keyframes[self.min_viewing_angle_index].kf_id
        self.min_viewing_angle_color = self.visible_keyframes[self.min_viewing_angle_index].color
        self.min_distance_index = int(np.argmin(di))
        self.min_distance_id = self.visible_keyframes[self.min_distance_index].kf_id
        self.min_distance_color = self.visible_keyframes[self.min_distance_index].color


@dataclass
class FaceInfo:
    visible_keyframes: list = field(default_factory=list)
    max_area_index: int = -1
    max_area_id: int = -1
    min_viewing_angle_index: int = -1
    min_viewing_angle_id: int = -1
    min_distance_index: int = -1
    min_distance_id: int = -1

    def CalcStat(self):  # visibility_tester.cc:202-224
        if not self.visible_keyframes:
            return
        a = [f.area for f in self.visible_keyframes]
        va = [f.viewing_angle for f in self.visible_keyframes]
        di = [f.distance for f in self.visible_keyframes]
        self.max_area_index = int(np.argmax(a))
        self.max_area_id = self.visible_keyframes[self.max_area_index].kf_id
        self.min_viewing_angle_index = int(np.argmin(va))
        self.min_viewing_angle_id = self.visible_keyframes[self.min_viewing_angle_index].kf_id
        self.min_distance_index = int(np.argmin(di))
        self.min_distance_id = self.visible_keyframes[self.min_distance_index].kf_id


class VisibilityInfo:
    def __init__(self, num_vertices: int, num_faces: int):
        self.vertex_info_list = [VertexInfo() for _ in range(num_vertices)]
        self.face_info_list = [FaceInfo() for _ in range(num_faces)]

    def CalcStatVertexInfo(self):
        for v in self.vertex_info_list:
            v.CalcStat()

    def CalcStatFaceInfo(self):
        for f in self.face_info_list:
            f.CalcStat()


def _area(tri) -> float:
    """0.5 * |EdgeFunction(p0, p1, p2)| in float (util/raster_util.h)."""
    (ax, ay), (bx, by), (cx, cy) = [(F32(p[0]), F32(p[1])) for p in tri]
    e = (cx - ax) * (by - ay) - (cy - ay) * (bx - ax)
    return float(F32(0.5) * abs(F32(e)))


class VisibilityTester:
    """ugu::VisibilityTester's interface (visibility_tester.h:216-265)."""

    def __init__(self, option: VisibilityTesterOption | None = None, device: int = 0):
        self._ctx = Context(device)
        self._option = option or VisibilityTesterOption()
        self._mesh = None
        self._normals = None
        self._initialized = False
        self._keyframe = None

    def set_option(self, option: VisibilityTesterOption) -> None:
        self._option = option

    def set_data(self, vertices, normals, indices) -> None:  # :310-317
        from .scenes import Mesh
        self._initialized = False
        self._mesh = Mesh(vertices=np.ascontiguousarray(vertices, np.float32),
                          vertex_indices=np.ascontiguousarray(indices, np.int32))
        self._normals = np.ascontiguousarray(normals, np.float32)

    def PrepareData(self) -> bool:  # :319-339
        if (self._mesh is None or len(self._mesh.vertices) == 0 or len(self._normals) == 0
                or len(self._mesh.vertex_indices) == 0):
            return False
        if self._ctx.set_mesh(0, self._mesh) != capi.OK:
            return False
        self._initialized = True
        return True

    def set_keyframe(self, keyframe: Keyframe) -> None:
        self._keyframe = keyframe

    def raw(self, keyframes, facewise: bool) -> dict:
        """The device results for all keyframes, keyframe-major arrays."""
        if not self._initialized:
            raise RuntimeError("mesh has not been initialized")
        keep, descs = [], []
        for kf in keyframes:
            d = capi.KeyframeDesc()
            d.id = int(kf.id)
            d.camera = capi.camera_struct(kf.camera)
            d.w2c_linear[:] = [float(x) for x in capi.w2c_linear(kf.camera).reshape(-1)]
            for name, a, dt in (("color", kf.color, np.uint8), ("depth", kf.depth, np.float32),
                                ("mask", kf.mask, np.uint8)):
                if a is not None:
                    a = np.ascontiguousarray(a, dt)
                    keep.append(a)
                    setattr(d, name, a.ctypes.data)
            descs.append(d)
        K = len(keyframes)
        items = 3 * self._mesh.num_faces if facewise else self._mesh.num_vertices
        res = {"visible": np.zeros((K, items), np.uint8),
               "projected_pos": np.zeros((K, items, 2), np.float32),
               "viewing_angle": np.zeros((K, items), np.float32),
               "distance": np.zeros((K, items), np.float32),
               "color": np.zeros((K, items, 3), np.float32),
               "intensity": np.zeros((K, items), np.float32)}
        out = capi.VisibilityOut(*[res[k].ctypes.data for k in
                                   ("visible", "projected_pos", "viewing_angle", "distance",
                                    "color", "intensity")])
        self._ctx.check(self._ctx.test_visibility(0, self._normals, descs,
                                                  self._option.to_struct(), facewise, out))
        return res

    def Test(self, info: VisibilityInfo, facewise: bool = True, keyframes=None) -> bool:
        """Test(info, facewise) for the keyframe set by set_keyframe, or
        Test(keyframes, info, facewise) (:670-731) for a list, in one launch."""
        kfs = keyframes if keyframes is not None else [self._keyframe]
        if not kfs or any(k is None for k in kfs):
            return False
        res = self.raw(kfs, facewise)
        F = self._mesh.vertex_indices
        for k, kf in enumerate(kfs):
            vis = res["visible"][k]

            def rec(i):
                return VertexInfoPerKeyframe(int(kf.id), res["color"][k, i].copy(),
                                             float(res["intensity"][k, i]),
                                             res["projected_pos"][k, i].copy(),
                                             float(res["viewing_angle"][k, i]),
                                             float(res["distance"][k, i]))
            if not facewise:
                for i in np.nonzero(vis)[0]:
                    info.vertex_info_list[i].visible_keyframes.append(rec(i))
                if self._option.collect_face_info:
                    for f in range(len(F)):  # TestFaces (:551-604)
                        vinf = []
                        for j in range(3):
                            vi = info.vertex_info_list[F[f, j]]
                            idx = vi.VisibleFrom(kf.id)
                            if idx < 0:
                                break
                            vinf.append(vi.visible_keyframes[idx])
                        if len(vinf) < 3:
                            continue
                        self._face(info, kf.id, f, vinf)
            else:  # TestFacewiseVertices (:606-668), faces in order
                done = np.zeros(len(info.vertex_info_list), bool)
                for f in range(len(F)):
                    vinf = []
                    for j in range(3):
                        i = 3 * f + j
                        if not vis[i]:
                            break
                        r = rec(i)
                        if not done[F[f, j]]:
                            done[F[f, j]] = True
                            info.vertex_info_list[F[f, j]].visible_keyframes.append(r)
                        vinf.append(r)
                    if len(vinf) < 3:
                        continue
                    self._face(info, kf.id, f, vinf)
        if self._option.calc_stat_vertex_info:
            info.CalcStatVertexInfo()
        if self._option.calc_stat_face_info:
            info.CalcStatFaceInfo()
        return True

    @staticmethod
    def _face(info, kf_id, f, vinf):
        va = F32(0.0)
        di = F32(0.0)
        with np.errstate(over="ignore"):  # FLT_MAX distances sum to inf, as in float
            for v in vinf:
                va = F32(va + F32(v.viewing_angle))
                di = F32(di + F32(v.distance))
        tri = np.array([v.projected_pos for v in vinf], np.float32)
        info.face_info_list[f].visible_keyframes.append(
            FaceInfoPerKeyframe(int(kf_id), int(f), _area(tri), float(va / F32(3)),
                                float(di / F32(3)), tri))
