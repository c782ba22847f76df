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
computes CalcStat's statistics (:68-176 and :202-224) with the float
arithmetic of ugu's math helpers (include/ugu/util/math_util.h).  One case
is not pinned: Median of an odd count >= 5 without force_org_val averages
the element std::nth_element leaves just below the middle, which the C++
standard does not fix; this takes the sorted one.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .rasterizer import Context

F32 = np.float32


def first_min(vals) -> int:
    """Index std::min_element returns: the first minimum under `<`."""
    idx = 0
    for i in range(1, len(vals)):
        if vals[i] < vals[idx]:
            idx = i
    return idx


def normalize_weights(weights):
    """NormalizeWeights (math_util.h:28-48): float weights plus 1e-6, divided
    by their float sum when it exceeds 1e-6, else all 1 / n."""
    nw = [F32(F32(w) + F32(1e-6)) for w in weights]
    total = F32(0.0)
    for w in nw:
        total = F32(total + w)
    if float(total) > 0.000001:
        return [F32(w / total) for w in nw]
    return [F32(F32(1.0) / F32(len(nw)))] * len(nw)


def weighted_average(data, weights) -> np.ndarray:
    """WeightedAverage (math_util.h:51-70): float products of the normalised
    weights summed in double, then cast to float."""
    nw = normalize_weights(weights)
    acc = [0.0, 0.0, 0.0]
    for d, w in zip(data, nw):
        for k in range(3):
            acc[k] += float(F32(F32(d[k]) * w))
    return np.array(acc, np.float32)


def weighted_median(data, weights):
    """WeightedMedian (math_util.h:72-100): the element at which the float
    running sum of the ascending normalised weights first exceeds 0.5 (the
    first element when it never does).  The sort is stable, which is the
    order std::sort gives for up to 16 elements (insertion sort); for more,
    and only among equal weights, the C++ order is not fixed."""
    nw = normalize_weights(weights)
    order = sorted(range(len(data)), key=lambda i: float(nw[i]))
    total, index = F32(0.0), 0
    for i, j in enumerate(order):
        total = F32(total + nw[j])
        if total > F32(0.5):
            index = i
            break
    return data[order[index]]


def median(data, force_org_val: bool = False):
    """Median (math_util.h:102-124) of floats: one value as is; two values
    averaged (the first one with force_org_val); otherwise the (n/2)-th
    smallest for an even count or force_org_val (not the mean of the two
    middle ones), and for an odd count the mean of the middle one and the
    next larger one."""
    n = len(data)
    if n == 1:
        return F32(data[0])
    if n == 2:
        return F32(data[0]) if force_org_val else F32(F32(F32(data[0]) + F32(data[1])) * F32(0.5))
    srt = sorted(F32(x) for x in data)
    h = n // 2
    if force_org_val or n % 2 == 0:
        return srt[h]
    return F32(F32(srt[h] + srt[h + 1]) * F32(0.5))


def median_color(colors) -> np.ndarray:
    """MedianColor (src/util/math_util.cc:44-56): Median per channel."""
    return np.array([median([c[k] for c in colors]) for k in range(3)], np.float32)


def mode(colors, weights=None):
    """Both Mode overloads (math_util.h:127-180): counts (or float sums of
    `weights`) per distinct colour in visit order; the mode is the first
    colour whose total exceeds every earlier best.  Returns (mode, total,
    occurrence dict keyed by colour tuples)."""
    occ, best, freq = {}, None, (F32(0.0) if weights is not None else 0)
    for i, c in enumerate(colors):
        key = tuple(float(F32(x)) for x in c)
        if weights is None:
            occ[key] = occ.get(key, 0) + 1
        else:
            occ[key] = F32(occ.get(key, F32(0.0)) + F32(weights[i]))
        if freq < occ[key]:
            freq = occ[key]
            best = np.array(key, np.float32)
    return best, freq, occ


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
    """VertexInfo (visibility_tester.h:75-126)."""
    visible_keyframes: list = field(default_factory=list)
    mean_color: np.ndarray | None = None
    median_color: np.ndarray | None = None
    min_viewing_angle_index: int = -1
    min_viewing_angle_id: int = -1
    min_viewing_angle_color: np.ndarray | None = None
    mean_viewing_angle_color: np.ndarray | None = None    # weighted by 1 / viewing angle
    median_viewing_angle_color: np.ndarray | None = None  # weighted by 1 / viewing angle
    min_distance_index: int = -1
    min_distance_id: int = -1
    min_distance_color: np.ndarray | None = None
    mean_distance_color: np.ndarray | None = None    # weighted by 1 / distance
    median_distance_color: np.ndarray | None = None  # weighted by 1 / distance
    min_intensity: float = float(np.finfo(np.float32).max)
    median_intensity: float = float(np.finfo(np.float32).max)
    median_intensity_color: np.ndarray | None = None
    min_intensity_color: np.ndarray | None = None
    mean_viewing_angle: float = -1.0
    median_viewing_angle: float = -1.0
    mean_distance: float = -1.0
    median_distance: float = -1.0
    mode: np.ndarray | None = None
    mode_frequency: int = -1
    mode_viewing_angle_color: np.ndarray | None = None
    mode_frequency_viewing_angle_color: float = -1.0
    occurrence: dict = field(default_factory=dict)
    occurrence_viewing_angle: dict = field(default_factory=dict)

    def VisibleFrom(self, kf_id: int) -> int:  # visibility_tester.cc:178-194
        for i, v in enumerate(self.visible_keyframes):
            if v.kf_id == kf_id:
                return i
        return -1

    def CalcStat(self):  # visibility_tester.cc:68-176
        kfs = self.visible_keyframes
        if not kfs:
            return
        n = F32(len(kfs))
        colors = [np.asarray(kf.color, np.float32) for kf in kfs]
        dist = [F32(kf.distance) for kf in kfs]
        va = [F32(kf.viewing_angle) for kf in kfs]
        inten = [F32(kf.intensity) for kf in kfs]
        # float arithmetic as in C++: FLT_MAX distances sum to inf, 1 / 0 is
        # inf, and so on, without warnings
        with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
            mc = np.zeros(3, np.float32)
            md, mva = F32(0.0), F32(0.0)
            for kf in kfs:  # float sums in visit order
                mc = (mc + np.asarray(kf.color, np.float32)).astype(np.float32)
                md = F32(md + F32(kf.distance))
                mva = F32(mva + F32(kf.viewing_angle))
            self.mean_color = (mc / n).astype(np.float32)
            self.mean_distance = float(F32(md / n))
            self.mean_viewing_angle = float(F32(mva / n))
            inv_d = [F32(F32(1.0) / d) for d in dist]
            inv_va = [F32(F32(1.0) / a) for a in va]
            i = first_min(va)
            self.min_viewing_angle_index, self.min_viewing_angle_id = i, kfs[i].kf_id
            self.min_viewing_angle_color = kfs[i].color
            i = first_min(dist)
            self.min_distance_index, self.min_distance_id = i, kfs[i].kf_id
            self.min_distance_color = kfs[i].color
            self.median_viewing_angle = float(median(va))
            self.median_distance = float(median(dist))
            self.median_color = median_color(colors)
            self.mean_viewing_angle_color = weighted_average(colors, inv_va)
            self.mean_distance_color = weighted_average(colors, inv_d)
            self.median_viewing_angle_color = weighted_median(colors, inv_va)
            self.median_distance_color = weighted_median(colors, inv_d)
            i = first_min(inten)
            self.min_intensity, self.min_intensity_color = float(inten[i]), colors[i]
            mi = median(inten, True)
            self.median_intensity = float(mi)
            j = next((k for k, v in enumerate(inten) if v == mi), len(inten))  # std::find
            self.median_intensity_color = colors[j] if j < len(colors) else None
            self.mode, self.mode_frequency, self.occurrence = mode(colors)
            (self.mode_viewing_angle_color, f,
             self.occurrence_viewing_angle) = mode(colors, inv_va)
            self.mode_frequency_viewing_angle_color = float(f)


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
        a = [F32(f.area) for f in self.visible_keyframes]
        va = [F32(f.viewing_angle) for f in self.visible_keyframes]
        di = [F32(f.distance) for f in self.visible_keyframes]
        self.max_area_index = first_min([-x for x in a])  # std::max_element: first maximum
        self.max_area_id = self.visible_keyframes[self.max_area_index].kf_id
        self.min_viewing_angle_index = first_min(va)
        self.min_viewing_angle_id = self.visible_keyframes[self.min_viewing_angle_index].kf_id
        self.min_distance_index = first_min(di)
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


def tester_option(option: VisibilityTesterOption) -> VisibilityTesterOption:
    """The option a VisibilityTester keeps of `option`: its constructor and
    set_option copy it with VisibilityTesterOption::CopyTo
    (visibility_tester.cc:44-53, 297-308), which copies
    backface_culling_angle_rad_th, use_mask, use_depth, interp and the three
    statistics switches only.  max_viewing_angle,
    max_distance_from_camera_to_vertex, max_depth_difference and eps keep
    their defaults, whatever the caller set."""
    t = VisibilityTesterOption()
    for k in ("backface_culling_angle_rad_th", "use_mask", "use_depth", "interp",
              "calc_stat_vertex_info", "collect_face_info", "calc_stat_face_info"):
        setattr(t, k, getattr(option, k))
    return t


class VisibilityTester:
    """ugu::VisibilityTester's interface (visibility_tester.h:216-265)."""

    def __init__(self, option: VisibilityTesterOption | None = None, device: int = 0):
        self._ctx = Context(device)
        self._option = tester_option(option) if option is not None else VisibilityTesterOption()
        self._mesh = None
        self._normals = None
        self._initialized = False
        self._keyframe = None

    def set_option(self, option: VisibilityTesterOption) -> None:
        self._option = tester_option(option)

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

    def raw(self, keyframes, facewise: bool, option: VisibilityTesterOption | None = None) -> dict:
        """The device results for all keyframes, keyframe-major arrays.
        `option`, when given, goes to the device as it is (every threshold
        of ugu_gpu_test_visibility); by default the tester's own."""
        opt = option if option is not None else self._option
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
        self._ctx.check(self._ctx.test_visibility(0, self._normals, descs, opt.to_struct(),
                                                  facewise, out))
        return res

    def Test(self, info: VisibilityInfo, facewise: bool = True, keyframes=None) -> bool:
        """Test(info, facewise) for the keyframe set by set_keyframe, or
        Test(keyframes, info, facewise) (:670-731) for a list, in one launch."""
        kfs = keyframes if keyframes is not None else [self._keyframe]
        if not kfs or any(k is None for k in kfs):
            return False
        res = self.raw(kfs, facewise)
        assemble_visibility_info(info, [int(kf.id) for kf in kfs], res,
                                 self._mesh.vertex_indices, self._option, facewise)
        return True


def assemble_visibility_info(info: VisibilityInfo, kf_ids, res: dict, faces,
                             option: VisibilityTesterOption, facewise: bool) -> None:
    """The host half of VisibilityTester::Test(keyframes, info, facewise)
    (visibility_tester.cc:670-731): the per-keyframe results `res`
    (keyframe-major arrays, as VisibilityTester.raw returns them) appended to
    `info` keyframe by keyframe as TestVertices / TestFaces (:416-604) or
    TestFacewiseVertices (:606-668) append them, then the statistics."""
    F = np.asarray(faces)
    for k, kid in enumerate(kf_ids):
        vis = res["visible"][k]

        def rec(i):
            return VertexInfoPerKeyframe(int(kid), res["color"][k, i].copy(),
                                         float(res["intensity"][k, i]),
                                         res["projected_pos"][k, i].copy(),
                                         float(res["viewing_angle"][k, i]),
                                         float(res["distance"][k, i]))
        if not facewise:
            for i in np.nonzero(vis)[0]:
                info.vertex_info_list[i].visible_keyframes.append(rec(i))
            if option.collect_face_info:
                for f in range(len(F)):  # TestFaces (:551-604)
                    vinf = []
                    for j in range(3):
                        vi = info.vertex_info_list[F[f, j]]
                        idx = vi.VisibleFrom(kid)
                        if idx < 0:
                            break
                        vinf.append(vi.visible_keyframes[idx])
                    if len(vinf) < 3:
                        continue
                    _face_record(info, kid, f, vinf)
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
                _face_record(info, kid, f, vinf)
    if option.calc_stat_vertex_info:
        info.CalcStatVertexInfo()
    if option.calc_stat_face_info:
        info.CalcStatFaceInfo()


def _face_record(info, kf_id, f, vinf):
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


# --- TextureMapping (include/ugu/texturing/texture_mapper.h,
#     src/texturing/texture_mapper.cc) --------------------------------------

class ViewSelectionCriteria:  # visibility_tester.h:23-37
    kMinViewingAngle = 0
    kMinDistance = 1
    kMaxArea = 6


class TexturingOutputUvType:  # texture_mapper.h:14-19
    kGenerateSimpleTile = 0
    kUseOriginalMeshUv = 1
    kGenerateSimpleTriangles = 2
    kGenerateSimpleCharts = 3


@dataclass
class TextureMappingOption:
    """TextureMappingOption (texture_mapper.h:22-30), same defaults."""
    criteria: int = ViewSelectionCriteria.kMaxArea
    type: int = 0  # TextureMappingType::kSimpleProjection
    uv_type: int = TexturingOutputUvType.kGenerateSimpleTile
    texture_base_name: str = "ugutex"
    tex_w: int = 1024
    tex_h: int = 1024
    padding_kernel: int = 3


def best_keyframes(info: VisibilityInfo, criteria: int):
    """Each face's best keyframe (texture_mapper.cc:938-970): the
    FaceInfoPerKeyframe at FaceInfo's min-viewing-angle, min-distance or
    max-area index.  Returns (kf id per face, -1 for faces seen by none;
    projected triangle per face, F x 3 x 2)."""
    pick = {ViewSelectionCriteria.kMinViewingAngle: "min_viewing_angle_index",
            ViewSelectionCriteria.kMinDistance: "min_distance_index",
            ViewSelectionCriteria.kMaxArea: "max_area_index"}.get(criteria)
    if pick is None:
        raise ValueError(f"ViewSelectionCriteria {criteria} is not implemented")
    F = len(info.face_info_list)
    face_kf = np.full(F, -1, np.int32)
    face_tri = np.zeros((F, 3, 2), np.float32)
    for f, fi in enumerate(info.face_info_list):
        if not fi.visible_keyframes:
            continue
        best = fi.visible_keyframes[getattr(fi, pick)]
        face_kf[f] = best.kf_id
        face_tri[f] = np.asarray(best.projected_tri, np.float32)
    return face_kf, face_tri


def simple_tile_layout(keyframes, face_kf, face_tri):
    """GenerateSimpleTileTextureAndUv's layout (texture_mapper.cc:62-141):
    the keyframe images tiled x_tiles = (int)sqrt(n) wide and n / x_tiles
    high, and each face's uv: its projected triangle moved to its best
    keyframe's tile, (x + 0.5) / tex_w and 1 - (y + 0.5) / tex_h, in float.
    A keyframe id maps to its position in the list (an unknown id to 0, as
    the reference's std::unordered_map::operator[] does); faces seen by no
    keyframe get zero uv.  Returns (x_tiles, y_tiles, uv F*3 x 2), or None
    when the images would not fill whole rows of tiles or differ in size
    (the reference then writes past its texture)."""
    n = len(keyframes)
    if n == 0:
        return None
    x_tiles = int(math.sqrt(float(n)))
    x_tiles = n if n < x_tiles else x_tiles
    y_tiles = n // x_tiles
    h, w = keyframes[0].color.shape[:2]
    if n % x_tiles or any(k.color.shape[:2] != (h, w) for k in keyframes):
        return None
    tex_w, tex_h = F32(x_tiles * w), F32(y_tiles * h)
    index = {}
    for i, k in enumerate(keyframes):
        index.setdefault(int(k.id), i)  # std::unordered_map::emplace keeps the first
    F = len(face_kf)
    uv = np.zeros((F, 3, 2), F32)
    for f in range(F):
        if face_kf[f] < 0:
            continue
        i = index.get(int(face_kf[f]), 0)
        tx, ty = F32((i % x_tiles) * w), F32((i // x_tiles) * h)
        for j in range(3):
            x = F32(face_tri[f, j, 0]) + tx
            y = F32(face_tri[f, j, 1]) + ty
            uv[f, j, 0] = (x + F32(0.5)) / tex_w
            uv[f, j, 1] = F32(1.0) - ((y + F32(0.5)) / tex_h)
    return x_tiles, y_tiles, uv.reshape(-1, 2)


def simple_triangles_layout(face_kf, tex_w: int, tex_h: int):
    """GenerateSimpleTrianglesTextureAndUv's layout (texture_mapper.cc:
    347-440): faces 2r and 2r + 1 share rectangle r of sq_len + 2 by
    sq_len + 1 texels (2 texels apart), the largest sq_len <= 100 for which
    all fit; the even face takes the upper-right triangle shifted right by
    2, the odd one the lower-left shifted down by 1.  Returns (target
    triangles F x 3 x 2 in texel coordinates, uv F*3 x 2: (t + 0.5) / size,
    flipped in y; zeros for faces seen by no keyframe), or None where the
    reference returns false (fewer than 6 texels per rectangle, sq_len
    under 3)."""
    pad = 2
    F = len(face_kf)
    rect_num = (F + 1) // 2
    if rect_num == 0:
        return np.zeros((0, 3, 2), F32), np.zeros((0, 2), F32)
    pix_per_rect = tex_h * tex_w // rect_num
    if pix_per_rect < 6:
        return None
    sq_len = min(int(math.sqrt(float(pix_per_rect))), 100)

    def fits(q):
        return (tex_w // (q + 2 + pad)) * (tex_h // (q + 1 + pad))
    while fits(sq_len) < rect_num:
        sq_len -= 1
        if sq_len < 3:
            return None
    rect_w, rect_h = sq_len + 2, sq_len + 1
    rect_w_num = tex_w // (rect_w + pad)
    target = np.zeros((F, 3, 2), F32)
    uv = np.zeros((F, 3, 2), F32)
    for i in range(F):
        if face_kf[i] < 0:
            continue
        rid = i // 2
        rx, ry = rid % rect_w_num, rid // rect_w_num
        if i % 2 == 0:
            x0 = (rect_w + pad) * rx + 2
            y0 = (rect_h + pad) * ry
            x1, y1 = x0 + sq_len - 1, y0 + sq_len - 1
            t = [(x0, y0), (x1, y0), (x1, y1)]
        else:
            x0 = (rect_w + pad) * rx
            y0 = (rect_h + pad) * ry + 1
            x1, y1 = x0 + sq_len - 1, y0 + sq_len - 1
            t = [(x0, y0), (x0, y1), (x1, y1)]
        for j, (x, y) in enumerate(t):
            target[i, j] = (x, y)
            uv[i, j, 0] = (F32(x) + F32(0.5)) / F32(tex_w)
            uv[i, j, 1] = F32(1.0) - ((F32(y) + F32(0.5)) / F32(tex_h))
    return target, uv.reshape(-1, 2)


def bin_packing_2d(rects, x_min: int, x_max: int, y_min: int, y_max: int):
    """BinPacking2D (src/discrete/bin_packer_2d.cc:14-113): guillotine
    packing of (width, height) rectangles in the given order into the free
    rectangle (x_min, y_min, x_max, y_max) (x, y, width, height).  Each
    rectangle takes the free one whose area exceeds its own the least
    (the first of equals); a larger one is cut across the longer leftover
    side, the remainder appended before the piece, until one fits exactly.
    Returns (packed (x, y, w, h) list, free rectangles), or None when a
    rectangle finds no room."""
    free = [(x_min, y_min, x_max, y_max)]
    packed = []
    for (w, h) in rects:
        while True:
            best, best_i = None, -1
            best_diff = 2 ** 31 - 1
            for i, (fx, fy, fw, fh) in enumerate(free):
                if h <= fh and w <= fw and fw * fh - w * h < best_diff:
                    best_diff = fw * fh - w * h
                    best, best_i = (fx, fy, fw, fh), i
            if best_i < 0 or best[2] * best[3] < w * h:
                return None
            fx, fy, fw, fh = best
            if fw == w and fh == h:
                packed.append(best)
                del free[best_i]
                break
            if fh - h > fw - w:  # CutRect: across the longer leftover side
                cut1, cut2 = (fx, fy, fw, h), (fx, fy + h, fw, fh - h)
            else:
                cut1, cut2 = (fx, fy, w, fh), (fx + w, fy, fw - w, fh)
            del free[best_i]
            free.append(cut2)
            free.append(cut1)
    return packed, free


def simple_charts_layout(vertex_indices, face_kf, face_tri, keyframes, tex_w: int, tex_h: int):
    """GenerateSimpleChartsTextureAndUv with GenerateAtlas
    (texture_mapper.cc:476-922): charts are the faces reachable from the
    lowest unselected face over shared edges (FaceAdjacency,
    include/ugu/face_adjacency.h: a face's neighbours own the reversed
    directed edges; duplicate directed edges sum, as setFromTriplets does)
    that have the seed's best keyframe.  A visible chart's patch is the
    bounding box of its projected triangles (floor / ceil) copied from the
    keyframe image with a 1-texel border replicated (PaddingBorderSimple);
    its vertices keep one texture position each (the first face's, in
    vertex order as std::map keeps them).  Visible charts are packed by
    patch area, largest first (std::sort; the mirror's sort is stable, so
    charts of equal area keep their chart order where libstdc++'s is
    unspecified), with BinPacking2D into the texture less a 1-texel edge,
    which grows by sqrt(2) steps up to 8192 until everything fits.  Faces
    of unseen charts share one uv at the first free rectangle (or 0, 0).
    Returns (texture H x W x 3, uv, uv_indices F x 3, mask H x W: 255 on
    the patches), or None where the reference fails (no packing within 8192) or reads past its arrays (a
    patch outside its keyframe image, an edge sum naming no face)."""
    from collections import deque
    vi = np.asarray(vertex_indices, np.int64)
    F = len(vi)
    edges = {}
    for f in range(F):
        a, b, c = (int(x) for x in vi[f])
        for e in ((a, b), (b, c), (c, a)):
            edges[e] = edges.get(e, 0) + f + 1
    selected = np.zeros(F, bool)
    charts = []  # (kf, faces) in the order of their seeds
    for seed in range(F):
        if selected[seed]:
            continue
        kf = int(face_kf[seed])
        faces = [seed]
        selected[seed] = True
        queue = deque([seed])
        while queue:
            fid = queue.popleft()
            a, b, c = (int(x) for x in vi[fid])
            adjacent = [edges.get(e, 0) - 1 for e in ((b, a), (c, b), (a, c))]
            adjacent = [g for g in adjacent if g >= 0]
            for e in ((a, b), (b, c), (c, a)):  # RemoveFace
                if e in edges:
                    edges[e] = 0
            if any(g >= F for g in adjacent):
                return None
            add = [g for g in adjacent if int(face_kf[g]) == kf and not selected[g]]
            for g in add:
                queue.append(g)
                faces.append(g)
                selected[g] = True
        charts.append((kf, faces))
    pad = 1
    valid = []  # (area, patch, vertex ids, positions, face uv-index lists)
    invalid_faces = []
    for kf, faces in charts:
        if kf < 0:
            invalid_faces.extend(faces)
            continue
        tris = np.asarray(face_tri, F32)[faces]  # n x 3 x 2
        xmin, xmax = int(math.floor(tris[:, :, 0].min())), int(math.ceil(tris[:, :, 0].max()))
        ymin, ymax = int(math.floor(tris[:, :, 1].min())), int(math.ceil(tris[:, :, 1].max()))
        img = keyframes[kf].color
        if xmin < 0 or ymin < 0 or xmax >= img.shape[1] or ymax >= img.shape[0]:
            return None
        ph, pw = ymax - ymin + 1 + 2 * pad, xmax - xmin + 1 + 2 * pad
        patch = np.zeros((ph, pw, 3), np.uint8)
        patch[pad:pad + ymax - ymin + 1, pad:pad + xmax - xmin + 1] = img[ymin:ymax + 1,
                                                                          xmin:xmax + 1]
        patch[:pad] = patch[pad]  # PaddingBorderSimple (:203-231)
        patch[ph - pad:] = patch[ph - pad - 1]
        patch[:, :pad] = patch[:, pad:pad + 1]
        patch[:, pw - pad:] = patch[:, pw - pad - 1:pw - pad]
        pos = {}
        for k, f in enumerate(faces):
            for j in range(3):
                p = (F32(tris[k, j, 0]) - F32(xmin) + F32(pad),
                     F32(tris[k, j, 1]) - F32(ymin) + F32(pad))
                pos.setdefault(int(vi[f, j]), p)
        vids = sorted(pos)
        new = {v: i for i, v in enumerate(vids)}
        valid.append((ph * pw, patch, [pos[v] for v in vids],
                      [(f, [new[int(vi[f, j])] for j in range(3)]) for f in faces]))
    valid.sort(key=lambda c: -c[0])
    rects = [(c[1].shape[1], c[1].shape[0]) for c in valid]
    cur_w, cur_h, tries = int(tex_w), int(tex_h), 0
    ratio = float(F32(math.sqrt(2.0)))
    while True:
        got = bin_packing_2d(rects, 1, cur_w - 1, 1, cur_h - 1)
        if got is not None:
            break
        tries += 1
        cur_w = int(tex_w * math.pow(ratio, tries))
        cur_h = int(tex_h * math.pow(ratio, tries))
        if 8192 < cur_w or 8192 < cur_h:
            return None
    packed, free = got
    tex = np.zeros((cur_h, cur_w, 3), np.uint8)
    mask = np.zeros((cur_h, cur_w), np.uint8)
    uv = []
    uv_indices = np.zeros((F, 3), np.int32)
    cols, rows = F32(cur_w), F32(cur_h)
    for (area, patch, positions, face_idx), (rx, ry, rw, rh) in zip(valid, packed):
        tex[ry:ry + patch.shape[0], rx:rx + patch.shape[1]] = patch
        mask[ry:ry + patch.shape[0], rx:rx + patch.shape[1]] = 255
        off = len(uv)
        for (px, py) in positions:
            uv.append(((px + F32(rx) + F32(0.5)) / cols,
                       F32(1.0) - ((py + F32(ry) + F32(0.5)) / rows)))
        for f, idx in face_idx:
            uv_indices[f] = [off + k for k in idx]
    inv = (F32(0.0), F32(0.0))
    if free:
        inv = ((F32(free[0][0]) + F32(0.5)) / cols, F32(1.0) - ((F32(free[0][1]) + F32(0.5)) / rows))
    uv.extend([inv, inv, inv])
    for f in invalid_faces:
        uv_indices[f] = [len(uv) - 3, len(uv) - 2, len(uv) - 1]
    return tex, np.asarray(uv, F32).reshape(-1, 2), uv_indices, mask


def _keyframe_descs(keyframes):
    descs, keep = [], []
    for kf in keyframes:
        d = capi.KeyframeDesc()
        d.id = int(kf.id)
        d.camera = capi.camera_struct(kf.camera)
        c = np.ascontiguousarray(kf.color, np.uint8)
        keep.append(c)
        d.color = c.ctypes.data
        descs.append(d)
    return descs, keep


def TextureMapping(keyframes, info: VisibilityInfo, mesh, option: TextureMappingOption,
                   ctx: Context | None = None, slot: int = 0) -> bool:
    """TextureMapping (texture_mapper.cc:1009-1017) with kSimpleProjection,
    each face textured from its best keyframe (:924-970), for three uv
    types:
      kGenerateSimpleTile (the default): the keyframe images tiled into one
        texture on the GPU (ugu_gpu_tile_images), the faces' uv moved to
        their keyframe's tile (simple_tile_layout);
      kUseOriginalMeshUv: a tex_h x tex_w texture drawn on the GPU on the
        mesh's own uv (ugu_gpu_texture_mapping), then padded;
      kGenerateSimpleTriangles: every visible face drawn on the GPU into
        its own half-rectangle of a tex_h x tex_w texture
        (simple_triangles_layout, ugu_gpu_texture_mapping_targets), padded
        with a 3-texel window; new uv and uv indices;
      kGenerateSimpleCharts: charts of edge-connected faces sharing a best
        keyframe, each a padded bounding-box patch of that keyframe's image,
        bin-packed into a texture that grows from tex_h x tex_w as needed
        (simple_charts_layout: host work, as in the reference); new uv and
        uv indices.
    Like the reference, it sets the mesh's one material to the texture and
    every face's material id to 0; the texture's mask (255 where a face, a
    patch or the padding wrote; all 255 for tiles) is left in
    mesh.texture_mask.  A layout the reference rejects or would overrun
    returns False."""
    if option.type != 0 or option.uv_type not in (TexturingOutputUvType.kGenerateSimpleTile,
                                                  TexturingOutputUvType.kUseOriginalMeshUv,
                                                  TexturingOutputUvType.kGenerateSimpleTriangles,
                                                  TexturingOutputUvType.kGenerateSimpleCharts):
        return False
    face_kf, face_tri = best_keyframes(info, option.criteria)
    F = len(mesh.vertex_indices)
    if option.uv_type == TexturingOutputUvType.kGenerateSimpleTile:
        lay = simple_tile_layout(keyframes, face_kf, face_tri)
        if lay is None:
            return False
        x_tiles, y_tiles, uv = lay
        ctx = ctx or Context(0)
        descs, keep = _keyframe_descs(keyframes)
        h, w = keyframes[0].color.shape[:2]
        tex = np.zeros((y_tiles * h, x_tiles * w, 3), np.uint8)
        ctx.check(ctx.tile_images(descs, x_tiles, tex))
        mesh.uv = uv
        mesh.uv_indices = np.arange(3 * F, dtype=np.int32).reshape(-1, 3)
        mesh.textures = [tex]
        mesh.textures_f32 = [None]
        mesh.material_ids = np.zeros(F, np.int32)
        mesh.texture_mask = np.full(tex.shape[:2], 255, np.uint8)
        return True
    if option.uv_type == TexturingOutputUvType.kGenerateSimpleCharts:
        lay = simple_charts_layout(mesh.vertex_indices, face_kf, face_tri, keyframes,
                                   int(option.tex_w), int(option.tex_h))
        if lay is None:
            return False
        tex, uv, uv_indices, mask = lay
        mesh.uv = uv
        mesh.uv_indices = uv_indices
        mesh.textures = [tex]
        mesh.textures_f32 = [None]
        mesh.material_ids = np.zeros(F, np.int32)
        mesh.texture_mask = mask
        return True
    if option.uv_type == TexturingOutputUvType.kGenerateSimpleTriangles:
        lay = simple_triangles_layout(face_kf, int(option.tex_w), int(option.tex_h))
        if lay is None:
            return False
        target, uv = lay
        ctx = ctx or Context(0)
        descs, keep = _keyframe_descs(keyframes)
        tex = np.zeros((option.tex_h, option.tex_w, 3), np.uint8)
        mask = np.zeros((option.tex_h, option.tex_w), np.uint8)
        opt = capi.TextureOption(int(option.tex_w), int(option.tex_h), 3)  # :430
        ctx.check(ctx.texture_mapping_targets(target.reshape(-1, 6), descs, face_kf,
                                              face_tri.reshape(-1, 6), opt, tex, mask))
        mesh.uv = uv
        mesh.uv_indices = np.arange(3 * F, dtype=np.int32).reshape(-1, 3)
        mesh.textures = [tex]
        mesh.textures_f32 = [None]
        mesh.material_ids = np.zeros(F, np.int32)
        mesh.texture_mask = mask
        return True
    if (mesh.uv is None or len(mesh.uv) == 0 or mesh.uv_indices is None
            or len(mesh.uv_indices) != len(mesh.vertex_indices)):
        return False  # :986-993
    ctx = ctx or Context(0)
    ctx.check(ctx.set_mesh(slot, mesh))
    descs, keep = _keyframe_descs(keyframes)
    tex = np.zeros((option.tex_h, option.tex_w, 3), np.uint8)
    mask = np.zeros((option.tex_h, option.tex_w), np.uint8)
    opt = capi.TextureOption(int(option.tex_w), int(option.tex_h), int(option.padding_kernel))
    ctx.check(ctx.texture_mapping(slot, descs, face_kf, face_tri.reshape(-1, 6), opt, tex, mask))
    mesh.textures = [tex]
    mesh.textures_f32 = [None]
    mesh.material_ids = np.zeros(len(mesh.vertex_indices), np.int32)
    mesh.texture_mask = mask
    return True
