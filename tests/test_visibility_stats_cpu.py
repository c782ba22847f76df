"""VertexInfo::CalcStat's statistics in the Python mirror of ugu's
VisibilityTester (ugu_gb300/visibility.py), against the rules of ugu's
math helpers (include/ugu/util/math_util.h:28-180, src/util/math_util.cc:44-56)
and of visibility_tester.cc:68-176, on hand-made inputs whose results follow
from those rules: the median's quirks (no averaging for an even count, the
first value for two with force_org_val), normalised weights with their
1e-6 offset, the weighted median's running sum, the first-best mode, and
float sums in visit order."""
import numpy as np

from ugu_gb300 import visibility as vis

F32 = np.float32


def test_first_min_is_std_min_element():
    assert vis.first_min([3.0, 1.0, 1.0, 2.0]) == 1
    assert vis.first_min([F32("nan"), 1.0, 0.0]) == 0  # nothing is < NaN
    assert vis.first_min([1.0, F32("nan"), 0.0]) == 2


def test_median_rules():
    assert vis.median([7.0]) == F32(7.0)
    assert vis.median([5.0, 1.0]) == F32(3.0)
    assert vis.median([5.0, 1.0], True) == F32(5.0)   # the first value, unsorted
    assert vis.median([3.0, 1.0, 2.0]) == F32(2.5)     # (middle + next) / 2
    assert vis.median([4.0, 1.0, 3.0, 2.0]) == F32(3.0)  # the upper middle, not 2.5
    assert vis.median([5.0, 4.0, 3.0, 2.0, 1.0], True) == F32(3.0)
    assert vis.median([5.0, 4.0, 3.0, 2.0, 1.0]) == F32(3.5)
    c = vis.median_color([[0, 10, 5], [2, 30, 5], [1, 20, 5]])
    assert np.array_equal(c, np.array([1.5, 25.0, 5.0], np.float32))


def test_normalize_weights():
    nw = vis.normalize_weights([1.0, 3.0])
    assert nw[0].dtype == np.float32
    s = F32(F32(1.0) + F32(1e-6)) + F32(F32(3.0) + F32(1e-6))
    assert nw[0] == F32(F32(F32(1.0) + F32(1e-6)) / F32(s))
    # a sum at or below 1e-6: even weights
    assert vis.normalize_weights([-1e-6, -1e-6, -1e-6]) == [F32(F32(1.0) / F32(3))] * 3


def test_weighted_average_and_median():
    data = [np.array(c, np.float32) for c in ([0, 0, 0], [10, 20, 30], [100, 100, 100])]
    avg = vis.weighted_average(data[:2], [1.0, 3.0])
    assert np.allclose(avg, [7.5, 15.0, 22.5], rtol=1e-5)
    # equal weights: the plain mean, summed in double
    assert np.allclose(vis.weighted_average(data, [2.0, 2.0, 2.0]), [110 / 3, 40.0, 130 / 3],
                       rtol=1e-6)
    # ascending weights 0.1 (A), 0.3 (C), 0.6 (B): the running sum passes 0.5 at B
    assert vis.weighted_median(data, [1.0, 6.0, 3.0]) is data[1]
    # four equal weights: 0.25, 0.5 (not above 0.5), 0.75 -> the third, in input order
    four = data + [np.array([7, 7, 7], np.float32)]
    assert vis.weighted_median(four, [1.0, 1.0, 1.0, 1.0]) is four[2]


def test_mode_first_best():
    a, b, c = (np.array(x, np.float32) for x in ([1, 2, 3], [4, 5, 6], [7, 8, 9]))
    m, f, occ = vis.mode([a, b, b, a, c])
    assert np.array_equal(m, b) and f == 2  # a reaches 2 later, not above b's 2
    assert occ[(1.0, 2.0, 3.0)] == 2 and occ[(7.0, 8.0, 9.0)] == 1
    m, f, occ = vis.mode([a, b, b, a, c], [3.0, 1.0, 1.0, 1.0, 0.5])
    assert np.array_equal(m, a) and f == F32(4.0)


def _kf(kid, color, intensity, va, dist):
    return vis.VertexInfoPerKeyframe(kid, np.array(color, np.float32), float(F32(intensity)),
                                     np.zeros(2, np.float32), float(F32(va)), float(F32(dist)))


def test_vertex_calc_stat():
    rng = np.random.default_rng(3)
    kfs = [_kf(10 + i, rng.integers(0, 256, 3).astype(np.float32), rng.uniform(0, 255),
               rng.uniform(0.05, 1.5), rng.uniform(0.5, 4.0)) for i in range(11)]
    kfs.append(_kf(99, kfs[3].color, kfs[3].intensity, 2.0, 9.0))  # a repeated colour
    v = vis.VertexInfo(visible_keyframes=list(kfs))
    v.CalcStat()
    # float sums in visit order, then one float division
    s = F32(0.0)
    for kf in kfs:
        s = F32(s + F32(kf.distance))
    assert v.mean_distance == float(F32(s / F32(len(kfs))))
    mc = np.zeros(3, np.float32)
    for kf in kfs:
        mc = (mc + kf.color).astype(np.float32)
    assert np.array_equal(v.mean_color, (mc / F32(len(kfs))).astype(np.float32))
    va = [kf.viewing_angle for kf in kfs]
    i = int(np.argmin(va))
    assert (v.min_viewing_angle_index, v.min_viewing_angle_id) == (i, kfs[i].kf_id)
    assert v.median_viewing_angle == float(vis.median([F32(x) for x in va]))
    inten = [F32(kf.intensity) for kf in kfs]
    assert v.min_intensity == float(min(inten))
    assert v.median_intensity == float(sorted(inten)[len(inten) // 2])
    assert np.array_equal(v.median_intensity_color,
                          kfs[[F32(x) for x in inten].index(F32(v.median_intensity))].color)
    assert np.array_equal(v.mode, kfs[3].color) and v.mode_frequency == 2
    assert v.mean_viewing_angle_color.shape == (3,) and v.median_distance_color is not None
    # the mean weighted by 1 / distance leans to the nearest keyframes
    w = np.array([1.0 / kf.distance for kf in kfs])
    ref = (np.array([kf.color for kf in kfs], np.float64) * (w / w.sum())[:, None]).sum(0)
    assert np.allclose(v.mean_distance_color, ref, rtol=1e-4)


def test_vertex_calc_stat_float_overflow_is_silent():
    """The tester's no-hit quirk reports FLT_MAX distances: their float sum
    is inf, as in C++, and no warning is raised."""
    import warnings
    big = float(np.finfo(np.float32).max)
    v = vis.VertexInfo(visible_keyframes=[_kf(1, [1, 2, 3], 10, 0.5, big),
                                          _kf(2, [4, 5, 6], 20, 0.0, big)])
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        v.CalcStat()
    assert v.mean_distance == float("inf")
    assert v.min_viewing_angle_index == 1


def test_face_calc_stat_first_max_area():
    f = vis.FaceInfo(visible_keyframes=[
        vis.FaceInfoPerKeyframe(1, 0, 4.0, 0.5, 2.0, np.zeros((3, 2), np.float32)),
        vis.FaceInfoPerKeyframe(2, 0, 9.0, 0.2, 3.0, np.zeros((3, 2), np.float32)),
        vis.FaceInfoPerKeyframe(3, 0, 9.0, 0.2, 1.0, np.zeros((3, 2), np.float32))])
    f.CalcStat()
    assert (f.max_area_index, f.max_area_id) == (1, 2)          # the first of the equal maxima
    assert (f.min_viewing_angle_index, f.min_viewing_angle_id) == (1, 2)
    assert (f.min_distance_index, f.min_distance_id) == (2, 3)
