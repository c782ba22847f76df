// geom_util.h override -- TEST INFRASTRUCTURE ONLY.
//
// The reference's include/ugu/util/geom_util.h pulls in face adjacency
// (Eigen's sparse module and dynamic matrices), lines and planes, none of
// which the Eigen-compatible shim provides.  The raytracer and the naive BVH
// (src/renderer/cpu/raytracer.cc, include/ugu/accel/bvh_naive.h,
// bvh_base.h) use only the declarations below; this header, first on the
// include path, stands in for it so that those sources compile unmodified.
// Declarations follow include/ugu/util/geom_util.h:95-135 and 153-172;
// the ray-triangle test is restated in geom_min.cc.
#pragma once

#include <cstdint>
#include <numeric>
#include <optional>
#include <set>
#include <vector>

#include "ugu/mesh.h"

namespace ugu {

void SetRandomUniformVertexColor(MeshPtr mesh, int seed = 0);
MeshPtr MakeCube(const Eigen::Vector3f& length);

// Success: (t, u, v), failure: nullopt (geom_util.h:100-115)
std::optional<Eigen::Vector3f> Intersect(const Eigen::Vector3f& origin, const Eigen::Vector3f& ray,
                                         const Eigen::Vector3f& v0, const Eigen::Vector3f& v1,
                                         const Eigen::Vector3f& v2, const float kEpsilon = 1e-6f,
                                         bool standard_barycentric = true);
std::optional<Eigen::Vector3d> Intersect(const Eigen::Vector3d& origin, const Eigen::Vector3d& ray,
                                         const Eigen::Vector3d& v0, const Eigen::Vector3d& v1,
                                         const Eigen::Vector3d& v2, const double kEpsilon = 1e-20,
                                         bool standard_barycentric = true);

// origin + ray * t == (1-u-v)*v0 + u*v1 + v*v2 (geom_util.h:117-124)
struct IntersectResult {
  float t = -1.f;
  float u = -1.f;
  float v = -1.f;
  uint32_t fid = uint32_t(~0);
};

std::vector<IntersectResult> Intersect(const Eigen::Vector3f& origin, const Eigen::Vector3f& ray,
                                       const std::vector<Eigen::Vector3f>& vertices,
                                       const std::vector<Eigen::Vector3i>& faces,
                                       int num_threads = 1, const float kEpsilon = 1e-10f,
                                       bool standard_barycentric = true);

// Componentwise bounds of a point set, the first point when it is the only
// one (geom_util.h:153-172).
template <typename T>
T ComputeMinBound(const std::vector<T>& points) {
  if (points.empty()) return T::Zero();
  T r = points[0];
  for (const T& p : points)
    for (int i = 0; i < r.rows(); ++i) r[i] = p[i] < r[i] ? p[i] : r[i];
  return r;
}

template <typename T>
T ComputeMaxBound(const std::vector<T>& points) {
  if (points.empty()) return T::Zero();
  T r = points[0];
  for (const T& p : points)
    for (int i = 0; i < r.rows(); ++i) r[i] = r[i] < p[i] ? p[i] : r[i];
  return r;
}

}  // namespace ugu
