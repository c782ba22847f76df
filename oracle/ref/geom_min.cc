// geom_min.cc -- TEST INFRASTRUCTURE ONLY.
//
// The ray-triangle intersection the naive BVH calls
// (src/util/geom_util.cc:60-115 and 1397-1481), restated for the
// raytracer's pinning build: src/util/geom_util.cc itself needs the parts
// of Eigen the shim does not provide.  Moller-Trumbore in the scalar type of
// the call, with the reference's checks and its conversion of (u, v) to the
// "standard" barycentric pair (weight of v0, weight of v1).
#include "ugu/util/geom_util.h"

namespace ugu {

namespace {

template <typename T>
std::optional<T> moller_trumbore(const T& origin, const T& ray, const T& v0, const T& v1,
                                 const T& v2, const typename T::Scalar eps, bool standard) {
  using S = typename T::Scalar;
  const T e1 = v1 - v0;
  const T e2 = v2 - v0;
  const T alpha = ray.cross(e2);
  const S det = e1.dot(alpha);
  if (-eps < det && det < eps) return std::nullopt;  // parallel or degenerate
  const S inv_det = S(1.0) / det;
  const T r = origin - v0;
  S u = alpha.dot(r) * inv_det;
  if (u < 0.0f || u > 1.0f) return std::nullopt;
  const T beta = r.cross(e1);
  S v = ray.dot(beta) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return std::nullopt;
  const S t = e2.dot(beta) * inv_det;
  if (t < 0.0f) return std::nullopt;
  if (standard) {
    const S w = 1 - u - v;
    v = u;
    u = w;
  }
  return T(t, u, v);
}

}  // namespace

std::optional<Eigen::Vector3f> Intersect(const Eigen::Vector3f& origin, const Eigen::Vector3f& ray,
                                         const Eigen::Vector3f& v0, const Eigen::Vector3f& v1,
                                         const Eigen::Vector3f& v2, const float eps,
                                         bool standard) {
  return moller_trumbore(origin, ray, v0, v1, v2, eps, standard);
}

std::optional<Eigen::Vector3d> Intersect(const Eigen::Vector3d& origin, const Eigen::Vector3d& ray,
                                         const Eigen::Vector3d& v0, const Eigen::Vector3d& v1,
                                         const Eigen::Vector3d& v2, const double eps,
                                         bool standard) {
  return moller_trumbore(origin, ray, v0, v1, v2, eps, standard);
}

// Every face the ray hits, in face order, tested in double (the
// single-threaded branch: the naive BVH calls it with one thread).
std::vector<IntersectResult> Intersect(const Eigen::Vector3f& origin, const Eigen::Vector3f& ray,
                                       const std::vector<Eigen::Vector3f>& vertices,
                                       const std::vector<Eigen::Vector3i>& faces, int num_threads,
                                       const float eps, bool standard) {
  (void)num_threads;
  std::vector<IntersectResult> results;
  for (size_t i = 0; i < faces.size(); ++i) {
    const Eigen::Vector3i& f = faces[i];
    auto hit = Intersect(origin.cast<double>(), ray.cast<double>(), vertices[f[0]].cast<double>(),
                         vertices[f[1]].cast<double>(), vertices[f[2]].cast<double>(),
                         double(eps), standard);
    if (hit) {
      const Eigen::Vector3f tuv = hit.value().cast<float>();
      IntersectResult r;
      r.fid = static_cast<uint32_t>(i);
      r.t = tuv[0];
      r.u = tuv[1];
      r.v = tuv[2];
      results.emplace_back(r);
    }
  }
  return results;
}

}  // namespace ugu
