// bvh.cu -- host build of the raytracer's bounding-volume hierarchy.
//
// ugu::Raytracer builds ugu::BvhNaive (include/ugu/accel/bvh_naive.h:34-216)
// when nanort is absent, which it is in the reference checkout.  Its tree
// decides which face wins a tie in ray distance: Intersect collects the hits
// of every leaf it reaches in depth-first order (left child first), then
// std::sort orders them by t, and for the handful of hits a ray makes
// std::sort keeps equal keys in that collection order.  So the tree is built
// here the same way, with the same std::sort on the same keys:
//   * a node with <= leaf_faces faces (or at depth 256) is a leaf
//     (bvh_naive.h:137-147);
//   * otherwise the faces are sorted by their centroid's coordinate on axis
//     depth % 3, the centroid summed in float from zero and divided by 3
//     (bvh_naive.h:164-205); the right child takes sorted[n/2, n) and the
//     left child sorted[0, n - n/2), so an odd node puts its middle face in
//     both children (bvh_naive.h:200-203);
//   * a node's box spans the vertices of all its faces (bvh_naive.h:151-157).
// The flattened tree lists the nodes in depth-first order and the leaves'
// faces in traversal order; a leaf entry's index is therefore its rank in
// the reference's hit order.  Leaf boxes (the reference tests none) are
// added for pruning only.  Leaves hold up to 4 faces for ugu::Raytracer and
// up to 5 for ugu::VisibilityTester (visibility_tester.cc:285-294).
#include <algorithm>
#include <cfloat>
#include <cstddef>
#include <cstring>
#include <vector>

#include "internal.cuh"

namespace ugu_gpu {

namespace {

constexpr int kMaxTreeDepth = 256;  // BvhNaive::m_max_tree_depth

struct Builder {
  const float* V;
  const int32_t* F;
  unsigned leaf_faces;  // BvhNaive::m_min_leaf_primitives
  std::vector<float> centre[3];
  HostBvh* out;

  void bounds(const std::vector<size_t>& ids, float lo[3], float hi[3]) const {
    for (int k = 0; k < 3; ++k) {
      lo[k] = FLT_MAX;
      hi[k] = -FLT_MAX;
    }
    for (size_t f : ids)
      for (int j = 0; j < 3; ++j) {
        const float* p = V + 3 * (size_t)F[3 * f + j];
        for (int k = 0; k < 3; ++k) {
          lo[k] = p[k] < lo[k] ? p[k] : lo[k];
          hi[k] = hi[k] < p[k] ? p[k] : hi[k];
        }
      }
  }

  // Appends the subtree of `ids` in depth-first order; returns its index.
  int build(const std::vector<size_t>& ids, int depth) {
    const int idx = (int)(out->nodes.size() / 2);
    out->nodes.resize(out->nodes.size() + 2);
    out->depth = std::max(out->depth, depth);
    float lo[3], hi[3];
    bounds(ids, lo, hi);
    int a, b;
    if ((unsigned)ids.size() <= leaf_faces || depth >= kMaxTreeDepth) {
      const int first = (int)(out->tris.size() / 3);
      for (size_t f : ids) {
        for (int j = 0; j < 3; ++j) {
          const float* p = V + 3 * (size_t)F[3 * f + j];
          float4 e;
          e.x = p[0];
          e.y = p[1];
          e.z = p[2];
          int32_t w = j == 0 ? (int32_t)f : 0;
          std::memcpy(&e.w, &w, 4);
          out->tris.push_back(e);
        }
      }
      a = -1 - first;
      b = (int)ids.size();
    } else {
      const int axis = depth % 3;
      const std::vector<float>& c = centre[axis];
      std::vector<size_t> left = ids;
      std::sort(left.begin(), left.end(), [&](const size_t& l, const size_t& r) {
        return c[l] < c[r];
      });
      const size_t mid = ids.size() / 2;
      std::vector<size_t> right(left.begin() + (std::ptrdiff_t)mid, left.end());
      left.resize(left.size() - mid);
      a = build(left, depth + 1);
      b = build(right, depth + 1);
    }
    float4& n0 = out->nodes[2 * (size_t)idx];
    float4& n1 = out->nodes[2 * (size_t)idx + 1];
    n0.x = lo[0];
    n0.y = lo[1];
    n0.z = lo[2];
    std::memcpy(&n0.w, &a, 4);
    n1.x = hi[0];
    n1.y = hi[1];
    n1.z = hi[2];
    std::memcpy(&n1.w, &b, 4);
    return idx;
  }
};

}  // namespace

bool build_bvh(const float* vertices, const int32_t* faces, int num_faces, HostBvh& out,
               int leaf_faces) {
  out.nodes.clear();
  out.tris.clear();
  out.depth = 0;
  if (num_faces <= 0) return false;
  Builder b;
  b.V = vertices;
  b.F = faces;
  b.leaf_faces = (unsigned)leaf_faces;
  b.out = &out;
  for (int k = 0; k < 3; ++k) b.centre[k].resize((size_t)num_faces);
  for (int f = 0; f < num_faces; ++f)
    for (int k = 0; k < 3; ++k) {
      // T center = Zero; center += v_i (i = 0..2); center /= 3.0f
      float s = 0.0f;
      for (int j = 0; j < 3; ++j) s += vertices[3 * (size_t)faces[3 * f + j] + k];
      b.centre[k][(size_t)f] = s / 3.0f;
    }
  std::vector<size_t> ids((size_t)num_faces);
  for (size_t i = 0; i < ids.size(); ++i) ids[i] = i;
  b.build(ids, 0);
  return out.depth <= kMaxBvhDepth;
}

}  // namespace ugu_gpu
