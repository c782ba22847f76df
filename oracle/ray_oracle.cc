/* ray_oracle.cc -- TEST INFRASTRUCTURE ONLY.
 *
 * The hit search of ugu::Raytracer (src/renderer/cpu/raytracer.cc:146-157)
 * restated on the CPU: ugu::BvhNaive (include/ugu/accel/bvh_naive.h), the
 * naive BVH the reference builds without nanort, and its recursive
 * Intersect.  C++ because the result of a tie in ray distance depends on
 * std::sort, both in the build (faces sorted by centroid) and in the hit
 * list (sorted by t): the same calls on the same keys reproduce it.
 *   Build (bvh_naive.h:34-216): a node with <= 4 faces, or at depth 256, is
 *   a leaf; otherwise its faces are sorted by centroid coordinate on axis
 *   depth % 3, the right child takes sorted[n/2, n) and the left child
 *   sorted[0, n - n/2).  An inner node's box spans its faces' vertices.
 *   Intersect (bvh_naive.h:218-246): at a leaf, every face is tested; at an
 *   inner node, the ray is tested against the 12 triangles of the box
 *   (bvh_base.h:23-80) and, on any hit, the left then the right subtree's
 *   hits are collected.  The hits are sorted by t with std::sort and the
 *   first is kept (bvh_naive.h:99-111).
 *   Ray-triangle test (src/util/geom_util.cc:60-115, 1417-1481):
 *   Moller-Trumbore in double from the float inputs, det epsilon = the
 *   BVH's 1e-8f, (t, u, v) cast to float with (u, v) turned into the weights
 *   of v0 and v1.
 */
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

#include "raster_oracle.h"

namespace {

// Eigen's 3-term dot: a0 b0 + (a1 b1 + a2 b2).
double dot3d(const double* a, const double* b) {
  return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]);
}
void cross3d(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

struct Hit {
  float t, u, v;
  uint32_t fid;
};

// geom_util.cc:60-115 in double, standard barycentric conversion.
bool moller_trumbore(const float* org, const float* dir, const float* a, const float* b,
                     const float* c, double eps, float* out) {
  const double O[3] = {org[0], org[1], org[2]}, D[3] = {dir[0], dir[1], dir[2]};
  const double A[3] = {a[0], a[1], a[2]}, B[3] = {b[0], b[1], b[2]}, C[3] = {c[0], c[1], c[2]};
  const double e1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
  const double e2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
  double alpha[3];
  cross3d(D, e2, alpha);
  const double det = dot3d(e1, alpha);
  if (-eps < det && det < eps) return false;
  const double inv = 1.0 / det;
  const double r[3] = {O[0] - A[0], O[1] - A[1], O[2] - A[2]};
  double u = dot3d(alpha, r) * inv;
  if (u < 0.0 || u > 1.0) return false;
  double beta[3];
  cross3d(r, e1, beta);
  double v = dot3d(D, beta) * inv;
  if (v < 0.0 || u + v > 1.0) return false;
  const double t = dot3d(e2, beta) * inv;
  if (t < 0.0) return false;
  const double w = 1 - u - v;
  out[0] = (float)t;
  out[1] = (float)w;
  out[2] = (float)u;
  return true;
}

struct Node {
  bool leaf = false;
  float lo[3], hi[3];
  int child[2] = {-1, -1};
  std::vector<size_t> faces;
  float box[24][3];  // the 24 corner copies of the box mesh
};

// The box mesh of bvh_base.h:23-80: 24 vertices (4 per side), 12 triangles,
// as (corner selector per axis: 0 = min, 1 = max) and index triples.
const int kBoxCorner[24][3] = {
    {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1},  // 0-3   y = max
    {0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1},  // 4-7   y = min
    {1, 1, 0}, {1, 1, 1}, {1, 0, 1}, {1, 0, 0},  // 8-11  = 1, 2, 6, 5
    {0, 1, 0}, {0, 1, 1}, {0, 0, 1}, {0, 0, 0},  // 12-15 = 0, 3, 7, 4
    {0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 0},  // 16-19 = 0, 1, 5, 4
    {0, 1, 1}, {1, 1, 1}, {1, 0, 1}, {0, 0, 1},  // 20-23 = 3, 2, 6, 7
};
const int kBoxTri[12][3] = {{0, 2, 1},    {0, 3, 2},    {4, 5, 6},    {4, 6, 7},
                            {8, 9, 10},   {8, 10, 11},  {12, 14, 13}, {12, 15, 14},
                            {16, 17, 18}, {16, 18, 19}, {20, 22, 21}, {20, 23, 22}};

const double kEps = (double)1e-8f;  // BvhNaive::m_epsilon

struct Bvh {
  const float* V;
  const int32_t* F;
  size_t leaf_faces = 4;  // BvhNaive::m_min_leaf_primitives
  std::vector<float> centre[3];
  std::vector<Node> nodes;

  int build(const std::vector<size_t>& ids, int depth) {
    const int idx = (int)nodes.size();
    nodes.emplace_back();
    if (ids.size() <= leaf_faces || depth >= 256) {
      nodes[idx].leaf = true;
      nodes[idx].faces = ids;
      return idx;
    }
    const int axis = depth % 3;
    const std::vector<float>& c = centre[axis];
    std::vector<size_t> left = ids;
    std::sort(left.begin(), left.end(),
              [&](const size_t& l, const size_t& r) { return c[l] < c[r]; });
    const size_t mid = ids.size() / 2;
    std::vector<size_t> right(left.begin() + (std::ptrdiff_t)mid, left.end());
    left.resize(left.size() - mid);
    // box of every vertex of the node's faces (ComputeMin/MaxBound)
    float lo[3], hi[3];
    const float* p0 = V + 3 * (size_t)F[3 * ids[0]];
    for (int k = 0; k < 3; ++k) lo[k] = hi[k] = p0[k];
    for (size_t f : ids)
      for (int j = 0; j < 3; ++j) {
        const float* p = V + 3 * (size_t)F[3 * f + j];
        for (int k = 0; k < 3; ++k) {
          lo[k] = p[k] < lo[k] ? p[k] : lo[k];
          hi[k] = hi[k] < p[k] ? p[k] : hi[k];
        }
      }
    for (int k = 0; k < 3; ++k) {
      nodes[idx].lo[k] = lo[k];
      nodes[idx].hi[k] = hi[k];
    }
    for (int i = 0; i < 24; ++i)
      for (int k = 0; k < 3; ++k) nodes[idx].box[i][k] = kBoxCorner[i][k] ? hi[k] : lo[k];
    const int a = build(left, depth + 1);
    const int b = build(right, depth + 1);
    nodes[idx].child[0] = a;
    nodes[idx].child[1] = b;
    return idx;
  }

  void intersect(int n, const float* org, const float* dir, std::vector<Hit>& out) const {
    const Node& nd = nodes[n];
    float tuv[3];
    if (nd.leaf) {
      for (size_t f : nd.faces) {
        const int32_t* fi = F + 3 * f;
        if (moller_trumbore(org, dir, V + 3 * (size_t)fi[0], V + 3 * (size_t)fi[1],
                            V + 3 * (size_t)fi[2], kEps, tuv))
          out.push_back(Hit{tuv[0], tuv[1], tuv[2], (uint32_t)f});
      }
      return;
    }
    bool any = false;
    for (int i = 0; i < 12 && !any; ++i)
      any = moller_trumbore(org, dir, nd.box[kBoxTri[i][0]], nd.box[kBoxTri[i][1]],
                            nd.box[kBoxTri[i][2]], kEps, tuv);
    if (!any) return;
    intersect(nd.child[0], org, dir, out);
    intersect(nd.child[1], org, dir, out);
  }
};

Bvh* build_bvh(const float* vertices, int32_t num_faces, const int32_t* faces, size_t leaf) {
  if (num_faces <= 0) return nullptr;
  Bvh* b = new Bvh();
  b->leaf_faces = leaf;
  b->V = vertices;
  b->F = faces;
  for (int k = 0; k < 3; ++k) b->centre[k].resize((size_t)num_faces);
  for (int32_t f = 0; f < num_faces; ++f)
    for (int k = 0; k < 3; ++k) {
      float s = 0.0f;  // T center = Zero; center += v_i; center /= 3.0f
      for (int j = 0; j < 3; ++j) s += vertices[3 * (size_t)faces[3 * f + j] + k];
      b->centre[k][(size_t)f] = s / 3.0f;
    }
  std::vector<size_t> ids((size_t)num_faces);
  for (size_t i = 0; i < ids.size(); ++i) ids[i] = i;
  b->build(ids, 0);
  return b;
}

// Nearest t along the ray (results[0].t of bvh_naive.h:99-111), or -1.
float nearest_t(const Bvh* b, const float* org, const float* dir) {
  std::vector<Hit> hits;
  b->intersect(0, org, dir, hits);
  std::sort(hits.begin(), hits.end(), [](const Hit& l, const Hit& r) { return l.t < r.t; });
  return hits.empty() ? -1.0f : hits[0].t;
}

float dot3f(const float* a, const float* b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }

// VisibilityTester::TestVertex (visibility_tester.cc:416-529) for one
// keyframe and world point wp of vertex vid; false when not visible.  With
// the host's VisibilityInfo assembly on top, pinned bit for bit to the
// reference's own visibility_tester.cc built into oracle/_ref
// (tests/test_visibility.py).
bool test_vertex(const Bvh* bvh, const float* V, const float* N, int vid, const float* wp,
                 const oracle_keyframe& K, const oracle_vis_option& o, float* proj, float* angle,
                 float* dist_out, float* col, float* inten) {
  const oracle_camera& c = K.cam;
  float cp[3];
  for (int k = 0; k < 3; ++k) cp[k] = dot3f(&K.L[3 * k], wp) + c.w2c_t[k];
  const float x = c.fx / cp[2] * cp[0] + c.cx;  // PinholeCamera::Project
  const float y = c.fy / cp[2] * cp[1] + c.cy;
  const float d = cp[2];
  proj[0] = x;
  proj[1] = y;
  if (d < 0 || x < 0 || c.width - 1 < x || y < 0 || c.height - 1 < y) return false;
  const int nx = static_cast<int>(std::round(x)), ny = static_cast<int>(std::round(y));
  const size_t nn = (size_t)ny * c.width + nx;
  if (o.use_mask && K.mask[nn] != 255) return false;
  if (o.use_depth && K.depth[nn] < std::numeric_limits<float>::epsilon()) return false;
  // ray_w(float, float) (camera.h:438-448)
  float r[3] = {(x - c.cx) / c.fx, (y - c.cy) / c.fy, 1.0f};
  const float n2 = r[0] * r[0] + (r[1] * r[1] + r[2] * r[2]);
  if (n2 > 0.0f) {
    const float sq = std::sqrt(n2);
    for (int k = 0; k < 3; ++k) r[k] = r[k] / sq;
  }
  float ray[3];
  for (int k = 0; k < 3; ++k) ray[k] = dot3f(&c.c2w_R[3 * k], r);
  const float* org = c.c2w_t;
  const float dotv = -dot3f(&N[3 * vid], ray);
  const float va = std::acos(dotv);
  *angle = va;
  if (o.backface_th < va) return false;
  const float t = nearest_t(bvh, org, ray);
  float distance = std::numeric_limits<float>::max();
  float hit[3];
  const float* v = &V[3 * vid];
  if (t >= 0.0f) {
    distance = t;
    for (int k = 0; k < 3; ++k) hit[k] = org[k] + ray[k] * t;
    const float e[3] = {hit[0] - v[0], hit[1] - v[1], hit[2] - v[2]};
    const float dd = std::sqrt(dot3f(e, e));
    if (dd > o.eps) return false;
  } else {
    for (int k = 0; k < 3; ++k) hit[k] = v[k];
  }
  if (o.use_depth) {
    const float hz = dot3f(&K.L[6], hit) + c.w2c_t[2];
    if (o.max_depth_difference < std::abs(hz - K.depth[nn])) return false;
  }
  *dist_out = distance;
  if (distance > o.max_distance || va > o.max_viewing_angle) return false;
  if (o.interp == 0) {
    for (int k = 0; k < 3; ++k) col[k] = K.color[3 * nn + k];
  } else {  // BilinearInterpolation (util/image_util.h:155-195)
    int x0 = static_cast<int>(std::floor(x)), y0 = static_cast<int>(std::floor(y));
    int x1 = x0 + 1, y1 = y0 + 1;
    if (x0 < 0.0f) x0 = 0;
    if (y0 < 0.0f) y0 = 0;
    if (c.width <= x1) x1 = c.width - 1;
    if (c.height <= y1) y1 = c.height - 1;
    const float lu = x - x0, lv = y - y0;
    const size_t W = (size_t)c.width;
    for (int k = 0; k < 3; ++k) {
      const float cf = (1.0f - lu) * (1.0f - lv) * K.color[3 * (y0 * W + x0) + k] +
                       lu * (1.0f - lv) * K.color[3 * (y0 * W + x1) + k] +
                       (1.0f - lu) * lv * K.color[3 * (y1 * W + x0) + k] +
                       lu * lv * K.color[3 * (y1 * W + x1) + k];
      col[k] = static_cast<uint8_t>(cf);
    }
  }
  *inten = static_cast<float>(0.2989 * col[0] + 0.5870 * col[1] + 0.1140 * col[2]);
  return true;
}

}  // namespace

extern "C" {

void* oracle_bvh_build(const float* vertices, int32_t num_faces, const int32_t* faces) {
  return build_bvh(vertices, num_faces, faces, 4);
}

// VisibilityTester::Test's per-keyframe pass (:670-702): TestVertex for
// every (keyframe, vertex), or facewise every (keyframe, face corner) with
// the vertex moved 1e-3 toward the face centre (:606-668).  Outputs
// keyframe-major; the fields are those of VertexInfoPerKeyframe.
void oracle_test_visibility(const float* V, int32_t nv, const int32_t* F, int32_t nf,
                            const float* N, int32_t n_kf, const oracle_keyframe* kfs,
                            const oracle_vis_option* o, int32_t facewise, uint8_t* visible,
                            float* proj, float* angle, float* dist, float* color,
                            float* intensity) {
  Bvh* bvh = build_bvh(V, nf, F, 5);  // visibility_tester.cc:285-294
  if (!bvh) return;
  const int64_t items = facewise ? 3 * (int64_t)nf : (int64_t)nv;
  for (int32_t k = 0; k < n_kf; ++k)
    for (int64_t it = 0; it < items; ++it) {
      const int64_t out = k * items + it;
      int vid;
      float wp[3];
      if (facewise) {
        const int64_t f = it / 3;
        const int j = (int)(it % 3);
        vid = F[3 * f + j];
        float ctr[3] = {0.0f, 0.0f, 0.0f};
        for (int i = 0; i < 3; ++i)
          for (int q = 0; q < 3; ++q) ctr[q] += V[3 * F[3 * f + i] + q];
        for (int q = 0; q < 3; ++q) ctr[q] /= 3;
        for (int q = 0; q < 3; ++q) wp[q] = V[3 * vid + q] + (ctr[q] - V[3 * vid + q]) * 1e-3f;
      } else {
        vid = (int)it;
        for (int q = 0; q < 3; ++q) wp[q] = V[3 * vid + q];
      }
      float pj[2] = {0, 0}, a = 0, dd = 0, c3[3] = {0, 0, 0}, in = 0;
      const bool vis = test_vertex(bvh, V, N, vid, wp, kfs[k], *o, pj, &a, &dd, c3, &in);
      visible[out] = vis ? 1 : 0;
      proj[2 * out] = pj[0];
      proj[2 * out + 1] = pj[1];
      angle[out] = a;
      dist[out] = dd;
      for (int q = 0; q < 3; ++q) color[3 * out + q] = c3[q];
      intensity[out] = in;
    }
  delete bvh;
}

void oracle_bvh_free(void* bvh) { delete static_cast<Bvh*>(bvh); }

// The nearest hit (raytracer.cc:152-161): 1 and (t, u, v, fid), or 0.
// *sort_dependent (when not NULL) is 1 when the ray has more than 16 hits
// and several share the smallest t: std::sort keeps equal keys in
// collection order only up to 16 elements, so which of them the reference
// reports then depends on the standard library's partitioning.
int oracle_bvh_nearest(const void* bvh, const float* org, const float* dir, float* t, float* u,
                       float* v, int32_t* fid, int32_t* sort_dependent) {
  const Bvh* b = static_cast<const Bvh*>(bvh);
  std::vector<Hit> hits;
  b->intersect(0, org, dir, hits);
  std::sort(hits.begin(), hits.end(), [](const Hit& l, const Hit& r) { return l.t < r.t; });
  if (sort_dependent)
    *sort_dependent = hits.size() > 16 && hits[1].t == hits[0].t ? 1 : 0;
  if (hits.empty()) return 0;
  *t = hits[0].t;
  *u = hits[0].u;
  *v = hits[0].v;
  *fid = (int32_t)hits[0].fid;
  return 1;
}

}  // extern "C"
