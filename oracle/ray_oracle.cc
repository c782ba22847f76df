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
#include <cstdint>
#include <vector>

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
  std::vector<float> centre[3];
  std::vector<Node> nodes;

  int build(const std::vector<size_t>& ids, int depth) {
    const int idx = (int)nodes.size();
    nodes.emplace_back();
    if (ids.size() <= 4 || depth >= 256) {
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

}  // namespace

extern "C" {

void* oracle_bvh_build(const float* vertices, int32_t num_faces, const int32_t* faces) {
  if (num_faces <= 0) return nullptr;
  Bvh* b = new Bvh();
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
