// ray.cu -- ugu::Raytracer::Impl::Render (src/renderer/cpu/raytracer.cc:127-224)
// for a group of views, one thread per pixel.
//
// Per pixel the reference casts the ray org_ray_w(x, y) + t ray_w(x, y)
// through its naive BVH, keeps the hit with the smallest float t (ties: the
// first in the tree's depth-first leaf order), and then:
//   * back-face culling: a nearest hit on a face whose normal points along
//     the ray leaves the pixel empty (:166-171);
//   * face_id = fid, mask = 255 for every face, face 0 included (:173-181);
//   * depth = (w2c_R (org + t ray) + w2c_t).z * depth_scale (:183-188);
//   * shading normal: the face normal, or (1 - u - v) n0 + u n1 + v n2 with
//     the hit's (u, v) (:190-201);
//   * the pixel shader with that (u, v) and light direction = ray (:211-218).
// The hit's (t, u, v) are the reference's: Moller-Trumbore in double from
// the float inputs (src/util/geom_util.cc:60-115, 1417-1481), cast to float,
// with (u, v) converted to (weight of v0, weight of v1).
//
// GB300 layout: the BVH lives in HBM as flat float4 arrays (nodes in
// depth-first order, leaf triangles in traversal order with their face id),
// read through L1/L2; each thread walks it with a small stack, a
// conservative float slab test per node and, per triangle, a float
// Moller-Trumbore with a forward error bound that only rejects what the
// double test would reject too.  Everything it cannot reject goes to the
// double test, so at most a few double tests run per ray on a part whose
// FP64 rate is a small fraction of its FP32 rate.
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>

#include "internal.cuh"
#include "shade.cuh"

namespace ugu_gpu {

namespace {

constexpr int kRayThreads = kRayTileW * kRayTileH;
constexpr int kStack = kMaxBvhDepth + 2;
// BvhNaive::m_epsilon (1e-8f) as the double Intersect receives it
constexpr double kDetEps = (double)1e-8f;

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// Eigen's 3-term dot (a0 b0 + (a1 b1 + a2 b2)) and cross product.
__device__ __forceinline__ double ddot(const double* a, const double* b) {
  return dadd(dmul(a[0], b[0]), dadd(dmul(a[1], b[1]), dmul(a[2], b[2])));
}
__device__ __forceinline__ void dcross(const double* a, const double* b, double* o) {
  o[0] = dsub(dmul(a[1], b[2]), dmul(a[2], b[1]));
  o[1] = dsub(dmul(a[2], b[0]), dmul(a[0], b[2]));
  o[2] = dsub(dmul(a[0], b[1]), dmul(a[1], b[0]));
}

// The reference's ray-triangle test in double (geom_util.cc:60-115) with
// the standard-barycentric conversion; (t, u, v) cast to float.
__device__ __noinline__ bool moller_trumbore_f64(float3 o, float3 d, float3 a, float3 b, float3 c,
                                                 float& t, float& u, float& v) {
  const double O[3] = {o.x, o.y, o.z}, D[3] = {d.x, d.y, d.z};
  const double A[3] = {a.x, a.y, a.z};
  const double e1[3] = {dsub(b.x, A[0]), dsub(b.y, A[1]), dsub(b.z, A[2])};
  const double e2[3] = {dsub(c.x, A[0]), dsub(c.y, A[1]), dsub(c.z, A[2])};
  double alpha[3];
  dcross(D, e2, alpha);
  const double det = ddot(e1, alpha);
  if (-kDetEps < det && det < kDetEps) return false;
  const double inv = __ddiv_rn(1.0, det);
  const double r[3] = {dsub(O[0], A[0]), dsub(O[1], A[1]), dsub(O[2], A[2])};
  const double uu = dmul(ddot(alpha, r), inv);
  if (uu < 0.0 || uu > 1.0) return false;
  double beta[3];
  dcross(r, e1, beta);
  const double vv = dmul(ddot(D, beta), inv);
  if (vv < 0.0 || dadd(uu, vv) > 1.0) return false;
  const double tt = dmul(ddot(e2, beta), inv);
  if (tt < 0.0) return false;
  const double w = dsub(dsub(1.0, uu), vv);
  t = __double2float_rn(tt);
  u = __double2float_rn(w);
  v = __double2float_rn(uu);
  return true;
}

// The same test in float with a forward error bound.  Each of det, u det,
// v det and t det is a sum of products formed with at most 7 roundings of
// its inputs, so it lies within 7 ulp of the same expression evaluated with
// absolute values; the bound below takes 64 ulp, far above the double
// test's own rounding.
struct MtFloat {
  float det, un, vn, tn;  // un, vn, tn multiplied by the sign of det
  float ad, lo, hi;       // |det| and the bounds of the exact |det|
  float eu, ev, et;
};

__device__ __forceinline__ MtFloat mt_float(float3 o, float3 d, float3 a, float3 b, float3 c) {
  const float g = 64.0f * 5.9604645e-8f;
  const float e1[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
  const float e2[3] = {c.x - a.x, c.y - a.y, c.z - a.z};
  const float D[3] = {d.x, d.y, d.z};
  const float r[3] = {o.x - a.x, o.y - a.y, o.z - a.z};
  float al[3], al_abs[3], be[3], be_abs[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const int j = (i + 1) % 3, k = (i + 2) % 3;
    al[i] = D[j] * e2[k] - D[k] * e2[j];
    al_abs[i] = fabsf(D[j] * e2[k]) + fabsf(D[k] * e2[j]);
    be[i] = r[j] * e1[k] - r[k] * e1[j];
    be_abs[i] = fabsf(r[j] * e1[k]) + fabsf(r[k] * e1[j]);
  }
  float det = 0.0f, md = 0.0f, un = 0.0f, mu = 0.0f, vn = 0.0f, mv = 0.0f, tn = 0.0f, mt = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    det += e1[i] * al[i];
    md += fabsf(e1[i]) * al_abs[i];
    un += al[i] * r[i];
    mu += al_abs[i] * fabsf(r[i]);
    vn += D[i] * be[i];
    mv += fabsf(D[i]) * be_abs[i];
    tn += e2[i] * be[i];
    mt += fabsf(e2[i]) * be_abs[i];
  }
  MtFloat q;
  const float s = det < 0.0f ? -1.0f : 1.0f;
  const float ed = g * md;
  q.det = det;
  q.ad = fabsf(det);
  q.lo = q.ad - ed;
  q.hi = q.ad + ed;
  q.un = s * un;
  q.vn = s * vn;
  q.tn = s * tn;
  q.eu = g * mu;
  q.ev = g * mv;
  q.et = g * mt;
  return q;
}

// What the double test does, as far as the float bound decides it:
// -1 certainly a miss, 1 certainly a hit, 0 undecided (run the double test).
// A hit needs |det| >= eps, 0 <= u <= 1, v >= 0, u + v <= 1 and t >= 0
// with u = un / |det| and so on.
__device__ __forceinline__ int mt_decide(const MtFloat& q) {
  const float eps = (float)kDetEps;
  if (q.hi < 0.999f * eps) return -1;  // |det| < eps: parallel or degenerate
  if (q.lo <= 0.0f) return 0;          // sign of det unknown
  if (q.un + q.eu < 0.0f || q.un - q.eu > q.hi) return -1;                  // u < 0, u > 1
  if (q.vn + q.ev < 0.0f || (q.un + q.vn) - (q.eu + q.ev) > q.hi) return -1;  // v, u + v
  if (q.tn + q.et < 0.0f) return -1;                                          // t < 0
  if (q.lo > 1.001f * eps && q.un - q.eu > 0.0f && q.un + q.eu < q.lo && q.vn - q.ev > 0.0f &&
      (q.un + q.vn) + (q.eu + q.ev) < q.lo && q.tn - q.et > 0.0f)
    return 1;
  return 0;
}

// The reference's box test (bvh_naive.h:232-238): the ray against the 12
// triangles of the box mesh (bvh_base.h:23-80) with the double test; the
// box counts as hit when any triangle is.  Corners: bit 0/1/2 set = max
// x/y/z.  Decided in float where the bound allows, in double otherwise.
__constant__ unsigned char kBoxCorner[24] = {2, 3, 7, 6, 0, 1, 5, 4, 3, 7, 5, 1,
                                             2, 6, 4, 0, 2, 3, 1, 0, 6, 7, 5, 4};
__constant__ unsigned char kBoxTri[12][3] = {{0, 2, 1},    {0, 3, 2},    {4, 5, 6},
                                             {4, 6, 7},    {8, 9, 10},   {8, 10, 11},
                                             {12, 14, 13}, {12, 15, 14}, {16, 17, 18},
                                             {16, 18, 19}, {20, 22, 21}, {20, 23, 22}};

__device__ __forceinline__ float3 box_corner(float4 lo, float4 hi, int k) {
  const unsigned c = kBoxCorner[k];
  return make_float3(c & 1 ? hi.x : lo.x, c & 2 ? hi.y : lo.y, c & 4 ? hi.z : lo.z);
}

// Triangles of the box mesh per face: x min, x max, y min, y max, z min,
// z max (bvh_base.h:23-80 lists y max, y min, x max, x min, z min, z max).
__constant__ unsigned char kFaceTri[6] = {6, 4, 2, 0, 8, 10};

// The rest of the reference box test: the triangles not in `done`
// classified in float, then the double test for every undecided one.
__device__ __noinline__ bool reference_box_rest(float4 lo, float4 hi, float3 o, float3 d,
                                                unsigned done, unsigned undecided) {
  for (int i = 0; i < 12; ++i) {
    if (done >> i & 1u) continue;
    const float3 a = box_corner(lo, hi, kBoxTri[i][0]);
    const float3 b = box_corner(lo, hi, kBoxTri[i][1]);
    const float3 c = box_corner(lo, hi, kBoxTri[i][2]);
    const int r = mt_decide(mt_float(o, d, a, b, c));
    if (r > 0) return true;
    if (r == 0) undecided |= 1u << i;
  }
  while (undecided) {
    const int i = __ffs(undecided) - 1;
    undecided &= undecided - 1;
    float t, u, v;
    if (moller_trumbore_f64(o, d, box_corner(lo, hi, kBoxTri[i][0]),
                            box_corner(lo, hi, kBoxTri[i][1]), box_corner(lo, hi, kBoxTri[i][2]),
                            t, u, v))
      return true;
  }
  return false;
}

// face = 2 * axis + (1 for the max side): the face the slab test says the
// ray enters through (or leaves through, from inside).  Its two triangles
// decide almost every box; the other ten only run when neither of them is
// certainly hit.
__device__ __forceinline__ bool reference_box_hit(float4 lo, float4 hi, float3 o, float3 d,
                                                  int face) {
  const int t0 = kFaceTri[face];
  unsigned undecided = 0;
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int i = t0 + j;
    const int r = mt_decide(mt_float(o, d, box_corner(lo, hi, kBoxTri[i][0]),
                                     box_corner(lo, hi, kBoxTri[i][1]),
                                     box_corner(lo, hi, kBoxTri[i][2])));
    if (r > 0) return true;
    if (r == 0) undecided |= 1u << i;
  }
  return reference_box_rest(lo, hi, o, d, 3u << t0, undecided);
}

// One axis of the slab test: the ray's parameters at the two planes.  A
// ray parallel to the axis (|d| < 1e-30: it moves less than 1e-23 over any
// distance a hit can have) is inside the slab for every t when lo <= o <=
// hi, including o exactly on a face plane, and outside for every t
// otherwise.
__device__ __forceinline__ void slab(float lo, float hi, float o, float d, float inv, float& t0,
                                     float& t1) {
  if (fabsf(d) >= 1e-30f) {
    t0 = (lo - o) * inv;
    t1 = (hi - o) * inv;
  } else {
    t0 = lo - o <= 0.0f ? -INFINITY : INFINITY;
    t1 = hi - o >= 0.0f ? INFINITY : -INFINITY;
  }
}

// Conservative slab test: -1 when the ray certainly misses the box at
// t >= 0 or certainly enters it beyond best_t (strictly, in float); else
// the face it enters through (leaves through, when tn < 0), as
// 2 * axis + (1 for the max side).  Each finite t is within 2e-7 of the
// exact plane crossing; the margins below take 1e-6.  An infinite tn (a
// miss) turns into NaN and fails the comparisons, as it should.
__device__ __forceinline__ int box_hit(float4 lo, float4 hi, float3 o, float3 d, float3 inv,
                                       float best_t, float& t_enter) {
  float t0[3], t1[3];
  slab(lo.x, hi.x, o.x, d.x, inv.x, t0[0], t1[0]);
  slab(lo.y, hi.y, o.y, d.y, inv.y, t0[1], t1[1]);
  slab(lo.z, hi.z, o.z, d.z, inv.z, t0[2], t1[2]);
  const float D[3] = {d.x, d.y, d.z};
  float tn = -INFINITY, tf = INFINITY;
  int an = 0, af = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float mn = fminf(t0[k], t1[k]), mx = fmaxf(t0[k], t1[k]);
    if (mn > tn) tn = mn, an = k;
    if (mx < tf) tf = mx, af = k;
  }
  const float tnc = tn - 1e-6f * fabsf(tn);
  const float tfc = tf + 1e-6f * fabsf(tf);
  if (!(tnc <= tfc && tfc >= 0.0f && !(tnc > best_t * (1.0f + 4e-6f)))) return -1;
  t_enter = tnc;
  return tn >= 0.0f ? 2 * an + (D[an] > 0.0f ? 0 : 1) : 2 * af + (D[af] > 0.0f ? 1 : 0);
}

// True when the reference's box test certainly hits: the ray crosses the
// plane of `face` at t > 0 at a point well inside the face, clear of its
// edges and of the diagonal that splits it into the box mesh's two
// triangles, and the face's determinant |d_k| * (its two side lengths) is
// above the test's epsilon.  The double test's own rounding (~1e-16 of the
// magnitudes) is far inside the float margins used here.  Diagonals
// (bvh_base.h:23-80, in face coordinates s, u of the two other axes in
// x, y, z order): y faces s = u, x and z faces s + u = 1.
__device__ __forceinline__ bool face_certain(float4 lo, float4 hi, float3 o, float3 d, float3 inv,
                                             int face) {
  const int k = face >> 1;
  const float L[3] = {lo.x, lo.y, lo.z}, H[3] = {hi.x, hi.y, hi.z};
  const float O[3] = {o.x, o.y, o.z}, D[3] = {d.x, d.y, d.z}, I[3] = {inv.x, inv.y, inv.z};
  if (fabsf(D[k]) < 1e-30f) return false;
  const float t = ((face & 1 ? H[k] : L[k]) - O[k]) * I[k];
  if (!(t > 0.0f)) return false;
  const int i = k == 0 ? 1 : 0, j = k == 2 ? 1 : 2;  // the face's axes, in order
  const float di = H[i] - L[i], dj = H[j] - L[j];
  if (!(di > 0.0f && dj > 0.0f) || di * dj * fabsf(D[k]) * (1.0f - 1e-5f) < 1.01f * (float)kDetEps)
    return false;
  const float pi = O[i] + t * D[i], pj = O[j] + t * D[j];
  const float ms = 2e-6f * (fabsf(O[i]) + fabsf(t * D[i]) + fabsf(L[i]) + fabsf(H[i])) / di + 1e-6f;
  const float mu = 2e-6f * (fabsf(O[j]) + fabsf(t * D[j]) + fabsf(L[j]) + fabsf(H[j])) / dj + 1e-6f;
  const float sc = (pi - L[i]) / di, uc = (pj - L[j]) / dj;
  if (!(sc > ms && sc < 1.0f - ms && uc > mu && uc < 1.0f - mu)) return false;
  const float diag = k == 1 ? sc - uc : sc + uc - 1.0f;
  return fabsf(diag) > ms + mu;
}

struct RayHit {
  float t, u, v;
  int32_t rank, fid;
};

__device__ __forceinline__ float3 ld3(const float4& q) { return make_float3(q.x, q.y, q.z); }

// Bounds [t_lo, t_hi] on the double test's t for a triangle the float test
// did not reject (t_hi = inf when the sign of det is undecided).
__device__ __forceinline__ void t_bounds(const MtFloat& q, float& t_lo, float& t_hi) {
  if (q.lo > 0.0f) {
    t_lo = fmaxf(0.0f, (q.tn - q.et) / q.hi) * (1.0f - 1e-6f);
    t_hi = (q.tn + q.et) / q.lo * (1.0f + 1e-6f);
  } else {
    t_lo = 0.0f;
    t_hi = INFINITY;
  }
}

// A triangle whose t is certainly above bound (1 + 4e-6) has a float t
// strictly above every float t <= bound: it can neither win nor tie.
__device__ __forceinline__ bool beyond(float t_lo, float bound) {
  return t_lo > bound * (1.0f + 4e-6f);
}

constexpr int kCand = 8;

// The double test on the pending candidates, nearest lower bound first,
// while one can still win or tie; updates the hit and the bound.
__device__ __forceinline__ void resolve(const float4* tris, float3 o, float3 d, int* ce, float* cl,
                                        int& n, RayHit& h, float& bound) {
  while (n > 0) {
    int j = 0;
    for (int k = 1; k < n; ++k)
      if (cl[k] < cl[j]) j = k;
    if (beyond(cl[j], bound)) break;  // so is every other candidate
    const int e = ce[j];
    ce[j] = ce[n - 1];
    cl[j] = cl[n - 1];
    --n;
    const float4 q0 = __ldg(&tris[3 * e]);
    float t, u, v;
    if (!moller_trumbore_f64(o, d, ld3(q0), ld3(__ldg(&tris[3 * e + 1])),
                             ld3(__ldg(&tris[3 * e + 2])), t, u, v))
      continue;
    if (t < h.t || (t == h.t && e < h.rank)) {
      h.t = t;
      h.u = u;
      h.v = v;
      h.rank = e;
      h.fid = __float_as_int(q0.w);
      bound = fminf(bound, t);
    }
  }
  n = 0;
}

// Nearest hit of the ray in the mesh's BVH: the smallest float t, ties to
// the lowest rank (the reference's depth-first collection order).  The
// traversal classifies triangles in float only; a certain hit bounds the
// nearest t (and prunes boxes), and the triangles that could still win or
// tie wait in a short list for the double test, run once per ray after the
// traversal (a full list is resolved on the spot).
__device__ RayHit trace(const float4* nodes, const float4* tris, float3 o, float3 d) {
  RayHit h;
  h.t = INFINITY;
  h.u = h.v = 0.0f;
  h.rank = INT_MAX;
  h.fid = -1;
  float bound = INFINITY;  // >= the smallest double-test t among the hits seen
  int ce[kCand];
  float cl[kCand];
  int nc = 0;
  const float3 inv = make_float3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);  // used where |d| >= 1e-30
  // stack entries: node << 3 | face (the face the slab test picked), and the
  // node's entry t, the pruning key once a closer hit is known
  int stack[kStack];
  float stack_t[kStack];
  int sp = 0;
  {
    float t0;
    const int f = box_hit(__ldg(&nodes[0]), __ldg(&nodes[1]), o, d, inv, bound, t0);
    if (f >= 0) {
      stack[0] = f;
      stack_t[0] = t0;
      sp = 1;
    }
  }
  while (sp > 0) {
    --sp;
    if (beyond(stack_t[sp], bound)) continue;
    const int n = stack[sp] >> 3, face = stack[sp] & 7;
    const float4 lo = __ldg(&nodes[2 * n]);
    const float4 hi = __ldg(&nodes[2 * n + 1]);
    const int a = __float_as_int(lo.w), b = __float_as_int(hi.w);
    if (a >= 0) {
      // the reference descends only when its own box test hits; the slab
      // test passed every box it can hit, not only those
      if (!face_certain(lo, hi, o, d, inv, face) && !reference_box_hit(lo, hi, o, d, face))
        continue;
      // children slab-tested here and pushed far first; the reference's
      // left-first order only matters through the ranks
      float ta, tb;
      const int fa = box_hit(__ldg(&nodes[2 * a]), __ldg(&nodes[2 * a + 1]), o, d, inv, bound, ta);
      const int fb = box_hit(__ldg(&nodes[2 * b]), __ldg(&nodes[2 * b + 1]), o, d, inv, bound, tb);
      if (sp + 2 > kStack) break;  // deeper than built trees go
      const bool a_first = fa >= 0 && (fb < 0 || ta <= tb);
      if (a_first) {
        if (fb >= 0) stack[sp] = b << 3 | fb, stack_t[sp++] = tb;
        stack[sp] = a << 3 | fa, stack_t[sp++] = ta;
      } else {
        if (fa >= 0) stack[sp] = a << 3 | fa, stack_t[sp++] = ta;
        if (fb >= 0) stack[sp] = b << 3 | fb, stack_t[sp++] = tb;
      }
      continue;
    }
    const int first = -1 - a;
    for (int e = first; e < first + b; ++e) {
      const float3 v0 = ld3(__ldg(&tris[3 * e]));
      const float3 v1 = ld3(__ldg(&tris[3 * e + 1]));
      const float3 v2 = ld3(__ldg(&tris[3 * e + 2]));
      const MtFloat q = mt_float(o, d, v0, v1, v2);
      const int r = mt_decide(q);
      if (r < 0) continue;
      float tl, th;
      t_bounds(q, tl, th);
      if (beyond(tl, bound)) continue;
      if (r > 0) bound = fminf(bound, th);
      if (nc == kCand) resolve(tris, o, d, ce, cl, nc, h, bound);
      ce[nc] = e;
      cl[nc] = tl;
      ++nc;
    }
  }
  resolve(tris, o, d, ce, cl, nc, h, bound);
  return h;
}

__global__ void __launch_bounds__(kRayThreads) k_ray(RayParams p) {
  __shared__ DevView sv;
  __shared__ DevMesh sm;
  {
    const int* src = reinterpret_cast<const int*>(&p.views[blockIdx.y]);
    int* dst = reinterpret_cast<int*>(&sv);
    for (int i = threadIdx.x; i < (int)(sizeof(DevView) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    const int* msrc = reinterpret_cast<const int*>(&p.meshes[sv.mesh]);
    int* mdst = reinterpret_cast<int*>(&sm);
    for (int i = threadIdx.x; i < (int)(sizeof(DevMesh) / 4); i += blockDim.x) mdst[i] = msrc[i];
    __syncthreads();
  }
  const Cam& c = sv.cam;
  const int tiles_x = (c.width + kRayTileW - 1) / kRayTileW;
  const int tiles_y = (c.height + kRayTileH - 1) / kRayTileH;
  if ((int64_t)blockIdx.x >= (int64_t)tiles_x * tiles_y) return;
  const int x = (int)(blockIdx.x % tiles_x) * kRayTileW + (int)(threadIdx.x % kRayTileW);
  const int y = (int)(blockIdx.x / tiles_x) * kRayTileH + (int)(threadIdx.x / kRayTileW);
  if (x >= c.width || y >= c.height) return;
  const int64_t pix = (int64_t)y * c.width + x;

  const float3 o = make_float3(c.T[0], c.T[1], c.T[2]);  // org_ray_w
  const float3 d = ray_w(c, x, y);
  const RayHit h = trace(sm.bvh_nodes, sm.bvh_tris, o, d);
  bool hit = h.fid >= 0;
  if (hit && p.backface_culling) {
    const float4 fn = __ldg(&sm.fnormals[h.fid]);
    if (dot3(fn.x, fn.y, fn.z, d.x, d.y, d.z) > 0.0f) hit = false;
  }
  const DevView& V = sv;
  if (V.face_id) V.face_id[pix] = hit ? h.fid : -1;
  if (V.mask) V.mask[pix] = hit ? 255 : 0;
  if (V.depth) {
    float z = 0.0f;
    if (hit) {
      const float hx = fadd(o.x, fmul(d.x, h.t));
      const float hy = fadd(o.y, fmul(d.y, h.t));
      const float hz = fadd(o.z, fmul(d.z, h.t));
      z = fmul(fadd(dot3(c.R[6], c.R[7], c.R[8], hx, hy, hz), c.t[2]), p.depth_scale);
    }
    V.depth[pix] = z;
  }
  if (V.color || V.normal || V.color_f32) {
    Shaded sh;
    sh.c[0] = sh.c[1] = sh.c[2] = 0;
    sh.cf[0] = sh.cf[1] = sh.cf[2] = 0.0f;
    sh.n[0] = sh.n[1] = sh.n[2] = 0.0f;
    if (hit) {
      float sn[3];
      if (p.shade.shading_normal == 0) {
        const float4 fn = __ldg(&sm.fnormals[h.fid]);
        sn[0] = fn.x;
        sn[1] = fn.y;
        sn[2] = fn.z;
      } else {  // (1.0f - u - v) * n0 + u * n1 + v * n2
        const int4 ni = __ldg(&sm.nidx[h.fid]);
        const float4 n0 = __ldg(&sm.normals[ni.x]);
        const float4 n1 = __ldg(&sm.normals[ni.y]);
        const float4 n2 = __ldg(&sm.normals[ni.z]);
        const float s0 = fsub(fsub(1.0f, h.u), h.v);
        sn[0] = fadd(fadd(fmul(s0, n0.x), fmul(h.u, n1.x)), fmul(h.v, n2.x));
        sn[1] = fadd(fadd(fmul(s0, n0.y), fmul(h.u, n1.y)), fmul(h.v, n2.y));
        sn[2] = fadd(fadd(fmul(s0, n0.z), fmul(h.u, n1.z)), fmul(h.v, n2.z));
      }
      shade_uv(p.shade, sm, c, h.fid, h.u, h.v, sn, x, y, sh);
    }
    if (V.color) {
      V.color[3 * pix + 0] = sh.c[0];
      V.color[3 * pix + 1] = sh.c[1];
      V.color[3 * pix + 2] = sh.c[2];
    }
    if (V.normal) {
      V.normal[3 * pix + 0] = sh.n[0];
      V.normal[3 * pix + 1] = sh.n[1];
      V.normal[3 * pix + 2] = sh.n[2];
    }
    if (V.color_f32) {
      V.color_f32[3 * pix + 0] = sh.cf[0];
      V.color_f32[3 * pix + 1] = sh.cf[1];
      V.color_f32[3 * pix + 2] = sh.cf[2];
    }
  }
}


// VisibilityTester::TestVertex (src/texturing/visibility_tester.cc:416-529)
// for one (keyframe, vertex) -- or, facewise (:606-668), one (keyframe,
// face corner) with the vertex moved 1e-3 of the way to the face centre.
// Float arithmetic in the reference's order; std::acos is acosf here (the
// host library's may differ by an ulp).
__global__ void __launch_bounds__(kRayThreads) k_visibility(VisParams p) {
  const int64_t item = (int64_t)blockIdx.x * kRayThreads + threadIdx.x;
  if (item >= p.items) return;
  const DevKeyframe& K = p.kfs[blockIdx.y];
  const Cam& c = K.cam;
  const DevMesh& m = *p.mesh;
  int vid;
  float3 wp;
  if (p.facewise) {
    const int f = (int)(item / 3), j = (int)(item - 3 * (int64_t)f);
    const int4 vi = __ldg(&m.vidx[f]);
    vid = j == 0 ? vi.x : (j == 1 ? vi.y : vi.z);
    const float4 a = __ldg(&m.vertices[vi.x]), b = __ldg(&m.vertices[vi.y]),
                 cc = __ldg(&m.vertices[vi.z]);
    // face_centers_: Zero, += each vertex, /= 3 (:327-333)
    const float3 ctr = make_float3(fdiv(fadd(fadd(fadd(0.0f, a.x), b.x), cc.x), 3.0f),
                                   fdiv(fadd(fadd(fadd(0.0f, a.y), b.y), cc.y), 3.0f),
                                   fdiv(fadd(fadd(fadd(0.0f, a.z), b.z), cc.z), 3.0f));
    const float4 v = __ldg(&m.vertices[vid]);
    // v_offset = (center - v) * 1e-3f; world_p = v + v_offset
    wp = make_float3(fadd(v.x, fmul(fsub(ctr.x, v.x), 1e-3f)),
                     fadd(v.y, fmul(fsub(ctr.y, v.y), 1e-3f)),
                     fadd(v.z, fmul(fsub(ctr.z, v.z), 1e-3f)));
  } else {
    vid = (int)item;
    const float4 v = __ldg(&m.vertices[vid]);
    wp = make_float3(v.x, v.y, v.z);
  }
  const float4 v4 = __ldg(&m.vertices[vid]);
  const int64_t out = (int64_t)blockIdx.y * p.items + item;
  uint8_t visible = 0;
  float px = 0.0f, py = 0.0f, angle = 0.0f, distance = 0.0f, intensity = 0.0f;
  float col[3] = {0.0f, 0.0f, 0.0f};
  do {
    // camera_p = w2c().cast<float>() * world_p; Project (camera.h:380-387)
    const float cx_ = fadd(dot3(K.L[0], K.L[1], K.L[2], wp.x, wp.y, wp.z), c.t[0]);
    const float cy_ = fadd(dot3(K.L[3], K.L[4], K.L[5], wp.x, wp.y, wp.z), c.t[1]);
    const float cz_ = fadd(dot3(K.L[6], K.L[7], K.L[8], wp.x, wp.y, wp.z), c.t[2]);
    px = fadd(fmul(fdiv(c.fx, cz_), cx_), c.cx);
    py = fadd(fmul(fdiv(c.fy, cz_), cy_), c.cy);
    if (cz_ < 0.0f || px < 0.0f || (float)(c.width - 1) < px || py < 0.0f ||
        (float)(c.height - 1) < py)
      break;
    const int nx = (int)roundf(px), ny = (int)roundf(py);
    const int64_t nn = (int64_t)ny * c.width + nx;
    if (p.use_mask && K.mask[nn] != 255) break;
    if (p.use_depth && K.depth[nn] < FLT_EPSILON) break;
    const float3 ray = ray_w_at(c, px, py);
    const float3 org = make_float3(c.T[0], c.T[1], c.T[2]);
    const float4 n4 = __ldg(&p.normals[vid]);
    const float dt = -dot3(n4.x, n4.y, n4.z, ray.x, ray.y, ray.z);
    angle = acosf(dt);
    if (p.backface_th < angle) break;
    const RayHit h = trace(m.vis_nodes, m.vis_tris, org, ray);
    distance = FLT_MAX;
    float3 hit;
    if (h.fid >= 0) {
      distance = h.t;
      hit = make_float3(fadd(org.x, fmul(ray.x, h.t)), fadd(org.y, fmul(ray.y, h.t)),
                        fadd(org.z, fmul(ray.z, h.t)));
      const float ex = fsub(hit.x, v4.x), ey = fsub(hit.y, v4.y), ez = fsub(hit.z, v4.z);
      const float dist = __fsqrt_rn(dot3(ex, ey, ez, ex, ey, ez));
      if (dist > p.eps) break;
    } else {
      hit = make_float3(v4.x, v4.y, v4.z);
    }
    if (p.use_depth) {
      const float hz = fadd(dot3(K.L[6], K.L[7], K.L[8], hit.x, hit.y, hit.z), c.t[2]);
      if (p.max_depth_difference < fabsf(fsub(hz, K.depth[nn]))) break;
    }
    if (distance > p.max_distance || angle > p.max_viewing_angle) break;
    if (p.interp == 0) {
      col[0] = K.color[3 * nn];
      col[1] = K.color[3 * nn + 1];
      col[2] = K.color[3 * nn + 2];
    } else {  // BilinearInterpolation (util/image_util.h:155-195)
      int x0 = (int)floorf(px), y0 = (int)floorf(py);
      int x1 = x0 + 1, y1 = y0 + 1;
      if (x0 < 0) x0 = 0;
      if (y0 < 0) y0 = 0;
      if (c.width <= x1) x1 = c.width - 1;
      if (c.height <= y1) y1 = c.height - 1;
      const float lu = fsub(px, (float)x0), lv = fsub(py, (float)y0);
      const uint8_t* im = K.color;
      const int64_t W = c.width;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float a00 = fmul(fmul(fsub(1.0f, lu), fsub(1.0f, lv)), (float)im[3 * (y0 * W + x0) + k]);
        const float a10 = fmul(fmul(lu, fsub(1.0f, lv)), (float)im[3 * (y0 * W + x1) + k]);
        const float a01 = fmul(fmul(fsub(1.0f, lu), lv), (float)im[3 * (y1 * W + x0) + k]);
        const float a11 = fmul(fmul(lu, lv), (float)im[3 * (y1 * W + x1) + k]);
        col[k] = (float)f2u8(fadd(fadd(fadd(a00, a10), a01), a11));
      }
    }
    // Color2Gray: (float)(0.2989 r + 0.5870 g + 0.1140 b) in double
    intensity = __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(0.2989, (double)col[0]),
                                                      __dmul_rn(0.5870, (double)col[1])),
                                            __dmul_rn(0.1140, (double)col[2])));
    visible = 1;
  } while (false);
  if (p.visible) p.visible[out] = visible;
  if (p.projected) {
    p.projected[2 * out] = px;
    p.projected[2 * out + 1] = py;
  }
  if (p.viewing_angle) p.viewing_angle[out] = angle;
  if (p.distance) p.distance[out] = distance;
  if (p.color) {
    p.color[3 * out] = col[0];
    p.color[3 * out + 1] = col[1];
    p.color[3 * out + 2] = col[2];
  }
  if (p.intensity) p.intensity[out] = intensity;
}

}  // namespace

void launch_visibility(const VisParams& p, cudaStream_t s) {
  if (p.items <= 0 || p.num_kf <= 0) return;
  k_visibility<<<dim3((unsigned)((p.items + kRayThreads - 1) / kRayThreads), (unsigned)p.num_kf),
                 kRayThreads, 0, s>>>(p);
}

void launch_ray(const RayParams& p, int64_t max_tiles, cudaStream_t s) {
  k_ray<<<dim3((unsigned)max_tiles, (unsigned)p.num_views), kRayThreads, 0, s>>>(p);
}

}  // namespace ugu_gpu
