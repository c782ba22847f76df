// exact.cuh -- IEEE binary32 arithmetic in the operation order of ugu's CPU
// rasterizer, so that face_id, mask and depth come out bit-identical.
//
// Every multiply/add/subtract/divide/sqrt below is an explicitly rounded
// intrinsic (__fmul_rn, __fadd_rn, __fsub_rn, __fdiv_rn, __fsqrt_rn): nvcc
// never contracts those into FMAs, whatever --fmad says.  Three-term sums of
// dot products and matrix-vector rows associate as a0 + (a1 + a2), which is
// how Eigen's unrolled size-3 reduction evaluates on x86-64.
#pragma once

#include <cstdint>
#include <cfloat>

namespace ugu_gpu {

#define UGU_HD __device__ __forceinline__

UGU_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
UGU_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
UGU_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
UGU_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }

UGU_HD float sum3(float a0, float a1, float a2) { return fadd(a0, fadd(a1, a2)); }

UGU_HD float dot3(float a0, float a1, float a2, float b0, float b1, float b2) {
  return sum3(fmul(a0, b0), fmul(a1, b1), fmul(a2, b2));
}

// rasterizer.cc:25-28: (c0 - a0) * (b1 - a1) - (c1 - a1) * (b0 - a0)
UGU_HD float edge_fn(float ax, float ay, float bx, float by, float cx, float cy) {
  return fsub(fmul(fsub(cx, ax), fsub(by, ay)), fmul(fsub(cy, ay), fsub(bx, ax)));
}

// std::min({a,b,c}) / std::max({a,b,c}) as min_element / max_element scan.
UGU_HD float min3_std(float a, float b, float c) {
  float m = a;
  if (b < m) m = b;
  if (c < m) m = c;
  return m;
}
UGU_HD float max3_std(float a, float b, float c) {
  float m = a;
  if (m < b) m = b;
  if (m < c) m = c;
  return m;
}

// float -> int32 with saturation and NaN -> 0 (cvt.rzi.s32.f32).  The
// reference's casts are undefined outside int32 range; this is the aarch64 /
// CUDA behaviour.
UGU_HD int32_t f2i_sat(float f) { return __float2int_rz(f); }

// static_cast<unsigned char>(float): low byte of the saturated int32.
UGU_HD uint8_t f2u8(float f) { return (uint8_t)(uint32_t)__float2int_rz(f); }

struct Cam {
  int32_t width, height;
  float fx, fy, cx, cy;
  float R[9];  // w2c rotation, row-major (float cast of w2c().rotation())
  float t[3];  // w2c translation
  float C[9];  // c2w rotation, row-major (PinholeCamera::c2w_R_f_)
  float T[3];  // c2w translation (PinholeCamera::c2w_t_f_), the raytracer's ray origin
};

// Loop A (rasterizer.cc:131-136) and PinholeCamera::Project
// (camera.h:380-387): p_c = R v + t; x = fx / z * x + cx; y = fy / z * y + cy.
UGU_HD float3 project(const Cam& c, float vx, float vy, float vz) {
  float px = fadd(dot3(c.R[0], c.R[1], c.R[2], vx, vy, vz), c.t[0]);
  float py = fadd(dot3(c.R[3], c.R[4], c.R[5], vx, vy, vz), c.t[1]);
  float pz = fadd(dot3(c.R[6], c.R[7], c.R[8], vx, vy, vz), c.t[2]);
  float3 o;
  o.x = fadd(fmul(fdiv(c.fx, pz), px), c.cx);
  o.y = fadd(fmul(fdiv(c.fy, pz), py), c.cy);
  o.z = pz;
  return o;
}

// PinholeCamera::ray_c + ray_w (camera.h:438-448) at an image point.
UGU_HD float3 ray_w_at(const Cam& c, float x, float y) {
  float d0 = fdiv(fsub(x, c.cx), c.fx);
  float d1 = fdiv(fsub(y, c.cy), c.fy);
  float d2 = 1.0f;
  float n2 = sum3(fmul(d0, d0), fmul(d1, d1), fmul(d2, d2));
  if (n2 > 0.0f) {
    float s = __fsqrt_rn(n2);
    d0 = fdiv(d0, s);
    d1 = fdiv(d1, s);
    d2 = fdiv(d2, s);
  }
  float3 r;
  r.x = dot3(c.C[0], c.C[1], c.C[2], d0, d1, d2);
  r.y = dot3(c.C[3], c.C[4], c.C[5], d0, d1, d2);
  r.z = dot3(c.C[6], c.C[7], c.C[8], d0, d1, d2);
  return r;
}

// The tabulated ray of pixel (x, y) (camera.h:482-513): the same value.
UGU_HD float3 ray_w(const Cam& c, int x, int y) { return ray_w_at(c, (float)x, (float)y); }

// Screen-space setup of one face for one view (rasterizer.cc:163-193).
struct FaceSetup {
  float3 v0, v1, v2;  // projected vertices (x, y, camera z)
  float area;
  int32_t x0, x1, y0, y1;  // inclusive pixel bbox, clamped to the image
};

// Returns false when the face is skipped: a vertex behind the camera
// (:170), the bbox off screen (:180-183), or |area| < FLT_MIN (:190-193).
UGU_HD bool face_setup(const Cam& c, float3 v0, float3 v1, float3 v2, FaceSetup& s) {
  if (v0.z < 0.0f || v1.z < 0.0f || v2.z < 0.0f) return false;
  float xmin = min3_std(v0.x, v1.x, v2.x);
  float ymin = min3_std(v0.y, v1.y, v2.y);
  float xmax = max3_std(v0.x, v1.x, v2.x);
  float ymax = max3_std(v0.y, v1.y, v2.y);
  if (xmin > (float)(c.width - 1) || xmax < 0.0f || ymin > (float)(c.height - 1) ||
      ymax < 0.0f)
    return false;
  s.x0 = max(0, f2i_sat(ceilf(xmin)));
  s.x1 = min(c.width - 1, f2i_sat(floorf(xmax)));
  s.y0 = max(0, f2i_sat(ceilf(ymin)));
  s.y1 = min(c.height - 1, f2i_sat(floorf(ymax)));
  s.area = edge_fn(v0.x, v0.y, v1.x, v1.y, v2.x, v2.y);
  if (fabsf(s.area) < FLT_MIN) return false;
  s.v0 = v0;
  s.v1 = v1;
  s.v2 = v2;
  return true;
}

// Edge functions at integer pixel (x, y) (rasterizer.cc:201-205).
struct Bary {
  float w0, w1, w2;
};
UGU_HD Bary edges_at(const FaceSetup& s, int x, int y) {
  float px = (float)x, py = (float)y;
  Bary b;
  b.w0 = edge_fn(s.v1.x, s.v1.y, s.v2.x, s.v2.y, px, py);
  b.w1 = edge_fn(s.v2.x, s.v2.y, s.v0.x, s.v0.y, px, py);
  b.w2 = edge_fn(s.v0.x, s.v0.y, s.v1.x, s.v1.y, px, py);
  return b;
}

// Inclusive coverage test with back faces kept (:206-207).
UGU_HD bool covered(const Bary& b, bool backface) {
  return (!backface && (b.w0 >= 0.0f && b.w1 >= 0.0f && b.w2 >= 0.0f)) ||
         (backface && (b.w0 <= 0.0f && b.w1 <= 0.0f && b.w2 <= 0.0f));
}

// Perspective-correct interpolation (:208-224); returns z, rewrites b.
UGU_HD float perspective(const FaceSetup& s, Bary& b) {
  float w0 = fdiv(b.w0, s.area);
  float w1 = fdiv(b.w1, s.area);
  float w2 = fdiv(b.w2, s.area);
  w0 = fdiv(w0, s.v0.z);
  w1 = fdiv(w1, s.v1.z);
  w2 = fdiv(w2, s.v2.z);
  float z = fdiv(1.0f, fadd(fadd(w0, w1), w2));
  b.w0 = fmul(w0, z);
  b.w1 = fmul(w1, z);
  b.w2 = fmul(w2, z);
  return z;
}

// The same weights when z is already known: z must be what perspective()
// returns for these inputs (the depth the z-test stored for the pixel), so
// that the result is bit-identical; one division fewer.
UGU_HD void perspective_at(const FaceSetup& s, Bary& b, float z) {
  const float w0 = fdiv(fdiv(b.w0, s.area), s.v0.z);
  const float w1 = fdiv(fdiv(b.w1, s.area), s.v1.z);
  const float w2 = fdiv(fdiv(b.w2, s.area), s.v2.z);
  b.w0 = fmul(w0, z);
  b.w1 = fmul(w1, z);
  b.w2 = fmul(w2, z);
}

// 64-bit z-buffer key: depth bits, then face id, then the back-face flag.
// For depths in [FLT_MIN, +inf] the unsigned order of the key is the order
// of (depth, face id): atomicMin keeps the nearest candidate and, on equal
// depth, the lowest face id -- the sequential loop's `z < d` rule.
constexpr unsigned long long kEmptyKey = ~0ull;

UGU_HD unsigned long long make_key(float z, int32_t fid, bool backface) {
  return ((unsigned long long)__float_as_uint(z) << 32) |
         ((unsigned long long)(uint32_t)fid << 1) | (backface ? 1ull : 0ull);
}
UGU_HD float key_depth(unsigned long long k) { return __uint_as_float((uint32_t)(k >> 32)); }
UGU_HD int32_t key_face(unsigned long long k) { return (int32_t)(((uint32_t)k) >> 1); }
UGU_HD bool key_backface(unsigned long long k) { return (k & 1ull) != 0; }

// A depth the min-reduction can order like the sequential z-test does.
UGU_HD bool orderable_depth(float z) { return z >= FLT_MIN; }

}  // namespace ugu_gpu
