// shade.cuh -- Loop C of ugu's rasterizer for one pixel (rasterizer.cc:254-299)
// and the pixel shaders (pixel_shader.h:215-422), in the reference's FP32
// operation order.  Shared by the global-z-buffer path, the tiled path and
// the raytracer.
#pragma once

#include "internal.cuh"

namespace ugu_gpu {


__device__ __forceinline__ int64_t texel_index(int64_t y, int64_t x, int32_t cols,
                                               int32_t rows) {
  // at<Vec3b>(y, x) reads texel y * cols + x (image.h:416-427); only an
  // address outside the allocation is clamped.
  int64_t i = y * (int64_t)cols + x;
  int64_t n = (int64_t)cols * (int64_t)rows;
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

__device__ __forceinline__ void fetch_texel(const DevTexture& t, int64_t i, float* o) {
  if (t.rgbf) {
    o[0] = __ldg(&t.rgbf[3 * i + 0]);
    o[1] = __ldg(&t.rgbf[3 * i + 1]);
    o[2] = __ldg(&t.rgbf[3 * i + 2]);
  } else {
    uint32_t v = __ldg(&t.rgba8[i]);
    o[0] = (float)(v & 0xffu);
    o[1] = (float)((v >> 8) & 0xffu);
    o[2] = (float)((v >> 16) & 0xffu);
  }
}


// The pixel shader of one pixel (pixel_shader.h:215-422) given the face,
// the colorizer's (u, v), the world-frame shading normal sn and the pixel;
// also the camera-frame normal w2c_R * sn (rasterizer.cc:282-289,
// raytracer.cc:192-199).
__device__ __forceinline__ void shade_uv(const ShadeOpts& p, const DevMesh& m, const Cam& c,
                                         int fid, float u, float v, const float sn[3], int x,
                                         int y, Shaded& out) {
  out.n[0] = dot3(c.R[0], c.R[1], c.R[2], sn[0], sn[1], sn[2]);
  out.n[1] = dot3(c.R[3], c.R[4], c.R[5], sn[0], sn[1], sn[2]);
  out.n[2] = dot3(c.R[6], c.R[7], c.R[8], sn[0], sn[1], sn[2]);

  // colorizer: weights (1 - u - v), u, v
  const float s0 = fsub(fsub(1.0f, u), v);
  float col[3] = {255.0f, 255.0f, 255.0f};
  if (p.diffuse_color == 2) {  // pixel_shader.h:234-256
    int4 vi = __ldg(&m.vidx[fid]);
    float4 c0 = __ldg(&m.vcolors[vi.x]);
    float4 c1 = __ldg(&m.vcolors[vi.y]);
    float4 c2 = __ldg(&m.vcolors[vi.z]);
    col[0] = fadd(fadd(fmul(s0, c0.x), fmul(u, c1.x)), fmul(v, c2.x));
    col[1] = fadd(fadd(fmul(s0, c0.y), fmul(u, c1.y)), fmul(v, c2.y));
    col[2] = fadd(fadd(fmul(s0, c0.z), fmul(u, c1.z)), fmul(v, c2.z));
  } else if (p.diffuse_color == 1) {  // pixel_shader.h:260-359
    const DevTexture t = m.textures[__ldg(&m.mat_ids[fid])];
    int4 ti = __ldg(&m.uvidx[fid]);
    float2 a = __ldg(&m.uv[ti.x]);
    float2 b = __ldg(&m.uv[ti.y]);
    float2 d = __ldg(&m.uv[ti.z]);
    float uvx = fadd(fadd(fmul(s0, a.x), fmul(u, b.x)), fmul(v, d.x));
    float uvy = fadd(fadd(fmul(s0, a.y), fmul(u, b.y)), fmul(v, d.y));
    float fx = fmul(uvx, (float)(t.width - 1));
    float fy = fmul(fsub(1.0f, uvy), (float)(t.height - 1));
    if (p.interp == 0) {
      int32_t tx = f2i_sat(roundf(fx));
      int32_t ty = f2i_sat(roundf(fy));
      fetch_texel(t, texel_index(ty, tx, t.width, t.height), col);
    } else {
      int32_t x0 = f2i_sat(floorf(fx));
      int32_t y0 = f2i_sat(floorf(fy));
      float lu = fsub(fx, (float)x0);
      float lv = fsub(fy, (float)y0);
      float t00[3], t10[3], t01[3], t11[3];
      // texel_index of the four taps: one linear address and its neighbours,
      // each clamped to the allocation on its own
      const int64_t n = (int64_t)t.width * t.height;
      const int64_t i00 = (int64_t)y0 * t.width + x0;
      auto clampi = [n](int64_t i) { return i < 0 ? (int64_t)0 : (i >= n ? n - 1 : i); };
      fetch_texel(t, clampi(i00), t00);
      fetch_texel(t, clampi(i00 + 1), t10);
      fetch_texel(t, clampi(i00 + t.width), t01);
      fetch_texel(t, clampi(i00 + t.width + 1), t11);
      const float a00 = fmul(fsub(1.0f, lu), fsub(1.0f, lv));
      const float a10 = fmul(lu, fsub(1.0f, lv));
      const float a01 = fmul(fsub(1.0f, lu), lv);
      const float a11 = fmul(lu, lv);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        col[k] = fadd(fadd(fadd(fmul(a00, t00[k]), fmul(a10, t10[k])), fmul(a01, t01[k])),
                      fmul(a11, t11[k]));
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    out.cf[k] = col[k];
    out.c[k] = p.diffuse_color == 0 ? (uint8_t)255 : f2u8(col[k]);
  }

  if (p.diffuse_shading != 0) {
    float3 r = ray_w(c, x, y);  // light_dir = ray_w (rasterizer.cc:293)
    if (p.diffuse_shading == 1) {  // pixel_shader.h:370-388
      float coeff = -dot3(r.x, r.y, r.z, sn[0], sn[1], sn[2]);
      if (coeff < 0.0f) coeff = 0.0f;
#pragma unroll
      for (int k = 0; k < 3; ++k) out.c[k] = f2u8(fmul(coeff, (float)out.c[k]));
    } else {  // pixel_shader.h:392-422
      float dot_light = -dot3(r.x, r.y, r.z, sn[0], sn[1], sn[2]);
      float theta_i = acosf(dot_light);
      float theta_r = acosf(dot_light);  // dot_ray == dot_light: ray_w is the light
      float bl[3] = {fsub(fmul(-sn[0], dot_light), r.x), fsub(fmul(-sn[1], dot_light), r.y),
                     fsub(fmul(-sn[2], dot_light), r.z)};
      float pdc = dot3(bl[0], bl[1], bl[2], bl[0], bl[1], bl[2]);
      float phi_diff_cos = (0.0f < pdc) ? pdc : 0.0f;
      float alpha = (theta_i < theta_r) ? theta_r : theta_i;
      float beta = (theta_r < theta_i) ? theta_r : theta_i;
      float dl = (0.0f < dot_light) ? dot_light : 0.0f;
      float coeff =
          fmul(dl, fadd(p.on_A, fmul(fmul(fmul(p.on_B, phi_diff_cos), sinf(alpha)), tanf(beta))));
#pragma unroll
      for (int k = 0; k < 3; ++k) out.c[k] = f2u8(fmul(coeff, (float)out.c[k]));
    }
  }
}

// Loop C body for a pixel whose final face id is > 0 (rasterizer.cc:254-299),
// given the winning face's projected vertices and area; with kDepth, the
// pixel's z-buffer depth `z` stands in for the one perspective() would
// recompute (bit-identical: the same inputs and operations).
template <bool kDepth>
__device__ __forceinline__ void shade_face_pixel_t(const ShadeOpts& p, const DevMesh& m,
                                                   const Cam& c, int fid, const FaceSetup& s,
                                                   int x, int y, float z, Shaded& out) {
  Bary w = edges_at(s, x, y);
  if (kDepth)
    perspective_at(s, w, z);
  else
    perspective(s, w);

  // shading normal (:268-279) from the stored weights
  float sn[3] = {0.0f, 0.0f, 0.0f};
  if (p.shading_normal == 0) {
    float4 fn = __ldg(&m.fnormals[fid]);
    sn[0] = fn.x;
    sn[1] = fn.y;
    sn[2] = fn.z;
  } else {
    int4 ni = __ldg(&m.nidx[fid]);
    float4 n0 = __ldg(&m.normals[ni.x]);
    float4 n1 = __ldg(&m.normals[ni.y]);
    float4 n2 = __ldg(&m.normals[ni.z]);
    sn[0] = fadd(fadd(fmul(w.w0, n0.x), fmul(w.w1, n1.x)), fmul(w.w2, n2.x));
    sn[1] = fadd(fadd(fmul(w.w0, n0.y), fmul(w.w1, n1.y)), fmul(w.w2, n2.y));
    sn[2] = fadd(fadd(fmul(w.w0, n0.z), fmul(w.w1, n1.z)), fmul(w.w2, n2.z));
  }
  // the colorizer's u = w1, v = w2
  shade_uv(p, m, c, fid, w.w1, w.w2, sn, x, y, out);
}

__device__ __forceinline__ void shade_face_pixel(const ShadeOpts& p, const DevMesh& m,
                                                 const Cam& c, int fid, const FaceSetup& s,
                                                 int x, int y, Shaded& out) {
  shade_face_pixel_t<false>(p, m, c, fid, s, x, y, 0.0f, out);
}


// Projected vertices and area of face `fid` (Loop A + rasterizer.cc:190).
__device__ __forceinline__ FaceSetup project_face(const DevMesh& m, const Cam& c, int fid) {
  FaceSetup s;
  int4 vi = __ldg(&m.vidx[fid]);
  float4 a = __ldg(&m.vertices[vi.x]);
  float4 b = __ldg(&m.vertices[vi.y]);
  float4 d = __ldg(&m.vertices[vi.z]);
  s.v0 = project(c, a.x, a.y, a.z);
  s.v1 = project(c, b.x, b.y, b.z);
  s.v2 = project(c, d.x, d.y, d.z);
  s.area = edge_fn(s.v0.x, s.v0.y, s.v1.x, s.v1.y, s.v2.x, s.v2.y);
  return s;
}

}  // namespace ugu_gpu
