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


// DiffuseVertexColorColorizer (pixel_shader.h:234-256): the colour at
// weights (s0, u, v) = (1 - u - v, u, v) of the face's vertex colours.
__device__ __forceinline__ void vertex_color(float s0, float u, float v, float4 c0, float4 c1,
                                             float4 c2, float col[3]) {
  col[0] = fadd(fadd(fmul(s0, c0.x), fmul(u, c1.x)), fmul(v, c2.x));
  col[1] = fadd(fadd(fmul(s0, c0.y), fmul(u, c1.y)), fmul(v, c2.y));
  col[2] = fadd(fadd(fmul(s0, c0.z), fmul(u, c1.z)), fmul(v, c2.z));
}

// DiffuseTextureNn/BilinearColorizer (pixel_shader.h:260-359): the texture
// colour at weights (s0, u, v) of the face's uvs a, b, d.
__device__ __forceinline__ void texture_color(const ShadeOpts& p, const DevTexture& t, float s0,
                                              float u, float v, float2 a, float2 b, float2 d,
                                              float col[3]) {
  const float uvx = fadd(fadd(fmul(s0, a.x), fmul(u, b.x)), fmul(v, d.x));
  const float uvy = fadd(fadd(fmul(s0, a.y), fmul(u, b.y)), fmul(v, d.y));
  const float fx = fmul(uvx, (float)(t.width - 1));
  const float fy = fmul(fsub(1.0f, uvy), (float)(t.height - 1));
  if (p.interp == 0) {
    const int32_t tx = f2i_sat(roundf(fx));
    const int32_t ty = f2i_sat(roundf(fy));
    fetch_texel(t, texel_index(ty, tx, t.width, t.height), col);
    return;
  }
  const int32_t x0 = f2i_sat(floorf(fx));
  const int32_t y0 = f2i_sat(floorf(fy));
  const float lu = fsub(fx, (float)x0);
  const float lv = fsub(fy, (float)y0);
  float t00[3], t10[3], t01[3], t11[3];
  // the four taps: one linear address and its neighbours (the unclamped
  // min + 1 of the reference), each clamped to the allocation on its own;
  // no clamp can apply when the cell lies inside the texture
  const int64_t i00 = (int64_t)y0 * t.width + x0;
  if ((unsigned)x0 < (unsigned)(t.width - 1) && (unsigned)y0 < (unsigned)(t.height - 1)) {
    fetch_texel(t, i00, t00);
    fetch_texel(t, i00 + 1, t10);
    fetch_texel(t, i00 + t.width, t01);
    fetch_texel(t, i00 + t.width + 1, t11);
  } else {
    const int64_t n = (int64_t)t.width * t.height;
    auto clampi = [n](int64_t i) { return i < 0 ? (int64_t)0 : (i >= n ? n - 1 : i); };
    fetch_texel(t, clampi(i00), t00);
    fetch_texel(t, clampi(i00 + 1), t10);
    fetch_texel(t, clampi(i00 + t.width), t01);
    fetch_texel(t, clampi(i00 + t.width + 1), t11);
  }
  const float a00 = fmul(fsub(1.0f, lu), fsub(1.0f, lv));
  const float a10 = fmul(lu, fsub(1.0f, lv));
  const float a01 = fmul(fsub(1.0f, lu), lv);
  const float a11 = fmul(lu, lv);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    col[k] = fadd(fadd(fadd(fmul(a00, t00[k]), fmul(a10, t10[k])), fmul(a01, t01[k])),
                  fmul(a11, t11[k]));
}

// The colorizer's result to 8 bits, then the diffuse shader (Lambertian
// pixel_shader.h:370-388 or Oren-Nayar :392-422) with light_dir = ray_w
// (rasterizer.cc:293).
__device__ __forceinline__ void finish_shading(const ShadeOpts& p, const Cam& c, const float sn[3],
                                               int x, int y, const float col[3], Shaded& out) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    out.cf[k] = col[k];
    out.c[k] = p.diffuse_color == 0 ? (uint8_t)255 : f2u8(col[k]);
  }
  if (p.diffuse_shading != 0) {
    float3 r = ray_w(c, x, y);
    if (p.diffuse_shading == 1) {
      float coeff = -dot3(r.x, r.y, r.z, sn[0], sn[1], sn[2]);
      if (coeff < 0.0f) coeff = 0.0f;
#pragma unroll
      for (int k = 0; k < 3; ++k) out.c[k] = f2u8(fmul(coeff, (float)out.c[k]));
    } else {
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

// The camera-frame normal w2c_R * sn (rasterizer.cc:282-289,
// raytracer.cc:192-199).
__device__ __forceinline__ void camera_normal(const Cam& c, const float sn[3], Shaded& out) {
  out.n[0] = dot3(c.R[0], c.R[1], c.R[2], sn[0], sn[1], sn[2]);
  out.n[1] = dot3(c.R[3], c.R[4], c.R[5], sn[0], sn[1], sn[2]);
  out.n[2] = dot3(c.R[6], c.R[7], c.R[8], sn[0], sn[1], sn[2]);
}

// The pixel shader of one pixel (pixel_shader.h:215-422) given the face,
// the colorizer's (u, v), the world-frame shading normal sn and the pixel;
// also the camera-frame normal w2c_R * sn.
__device__ __forceinline__ void shade_uv(const ShadeOpts& p, const DevMesh& m, const Cam& c,
                                         int fid, float u, float v, const float sn[3], int x,
                                         int y, Shaded& out) {
  camera_normal(c, sn, out);
  // colorizer: weights (1 - u - v), u, v
  const float s0 = fsub(fsub(1.0f, u), v);
  float col[3] = {255.0f, 255.0f, 255.0f};
  if (p.diffuse_color == 2) {
    const int4 vi = __ldg(&m.vidx[fid]);
    vertex_color(s0, u, v, __ldg(&m.vcolors[vi.x]), __ldg(&m.vcolors[vi.y]),
                 __ldg(&m.vcolors[vi.z]), col);
  } else if (p.diffuse_color == 1) {
    const DevTexture t = m.textures[__ldg(&m.mat_ids[fid])];
    const int4 ti = __ldg(&m.uvidx[fid]);
    texture_color(p, t, s0, u, v, __ldg(&m.uv[ti.x]), __ldg(&m.uv[ti.y]), __ldg(&m.uv[ti.z]),
                  col);
  }
  finish_shading(p, c, sn, x, y, col, out);
}

// Loop C (rasterizer.cc:254-299) for one pixel of the tiled resolve whose
// winning face fid > 0 and its depth z are known, for one colour source
// (kColor: 0 white, 1 texture, 2 vertex colour) and shading normal (kNormal:
// 0 face, 1 vertex).  The arithmetic is shade_face_pixel's with the
// z-buffer's depth standing in for the one perspective() would recompute
// (bit-identical: the same inputs and operations).  The face's gathers are
// issued in groups -- the vertex ranks and the normal and colour indices,
// then the projected vertices and uvs or colours, then the normals and the
// texels -- rather than one after another.  tex0 is the first material's
// texture: a mesh with one material has only material id 0
// (ugu_gpu_set_mesh checks every id), so its id is not read.
template <int kColor, int kNormal>
__device__ __forceinline__ void shade_tile_pixel_t(const ShadeOpts& p, const DevMesh& m,
                                                   const DevTexture& tex0, const Cam& c,
                                                   const float4* proj, int fid, int x, int y,
                                                   float z, Shaded& out) {
  const int4 vi = __ldg(&m.vidx_ranked[fid]);
  const int4 ni = kNormal ? __ldg(&m.nidx[fid]) : make_int4(0, 0, 0, 0);
  const float4 fn = kNormal ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : __ldg(&m.fnormals[fid]);
  const int4 ci = kColor == 2 ? __ldg(&m.vidx[fid])
                              : (kColor == 1 ? __ldg(&m.uvidx[fid]) : make_int4(0, 0, 0, 0));
  const int mat = (kColor == 1 && m.num_materials != 1) ? __ldg(&m.mat_ids[fid]) : 0;
  const float4 a = __ldg(&proj[vi.x]);
  const float4 b = __ldg(&proj[vi.y]);
  const float4 d = __ldg(&proj[vi.z]);
  float4 c0, c1, c2;
  float2 u0, u1, u2;
  if (kColor == 2) {
    c0 = __ldg(&m.vcolors[ci.x]);
    c1 = __ldg(&m.vcolors[ci.y]);
    c2 = __ldg(&m.vcolors[ci.z]);
  }
  if (kColor == 1) {
    u0 = __ldg(&m.uv[ci.x]);
    u1 = __ldg(&m.uv[ci.y]);
    u2 = __ldg(&m.uv[ci.z]);
  }
  // Loop C's weights (rasterizer.cc:208-224) with the z-buffer's depth
  FaceSetup s;
  s.v0 = make_float3(a.x, a.y, a.z);
  s.v1 = make_float3(b.x, b.y, b.z);
  s.v2 = make_float3(d.x, d.y, d.z);
  s.area = edge_fn(a.x, a.y, b.x, b.y, d.x, d.y);
  Bary w = edges_at(s, x, y);
  perspective_at(s, w, z);
  // shading normal (:268-279) from the weights; the vertex normals are
  // fetched only now, which keeps the kernel within its register budget
  float sn[3];
  if (kNormal) {
    const float4 n0 = __ldg(&m.normals[ni.x]);
    const float4 n1 = __ldg(&m.normals[ni.y]);
    const float4 n2 = __ldg(&m.normals[ni.z]);
    sn[0] = fadd(fadd(fmul(w.w0, n0.x), fmul(w.w1, n1.x)), fmul(w.w2, n2.x));
    sn[1] = fadd(fadd(fmul(w.w0, n0.y), fmul(w.w1, n1.y)), fmul(w.w2, n2.y));
    sn[2] = fadd(fadd(fmul(w.w0, n0.z), fmul(w.w1, n1.z)), fmul(w.w2, n2.z));
  } else {
    sn[0] = fn.x;
    sn[1] = fn.y;
    sn[2] = fn.z;
  }
  camera_normal(c, sn, out);
  // the colorizer's u = w1, v = w2
  const float u = w.w1, v = w.w2;
  const float s0 = fsub(fsub(1.0f, u), v);
  float col[3] = {255.0f, 255.0f, 255.0f};
  if (kColor == 2) vertex_color(s0, u, v, c0, c1, c2, col);
  if (kColor == 1) {
    const DevTexture t = m.num_materials == 1 ? tex0 : m.textures[mat];
    texture_color(p, t, s0, u, v, u0, u1, u2, col);
  }
  finish_shading(p, c, sn, x, y, col, out);
}

__device__ __forceinline__ void shade_tile_pixel(const ShadeOpts& p, const DevMesh& m,
                                                 const DevTexture& tex0, const Cam& c,
                                                 const float4* proj, int fid, int x, int y,
                                                 float z, Shaded& out) {
  if (p.diffuse_color == 1) {
    if (p.shading_normal)
      shade_tile_pixel_t<1, 1>(p, m, tex0, c, proj, fid, x, y, z, out);
    else
      shade_tile_pixel_t<1, 0>(p, m, tex0, c, proj, fid, x, y, z, out);
  } else if (p.diffuse_color == 2) {
    if (p.shading_normal)
      shade_tile_pixel_t<2, 1>(p, m, tex0, c, proj, fid, x, y, z, out);
    else
      shade_tile_pixel_t<2, 0>(p, m, tex0, c, proj, fid, x, y, z, out);
  } else {
    if (p.shading_normal)
      shade_tile_pixel_t<0, 1>(p, m, tex0, c, proj, fid, x, y, z, out);
    else
      shade_tile_pixel_t<0, 0>(p, m, tex0, c, proj, fid, x, y, z, out);
  }
}

// Loop C body for a pixel whose final face id is > 0 (rasterizer.cc:254-299),
// given the winning face's projected vertices and area (the global path's
// resolve).
__device__ __forceinline__ void shade_face_pixel(const ShadeOpts& p, const DevMesh& m,
                                                 const Cam& c, int fid, const FaceSetup& s,
                                                 int x, int y, Shaded& out) {
  Bary w = edges_at(s, x, y);
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
