// texmap.cu -- TextureMapping's texture on the mesh's own uv
// (src/texturing/texture_mapper.cc: TextureMappingSimple :924-1006 with
// kUseOriginalMeshUv, GenerateTextureOnOriginalUv :294-345), or on the
// triangles of a generated layout (kGenerateSimpleTriangles,
// GenerateSimpleTrianglesTextureAndUv :347-440: the host lays the faces
// out and passes their target triangles).
//
// The reference walks the faces in order and rasterizes each face's uv
// triangle into the texture (RasterizeTriangle, :234-292), sampling its
// best keyframe's colour image at the same barycentric point of the face's
// projected triangle; a later face overwrites an earlier one.  Here:
//   k_tm_cover  one warp per face, its lanes over the texels of the face's
//               box: every texel its uv triangle covers takes the face
//               number by atomicMax, so the last face in order wins, as in
//               the sequential loop;
//   k_tm_fill   one thread per texel: the winning face's weights at the
//               texel (the same float operations) and the bilinear sample
//               (BilinearInterpolation, include/ugu/util/image_util.h:156-192);
//   k_tm_pad    one thread per texel: PaddingSimple (:148-201), each empty
//               texel away from the border takes the float mean of the valid
//               texels of its kernel window, read from the unpadded copy.
// Each pass is HBM- or latency-bound on a few bytes per texel.
#include <cuda_runtime.h>

#include "internal.cuh"

namespace ugu_gpu {

namespace {

constexpr int kTmThreads = 256;

// The face's uv triangle in texel coordinates (:316-321).
struct UvTri {
  float x[3], y[3];
};

__device__ __forceinline__ UvTri uv_tri(const TexMapParams& p, int f) {
  UvTri t;
  if (p.face_target) {  // a layout's own triangle (the atlas uv types)
    const float* q = p.face_target + 6 * (int64_t)f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      t.x[j] = __ldg(&q[2 * j]);
      t.y[j] = __ldg(&q[2 * j + 1]);
    }
    return t;
  }
  const int4 ti = __ldg(&p.uvidx[f]);
  const int idx[3] = {ti.x, ti.y, ti.z};
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float2 u = __ldg(&p.uv[idx[j]]);
    t.x[j] = fsub(fmul(u.x, (float)p.tex_w), 0.5f);
    t.y[j] = fsub(fmul(fsub(1.0f, u.y), (float)p.tex_h), 0.5f);
  }
  return t;
}

// 1 / area, the area kept away from zero as the reference does (:238-242).
__device__ __forceinline__ float inv_area(const UvTri& t) {
  float area = edge_fn(t.x[0], t.y[0], t.x[1], t.y[1], t.x[2], t.y[2]);
  if (fabsf(area) < FLT_MIN) area = area > 0.0f ? FLT_MIN : -FLT_MIN;
  return fdiv(1.0f, area);
}

// The weights of texel (x, y); false outside the triangle (:262-276).
__device__ __forceinline__ bool tm_weights(const UvTri& t, float ia, int x, int y, float w[3]) {
  const float px = (float)x, py = (float)y;
  w[0] = fmul(edge_fn(t.x[1], t.y[1], t.x[2], t.y[2], px, py), ia);
  w[1] = fmul(edge_fn(t.x[2], t.y[2], t.x[0], t.y[0], px, py), ia);
  w[2] = fmul(edge_fn(t.x[0], t.y[0], t.x[1], t.y[1], px, py), ia);
  return !(w[0] < 0.0f || w[1] < 0.0f || w[2] < 0.0f);
}

// One warp per face (kTmThreads / 32 faces per block); the lanes take the
// box's texels in row-major order, 32 at a time.
__global__ void __launch_bounds__(kTmThreads) k_tm_cover(TexMapParams p) {
  const int64_t fw = (int64_t)blockIdx.x * (kTmThreads / 32) + threadIdx.x / 32;
  if (fw >= p.num_faces) return;
  const int f = (int)fw;
  if (__ldg(&p.face_kf[f]) < 0) return;
  const int lane = threadIdx.x & 31;
  const UvTri t = uv_tri(p, f);
  const float ia = inv_area(t);
  // the bounding box: int casts of min - 1 and max + 1, clamped (:245-256)
  auto clampi = [](int v, int hi) { return max(0, min(v, hi)); };
  const int x0 = clampi(f2i_sat(fsub(min3_std(t.x[0], t.x[1], t.x[2]), 1.0f)), p.tex_w - 1);
  const int x1 = clampi(f2i_sat(fadd(max3_std(t.x[0], t.x[1], t.x[2]), 1.0f)), p.tex_w - 1);
  const int y0 = clampi(f2i_sat(fsub(min3_std(t.y[0], t.y[1], t.y[2]), 1.0f)), p.tex_h - 1);
  const int y1 = clampi(f2i_sat(fadd(max3_std(t.y[0], t.y[1], t.y[2]), 1.0f)), p.tex_h - 1);
  const int bw = x1 - x0 + 1;
  const int64_t n = (int64_t)bw * (y1 - y0 + 1);
  for (int64_t k = lane; k < n; k += 32) {
    const int y = y0 + (int)(k / bw), x = x0 + (int)(k % bw);
    float w[3];
    if (tm_weights(t, ia, x, y, w)) atomicMax(&p.owner[(int64_t)y * p.tex_w + x], f);
  }
}

// BilinearInterpolation<Vec3b>: floor, the lower corner clamped at 0 and
// the upper one at the last column / row, float weights, truncation to a
// byte.  A read outside the image's allocation is clamped to it.
__device__ __forceinline__ void bilinear3(const DevKeyframe& k, float x, float y, uint8_t* out) {
  const int cols = k.cam.width, rows = k.cam.height;
  int xa = f2i_sat(floorf(x)), ya = f2i_sat(floorf(y));
  int xb = xa + 1, yb = ya + 1;
  if (xa < 0) xa = 0;
  if (ya < 0) ya = 0;
  if (cols <= xb) xb = cols - 1;
  if (rows <= yb) yb = rows - 1;
  const float lu = fsub(x, (float)xa), lv = fsub(y, (float)ya);
  const float nu = fsub(1.0f, lu), nv = fsub(1.0f, lv);
  const int64_t n = (int64_t)cols * rows;
  auto px = [&](int yy, int xx) {
    int64_t i = (int64_t)yy * cols + xx;
    i = i < 0 ? 0 : (i >= n ? n - 1 : i);
    return k.color + 3 * i;
  };
  const uint8_t *a = px(ya, xa), *b = px(ya, xb), *c = px(yb, xa), *d = px(yb, xb);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const float v = fadd(fadd(fadd(fmul(fmul(nu, nv), (float)a[ch]), fmul(fmul(lu, nv), (float)b[ch])),
                              fmul(fmul(nu, lv), (float)c[ch])),
                         fmul(fmul(lu, lv), (float)d[ch]));
    out[ch] = f2u8(v);
  }
}

__global__ void __launch_bounds__(kTmThreads) k_tm_fill(TexMapParams p) {
  const int64_t n = (int64_t)p.tex_w * p.tex_h;
  const int64_t i = (int64_t)blockIdx.x * kTmThreads + threadIdx.x;
  if (i >= n) return;
  const int f = p.owner[i];
  uint8_t rgb[3] = {0, 0, 0};
  uint8_t m = 0;
  if (f >= 0) {
    const int y = (int)(i / p.tex_w), x = (int)(i - (int64_t)y * p.tex_w);
    const UvTri t = uv_tri(p, f);
    float w[3];
    tm_weights(t, inv_area(t), x, y, w);  // covered: k_tm_cover tested the same values
    const float* s = p.face_tri + 6 * (int64_t)f;
    // src_pos = w0 * s0 + w1 * s1 + w2 * s2 (:279-281)
    const float sx = fadd(fadd(fmul(w[0], s[0]), fmul(w[1], s[2])), fmul(w[2], s[4]));
    const float sy = fadd(fadd(fmul(w[0], s[1]), fmul(w[1], s[3])), fmul(w[2], s[5]));
    bilinear3(p.kf[__ldg(&p.face_kf[f])], sx, sy, rgb);
    m = 255;
  }
  p.tex0[3 * i + 0] = rgb[0];
  p.tex0[3 * i + 1] = rgb[1];
  p.tex0[3 * i + 2] = rgb[2];
  p.mask0[i] = m;
}

__global__ void __launch_bounds__(kTmThreads) k_tm_pad(TexMapParams p) {
  const int64_t n = (int64_t)p.tex_w * p.tex_h;
  const int64_t i = (int64_t)blockIdx.x * kTmThreads + threadIdx.x;
  if (i >= n) return;
  const int y = (int)(i / p.tex_w), x = (int)(i - (int64_t)y * p.tex_w);
  uint8_t rgb[3] = {p.tex0[3 * i], p.tex0[3 * i + 1], p.tex0[3 * i + 2]};
  uint8_t m = p.mask0[i];
  const int hk = p.hk;
  if (m != 255 && y >= hk && y < p.tex_h - hk && x >= hk && x < p.tex_w - hk) {
    float sum[3] = {0.0f, 0.0f, 0.0f};
    int cnt = 0;
    for (int jj = -hk; jj <= hk; ++jj)
      for (int ii = -hk; ii <= hk; ++ii) {
        const int64_t q = (int64_t)(y + jj) * p.tex_w + (x + ii);
        if (p.mask0[q] != 255) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) sum[c] = fadd(sum[c], (float)p.tex0[3 * q + c]);
        ++cnt;
      }
    if (cnt) {
      m = 255;
#pragma unroll
      for (int c = 0; c < 3; ++c) rgb[c] = f2u8(fdiv(sum[c], (float)cnt));
    }
  }
  p.tex[3 * i + 0] = rgb[0];
  p.tex[3 * i + 1] = rgb[1];
  p.tex[3 * i + 2] = rgb[2];
  p.mask[i] = m;
}

}  // namespace

void launch_texture_mapping(const TexMapParams& p, cudaStream_t s) {
  const int64_t n = (int64_t)p.tex_w * p.tex_h;
  cudaMemsetAsync(p.owner, 0xff, sizeof(int32_t) * (size_t)n, s);  // -1: no face
  if (p.num_faces > 0)
    k_tm_cover<<<(unsigned)(((int64_t)p.num_faces + kTmThreads / 32 - 1) / (kTmThreads / 32)),
                 kTmThreads, 0, s>>>(p);
  const unsigned blocks = (unsigned)((n + kTmThreads - 1) / kTmThreads);
  k_tm_fill<<<blocks, kTmThreads, 0, s>>>(p);
  k_tm_pad<<<blocks, kTmThreads, 0, s>>>(p);
}

}  // namespace ugu_gpu
