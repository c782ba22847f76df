// vis.cu -- the image helpers ugu's examples apply to a render
// (examples/ex02_renderer.cc:146-154), as one elementwise device pass:
//   Depth2Gray         src/util/image_util.cc:392-411
//   Normal2Color       src/util/image_util.cc:413-446 (RGB order, no OpenCV)
//   FaceId2RandomColor src/util/image_util.cc:448-487 (RGB order)
//   ConvertTo<uint16_t> include/ugu/image_proc.h:453-475 (16-bit depth)
// Each is HBM-bound (a few bytes in and out per pixel); one thread per pixel
// with the arithmetic of the reference: float for Depth2Gray, double and
// round-half-away for Normal2Color, std::mt19937 seeded with the face id
// for the face colours.
#include <cuda_runtime.h>

#include "internal.cuh"
#include "shade.cuh"

namespace ugu_gpu {

namespace {

constexpr int kVisThreads = 256;

// static_cast<uint8_t>(double) as the Arm and x86 hosts compute it for the
// in-range values these helpers produce: truncation toward zero, low byte
// of the int32 conversion.
__device__ __forceinline__ uint8_t d2u8(double v) { return (uint8_t)(uint32_t)__double2int_rz(v); }

// The first three outputs of std::mt19937(seed) (MT19937, Matsumoto and
// Nishimura 1998): the seeding recurrence up to word 399, one twist of words
// 0..2 and the tempering.  Only words 0..3 and 397..399 of the initial state
// are needed for them.
__device__ __forceinline__ void mt19937_first3(uint32_t seed, uint32_t out[3]) {
  uint32_t lo[4], hi[3];
  uint32_t x = seed;
  lo[0] = x;
  for (uint32_t i = 1; i < 400; ++i) {
    x = 1812433253u * (x ^ (x >> 30)) + i;
    if (i < 4) lo[i] = x;
    if (i >= 397) hi[i - 397] = x;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const uint32_t y = (lo[k] & 0x80000000u) | (lo[k + 1] & 0x7fffffffu);
    uint32_t v = hi[k] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    v ^= v >> 11;
    v ^= (v << 7) & 0x9d2c5680u;
    v ^= (v << 15) & 0xefc60000u;
    v ^= v >> 18;
    out[k] = v;
  }
}

__global__ void __launch_bounds__(kVisThreads) k_vis(ugu_gpu_vis it) {
  const int64_t npx = (int64_t)it.width * it.height;
  const int64_t i = (int64_t)blockIdx.x * kVisThreads + threadIdx.x;
  if (i >= npx) return;
  if (it.depth) {
    const float d = it.depth[i];
    if (it.vis_depth) {
      const float inv_denom = fdiv(1.0f, fsub(it.max_d, it.min_d));
      float norm = fmul(fsub(d, it.min_d), inv_denom);
      norm = norm < 0.0f ? 0.0f : norm;  // std::max(norm, 0.0f)
      norm = 1.0f < norm ? 1.0f : norm;  // std::min(.., 1.0f)
      it.vis_depth[i] = f2u8(fmul(norm, 255.0f));
    }
    if (it.depth_u16) {  // static_cast<uint16_t>(double(1.0f) * double(d))
      const double v = __dmul_rn(1.0, (double)d);
      it.depth_u16[i] = (uint16_t)(uint32_t)__double2int_rz(v);
    }
  }
  if (it.normal && it.vis_normal) {
    double n[3] = {it.normal[3 * i], it.normal[3 * i + 1], it.normal[3 * i + 2]};
    float nf[3] = {it.normal[3 * i], it.normal[3 * i + 1], it.normal[3 * i + 2]};
    if (it.gl_coord) {
      nf[0] = fmul(nf[0], -1.0f);
      nf[2] = fmul(nf[2], -1.0f);
    }
    n[0] = nf[0];
    n[1] = nf[1];
    n[2] = nf[2];
    // round((n + 1.0) * 0.5 * 255) for x, y; round(-n * 127.0) + 128 for z
    it.vis_normal[3 * i + 0] = d2u8(round(__dmul_rn(__dmul_rn(__dadd_rn(n[0], 1.0), 0.5), 255.0)));
    it.vis_normal[3 * i + 1] = d2u8(round(__dmul_rn(__dmul_rn(__dadd_rn(n[1], 1.0), 0.5), 255.0)));
    it.vis_normal[3 * i + 2] = d2u8(__dadd_rn(round(__dmul_rn(-n[2], 127.0)), 128.0));
  }
  if (it.face_id && it.vis_face_id) {
    const int32_t fid = it.face_id[i];
    uint8_t c[3] = {0, 0, 0};
    if (fid >= 0) {
      uint32_t r[3];
      mt19937_first3((uint32_t)fid, r);
      c[0] = (uint8_t)(r[0] % 256);
      c[1] = (uint8_t)(r[1] % 256);
      c[2] = (uint8_t)(r[2] % 256);
    }
    it.vis_face_id[3 * i + 0] = c[0];
    it.vis_face_id[3 * i + 1] = c[1];
    it.vis_face_id[3 * i + 2] = c[2];
  }
}

}  // namespace

void launch_vis(const ugu_gpu_vis& item, cudaStream_t s) {
  const int64_t npx = (int64_t)item.width * item.height;
  if (npx <= 0) return;
  k_vis<<<(unsigned)((npx + kVisThreads - 1) / kVisThreads), kVisThreads, 0, s>>>(item);
}

}  // namespace ugu_gpu

// ---------------------------------------------------------------------------
// G-buffer channels (ugu_gpu_render_gbuffer): one thread per pixel of one
// view, from the face the render reported and the forward's own arithmetic
// (project_face, edges_at, perspective of exact.cuh / shade.cuh).
// ---------------------------------------------------------------------------

namespace ugu_gpu {

namespace {

__global__ void __launch_bounds__(kVisThreads) k_gbuffer(GbufParams p) {
  const Cam& c = p.cam;
  const DevMesh& m = *p.mesh;
  const int64_t npx = (int64_t)c.width * c.height;
  const int64_t i = (int64_t)blockIdx.x * kVisThreads + threadIdx.x;
  if (i >= npx) return;
  const int fid = p.face_id[i];
  float pw[3] = {0, 0, 0}, pc[3] = {0, 0, 0}, nw[3] = {0, 0, 0}, nc[3] = {0, 0, 0};
  float bary[3] = {0, 0, 0}, uv[3] = {0, 0, 0};
  uint8_t stencil = 0;
  if (fid < -1 || fid >= m.num_faces) {
    atomicAdd(p.bad_ids, 1ull);
  } else if (fid >= 0) {
    stencil = 255;
    const int y = (int)(i / c.width), x = (int)(i - (int64_t)y * c.width);
    const FaceSetup s = project_face(m, c, fid);
    Bary w = edges_at(s, x, y);
    perspective(s, w);
    bary[0] = w.w1;
    bary[1] = w.w2;
    bary[2] = fsub(fsub(1.0f, w.w1), w.w2);
    const int4 vi = __ldg(&m.vidx[fid]);
    const float4 P0 = __ldg(&m.vertices[vi.x]), P1 = __ldg(&m.vertices[vi.y]),
                 P2 = __ldg(&m.vertices[vi.z]);
    pw[0] = fadd(fadd(fmul(w.w0, P0.x), fmul(w.w1, P1.x)), fmul(w.w2, P2.x));
    pw[1] = fadd(fadd(fmul(w.w0, P0.y), fmul(w.w1, P1.y)), fmul(w.w2, P2.y));
    pw[2] = fadd(fadd(fmul(w.w0, P0.z), fmul(w.w1, P1.z)), fmul(w.w2, P2.z));
#pragma unroll
    for (int k = 0; k < 3; ++k)
      pc[k] = fadd(c.t[k], dot3(c.R[3 * k], c.R[3 * k + 1], c.R[3 * k + 2], pw[0], pw[1], pw[2]));
    float sn[3];
    if (p.shading_normal == 0) {
      const float4 fn = __ldg(&m.fnormals[fid]);
      sn[0] = fn.x;
      sn[1] = fn.y;
      sn[2] = fn.z;
    } else {
      const int4 ni = __ldg(&m.nidx[fid]);
      const float4 n0 = __ldg(&m.normals[ni.x]), n1 = __ldg(&m.normals[ni.y]),
                   n2 = __ldg(&m.normals[ni.z]);
      sn[0] = fadd(fadd(fmul(w.w0, n0.x), fmul(w.w1, n1.x)), fmul(w.w2, n2.x));
      sn[1] = fadd(fadd(fmul(w.w0, n0.y), fmul(w.w1, n1.y)), fmul(w.w2, n2.y));
      sn[2] = fadd(fadd(fmul(w.w0, n0.z), fmul(w.w1, n1.z)), fmul(w.w2, n2.z));
    }
    // Eigen's normalize: divide by sqrt(n . n) when it is > 0
    const float n2 = dot3(sn[0], sn[1], sn[2], sn[0], sn[1], sn[2]);
    if (n2 > 0.0f) {
      const float r = __fsqrt_rn(n2);
#pragma unroll
      for (int k = 0; k < 3; ++k) nw[k] = fdiv(sn[k], r);
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) nw[k] = sn[k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
      nc[k] = dot3(c.R[3 * k], c.R[3 * k + 1], c.R[3 * k + 2], nw[0], nw[1], nw[2]);
    if (m.uv) {  // the colorizer's weights (1 - u - v), u, v
      const float s0 = fsub(fsub(1.0f, w.w1), w.w2);
      const int4 ti = __ldg(&m.uvidx[fid]);
      const float2 a = __ldg(&m.uv[ti.x]), b = __ldg(&m.uv[ti.y]), d = __ldg(&m.uv[ti.z]);
      uv[0] = fadd(fadd(fmul(s0, a.x), fmul(w.w1, b.x)), fmul(w.w2, d.x));
      uv[1] = fadd(fadd(fmul(s0, a.y), fmul(w.w1, b.y)), fmul(w.w2, d.y));
      uv[2] = fsub(fsub(1.0f, uv[0]), uv[1]);
    }
  }
  auto put3 = [&](float* o, const float* v) {
    if (o) {
      o[3 * i + 0] = v[0];
      o[3 * i + 1] = v[1];
      o[3 * i + 2] = v[2];
    }
  };
  put3(p.pos_wld, pw);
  put3(p.pos_cam, pc);
  put3(p.normal_wld, nw);
  put3(p.normal_cam, nc);
  put3(p.bary, bary);
  put3(p.uv, uv);
  if (p.stencil) p.stencil[i] = stencil;
}

}  // namespace

void launch_gbuffer(const GbufParams& p, cudaStream_t s) {
  const int64_t npx = (int64_t)p.cam.width * p.cam.height;
  if (npx <= 0) return;
  k_gbuffer<<<(unsigned)((npx + kVisThreads - 1) / kVisThreads), kVisThreads, 0, s>>>(p);
}

}  // namespace ugu_gpu
