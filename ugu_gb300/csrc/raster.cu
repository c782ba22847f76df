// raster.cu -- the forward kernels of the GB300 rasterizer.
//
//   k_raster   one thread per (view, face): Loop A + the per-face culls of
//              Loop B (rasterizer.cc:131-193).  Faces whose screen bbox has
//              at most small_bbox_max pixels are rasterised right there;
//              larger faces are split into (face, tile) items.
//   k_tiles    persistent blocks over the (face, tile) items: one block per
//              item, one thread per pixel of the tile.
//   k_resolve  one thread per pixel: Loop C (rasterizer.cc:244-301) with the
//              pixel shaders of pixel_shader.h:215-422.
//
// The z-test of Loop B (rasterizer.cc:228-237) is a 64-bit atomicMin on
// (depth bits << 32 | face id << 1 | back-face bit), see exact.cuh.  The
// resolve recomputes the barycentrics of the winning face from its id
// instead of storing a weight image.
#include <cuda_runtime.h>

#include "internal.cuh"

namespace ugu_gpu {

namespace {

constexpr int kRasterThreads = 256;
constexpr int kResolveThreads = 256;
constexpr int kTileThreads = 256;

__device__ __forceinline__ void load_view(const RenderParams& p, int v, DevView& sv,
                                          DevMesh& sm) {
  // Cooperative copy of the view and mesh descriptors into shared memory.
  const int* src = reinterpret_cast<const int*>(&p.views[v]);
  int* dst = reinterpret_cast<int*>(&sv);
  for (int i = threadIdx.x; i < (int)(sizeof(DevView) / 4); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  const int* msrc = reinterpret_cast<const int*>(&p.meshes[sv.mesh]);
  int* mdst = reinterpret_cast<int*>(&sm);
  for (int i = threadIdx.x; i < (int)(sizeof(DevMesh) / 4); i += blockDim.x) mdst[i] = msrc[i];
  __syncthreads();
}

__device__ __forceinline__ bool setup_face(const DevMesh& m, const Cam& c, int f,
                                           FaceSetup& s) {
  int4 vi = __ldg(&m.vidx[f]);
  float4 a = __ldg(&m.vertices[vi.x]);
  float4 b = __ldg(&m.vertices[vi.y]);
  float4 d = __ldg(&m.vertices[vi.z]);
  float3 p0 = project(c, a.x, a.y, a.z);
  float3 p1 = project(c, b.x, b.y, b.z);
  float3 p2 = project(c, d.x, d.y, d.z);
  return face_setup(c, p0, p1, p2, s);
}

// One pixel test of Loop B's inner body (rasterizer.cc:196-237).
__device__ __forceinline__ void raster_pixel(const Cam& c, const FaceSetup& s, float4 fn,
                                             int f, int x, int y,
                                             unsigned long long* keys,
                                             DevCounters* counters) {
  float3 r = ray_w(c, x, y);
  bool bf = dot3(fn.x, fn.y, fn.z, r.x, r.y, r.z) > 0.0f;
  Bary b = edges_at(s, x, y);
  if (!covered(b, bf)) return;
  float z = perspective(s, b);
  if (!orderable_depth(z)) {
    atomicAdd(&counters->special, 1ull);
    return;
  }
  unsigned long long key = make_key(z, f, bf);
  unsigned long long* kp = keys + (int64_t)y * c.width + x;
  // Keys only decrease, so a stale value read here is never below the
  // current one: skipping the atomic when key >= it is always safe.
  if (key < __ldcg(kp)) atomicMin(kp, key);
}

__global__ void __launch_bounds__(kRasterThreads) k_raster(RenderParams p) {
  __shared__ DevView sv;
  __shared__ DevMesh sm;
  load_view(p, blockIdx.y, sv, sm);
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= sm.num_faces) return;
  const Cam& c = sv.cam;
  FaceSetup s;
  if (!setup_face(sm, c, f, s)) return;
  if (s.x1 < s.x0 || s.y1 < s.y0) return;
  const int64_t npx = (int64_t)(s.x1 - s.x0 + 1) * (int64_t)(s.y1 - s.y0 + 1);
  unsigned long long* keys = p.keys + sv.key_offset;
  if (npx <= p.small_bbox_max) {
    float4 fn = __ldg(&sm.fnormals[f]);
    for (int y = s.y0; y <= s.y1; ++y)
      for (int x = s.x0; x <= s.x1; ++x) raster_pixel(c, s, fn, f, x, y, keys, p.counters);
    return;
  }
  const int ts = p.tile_log2;
  const int tx0 = s.x0 >> ts, tx1 = s.x1 >> ts, ty0 = s.y0 >> ts, ty1 = s.y1 >> ts;
  const int ntx = tx1 - tx0 + 1;
  const int n = ntx * (ty1 - ty0 + 1);
  unsigned long long base = atomicAdd(&p.counters->tile_items, (unsigned long long)n);
  for (int k = 0; k < n; ++k) {
    unsigned long long slot = base + k;
    if (slot >= (unsigned long long)p.item_capacity) {
      atomicAdd(&p.counters->overflow, (unsigned long long)(n - k));
      break;
    }
    TileItem it;
    it.view = blockIdx.y;
    it.face = f;
    it.tx = tx0 + k % ntx;
    it.ty = ty0 + k / ntx;
    p.items[slot] = it;
  }
}

__global__ void __launch_bounds__(kTileThreads) k_tiles(RenderParams p) {
  __shared__ DevView sv;
  __shared__ DevMesh sm;
  __shared__ int cur_view;
  if (threadIdx.x == 0) cur_view = -1;
  __syncthreads();
  unsigned long long n = p.counters->tile_items;
  if (n > (unsigned long long)p.item_capacity) n = p.item_capacity;
  const int T = 1 << p.tile_log2;
  for (unsigned long long i = blockIdx.x; i < n; i += gridDim.x) {
    TileItem it = p.items[i];
    if (it.view != cur_view) {  // uniform across the block
      __syncthreads();
      load_view(p, it.view, sv, sm);
      if (threadIdx.x == 0) cur_view = it.view;
      __syncthreads();
    }
    const Cam& c = sv.cam;
    FaceSetup s;
    setup_face(sm, c, it.face, s);
    float4 fn = __ldg(&sm.fnormals[it.face]);
    const int xa = max(s.x0, it.tx * T), xb = min(s.x1, it.tx * T + T - 1);
    const int ya = max(s.y0, it.ty * T), yb = min(s.y1, it.ty * T + T - 1);
    const int w = xb - xa + 1, h = yb - ya + 1;
    unsigned long long* keys = p.keys + sv.key_offset;
    if (w > 0 && h > 0)
      for (int k = threadIdx.x; k < w * h; k += blockDim.x)
        raster_pixel(c, s, fn, it.face, xa + k % w, ya + k / w, keys, p.counters);
  }
}

// ---- resolve -------------------------------------------------------------

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

struct Shaded {
  uint8_t c[3];
  float cf[3];
  float n[3];
};

// Loop C body for a pixel whose final face id is > 0 (rasterizer.cc:254-299).
__device__ void shade_pixel(const RenderParams& p, const DevMesh& m, const Cam& c, int fid,
                            int x, int y, Shaded& out) {
  FaceSetup s;
  {
    int4 vi = __ldg(&m.vidx[fid]);
    float4 a = __ldg(&m.vertices[vi.x]);
    float4 b = __ldg(&m.vertices[vi.y]);
    float4 d = __ldg(&m.vertices[vi.z]);
    s.v0 = project(c, a.x, a.y, a.z);
    s.v1 = project(c, b.x, b.y, b.z);
    s.v2 = project(c, d.x, d.y, d.z);
    s.area = edge_fn(s.v0.x, s.v0.y, s.v1.x, s.v1.y, s.v2.x, s.v2.y);
  }
  Bary w = edges_at(s, x, y);
  perspective(s, w);

  // shading normal (:268-279) and its camera-frame copy (:282-289)
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
  out.n[0] = dot3(c.R[0], c.R[1], c.R[2], sn[0], sn[1], sn[2]);
  out.n[1] = dot3(c.R[3], c.R[4], c.R[5], sn[0], sn[1], sn[2]);
  out.n[2] = dot3(c.R[6], c.R[7], c.R[8], sn[0], sn[1], sn[2]);

  // colorizer: u = w1, v = w2, weights (1 - u - v), u, v
  const float u = w.w1, v = w.w2;
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
      fetch_texel(t, texel_index(y0, x0, t.width, t.height), t00);
      fetch_texel(t, texel_index(y0, (int64_t)x0 + 1, t.width, t.height), t10);
      fetch_texel(t, texel_index((int64_t)y0 + 1, x0, t.width, t.height), t01);
      fetch_texel(t, texel_index((int64_t)y0 + 1, (int64_t)x0 + 1, t.width, t.height), t11);
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

__global__ void __launch_bounds__(kResolveThreads) k_resolve(RenderParams p) {
  __shared__ DevView sv;
  __shared__ DevMesh sm;
  load_view(p, blockIdx.y, sv, sm);
  const Cam& c = sv.cam;
  const int64_t npx = (int64_t)c.width * c.height;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npx) return;
  const int x = (int)(i % c.width), y = (int)(i / c.width);
  unsigned long long* kp = p.keys + sv.key_offset + i;
  const unsigned long long key = __ldcg(kp);
  __stcg(kp, kEmptyKey);  // leave the z-buffer clear for the next view group
  float depth = 0.0f;
  int32_t fid = -1;
  Shaded sh;
  sh.c[0] = sh.c[1] = sh.c[2] = 0;
  sh.cf[0] = sh.cf[1] = sh.cf[2] = 0.0f;
  sh.n[0] = sh.n[1] = sh.n[2] = 0.0f;
  uint8_t mask = 0;
  if (key != kEmptyKey && !(p.backface_culling && key_backface(key))) {
    depth = key_depth(key);
    fid = key_face(key);
    if (fid > 0) {  // rasterizer.cc:254: face 0 is never shaded
      mask = 255;
      shade_pixel(p, sm, c, fid, x, y, sh);
    }
  }
  if (sv.depth) sv.depth[i] = depth;
  if (sv.face_id) sv.face_id[i] = fid;
  if (sv.mask) sv.mask[i] = mask;
  if (sv.color) {
    sv.color[3 * i + 0] = sh.c[0];
    sv.color[3 * i + 1] = sh.c[1];
    sv.color[3 * i + 2] = sh.c[2];
  }
  if (sv.normal) {
    sv.normal[3 * i + 0] = sh.n[0];
    sv.normal[3 * i + 1] = sh.n[1];
    sv.normal[3 * i + 2] = sh.n[2];
  }
  if (sv.color_f32) {
    sv.color_f32[3 * i + 0] = sh.cf[0];
    sv.color_f32[3 * i + 1] = sh.cf[1];
    sv.color_f32[3 * i + 2] = sh.cf[2];
  }
}

}  // namespace

void launch_raster(const RenderParams& p, int max_faces, int num_sms, cudaStream_t s) {
  (void)num_sms;
  dim3 grid((max_faces + kRasterThreads - 1) / kRasterThreads, p.num_views);
  k_raster<<<grid, kRasterThreads, 0, s>>>(p);
}

void launch_tiles(const RenderParams& p, int grid, cudaStream_t s) {
  k_tiles<<<grid, kTileThreads, 0, s>>>(p);
}

void launch_resolve(const RenderParams& p, int64_t max_pixels, cudaStream_t s) {
  dim3 grid((unsigned)((max_pixels + kResolveThreads - 1) / kResolveThreads), p.num_views);
  k_resolve<<<grid, kResolveThreads, 0, s>>>(p);
}

int raster_launches_per_group() { return 3; }

}  // namespace ugu_gpu
