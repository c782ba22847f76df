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
#include "shade.cuh"

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
                                             const RenderParams& p) {
  float3 r = ray_w(c, x, y);
  bool bf = dot3(fn.x, fn.y, fn.z, r.x, r.y, r.z) > 0.0f;
  Bary b = edges_at(s, x, y);
  if (!covered(b, bf)) return;
  float z = perspective(s, b);
  if (!orderable_depth(z)) {
    atomicAdd(&p.counters->special, 1ull);
    if (p.sticky) atomicOr(p.sticky, kStickySpecial);
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
      for (int x = s.x0; x <= s.x1; ++x) raster_pixel(c, s, fn, f, x, y, keys, p);
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
      if (p.sticky) atomicOr(p.sticky, kStickyOverflow);
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
        raster_pixel(c, s, fn, it.face, xa + k % w, ya + k / w, keys, p);
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
      shade_face_pixel(p.shade, sm, c, fid, project_face(sm, c, fid), x, y, sh);
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
  if (max_faces <= 0) return;  // no face to draw: k_resolve writes the empty images
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
