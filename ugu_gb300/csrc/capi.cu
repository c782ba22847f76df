// capi.cu -- the C ABI of include/ugu_gpu.h: context, mesh upload,
// validation, batched rendering, CUDA-graph plans.
//
// Validation follows ValidateAndInitBeforeRender
// (src/renderer/cpu/util_private.cc:12-90) case by case and in the same
// order; failures return the matching status code with the reference's
// message in ugu_gpu_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "internal.cuh"
#include "ugu_gpu.h"

using namespace ugu_gpu;

namespace {

// An NVTX range over a scope (NVTX 3 is header-only: without a tool attached
// the calls return at once).  Profilers group the kernels an entry point
// launches under its range, e.g. `ncu --nvtx --nvtx-include "ugu_gpu tile/"`
// for a direct render's tile kernels (a plan replays under its launch range).
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};

}  // namespace

namespace {

constexpr int kMaxMeshes = 16;
thread_local std::string g_create_error;

struct MeshSlot {
  bool present = false;
  DevMesh dev{};
  std::vector<ugu_gpu_device_texture> dev_tex;  // device texture pointers, host copy
  std::vector<void*> allocs;
  bool has_fnormals = false, has_normals = false, has_vcolors = false;
  bool has_uv = false, has_matids = false;
  int num_materials = 0;
  bool all_textures_nonempty = true;
  bool all_textures_f32 = false;
  int tex0_w = 0, tex0_h = 0;
  float centre[3] = {0.0f, 0.0f, 0.0f};  // bounding-box centre of the vertices
  size_t bytes = 0;
  // raytracer: host copies of positions and faces, its BVH built on first use
  std::vector<float> h_vertices;
  std::vector<int32_t> h_faces;
  bool bvh = false;
  bool vis_bvh = false;  // the visibility tester's tree (leaves of up to 5 faces)
};

// Device scratch of one render sequence.  A plan owns its own so that later
// renders on the context cannot move buffers a captured graph points at.
struct Scratch {
  unsigned long long* keys = nullptr;
  size_t keys_cap = 0;
  TileItem* items = nullptr;
  size_t items_cap = 0;
  DevCounters* counters = nullptr;
  DevCounters* h_counters = nullptr;  // pinned
  size_t counters_cap = 0;
  DevView* d_views = nullptr;
  DevView* h_views = nullptr;  // pinned
  size_t views_cap = 0;
  uint8_t* d_out = nullptr;  // device outputs of host-pointer renders
  size_t d_out_cap = 0;
  bool keys_dirty = false;
  // tiled path
  int32_t* tile_count = nullptr;  // 4 arrays: count, offsets (+1), lo cursor, hi cursor
  size_t tiles_cap = 0;
  long long* chunk_sums = nullptr;  // the tile-count scan's chunk sums, for tiles_cap tiles
  int2* entries = nullptr;  // entries_cap entries in tile order
  size_t entries_cap = 0;
  size_t entries_min = 0;  // capacity asked for by the last overflow
  float4* proj = nullptr;
  size_t proj_cap = 0;
  TileCounters* tcounters = nullptr;
  TileCounters* h_tcounters = nullptr;  // pinned
  size_t tcounters_cap = 0;
  bool tiles_dirty = false;
  // signature of the view list the entry and run lists were last sized for
  // by a sizing pass (asynchronous renders size before they enqueue)
  uint64_t sized_sig = 0;
  size_t list_min = size_t(1) << 22;  // capacity of the item / overflow lists
  // backward: per-view target pointers, hi + lo projection table
  void* proj64 = nullptr;    // 32 bytes per vertex of every view
  size_t proj64_cap = 0;     // vertices
  float* grad4 = nullptr;   // backward: RGBA texel-gradient scratch
  size_t grad4_cap = 0;     // texels
  const float** d_targets = nullptr;
  const float** h_targets = nullptr;  // pinned
  size_t targets_cap = 0;
};

struct Group {
  int first, count;
  int max_faces;
  int64_t max_pixels;
  int64_t tiles;     // tiled path: screen tiles of the group's views
  int64_t faces;     // tiled path: faces summed over the group's views
  int64_t vertices;  // tiled path: vertices summed over the group's views
  int max_vertices;
  int64_t ray_tiles;  // raytracer: the most kRayTileW x kRayTileH tiles of a view
};

}  // namespace

namespace ugu_gpu {
// Error message for ugu_gpu_last_error(NULL) from entry points without a context.
void set_thread_error(const char* msg) { g_create_error = msg; }
}  // namespace ugu_gpu

struct ugu_gpu_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // device-to-host copies of host-pointer renders
  // UGU_GPU_TIME_KERNELS: events around each tile-kernel launch of a render
  std::vector<cudaEvent_t> tile_events;
  bool time_tile = false;
  int timed_groups = 0;
  double tile_ms = 0.0;
  uint64_t tile_launches = 0;
  std::vector<cudaEvent_t> events;     // one per group of a host-pointer render, and one more
  std::string last_error;
  ugu_gpu_option opt{};
  MeshSlot meshes[kMaxMeshes];
  DevMesh* d_meshes = nullptr;
  ugu_gpu_tuning tuning{};
  Scratch scratch;
  uint64_t launches = 0;
  uint64_t special = 0;
  uint64_t large_items = 0;
  // counters of the last asynchronous plan replay, checked at synchronize
  ugu_gpu_plan* pending_plan = nullptr;
  // groups of the last UGU_GPU_ASYNC render, whose counters synchronize checks
  size_t pending_async_groups = 0;
  // sticky status word the kernels set (kStickyOverflow, kStickySpecial):
  // read and cleared by ugu_gpu_synchronize, so that no asynchronous render
  // or replay whose lists overflowed passes unreported
  unsigned long long* d_sticky = nullptr;
  // set while an asynchronous render or a plan is enqueued: only those use
  // the sticky word (a synchronous render checks and retries on its own)
  bool sticky_on = false;
  uint64_t mesh_generation = 0;  // bumped by every ugu_gpu_set_mesh
  // ugu_gpu_autotune's results, keyed by workload shape
  std::map<uint64_t, ugu_gpu_tuning> tuned;
  // set while a UGU_GPU_RAYTRACE render or plan is being prepared and enqueued
  bool raytrace = false;
  // plans created on this context and not destroyed yet (destroyed with it)
  std::vector<ugu_gpu_plan*> plans;
  // device staging of ugu_gpu_visualize / ugu_gpu_render_gbuffer with host
  // buffers, and the G-buffer pass's bad-id counter (device, then pinned)
  uint8_t* vis_buf = nullptr;
  size_t vis_cap = 0;
  unsigned long long* gbuf_bad = nullptr;
  unsigned long long* h_gbuf_bad = nullptr;
};

struct ugu_gpu_plan {
  ugu_gpu_context* ctx = nullptr;
  Scratch scratch;
  std::vector<Group> groups;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int kernels = 0;
  bool raytrace = false;
};

namespace {

int set_error(ugu_gpu_context* ctx, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx)
    ctx->last_error = buf;
  else
    g_create_error = buf;
  return code;
}

int cuda_fail(ugu_gpu_context* ctx, cudaError_t e, const char* what) {
  int code = (e == cudaErrorMemoryAllocation) ? UGU_GPU_ERR_OUT_OF_MEMORY : UGU_GPU_ERR_CUDA;
  return set_error(ctx, code, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(ctx, call, what)                            \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
  } while (0)

void free_slot(MeshSlot& s) {
  for (void* p : s.allocs) cudaFree(p);
  s = MeshSlot();
}

void free_scratch(Scratch& s) {
  cudaFree(s.keys);
  cudaFree(s.items);
  cudaFree(s.counters);
  cudaFreeHost(s.h_counters);
  cudaFree(s.d_views);
  cudaFreeHost(s.h_views);
  cudaFree(s.d_out);
  cudaFree(s.tile_count);
  cudaFree(s.chunk_sums);
  cudaFree(s.entries);
  cudaFree(s.proj);
  cudaFree(s.tcounters);
  cudaFreeHost(s.h_tcounters);
  cudaFree(s.proj64);
  cudaFree(s.grad4);
  cudaFree(s.d_targets);
  cudaFreeHost(s.h_targets);
  s = Scratch();
}

// Indices 0..n-1 sorted by the 30-bit Morton code of point(i) within the
// box [lo, hi] (stable: equal codes keep their order).
template <typename Point>
std::vector<int32_t> morton_sort(int64_t n, const float lo[3], const float hi[3], Point point) {
  std::vector<std::pair<uint32_t, int32_t>> key(n);
  auto spread = [](uint32_t x) {  // 10 bits -> every third bit of 30
    x &= 1023u;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
  };
  for (int64_t i = 0; i < n; ++i) {
    double c[3];
    point(i, c);
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
      const double ext = (double)hi[k] - (double)lo[k];
      double u = ext > 0.0 ? (c[k] - lo[k]) / ext : 0.0;
      if (!(u >= 0.0)) u = 0.0;  // NaN as well
      if (u > 1.0) u = 1.0;
      q[k] = (uint32_t)(u * 1023.0);
    }
    key[i] = {spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2), (int32_t)i};
  }
  std::stable_sort(key.begin(), key.end(),
                   [](const auto& a, const auto& b) { return a.first < b.first; });
  std::vector<int32_t> order(n);
  for (int64_t i = 0; i < n; ++i) order[i] = key[i].second;
  return order;
}

// The tiled path's spatial orders (results never depend on them): faces by
// centroid, vertices by position.  Projected vertices are stored by vertex
// rank, and two index copies refer to ranks: one in face order (shading),
// one in the faces' Morton order (binning and tile setup), so that a block's
// neighbouring faces and their vertices sit close together in memory.
struct SpatialOrder {
  std::vector<int32_t> face_order, vertex_order;
  std::vector<int4> vidx_ranked, vidx_morton;
  std::vector<float4> fnormals_morton;
};

SpatialOrder spatial_order(const ugu_gpu_mesh* m, const float lo[3], const float hi[3]) {
  const int64_t F = m->num_faces, V = m->num_vertices;
  const float* P = m->vertices;
  const int32_t* I = m->vertex_indices;
  SpatialOrder o;
  o.face_order = morton_sort(F, lo, hi, [&](int64_t f, double* c) {
    for (int k = 0; k < 3; ++k)
      c[k] = (P[3 * (int64_t)I[3 * f] + k] + P[3 * (int64_t)I[3 * f + 1] + k] +
              (double)P[3 * (int64_t)I[3 * f + 2] + k]) / 3.0;
  });
  o.vertex_order = morton_sort(V, lo, hi, [&](int64_t v, double* c) {
    for (int k = 0; k < 3; ++k) c[k] = P[3 * v + k];
  });
  std::vector<int32_t> rank(V);
  for (int64_t r = 0; r < V; ++r) rank[o.vertex_order[r]] = (int32_t)r;
  o.vidx_ranked.resize(F);
  o.vidx_morton.resize(F);
  for (int64_t f = 0; f < F; ++f)
    o.vidx_ranked[f] = make_int4(rank[I[3 * f]], rank[I[3 * f + 1]], rank[I[3 * f + 2]], 0);
  for (int64_t i = 0; i < F; ++i) o.vidx_morton[i] = o.vidx_ranked[o.face_order[i]];
  if (m->face_normals) {
    o.fnormals_morton.resize(F);
    for (int64_t i = 0; i < F; ++i) {
      const float* n = m->face_normals + 3 * (int64_t)o.face_order[i];
      o.fnormals_morton[i] = make_float4(n[0], n[1], n[2], 0.0f);
    }
  }
  return o;
}

template <typename T>
int upload(ugu_gpu_context* ctx, MeshSlot& slot, const std::vector<T>& h, const T** out) {
  *out = nullptr;
  if (h.empty()) return UGU_GPU_OK;
  void* p = nullptr;
  CK(ctx, cudaMalloc(&p, h.size() * sizeof(T)), "cudaMalloc(mesh)");
  slot.allocs.push_back(p);
  slot.bytes += h.size() * sizeof(T);
  CK(ctx, cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice),
     "cudaMemcpy(mesh)");
  *out = static_cast<const T*>(p);
  return UGU_GPU_OK;
}

bool indices_ok(const int32_t* idx, int64_t n, int32_t limit) {
  for (int64_t i = 0; i < n; ++i)
    if (idx[i] < 0 || idx[i] >= limit) return false;
  return true;
}

int check_option(ugu_gpu_context* ctx, const ugu_gpu_option& o) {
  if (o.diffuse_color < 0 || o.diffuse_color > 2 || o.interp < 0 || o.interp > 1 ||
      o.shading_normal < 0 || o.shading_normal > 1 || o.diffuse_shading < 0 ||
      o.diffuse_shading > 2)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "option enum out of range");
  return UGU_GPU_OK;
}

// ValidateAndInitBeforeRender (util_private.cc:19-67) for one view.
int validate_view(ugu_gpu_context* ctx, const ugu_gpu_view& v, bool any_output) {
  if (v.mesh < 0 || v.mesh >= kMaxMeshes || !ctx->meshes[v.mesh].present)
    return set_error(ctx, UGU_GPU_ERR_NOT_PREPARED, "mesh has not been initialized");
  const MeshSlot& m = ctx->meshes[v.mesh];
  const ugu_gpu_option& o = ctx->opt;
  if (o.backface_culling && !m.has_fnormals)
    return set_error(ctx, UGU_GPU_ERR_NO_FACE_NORMALS,
                     "specified back-face culling but face normal is empty.");
  if (o.diffuse_color == 1 && m.num_materials == 0)
    return set_error(ctx, UGU_GPU_ERR_NO_TEXTURE,
                     "specified texture as diffuse color but texture is empty.");
  if (o.diffuse_color == 1 && !m.all_textures_nonempty)
    return set_error(ctx, UGU_GPU_ERR_EMPTY_TEXTURE,
                     "specified texture as diffuse color but a texture is empty.");
  if (o.diffuse_color == 2 && !m.has_vcolors)
    return set_error(ctx, UGU_GPU_ERR_NO_VERTEX_COLORS,
                     "specified vertex color as diffuse color but vertex color is empty.");
  if (o.shading_normal == 0 && !m.has_fnormals)
    return set_error(ctx, UGU_GPU_ERR_NO_FACE_NORMALS_FOR_SHADING,
                     "specified face normal as shading normal but face normal is empty.");
  if (o.shading_normal == 1 && !m.has_normals)
    return set_error(ctx, UGU_GPU_ERR_NO_VERTEX_NORMALS,
                     "specified vertex normal as shading normal but vertex normal is empty.");
  if (!any_output)
    return set_error(ctx, UGU_GPU_ERR_NO_OUTPUT, "all arguments are nullptr. nothing to do");
  // Preconditions the reference leaves undefined (it would read past its
  // arrays): the z pass reads face normals for the back-face test
  // (rasterizer.cc:199); the texture path reads uv, uv_indices and
  // material_ids.  A mesh without faces reads none of them.
  const bool has_faces = m.dev.num_faces > 0;
  if (has_faces && !m.has_fnormals)
    return set_error(ctx, UGU_GPU_ERR_NO_FACE_NORMALS,
                     "face normals are required: the z pass reads them for every face");
  if (has_faces && o.diffuse_color == 1 && (!m.has_uv || !m.has_matids))
    return set_error(ctx, UGU_GPU_ERR_NO_TEXTURE,
                     "texture colour needs uv, uv_indices and material_ids");
  const ugu_gpu_camera& c = v.camera;
  if (c.width <= 0 || c.height <= 0 || (int64_t)c.width * c.height > (int64_t)1 << 31)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad image size %dx%d", c.width,
                     c.height);
  return UGU_GPU_OK;
}

bool any_image(const ugu_gpu_images& im) {
  return im.color || im.depth || im.normal || im.mask || im.face_id || im.color_f32;
}

void fill_cam(Cam& d, const ugu_gpu_camera& c) {
  d.width = c.width;
  d.height = c.height;
  d.fx = c.fx;
  d.fy = c.fy;
  d.cx = c.cx;
  d.cy = c.cy;
  std::memcpy(d.R, c.w2c_R, sizeof(d.R));
  std::memcpy(d.t, c.w2c_t, sizeof(d.t));
  std::memcpy(d.C, c.c2w_R, sizeof(d.C));
  std::memcpy(d.T, c.c2w_t, sizeof(d.T));
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

size_t host_bytes_of_view(const ugu_gpu_images& im, int64_t px) {
  size_t b = 0;
  if (im.color) b += align256(3 * px);
  if (im.depth) b += align256(4 * px);
  if (im.normal) b += align256(12 * px);
  if (im.mask) b += align256(px);
  if (im.face_id) b += align256(4 * px);
  if (im.color_f32) b += align256(12 * px);
  return b;
}

int64_t tiles_of(const ugu_gpu_camera& c, int tlog) {
  const int64_t T = int64_t(1) << tlog;
  return ((c.width + T - 1) / T) * ((c.height + T - 1) / T);
}

// The tile edge (log2) of one view on the tiled path: 16 pixels for views
// of at most small_view_pixels pixels, else the tuning's.
int view_tile_log2(const ugu_gpu_tuning& t, const ugu_gpu_camera& c) {
  return t.small_view_pixels > 0 && (int64_t)c.width * c.height <= t.small_view_pixels
             ? 4
             : t.tile_log2;
}

// Views split into launch groups: per view (the baseline), by z-buffer
// pixels (global path) or all together (tiled path).  Renders into host
// buffers are cut into groups of at most kHostChunkPixels so that each
// group's copy to the host overlaps the next group's kernels.
constexpr int64_t kHostChunkPixels = int64_t(4) << 20;

std::vector<Group> make_groups(ugu_gpu_context* ctx, int n, const ugu_gpu_view* views,
                               bool per_view, bool host_outputs = false) {
  const ugu_gpu_tuning& t = ctx->tuning;
  int64_t limit = t.path == UGU_GPU_PATH_GLOBAL ? (int64_t)t.group_pixels : INT64_MAX;
  if (host_outputs) limit = std::min(limit, kHostChunkPixels);
  std::vector<Group> g;
  Group cur{0, 0, 0, 0, 0, 0, 0, 0};
  int64_t acc = 0;
  for (int i = 0; i < n; ++i) {
    int64_t px = (int64_t)views[i].camera.width * views[i].camera.height;
    bool full = cur.count > 0 && (per_view || acc + px > limit);
    if (full) {
      g.push_back(cur);
      cur = Group{i, 0, 0, 0, 0, 0, 0, 0};
      acc = 0;
    }
    const int F = ctx->meshes[views[i].mesh].dev.num_faces;
    const int V = ctx->meshes[views[i].mesh].dev.num_vertices;
    cur.count++;
    acc += px;
    cur.max_faces = std::max(cur.max_faces, F);
    cur.max_vertices = std::max(cur.max_vertices, V);
    cur.max_pixels = std::max(cur.max_pixels, px);
    cur.tiles += tiles_of(views[i].camera, view_tile_log2(t, views[i].camera));
    cur.ray_tiles = std::max(cur.ray_tiles,
                             (int64_t)((views[i].camera.width + kRayTileW - 1) / kRayTileW) *
                                 ((views[i].camera.height + kRayTileH - 1) / kRayTileH));
    cur.faces += F;
    cur.vertices += V;
  }
  if (cur.count) g.push_back(cur);
  return g;
}

int64_t group_key_count(const std::vector<Group>& groups, const ugu_gpu_view* views) {
  int64_t mx = 0;
  for (const Group& gr : groups) {
    int64_t acc = 0;
    for (int i = gr.first; i < gr.first + gr.count; ++i)
      acc += (int64_t)views[i].camera.width * views[i].camera.height;
    mx = std::max(mx, acc);
  }
  return mx;
}

int ensure_tiled(ugu_gpu_context* ctx, Scratch& s, const std::vector<Group>& groups) {
  size_t tiles = 0, verts = 0, faces = 0;
  for (const Group& g : groups) {
    tiles = std::max(tiles, (size_t)g.tiles);
    verts = std::max(verts, (size_t)g.vertices);
    faces = std::max(faces, (size_t)g.faces);
  }
  if (tiles > s.tiles_cap) {
    cudaFree(s.tile_count);
    cudaFree(s.chunk_sums);
    s.tile_count = nullptr;
    s.chunk_sums = nullptr;
    s.tiles_cap = 0;
    CK(ctx, cudaMalloc(&s.tile_count, (4 * tiles + 1) * sizeof(int32_t)),
       "cudaMalloc(tile offsets)");
    CK(ctx, cudaMalloc(&s.chunk_sums, scan_chunks((int64_t)tiles) * sizeof(long long)),
       "cudaMalloc(scan chunk sums)");
    s.tiles_cap = tiles;
    s.tiles_dirty = true;
  }
  if (verts > s.proj_cap) {
    cudaFree(s.proj);
    s.proj = nullptr;
    s.proj_cap = 0;
    CK(ctx, cudaMalloc(&s.proj, verts * sizeof(float4)), "cudaMalloc(projected vertices)");
    s.proj_cap = verts;
  }
  // (face, tile) entries: most faces touch one tile; a render that needs more
  // reports how many, and the next attempt allocates that
  const size_t want = std::min<size_t>(s.entries_min ? s.entries_min : faces + faces / 4 + 4096,
                                       (size_t)INT32_MAX);
  if (want > s.entries_cap) {
    cudaFree(s.entries);
    s.entries = nullptr;
    s.entries_cap = 0;
    CK(ctx, cudaMalloc(&s.entries, want * sizeof(int2)), "cudaMalloc(tile entries)");
    s.entries_cap = want;
  }
  if (groups.size() > s.tcounters_cap) {
    cudaFree(s.tcounters);
    cudaFreeHost(s.h_tcounters);
    s.tcounters = nullptr;
    s.h_tcounters = nullptr;
    s.tcounters_cap = 0;
    CK(ctx, cudaMalloc(&s.tcounters, groups.size() * sizeof(TileCounters)),
       "cudaMalloc(tile counters)");
    CK(ctx, cudaMallocHost(&s.h_tcounters, groups.size() * sizeof(TileCounters)),
       "cudaMallocHost(tile counters)");
    s.tcounters_cap = groups.size();
  }
  if (s.tiles_dirty) {
    CK(ctx, cudaMemsetAsync(s.tile_count, 0, s.tiles_cap * sizeof(int32_t), ctx->stream),
       "cudaMemsetAsync(tile counts)");
    s.tiles_dirty = false;
  }
  return UGU_GPU_OK;
}

int ensure_scratch(ugu_gpu_context* ctx, Scratch& s, size_t nkeys, size_t nviews,
                   size_t ngroups, size_t out_bytes) {
  if (ctx->tuning.path != UGU_GPU_PATH_GLOBAL) nkeys = 0;
  if (nkeys > s.keys_cap) {
    cudaFree(s.keys);
    s.keys = nullptr;
    s.keys_cap = 0;
    CK(ctx, cudaMalloc(&s.keys, nkeys * sizeof(unsigned long long)), "cudaMalloc(z-buffer)");
    s.keys_cap = nkeys;
    s.keys_dirty = true;
  }
  if (s.keys_dirty) {
    CK(ctx, cudaMemsetAsync(s.keys, 0xff, s.keys_cap * sizeof(unsigned long long), ctx->stream),
       "cudaMemsetAsync(z-buffer)");
    s.keys_dirty = false;
  }
  if (s.items_cap < s.list_min && ctx->tuning.path == UGU_GPU_PATH_GLOBAL) {
    cudaFree(s.items);
    s.items = nullptr;
    s.items_cap = 0;
    size_t cap = s.list_min;
    CK(ctx, cudaMalloc(&s.items, cap * sizeof(TileItem)), "cudaMalloc(tile items)");
    s.items_cap = cap;
  }
  if (ngroups > s.counters_cap) {
    cudaFree(s.counters);
    cudaFreeHost(s.h_counters);
    s.counters = nullptr;
    s.h_counters = nullptr;
    s.counters_cap = 0;
    CK(ctx, cudaMalloc(&s.counters, ngroups * sizeof(DevCounters)), "cudaMalloc(counters)");
    CK(ctx, cudaMallocHost(&s.h_counters, ngroups * sizeof(DevCounters)),
       "cudaMallocHost(counters)");
    s.counters_cap = ngroups;
  }
  if (nviews > s.views_cap) {
    cudaFree(s.d_views);
    cudaFreeHost(s.h_views);
    s.d_views = nullptr;
    s.h_views = nullptr;
    s.views_cap = 0;
    CK(ctx, cudaMalloc(&s.d_views, nviews * sizeof(DevView)), "cudaMalloc(views)");
    CK(ctx, cudaMallocHost(&s.h_views, nviews * sizeof(DevView)), "cudaMallocHost(views)");
    s.views_cap = nviews;
  }
  if (out_bytes > s.d_out_cap) {
    cudaFree(s.d_out);
    s.d_out = nullptr;
    s.d_out_cap = 0;
    CK(ctx, cudaMalloc(&s.d_out, out_bytes), "cudaMalloc(output staging)");
    s.d_out_cap = out_bytes;
  }
  return UGU_GPU_OK;
}

ShadeOpts shade_opts(const ugu_gpu_option& o) {
  ShadeOpts p;
  p.diffuse_color = o.diffuse_color;
  p.interp = o.interp;
  p.shading_normal = o.shading_normal;
  p.diffuse_shading = o.diffuse_shading;
  // OrenNayarParam (pixel_shader.h:143-148), in float like the reference
  float sigma_2 = o.oren_nayar_sigma * o.oren_nayar_sigma;
  p.on_A = 1.0f - (0.5f * sigma_2 / (sigma_2 + 0.33f));
  p.on_B = 0.45f * sigma_2 / (sigma_2 + 0.09f);
  return p;
}

RenderParams base_params(ugu_gpu_context* ctx, const Scratch& s) {
  RenderParams p{};
  const ugu_gpu_option& o = ctx->opt;
  p.meshes = ctx->d_meshes;
  p.shade = shade_opts(o);
  p.backface_culling = o.backface_culling ? 1 : 0;
  p.keys = s.keys;
  p.items = s.items;
  p.item_capacity = (int64_t)s.items_cap;
  p.tile_log2 = ctx->tuning.tile_log2;
  p.small_bbox_max = ctx->tuning.small_bbox_max;
  p.sticky = ctx->sticky_on ? ctx->d_sticky : nullptr;
  return p;
}

int persistent_grid(ugu_gpu_context* ctx, int blocks_per_sm) {
  const int per_sm = ctx->tuning.ctas_per_sm > 0 ? std::min(ctx->tuning.ctas_per_sm, blocks_per_sm)
                                                 : blocks_per_sm;
  return ctx->num_sms * std::max(per_sm, 1);
}

// An entry capacity that holds what a render reported, with room to spare;
// the next ensure_tiled allocates it.
void want_capacity(Scratch& s, const TileCounters& c) {
  const size_t e = (size_t)c.total_entries;
  s.entries_min = std::max(s.entries_min, e + e / 8 + 4096);
}

TileParams tile_params(ugu_gpu_context* ctx, Scratch& s, const Group& gr, size_t gi) {
  const ugu_gpu_option& o = ctx->opt;
  TileParams p{};
  p.meshes = ctx->d_meshes;
  p.views = s.d_views + gr.first;
  p.num_views = gr.count;
  p.shade = shade_opts(o);
  p.backface_culling = o.backface_culling ? 1 : 0;
  p.total_tiles = (int32_t)gr.tiles;
  p.max_vertices = gr.max_vertices;
  p.split_class = ctx->tuning.split_class > 0 ? ctx->tuning.split_class : 64;
  p.bin_faces = ctx->tuning.bin_faces > 0 ? ctx->tuning.bin_faces : 2;
  p.entry_cap = (int64_t)s.entries_cap;
  p.proj = s.proj;
  p.tile_count = s.tile_count;
  p.tile_off = s.tile_count + s.tiles_cap;
  p.tile_lo = p.tile_off + s.tiles_cap + 1;
  p.tile_hi = p.tile_lo + s.tiles_cap;
  p.entries = s.entries;
  p.chunk_sums = s.chunk_sums;
  p.counters = s.tcounters + gi;
  p.sticky = ctx->sticky_on ? ctx->d_sticky : nullptr;
  return p;
}

// Enqueue one group's kernels (no synchronisation); returns how many.
int enqueue_group(ugu_gpu_context* ctx, Scratch& s, const Group& gr, size_t gi) {
  if (ctx->raytrace) {
    RayParams p{};
    p.meshes = ctx->d_meshes;
    p.views = s.d_views + gr.first;
    p.num_views = gr.count;
    p.shade = shade_opts(ctx->opt);
    p.backface_culling = ctx->opt.backface_culling ? 1 : 0;
    p.depth_scale = ctx->opt.depth_scale;
    launch_ray(p, gr.ray_tiles, ctx->stream);
    return 1;
  }
  if (ctx->tuning.path != UGU_GPU_PATH_GLOBAL) {
    TileParams p = tile_params(ctx, s, gr, gi);
    cudaMemsetAsync(p.counters, 0, sizeof(TileCounters), ctx->stream);
    {
      Range r("ugu_gpu bin");
      launch_bin(p, gr.max_faces, ctx->stream);
    }
    const bool timed = ctx->time_tile && 2 * (size_t)(gi + 1) <= ctx->tile_events.size();
    if (timed) cudaEventRecord(ctx->tile_events[2 * gi], ctx->stream);
    {
      Range r("ugu_gpu tile");
      launch_tile(p, persistent_grid(ctx, tile_kernel_blocks_per_sm()), ctx->stream);
    }
    if (timed) {
      cudaEventRecord(ctx->tile_events[2 * gi + 1], ctx->stream);
      ctx->timed_groups = (int)gi + 1;
    }
    return kBinKernels + 1;
  }
  RenderParams p = base_params(ctx, s);
  p.views = s.d_views + gr.first;
  p.num_views = gr.count;
  p.counters = s.counters + gi;
  launch_raster(p, gr.max_faces, ctx->num_sms, ctx->stream);
  launch_tiles(p, ctx->num_sms * 8, ctx->stream);
  launch_resolve(p, gr.max_pixels, ctx->stream);
  return 3;
}

// Tiled path: count the (face, tile) entries of every group without
// rendering, and make the entry buffer hold the largest count with room to
// spare (a plan sizes its buffer this way before capture).
int size_tiled(ugu_gpu_context* ctx, Scratch& s, const std::vector<Group>& groups) {
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    TileParams p = tile_params(ctx, s, groups[gi], gi);
    CK(ctx, cudaMemsetAsync(p.counters, 0, sizeof(TileCounters), ctx->stream),
       "cudaMemsetAsync(tile counters)");
    launch_size(p, groups[gi].max_faces, ctx->stream);
  }
  CK(ctx, cudaGetLastError(), "kernel launch");
  CK(ctx, cudaMemcpyAsync(s.h_tcounters, s.tcounters, groups.size() * sizeof(TileCounters),
                          cudaMemcpyDeviceToHost, ctx->stream),
     "cudaMemcpyAsync(tile counters)");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "sizing pass");
  for (size_t gi = 0; gi < groups.size(); ++gi) want_capacity(s, s.h_tcounters[gi]);
  return ensure_tiled(ctx, s, groups);
}

// Fill s.h_views for the views; host-pointer outputs get device staging.
void fill_views(ugu_gpu_context* ctx, Scratch& s, const std::vector<Group>& groups,
                const ugu_gpu_view* views, bool device_ptrs) {
  size_t off = 0;
  for (const Group& gr : groups) {
    int64_t key_off = 0, tile_base = 0, proj_off = 0;
    for (int i = gr.first; i < gr.first + gr.count; ++i) {
      const ugu_gpu_view& v = views[i];
      DevView& d = s.h_views[i];
      std::memset(&d, 0, sizeof(d));
      fill_cam(d.cam, v.camera);
      d.mesh = v.mesh;
      d.key_offset = key_off;
      int64_t px = (int64_t)v.camera.width * v.camera.height;
      key_off += px;
      const int tlog = view_tile_log2(ctx->tuning, v.camera);
      const int T = 1 << tlog;
      d.tile_log2 = tlog;
      d.tiles_x = (v.camera.width + T - 1) / T;
      d.tile_base = (int32_t)tile_base;
      tile_base += tiles_of(v.camera, tlog);
      d.proj_offset = proj_off;
      proj_off += ctx->meshes[v.mesh].dev.num_vertices;
      // camera depth of the mesh's bounding-box centre (a draw-order split only)
      const float* ce = ctx->meshes[v.mesh].centre;
      d.split_z = d.cam.R[6] * ce[0] + d.cam.R[7] * ce[1] + d.cam.R[8] * ce[2] + d.cam.t[2];
      if (device_ptrs) {
        d.color = v.images.color;
        d.depth = v.images.depth;
        d.normal = v.images.normal;
        d.mask = v.images.mask;
        d.face_id = v.images.face_id;
        d.color_f32 = v.images.color_f32;
      }
    }
    if (device_ptrs) continue;
    // Host outputs: the group's staging is laid out output by output, each
    // output's views back to back in view order, so that views whose host
    // buffers are back to back as well are copied with one call (copy_back).
    // The kernels' stores are scalar: 4-byte alignment is all they need.
    // This packing never takes more than one 256-byte-aligned block per
    // output and view (host_bytes_of_view).
    auto stage = [&](size_t bytes_per_px, bool (*wants)(const ugu_gpu_images&),
                     void (*set)(DevView&, uint8_t*)) {
      size_t run = 0;
      for (int i = gr.first; i < gr.first + gr.count; ++i) {
        if (!wants(views[i].images)) continue;
        set(s.h_views[i], s.d_out + off + run);
        run += bytes_per_px * (size_t)views[i].camera.width * views[i].camera.height;
      }
      off += align256(run);
    };
    stage(3, [](const ugu_gpu_images& m) { return m.color != nullptr; },
          [](DevView& d, uint8_t* p) { d.color = p; });
    stage(4, [](const ugu_gpu_images& m) { return m.depth != nullptr; },
          [](DevView& d, uint8_t* p) { d.depth = reinterpret_cast<float*>(p); });
    stage(12, [](const ugu_gpu_images& m) { return m.normal != nullptr; },
          [](DevView& d, uint8_t* p) { d.normal = reinterpret_cast<float*>(p); });
    stage(1, [](const ugu_gpu_images& m) { return m.mask != nullptr; },
          [](DevView& d, uint8_t* p) { d.mask = p; });
    stage(4, [](const ugu_gpu_images& m) { return m.face_id != nullptr; },
          [](DevView& d, uint8_t* p) { d.face_id = reinterpret_cast<int32_t*>(p); });
    stage(12, [](const ugu_gpu_images& m) { return m.color_f32 != nullptr; },
          [](DevView& d, uint8_t* p) { d.color_f32 = reinterpret_cast<float*>(p); });
  }
}

// The group's outputs to the caller's host buffers, one copy per output and
// run of views whose host buffers follow one another (their staging does,
// fill_views), so that a caller with one buffer per output for all views
// costs one copy per output and group.
int copy_back(ugu_gpu_context* ctx, const Scratch& s, int first, int count,
              const ugu_gpu_view* views, cudaStream_t stream) {
  auto out = [&](size_t bytes_per_px, void* (*host)(const ugu_gpu_images&),
                 const void* (*dev)(const DevView&)) -> int {
    uint8_t* dst = nullptr;
    const uint8_t* src = nullptr;
    size_t bytes = 0;
    auto flush = [&]() -> int {
      if (bytes)
        CK(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream),
           "cudaMemcpyAsync(output)");
      bytes = 0;
      return UGU_GPU_OK;
    };
    for (int i = first; i < first + count; ++i) {
      uint8_t* h = static_cast<uint8_t*>(host(views[i].images));
      if (!h) continue;
      const uint8_t* d = static_cast<const uint8_t*>(dev(s.h_views[i]));
      const size_t b = bytes_per_px * (size_t)views[i].camera.width * views[i].camera.height;
      if (bytes && h == dst + bytes && d == src + bytes) {
        bytes += b;
        continue;
      }
      int rc = flush();
      if (rc) return rc;
      dst = h;
      src = d;
      bytes = b;
    }
    return flush();
  };
  int rc;
  if ((rc = out(3, [](const ugu_gpu_images& m) -> void* { return m.color; },
                [](const DevView& d) -> const void* { return d.color; })))
    return rc;
  if ((rc = out(4, [](const ugu_gpu_images& m) -> void* { return m.depth; },
                [](const DevView& d) -> const void* { return d.depth; })))
    return rc;
  if ((rc = out(12, [](const ugu_gpu_images& m) -> void* { return m.normal; },
                [](const DevView& d) -> const void* { return d.normal; })))
    return rc;
  if ((rc = out(1, [](const ugu_gpu_images& m) -> void* { return m.mask; },
                [](const DevView& d) -> const void* { return d.mask; })))
    return rc;
  if ((rc = out(4, [](const ugu_gpu_images& m) -> void* { return m.face_id; },
                [](const DevView& d) -> const void* { return d.face_id; })))
    return rc;
  return out(12, [](const ugu_gpu_images& m) -> void* { return m.color_f32; },
             [](const DevView& d) -> const void* { return d.color_f32; });
}

int check_counters(ugu_gpu_context* ctx, Scratch& s, size_t ngroups) {
  uint64_t special = 0, overflow = 0, items = 0;
  for (size_t g = 0; g < ngroups; ++g) {
    if (ctx->tuning.path == UGU_GPU_PATH_GLOBAL) {
      special += s.h_counters[g].special;
      overflow += s.h_counters[g].overflow;
      items += s.h_counters[g].tile_items;
    } else {
      special += s.h_tcounters[g].special;
      if (s.h_tcounters[g].invalid)
        return set_error(ctx, UGU_GPU_ERR_CUDA,
                         "internal error: %u invalid tile entries (outputs not valid)",
                         s.h_tcounters[g].invalid);
      if (s.h_tcounters[g].dropped) {
        // the next attempt allocates what this render reported it needs
        overflow += s.h_tcounters[g].total_entries;
        want_capacity(s, s.h_tcounters[g]);
      }
      items += s.h_tcounters[g].total_entries;
    }
  }
  ctx->special += special;
  ctx->large_items = items;
  if (overflow)
    return set_error(ctx, UGU_GPU_ERR_CAPACITY, "%llu tile items exceeded the capacity",
                     (unsigned long long)overflow);
  if (special)
    return set_error(ctx, UGU_GPU_ERR_DEGENERATE_DEPTH,
                     "%llu covered samples had depth < FLT_MIN or NaN (a vertex at z ~ 0)",
                     (unsigned long long)special);
  return UGU_GPU_OK;
}

int validate_views(ugu_gpu_context* ctx, int n, const ugu_gpu_view* views) {
  int rc = check_option(ctx, ctx->opt);
  if (rc) return rc;
  for (int i = 0; i < n; ++i) {
    rc = validate_view(ctx, views[i], any_image(views[i].images));
    if (rc) return rc;
  }
  return UGU_GPU_OK;
}

int prepare_scratch(ugu_gpu_context* ctx, Scratch& s, const std::vector<Group>& groups,
                    const ugu_gpu_view* views, int n, size_t out_bytes) {
  if (ctx->raytrace) return ensure_scratch(ctx, s, 0, (size_t)n, groups.size(), out_bytes);
  int rc = ensure_scratch(ctx, s, (size_t)group_key_count(groups, views), (size_t)n,
                          groups.size(), out_bytes);
  if (rc || ctx->tuning.path == UGU_GPU_PATH_GLOBAL) return rc;
  return ensure_tiled(ctx, s, groups);
}

// Everything one render enqueues once its view table is on the device.  With
// host outputs, each group's copies run on the copy stream as soon as the
// group's kernels are done, overlapping the next group's kernels; the
// render stream then waits for the last copy.
int enqueue_render(ugu_gpu_context* ctx, Scratch& s, const std::vector<Group>& groups,
                   const ugu_gpu_view* views, int n, bool dev, int* kernels) {
  const bool global = ctx->tuning.path == UGU_GPU_PATH_GLOBAL && !ctx->raytrace;
  if (global)
    CK(ctx, cudaMemsetAsync(s.counters, 0, groups.size() * sizeof(DevCounters), ctx->stream),
       "cudaMemsetAsync(counters)");
  if (!dev) {
    while (ctx->events.size() < groups.size() + 1) {
      cudaEvent_t e;
      CK(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
      ctx->events.push_back(e);
    }
  }
  int nk = 0;
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    nk += enqueue_group(ctx, s, groups[gi], gi);
    if (!dev) {
      CK(ctx, cudaEventRecord(ctx->events[gi], ctx->stream), "cudaEventRecord");
      CK(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->events[gi], 0), "cudaStreamWaitEvent");
      int rc = copy_back(ctx, s, groups[gi].first, groups[gi].count, views, ctx->copy_stream);
      if (rc) return rc;
    }
  }
  CK(ctx, cudaGetLastError(), "kernel launch");
  *kernels = nk;
  (void)n;
  if (!dev) {
    cudaEvent_t done = ctx->events[groups.size()];
    CK(ctx, cudaEventRecord(done, ctx->copy_stream), "cudaEventRecord");
    CK(ctx, cudaStreamWaitEvent(ctx->stream, done, 0), "cudaStreamWaitEvent");
  }
  if (ctx->raytrace) return UGU_GPU_OK;  // the ray kernel keeps no counters
  if (global)
    CK(ctx, cudaMemcpyAsync(s.h_counters, s.counters, groups.size() * sizeof(DevCounters),
                            cudaMemcpyDeviceToHost, ctx->stream),
       "cudaMemcpyAsync(counters)");
  else
    CK(ctx, cudaMemcpyAsync(s.h_tcounters, s.tcounters, groups.size() * sizeof(TileCounters),
                            cudaMemcpyDeviceToHost, ctx->stream),
       "cudaMemcpyAsync(tile counters)");
  return UGU_GPU_OK;
}

// Raytracer::PrepareMesh (raytracer.cc:90-110) for one slot, on first use:
// the naive BVH built on the host and uploaded with the mesh.
int ensure_bvh(ugu_gpu_context* ctx, int slot) {
  MeshSlot& s = ctx->meshes[slot];
  if (s.bvh) return UGU_GPU_OK;
  if (s.h_vertices.empty() || s.h_faces.empty())
    return set_error(ctx, UGU_GPU_ERR_NOT_PREPARED, "mesh is empty");
  HostBvh hb;
  if (!build_bvh(s.h_vertices.data(), s.h_faces.data(), (int)(s.h_faces.size() / 3), hb))
    return set_error(ctx, UGU_GPU_ERR_CAPACITY, "BVH deeper than %d levels", kMaxBvhDepth);
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  int rc;
  if ((rc = upload(ctx, s, hb.nodes, &s.dev.bvh_nodes))) return rc;
  if ((rc = upload(ctx, s, hb.tris, &s.dev.bvh_tris))) return rc;
  s.dev.bvh_depth = hb.depth;
  s.dev.bvh_entries = (int32_t)(hb.tris.size() / 3);
  CK(ctx, cudaMemcpy(ctx->d_meshes + slot, &s.dev, sizeof(DevMesh), cudaMemcpyHostToDevice),
     "cudaMemcpy(mesh table)");
  s.bvh = true;
  return UGU_GPU_OK;
}

// VisibilityTester::PrepareData's tree (visibility_tester.cc:319-339) for
// one slot, on first use.
int ensure_vis_bvh(ugu_gpu_context* ctx, int slot) {
  MeshSlot& s = ctx->meshes[slot];
  if (s.vis_bvh) return UGU_GPU_OK;
  if (s.h_vertices.empty() || s.h_faces.empty())
    return set_error(ctx, UGU_GPU_ERR_NOT_PREPARED, "mesh is empty");
  HostBvh hb;
  if (!build_bvh(s.h_vertices.data(), s.h_faces.data(), (int)(s.h_faces.size() / 3), hb, 5))
    return set_error(ctx, UGU_GPU_ERR_CAPACITY, "BVH deeper than %d levels", kMaxBvhDepth);
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  int rc;
  if ((rc = upload(ctx, s, hb.nodes, &s.dev.vis_nodes))) return rc;
  if ((rc = upload(ctx, s, hb.tris, &s.dev.vis_tris))) return rc;
  CK(ctx, cudaMemcpy(ctx->d_meshes + slot, &s.dev, sizeof(DevMesh), cudaMemcpyHostToDevice),
     "cudaMemcpy(mesh table)");
  s.vis_bvh = true;
  return UGU_GPU_OK;
}

// The raytracer mode of the context for the lifetime of one call.
struct RayMode {
  ugu_gpu_context* ctx;
  RayMode(ugu_gpu_context* c, bool on) : ctx(c) { ctx->raytrace = on; }
  ~RayMode() { ctx->raytrace = false; }
};

int ensure_bvhs(ugu_gpu_context* ctx, int n, const ugu_gpu_view* views) {
  for (int i = 0; i < n; ++i) {
    int rc = ensure_bvh(ctx, views[i].mesh);
    if (rc) return rc;
  }
  return UGU_GPU_OK;
}

// FNV-1a over what decides a tiled render's entry and run counts: the views'
// meshes and cameras, the mesh uploads and the tuning.
uint64_t view_list_signature(const ugu_gpu_context* ctx, int n, const ugu_gpu_view* views,
                             uint32_t flags) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&h](const void* p, size_t len) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < len; ++i) h = (h ^ b[i]) * 1099511628211ull;
  };
  mix(&n, sizeof(n));
  mix(&flags, sizeof(flags));
  mix(&ctx->mesh_generation, sizeof(ctx->mesh_generation));
  mix(&ctx->tuning, sizeof(ctx->tuning));
  for (int i = 0; i < n; ++i) {
    mix(&views[i].mesh, sizeof(views[i].mesh));
    mix(&views[i].camera, sizeof(views[i].camera));
  }
  return h | 1ull;  // never 0, the "not sized" value
}

int render_impl(ugu_gpu_context* ctx, int n, const ugu_gpu_view* views, uint32_t flags) {
  Range range("ugu_gpu render");
  if (n < 0 || (n > 0 && !views))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad view list");
  if (n == 0) return UGU_GPU_OK;
  int rc = validate_views(ctx, n, views);
  if (rc) return rc;
  const bool ray = (flags & UGU_GPU_RAYTRACE) != 0;
  if (ray && (rc = ensure_bvhs(ctx, n, views))) return rc;
  RayMode mode(ctx, ray);
  const bool dev = (flags & UGU_GPU_DEVICE_POINTERS) != 0;
  if ((flags & UGU_GPU_ASYNC) && !dev)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "UGU_GPU_ASYNC needs device pointers");
  if ((flags & UGU_GPU_TIME_KERNELS) && (flags & UGU_GPU_ASYNC))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                     "UGU_GPU_TIME_KERNELS reads its events at the end of the render (no ASYNC)");
  std::vector<Group> groups =
      make_groups(ctx, n, views, (flags & UGU_GPU_PER_VIEW) != 0, !dev);
  size_t out_bytes = 0;
  if (!dev)
    for (int i = 0; i < n; ++i)
      out_bytes += host_bytes_of_view(views[i].images,
                                      (int64_t)views[i].camera.width * views[i].camera.height);
  Scratch& s = ctx->scratch;
  for (int attempt = 0;; ++attempt) {
    rc = prepare_scratch(ctx, s, groups, views, n, out_bytes);
    if (rc) return rc;
    // The pinned view table may still be read by a previous asynchronous copy.
    CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    fill_views(ctx, s, groups, views, dev);
    CK(ctx, cudaMemcpyAsync(s.d_views, s.h_views, n * sizeof(DevView), cudaMemcpyHostToDevice,
                            ctx->stream),
       "cudaMemcpyAsync(views)");
    // An asynchronous render cannot be retried once its lists overflowed, so
    // on the tiled path it first counts its entries with a sizing pass (as a
    // plan does), unless these very views were sized last.
    const bool async = (flags & UGU_GPU_ASYNC) != 0;
    if (async && !ray && ctx->tuning.path != UGU_GPU_PATH_GLOBAL) {
      const uint64_t sig = view_list_signature(ctx, n, views, flags);
      if (sig != s.sized_sig) {
        if ((rc = size_tiled(ctx, s, groups))) return rc;
        s.sized_sig = sig;
      }
    }
    int kernels = 0;
    ctx->time_tile = (flags & UGU_GPU_TIME_KERNELS) != 0;
    ctx->timed_groups = 0;
    while (ctx->time_tile && ctx->tile_events.size() < 2 * groups.size()) {
      cudaEvent_t e;
      CK(ctx, cudaEventCreate(&e), "cudaEventCreate");
      ctx->tile_events.push_back(e);
    }
    ctx->sticky_on = async;
    rc = enqueue_render(ctx, s, groups, views, n, dev, &kernels);
    ctx->sticky_on = false;
    ctx->time_tile = false;
    if (rc) {
      s.keys_dirty = s.tiles_dirty = true;
      return rc;
    }
    ctx->launches += kernels;
    if (async) {
      ctx->pending_async_groups = ray ? 0 : groups.size();
      return UGU_GPU_OK;
    }
    CK(ctx, cudaStreamSynchronize(ctx->stream), "render");
    if (ray) return UGU_GPU_OK;
    rc = check_counters(ctx, s, groups.size());
    if (!rc)
      for (int g = 0; g < ctx->timed_groups; ++g) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ctx->tile_events[2 * g], ctx->tile_events[2 * g + 1]) ==
            cudaSuccess) {
          ctx->tile_ms += ms;
          ++ctx->tile_launches;
        }
      }
    if (rc == UGU_GPU_ERR_CAPACITY && attempt == 0) {
      // a list overflowed: grow it (the tiled path knows the exact need) and
      // render again
      if (ctx->tuning.path == UGU_GPU_PATH_GLOBAL) s.list_min *= 8;
      s.keys_dirty = s.tiles_dirty = true;
      continue;
    }
    return rc;
  }
}

}  // namespace

extern "C" {

int ugu_gpu_abi_version(void) { return UGU_GPU_ABI_VERSION; }

const char* ugu_gpu_last_error(const ugu_gpu_context* ctx) {
  return ctx ? ctx->last_error.c_str() : g_create_error.c_str();
}

int ugu_gpu_create(int32_t device, ugu_gpu_context** out) {
  if (!out) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return set_error(nullptr, UGU_GPU_ERR_NO_DEVICE, "no CUDA device: %s",
                     e == cudaSuccess ? "count is 0" : cudaGetErrorString(e));
  if (device < 0 || device >= count)
    return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "device %d of %d", device, count);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return set_error(nullptr, UGU_GPU_ERR_CUDA, "cudaSetDevice: %s",
                                         cudaGetErrorString(e));
  ugu_gpu_context* ctx = new ugu_gpu_context();
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_meshes, kMaxMeshes * sizeof(DevMesh));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_meshes, 0, kMaxMeshes * sizeof(DevMesh));
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_sticky, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_sticky, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) {
    set_error(nullptr, UGU_GPU_ERR_CUDA, "context setup: %s", cudaGetErrorString(e));
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    cudaFree(ctx->d_meshes);
    cudaFree(ctx->d_sticky);
    delete ctx;
    return UGU_GPU_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  // occupancy queries happen here, never inside a stream capture
  tile_kernel_blocks_per_sm();
  ctx->opt.diffuse_color = 0;
  ctx->opt.interp = 1;
  ctx->opt.shading_normal = 1;
  ctx->opt.diffuse_shading = 0;
  ctx->opt.depth_scale = 1.0f;
  ctx->opt.backface_culling = 1;
  ctx->opt.oren_nayar_sigma = 0.3f;
  ctx->tuning.path = UGU_GPU_PATH_TILED;
  ctx->tuning.tile_log2 = 5;
  ctx->tuning.entry_capacity = 0;
  ctx->tuning.small_bbox_max = 256;
  ctx->tuning.group_pixels = 4 << 20;
  ctx->tuning.ctas_per_sm = 0;
  // the thresholds the autotuner most often keeps on large view batches
  ctx->tuning.split_class = 256;
  ctx->tuning.bin_faces = 4;
  ctx->tuning.small_view_pixels = 640 * 480;
  *out = ctx;
  return UGU_GPU_OK;
}

int ugu_gpu_destroy(ugu_gpu_context* ctx) {
  if (!ctx) return UGU_GPU_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  while (!ctx->plans.empty()) ugu_gpu_plan_destroy(ctx->plans.back());
  for (MeshSlot& s : ctx->meshes) free_slot(s);
  free_scratch(ctx->scratch);
  cudaFree(ctx->d_meshes);
  cudaFree(ctx->d_sticky);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->tile_events) cudaEventDestroy(e);
  cudaFree(ctx->vis_buf);
  cudaFree(ctx->gbuf_bad);
  cudaFreeHost(ctx->h_gbuf_bad);
  delete ctx;
  return UGU_GPU_OK;
}

int ugu_gpu_set_option(ugu_gpu_context* ctx, const ugu_gpu_option* opt) {
  if (!ctx || !opt) return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL argument");
  int rc = check_option(ctx, *opt);
  if (rc) return rc;
  ctx->opt = *opt;
  return UGU_GPU_OK;
}

int ugu_gpu_set_mesh(ugu_gpu_context* ctx, int32_t slot, const ugu_gpu_mesh* m) {
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  if (slot < 0 || slot >= kMaxMeshes)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "mesh slot %d out of [0, %d)", slot,
                     kMaxMeshes);
  cudaSetDevice(ctx->device);
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  MeshSlot& s = ctx->meshes[slot];
  free_slot(s);
  ++ctx->mesh_generation;
  DevMesh empty{};
  CK(ctx, cudaMemcpy(ctx->d_meshes + slot, &empty, sizeof(DevMesh), cudaMemcpyHostToDevice),
     "cudaMemcpy(mesh table)");
  if (!m) return UGU_GPU_OK;
  if (m->num_vertices < 0 || m->num_faces < 0 || m->num_normals < 0 || m->num_uv < 0 ||
      m->num_materials < 0)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "negative count");
  if ((m->num_vertices && !m->vertices) || (m->num_faces && !m->vertex_indices))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "vertices or faces are NULL");
  const int64_t F = m->num_faces, V = m->num_vertices;
  if (!indices_ok(m->vertex_indices, 3 * F, m->num_vertices))
    return set_error(ctx, UGU_GPU_ERR_INDEX_OUT_OF_RANGE, "vertex index out of range");
  const bool has_normals = m->num_normals > 0 && m->normals && m->normal_indices;
  if (has_normals && !indices_ok(m->normal_indices, 3 * F, m->num_normals))
    return set_error(ctx, UGU_GPU_ERR_INDEX_OUT_OF_RANGE, "normal index out of range");
  const bool has_uv = m->num_uv > 0 && m->uv && m->uv_indices;
  if (has_uv && !indices_ok(m->uv_indices, 3 * F, m->num_uv))
    return set_error(ctx, UGU_GPU_ERR_INDEX_OUT_OF_RANGE, "uv index out of range");
  if (m->material_ids && !indices_ok(m->material_ids, F, std::max(m->num_materials, 0)))
    return set_error(ctx, UGU_GPU_ERR_INDEX_OUT_OF_RANGE, "material id out of range");
  if (m->num_materials > 0 && !m->materials)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "materials is NULL");

  std::vector<float4> v4(V);
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < V; ++i) {
    v4[i] = make_float4(m->vertices[3 * i], m->vertices[3 * i + 1], m->vertices[3 * i + 2], 0.f);
    for (int k = 0; k < 3; ++k) {
      const float x = m->vertices[3 * i + k];
      if (x < lo[k]) lo[k] = x;  // NaN coordinates are skipped
      if (x > hi[k]) hi[k] = x;
    }
  }
  float centre[3];
  for (int k = 0; k < 3; ++k)
    centre[k] = (V > 0 && std::isfinite(lo[k]) && std::isfinite(hi[k])) ? 0.5f * (lo[k] + hi[k])
                                                                         : 0.0f;
  auto pad3i = [&](const int32_t* a) {
    std::vector<int4> o(F);
    for (int64_t i = 0; i < F; ++i) o[i] = make_int4(a[3 * i], a[3 * i + 1], a[3 * i + 2], 0);
    return o;
  };
  auto pad3f = [&](const float* a, int64_t n) {
    std::vector<float4> o(n);
    for (int64_t i = 0; i < n; ++i) o[i] = make_float4(a[3 * i], a[3 * i + 1], a[3 * i + 2], 0.f);
    return o;
  };
  int rc;
  DevMesh& d = s.dev;
  d.num_vertices = m->num_vertices;
  d.num_faces = m->num_faces;
  if ((rc = upload(ctx, s, v4, &d.vertices))) return rc;
  if ((rc = upload(ctx, s, pad3i(m->vertex_indices), &d.vidx))) return rc;
  {
    SpatialOrder so = spatial_order(m, lo, hi);
    if ((rc = upload(ctx, s, so.face_order, &d.order))) return rc;
    if ((rc = upload(ctx, s, so.vertex_order, &d.vorder))) return rc;
    if ((rc = upload(ctx, s, so.vidx_ranked, &d.vidx_ranked))) return rc;
    if ((rc = upload(ctx, s, so.vidx_morton, &d.vidx_morton))) return rc;
    if ((rc = upload(ctx, s, so.fnormals_morton, &d.fnormals_morton))) return rc;
  }
  if (m->face_normals && F > 0) {
    if ((rc = upload(ctx, s, pad3f(m->face_normals, F), &d.fnormals))) return rc;
    s.has_fnormals = true;
  }
  if (has_normals) {
    d.num_normals = m->num_normals;
    if ((rc = upload(ctx, s, pad3f(m->normals, m->num_normals), &d.normals))) return rc;
    if ((rc = upload(ctx, s, pad3i(m->normal_indices), &d.nidx))) return rc;
    s.has_normals = true;
  }
  if (m->vertex_colors && V > 0) {
    if ((rc = upload(ctx, s, pad3f(m->vertex_colors, V), &d.vcolors))) return rc;
    s.has_vcolors = true;
  }
  if (has_uv) {
    d.num_uv = m->num_uv;
    std::vector<float2> uv(m->num_uv);
    for (int i = 0; i < m->num_uv; ++i) uv[i] = make_float2(m->uv[2 * i], m->uv[2 * i + 1]);
    if ((rc = upload(ctx, s, uv, &d.uv))) return rc;
    if ((rc = upload(ctx, s, pad3i(m->uv_indices), &d.uvidx))) return rc;
    s.has_uv = true;
  }
  if (m->material_ids && F > 0) {
    std::vector<int32_t> mi(m->material_ids, m->material_ids + F);
    if ((rc = upload(ctx, s, mi, &d.mat_ids))) return rc;
    s.has_matids = true;
  }
  s.num_materials = m->num_materials;
  d.num_materials = m->num_materials;
  if (m->num_materials > 0) {
    std::vector<DevTexture> tex(m->num_materials);
    s.all_textures_f32 = true;
    for (int i = 0; i < m->num_materials; ++i) {
      const ugu_gpu_texture& t = m->materials[i];
      DevTexture& dt = tex[i];
      dt.width = t.width;
      dt.height = t.height;
      dt.rgba8 = nullptr;
      dt.rgbf = nullptr;
      if (t.width < 1 || t.height < 1 || (!t.rgb8 && !t.rgb_f32)) {
        s.all_textures_nonempty = false;
        s.all_textures_f32 = false;
        continue;
      }
      const int64_t n = (int64_t)t.width * t.height;
      if (t.rgb8) {
        std::vector<uint32_t> rgba(n);
        for (int64_t k = 0; k < n; ++k)
          rgba[k] = (uint32_t)t.rgb8[3 * k] | ((uint32_t)t.rgb8[3 * k + 1] << 8) |
                    ((uint32_t)t.rgb8[3 * k + 2] << 16);
        if ((rc = upload(ctx, s, rgba, &dt.rgba8))) return rc;
      }
      if (t.rgb_f32) {
        std::vector<float> f(t.rgb_f32, t.rgb_f32 + 3 * n);
        if ((rc = upload(ctx, s, f, &dt.rgbf))) return rc;
      } else {
        s.all_textures_f32 = false;
      }
      if (i == 0) {
        s.tex0_w = t.width;
        s.tex0_h = t.height;
      }
    }
    if ((rc = upload(ctx, s, tex, &d.textures))) return rc;
    s.dev_tex.resize(tex.size());
    for (size_t i = 0; i < tex.size(); ++i)
      s.dev_tex[i] = {tex[i].width, tex[i].height, tex[i].rgba8, tex[i].rgbf};
  }
  CK(ctx, cudaMemcpy(ctx->d_meshes + slot, &d, sizeof(DevMesh), cudaMemcpyHostToDevice),
     "cudaMemcpy(mesh table)");
  for (int k = 0; k < 3; ++k) s.centre[k] = centre[k];
  s.h_vertices.assign(m->vertices, m->vertices + 3 * V);
  s.h_faces.assign(m->vertex_indices, m->vertex_indices + 3 * F);
  s.present = true;
  return UGU_GPU_OK;
}

int ugu_gpu_render(ugu_gpu_context* ctx, int32_t mesh, const ugu_gpu_camera* cam,
                   const ugu_gpu_images* images) {
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  if (!cam) return set_error(ctx, UGU_GPU_ERR_NO_CAMERA, "camera has not been set");
  if (!images) return set_error(ctx, UGU_GPU_ERR_NO_OUTPUT, "all arguments are nullptr. nothing to do");
  cudaSetDevice(ctx->device);
  ugu_gpu_view v;
  v.mesh = mesh;
  v.camera = *cam;
  v.images = *images;
  return render_impl(ctx, 1, &v, 0);
}

int ugu_gpu_render_views(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_view* views,
                         uint32_t flags) {
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  cudaSetDevice(ctx->device);
  return render_impl(ctx, n, views, flags);
}

int ugu_gpu_plan_create(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_view* views,
                        uint32_t flags, ugu_gpu_plan** out) {
  Range range("ugu_gpu plan create");
  if (!ctx || !out || n <= 0 || !views)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad plan arguments");
  *out = nullptr;
  if (!(flags & UGU_GPU_DEVICE_POINTERS))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "a plan needs device pointers");
  cudaSetDevice(ctx->device);
  int rc = validate_views(ctx, n, views);
  if (rc) return rc;
  const bool ray = (flags & UGU_GPU_RAYTRACE) != 0;
  if (ray && (rc = ensure_bvhs(ctx, n, views))) return rc;
  RayMode mode(ctx, ray);
  ugu_gpu_plan* plan = new ugu_gpu_plan();
  plan->ctx = ctx;
  plan->raytrace = ray;
  plan->groups = make_groups(ctx, n, views, (flags & UGU_GPU_PER_VIEW) != 0);
  Scratch& s = plan->scratch;
  rc = prepare_scratch(ctx, s, plan->groups, views, n, 0);
  if (!rc) {
    fill_views(ctx, s, plan->groups, views, true);
    cudaError_t e = cudaMemcpyAsync(s.d_views, s.h_views, n * sizeof(DevView),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "plan views");
  }
  if (!rc && !ray && ctx->tuning.path != UGU_GPU_PATH_GLOBAL) rc = size_tiled(ctx, s, plan->groups);
  if (!rc) {
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "cudaStreamBeginCapture");
  }
  if (!rc) {
    int k = 0;
    ctx->sticky_on = true;
    rc = enqueue_render(ctx, s, plan->groups, views, n, true, &k);
    ctx->sticky_on = false;
    plan->kernels = k;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &plan->graph);
    if (!rc && e != cudaSuccess) rc = cuda_fail(ctx, e, "cudaStreamEndCapture");
  }
  if (!rc) {
    cudaError_t e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "cudaGraphInstantiate");
  }
  if (rc) {
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    free_scratch(plan->scratch);
    delete plan;
    return rc;
  }
  ctx->plans.push_back(plan);
  *out = plan;
  return UGU_GPU_OK;
}

int ugu_gpu_plan_launch(ugu_gpu_plan* plan) {
  Range range("ugu_gpu plan launch");
  if (!plan) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL plan");
  ugu_gpu_context* ctx = plan->ctx;
  CK(ctx, cudaGraphLaunch(plan->exec, ctx->stream), "cudaGraphLaunch");
  ctx->launches += plan->kernels;
  ctx->pending_plan = plan;
  return UGU_GPU_OK;
}

int ugu_gpu_plan_destroy(ugu_gpu_plan* plan) {
  if (!plan) return UGU_GPU_OK;
  ugu_gpu_context* ctx = plan->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->pending_plan == plan) ctx->pending_plan = nullptr;
  ctx->plans.erase(std::remove(ctx->plans.begin(), ctx->plans.end(), plan), ctx->plans.end());
  cudaGraphExecDestroy(plan->exec);
  cudaGraphDestroy(plan->graph);
  free_scratch(plan->scratch);
  delete plan;
  return UGU_GPU_OK;
}

// TextureMapping with kUseOriginalMeshUv (texture_mapper.cc:924-1006,
// :294-345); texmap.cu draws the texture.
namespace {

// The texture of TextureMapping for F faces: target triangles from the
// mesh slot's uv (uv, uvidx) or given per face (face_target, texel
// coordinates, host or device as the flags say).
int texture_mapping_impl(ugu_gpu_context* ctx, int F, const float2* uv, const int4* uvidx,
                         const float* face_target, int32_t n, const ugu_gpu_keyframe* keyframes,
                         const int32_t* face_kf, const float* face_tri,
                         const ugu_gpu_texture_option* option, uint8_t* texture, uint8_t* mask,
                         uint32_t flags) {
  const bool dev = (flags & UGU_GPU_DEVICE_POINTERS) != 0;
  for (int k = 0; k < n; ++k)
    if (!keyframes[k].color || keyframes[k].camera.width <= 0 || keyframes[k].camera.height <= 0)
      return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "keyframe color is empty");
  if (!dev)  // the reference indexes the keyframe list by id: an id past it is an error here
    for (int f = 0; f < F; ++f)
      if (face_kf[f] >= n)
        return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                         "face %d: keyframe id %d is not an index of the %d keyframes", f,
                         face_kf[f], n);
  const size_t texels = (size_t)option->tex_w * option->tex_h;
  size_t img_bytes = 0;
  if (!dev)
    for (int k = 0; k < n; ++k)
      img_bytes += align256(3 * (size_t)keyframes[k].camera.width * keyframes[k].camera.height);
  const size_t total = align256(sizeof(DevKeyframe) * (size_t)std::max(n, 1)) + img_bytes +
                       (dev ? 0 : align256(4 * (size_t)F) + align256(24 * (size_t)F)) +
                       (dev || !face_target ? 0 : align256(24 * (size_t)F)) +
                       align256(4 * texels) + align256(3 * texels) + align256(texels) +
                       (dev ? 0 : align256(3 * texels) + align256(texels));
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (total > ctx->vis_cap) {
    cudaFree(ctx->vis_buf);
    ctx->vis_buf = nullptr;
    ctx->vis_cap = 0;
    CK(ctx, cudaMalloc(&ctx->vis_buf, total), "cudaMalloc(texture mapping buffers)");
    ctx->vis_cap = total;
  }
  uint8_t* q = ctx->vis_buf;
  auto take = [&](size_t bytes) {
    uint8_t* r = q;
    q += align256(bytes);
    return r;
  };
  DevKeyframe* d_kfs = reinterpret_cast<DevKeyframe*>(take(sizeof(DevKeyframe) * std::max(n, 1)));
  std::vector<DevKeyframe> hk((size_t)std::max(n, 1));
  for (int k = 0; k < n; ++k) {
    DevKeyframe& d = hk[k];
    std::memset(&d, 0, sizeof(d));
    fill_cam(d.cam, keyframes[k].camera);
    d.id = keyframes[k].id;
    if (dev) {
      d.color = keyframes[k].color;
      continue;
    }
    const size_t px = (size_t)keyframes[k].camera.width * keyframes[k].camera.height;
    uint8_t* c = take(3 * px);
    CK(ctx, cudaMemcpyAsync(c, keyframes[k].color, 3 * px, cudaMemcpyHostToDevice, ctx->stream),
       "cudaMemcpyAsync(keyframe color)");
    d.color = c;
  }
  CK(ctx, cudaMemcpyAsync(d_kfs, hk.data(), sizeof(DevKeyframe) * hk.size(),
                          cudaMemcpyHostToDevice, ctx->stream),
     "cudaMemcpyAsync(keyframes)");
  TexMapParams p{};
  p.uv = uv;
  p.uvidx = uvidx;
  p.face_target = face_target;
  p.num_faces = F;
  p.kf = d_kfs;
  p.tex_w = option->tex_w;
  p.tex_h = option->tex_h;
  p.hk = option->padding_kernel / 2;
  if (dev) {
    p.face_kf = face_kf;
    p.face_tri = face_tri;
  } else {
    int32_t* fk = reinterpret_cast<int32_t*>(take(4 * (size_t)F));
    float* ft = reinterpret_cast<float*>(take(24 * (size_t)F));
    CK(ctx, cudaMemcpyAsync(fk, face_kf, 4 * (size_t)F, cudaMemcpyHostToDevice, ctx->stream),
       "cudaMemcpyAsync(face keyframes)");
    CK(ctx, cudaMemcpyAsync(ft, face_tri, 24 * (size_t)F, cudaMemcpyHostToDevice, ctx->stream),
       "cudaMemcpyAsync(face triangles)");
    p.face_kf = fk;
    p.face_tri = ft;
    if (face_target) {
      float* tt = reinterpret_cast<float*>(take(24 * (size_t)F));
      CK(ctx, cudaMemcpyAsync(tt, face_target, 24 * (size_t)F, cudaMemcpyHostToDevice,
                              ctx->stream),
         "cudaMemcpyAsync(face targets)");
      p.face_target = tt;
    }
  }
  p.owner = reinterpret_cast<int32_t*>(take(4 * texels));
  p.tex0 = take(3 * texels);
  p.mask0 = take(texels);
  p.tex = dev ? texture : take(3 * texels);
  p.mask = dev ? mask : take(texels);
  launch_texture_mapping(p, ctx->stream);
  CK(ctx, cudaGetLastError(), "texture mapping launch");
  ctx->launches += F > 0 ? 3 : 2;
  if (!dev) {
    CK(ctx, cudaMemcpyAsync(texture, p.tex, 3 * texels, cudaMemcpyDeviceToHost, ctx->stream),
       "cudaMemcpyAsync(texture)");
    CK(ctx, cudaMemcpyAsync(mask, p.mask, texels, cudaMemcpyDeviceToHost, ctx->stream),
       "cudaMemcpyAsync(texture mask)");
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream), "texture mapping");
  return UGU_GPU_OK;
}

bool texmap_args_ok(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_keyframe* keyframes,
                    const int32_t* face_kf, const float* face_tri,
                    const ugu_gpu_texture_option* option, const uint8_t* texture,
                    const uint8_t* mask) {
  if (n < 0 || (n > 0 && !keyframes) || !face_kf || !face_tri || !option || !texture || !mask) {
    set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad keyframes, face arrays, option or output");
    return false;
  }
  if (option->tex_w <= 0 || option->tex_h <= 0 || option->padding_kernel < 0) {
    set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad texture size or padding kernel");
    return false;
  }
  return true;
}

}  // namespace

int ugu_gpu_texture_mapping(ugu_gpu_context* ctx, int32_t mesh, int32_t n,
                            const ugu_gpu_keyframe* keyframes, const int32_t* face_kf,
                            const float* face_tri, const ugu_gpu_texture_option* option,
                            uint8_t* texture, uint8_t* mask, uint32_t flags) {
  Range range("ugu_gpu texture mapping");
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  cudaSetDevice(ctx->device);
  if (!texmap_args_ok(ctx, n, keyframes, face_kf, face_tri, option, texture, mask))
    return UGU_GPU_ERR_INVALID_ARGUMENT;
  if (mesh < 0 || mesh >= kMaxMeshes || !ctx->meshes[mesh].present)
    return set_error(ctx, UGU_GPU_ERR_NOT_PREPARED, "mesh has not been initialized");
  MeshSlot& ms = ctx->meshes[mesh];
  if (!ms.dev.uv || !ms.dev.uvidx)  // :986-993
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                     "OutputUvType kUseOriginalMeshUv is specified but UV on mesh is invalid");
  return texture_mapping_impl(ctx, ms.dev.num_faces, ms.dev.uv, ms.dev.uvidx, nullptr, n,
                              keyframes, face_kf, face_tri, option, texture, mask, flags);
}

// GenerateSimpleTrianglesTextureAndUv (texture_mapper.cc:347-440): the
// faces' target triangles come from the caller's layout.
int ugu_gpu_texture_mapping_targets(ugu_gpu_context* ctx, int32_t num_faces,
                                    const float* face_target, int32_t n,
                                    const ugu_gpu_keyframe* keyframes, const int32_t* face_kf,
                                    const float* face_tri, const ugu_gpu_texture_option* option,
                                    uint8_t* texture, uint8_t* mask, uint32_t flags) {
  Range range("ugu_gpu texture mapping");
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  cudaSetDevice(ctx->device);
  if (num_faces < 0 || (num_faces > 0 && !face_target))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad face count or target triangles");
  if (!texmap_args_ok(ctx, n, keyframes, face_kf, face_tri, option, texture, mask))
    return UGU_GPU_ERR_INVALID_ARGUMENT;
  return texture_mapping_impl(ctx, num_faces, nullptr, nullptr, face_target, n, keyframes,
                              face_kf, face_tri, option, texture, mask, flags);
}

// MakeTiledImage (texture_mapper.cc:29-60): keyframe image i is copied to
// tile (i % x_tiles, i / x_tiles) of a texture x_tiles images wide, one
// two-dimensional copy per keyframe.  Every image must have the first
// one's size, and the n images must fill whole rows of tiles (elsewhere the
// reference writes past its texture).
int ugu_gpu_tile_images(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_keyframe* keyframes,
                        int32_t x_tiles, uint8_t* texture, uint32_t flags) {
  Range range("ugu_gpu tile images");
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  cudaSetDevice(ctx->device);
  if (n <= 0 || !keyframes || !texture || x_tiles <= 0 || n % x_tiles != 0)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                     "tiling needs keyframes that fill whole rows of %d tiles", x_tiles);
  const int w = keyframes[0].camera.width, h = keyframes[0].camera.height;
  for (int k = 0; k < n; ++k)
    if (!keyframes[k].color || keyframes[k].camera.width != w || keyframes[k].camera.height != h)
      return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                       "keyframe %d: every tiled image must have the first one's size", k);
  const bool dev = (flags & UGU_GPU_DEVICE_POINTERS) != 0;
  const size_t row = 3 * (size_t)w, pitch = row * (size_t)x_tiles;
  for (int k = 0; k < n; ++k) {
    uint8_t* dst = texture + (size_t)(k / x_tiles) * h * pitch + (size_t)(k % x_tiles) * row;
    CK(ctx, cudaMemcpy2DAsync(dst, pitch, keyframes[k].color, row, row, h,
                              dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToHost, ctx->stream),
       "cudaMemcpy2DAsync(tile)");
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream), "tiling");
  return UGU_GPU_OK;
}

int ugu_gpu_synchronize(ugu_gpu_context* ctx) {
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  int rc = UGU_GPU_OK;
  // the last asynchronous render's and replay's counters (an overflow grows
  // the lists for the next render), then what any earlier one left sticky
  if (ctx->pending_async_groups) {
    const size_t g = ctx->pending_async_groups;
    ctx->pending_async_groups = 0;
    rc = check_counters(ctx, ctx->scratch, g);
    if (rc == UGU_GPU_ERR_CAPACITY) ctx->scratch.sized_sig = 0;
  }
  if (ctx->pending_plan) {
    ugu_gpu_plan* p = ctx->pending_plan;
    ctx->pending_plan = nullptr;
    const int prc = p->raytrace ? UGU_GPU_OK : check_counters(ctx, p->scratch, p->groups.size());
    if (!rc) rc = prc;
  }
  unsigned long long sticky = 0;
  CK(ctx, cudaMemcpy(&sticky, ctx->d_sticky, sizeof(sticky), cudaMemcpyDeviceToHost),
     "cudaMemcpy(status)");
  if (sticky) {
    CK(ctx, cudaMemset(ctx->d_sticky, 0, sizeof(sticky)), "cudaMemset(status)");
    if (!rc && (sticky & kStickyOverflow))
      rc = set_error(ctx, UGU_GPU_ERR_CAPACITY,
                     "an asynchronous render overflowed its tile lists: its images are not "
                     "valid; render it again");
    if (!rc && (sticky & kStickySpecial))
      rc = set_error(ctx, UGU_GPU_ERR_DEGENERATE_DEPTH,
                     "an asynchronous render had covered samples with depth < FLT_MIN or NaN");
  }
  return rc;
}

int ugu_gpu_set_stream(ugu_gpu_context* ctx, void* stream) {
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return UGU_GPU_OK;
}

int ugu_gpu_set_tuning(ugu_gpu_context* ctx, const ugu_gpu_tuning* t) {
  if (!ctx || !t) return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL argument");
  const bool tiled = t->path == UGU_GPU_PATH_TILED;
  if ((t->path != UGU_GPU_PATH_TILED && t->path != UGU_GPU_PATH_GLOBAL) ||
      (tiled && (t->tile_log2 < 4 || t->tile_log2 > 5)) ||
      (!tiled && (t->tile_log2 < 3 || t->tile_log2 > 6)) || t->entry_capacity < 0 ||
      t->small_bbox_max < 0 || t->group_pixels < 1 || t->ctas_per_sm < 0 ||
      t->split_class < 0 || t->small_view_pixels < 0 ||
      !(t->bin_faces == 0 || t->bin_faces == 1 || t->bin_faces == 2 || t->bin_faces == 4))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "tuning out of range");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (t->tile_log2 != ctx->tuning.tile_log2 || t->entry_capacity != ctx->tuning.entry_capacity) {
    // tile arrays are laid out per tile size: start them and the entries afresh
    Scratch& s = ctx->scratch;
    cudaFree(s.tile_count);
    cudaFree(s.entries);
      s.tile_count = nullptr;
    s.entries = nullptr;
    s.tiles_cap = s.entries_cap = 0;
    s.entries_min = (size_t)t->entry_capacity;
  }
  ctx->tuning = *t;
  return UGU_GPU_OK;
}

int ugu_gpu_get_tuning(const ugu_gpu_context* ctx, ugu_gpu_tuning* t) {
  if (!ctx || !t) return UGU_GPU_ERR_INVALID_ARGUMENT;
  *t = ctx->tuning;
  return UGU_GPU_OK;
}

namespace {

// What the fastest tuning of a render depends on: the views' sizes and
// meshes (their face, vertex and texture sizes), the options and the device.
uint64_t workload_shape(const ugu_gpu_context* ctx, int n, const ugu_gpu_view* views) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&h](const void* p, size_t len) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < len; ++i) h = (h ^ b[i]) * 1099511628211ull;
  };
  mix(&n, sizeof(n));
  mix(&ctx->num_sms, sizeof(ctx->num_sms));
  mix(&ctx->opt, sizeof(ctx->opt));
  for (int i = 0; i < n; ++i) {
    const ugu_gpu_camera& c = views[i].camera;
    mix(&c.width, sizeof(c.width));
    mix(&c.height, sizeof(c.height));
    const DevMesh& m = ctx->meshes[views[i].mesh].dev;
    const int32_t dims[4] = {m.num_vertices, m.num_faces, ctx->meshes[views[i].mesh].tex0_w,
                             ctx->meshes[views[i].mesh].tex0_h};
    mix(dims, sizeof(dims));
  }
  return h;
}

const char* tuning_cache_file() {
  const char* f = std::getenv("UGU_GPU_TUNING_CACHE");
  return (f && *f) ? f : nullptr;
}

// One line per entry: the shape key in hex, then the tuning's ten fields.
bool read_cached_tuning(uint64_t key, ugu_gpu_tuning* t) {
  const char* fn = tuning_cache_file();
  if (!fn) return false;
  FILE* f = std::fopen(fn, "r");
  if (!f) return false;
  bool found = false;
  unsigned long long k = 0;
  ugu_gpu_tuning r{};
  while (std::fscanf(f, "%llx %d %d %d %d %d %d %d %d %d", &k, &r.path, &r.tile_log2,
                     &r.entry_capacity, &r.small_bbox_max, &r.group_pixels, &r.ctas_per_sm,
                     &r.split_class, &r.bin_faces, &r.small_view_pixels) == 10)
    if (k == key) {
      *t = r;  // the last entry for a key wins
      found = true;
    }
  std::fclose(f);
  return found;
}

void write_cached_tuning(uint64_t key, const ugu_gpu_tuning& t) {
  const char* fn = tuning_cache_file();
  if (!fn) return;
  FILE* f = std::fopen(fn, "a");
  if (!f) return;
  std::fprintf(f, "%llx %d %d %d %d %d %d %d %d %d\n", (unsigned long long)key, t.path,
               t.tile_log2, t.entry_capacity, t.small_bbox_max, t.group_pixels, t.ctas_per_sm,
               t.split_class, t.bin_faces, t.small_view_pixels);
  std::fclose(f);
}

}  // namespace

int ugu_gpu_autotune(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_view* views,
                     ugu_gpu_tuning* chosen) {
  Range range("ugu_gpu autotune");
  if (!ctx || n <= 0 || !views)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad autotune arguments");
  cudaSetDevice(ctx->device);
  int rc = validate_views(ctx, n, views);
  if (rc) return rc;
  const uint64_t key = workload_shape(ctx, n, views);
  ugu_gpu_tuning cached{};
  auto hit = ctx->tuned.find(key);
  if (hit != ctx->tuned.end() || read_cached_tuning(key, &cached)) {
    if (hit != ctx->tuned.end()) cached = hit->second;
    ctx->tuned[key] = cached;
    if ((rc = ugu_gpu_set_tuning(ctx, &cached))) return rc;
    if (chosen) *chosen = cached;
    return UGU_GPU_OK;
  }
  const ugu_gpu_tuning start = ctx->tuning;
  cudaEvent_t e0, e1;
  CK(ctx, cudaEventCreate(&e0), "cudaEventCreate");
  CK(ctx, cudaEventCreate(&e1), "cudaEventCreate");
  // The median of seven timed renders of the views on one candidate, after
  // an untimed one that sizes its lists; a failed candidate is skipped.
  // (Candidates often differ by about 1 %, within the spread of three.)
  constexpr int kTimed = 7;
  auto time_of = [&](const ugu_gpu_tuning& t, float* ms_out) -> int {
    int r = ugu_gpu_set_tuning(ctx, &t);
    if (!r) r = render_impl(ctx, n, views, UGU_GPU_DEVICE_POINTERS | UGU_GPU_ASYNC);
    if (!r) r = ugu_gpu_synchronize(ctx);
    float ms[kTimed];
    for (int k = 0; k < kTimed && !r; ++k) {
      cudaEventRecord(e0, ctx->stream);
      r = render_impl(ctx, n, views, UGU_GPU_DEVICE_POINTERS | UGU_GPU_ASYNC);
      cudaEventRecord(e1, ctx->stream);
      if (!r) r = ugu_gpu_synchronize(ctx);
      ms[k] = 0.0f;
      cudaEventElapsedTime(&ms[k], e0, e1);
    }
    if (r) return r;
    std::sort(ms, ms + kTimed);
    *ms_out = ms[kTimed / 2];
    return UGU_GPU_OK;
  };
  float best = 1e30f;
  ugu_gpu_tuning best_t = start;
  bool any = false;
  // in stage 2 a threshold moves off its current value only for a gain above
  // the timing noise, so that noise does not walk the search away from the
  // base values
  float margin = 1.0f;
  auto consider = [&](const ugu_gpu_tuning& t) {
    float ms = 0.0f;
    if (time_of(t, &ms) == UGU_GPU_OK && ms < best * margin) {
      best = ms;
      best_t = t;
      any = true;
    }
  };
  // Stage 1: the path and the tile size, each at the base thresholds (a new
  // context's).
  ugu_gpu_tuning base = start;
  base.entry_capacity = 0;
  base.ctas_per_sm = 0;
  base.split_class = 256;
  base.bin_faces = 4;
  base.small_view_pixels = 640 * 480;
  base.small_bbox_max = 256;
  base.group_pixels = 8 << 20;
  for (int tl : {4, 5}) {
    ugu_gpu_tuning t = base;
    t.path = UGU_GPU_PATH_TILED;
    t.tile_log2 = tl;
    consider(t);
  }
  {
    ugu_gpu_tuning t = base;
    t.path = UGU_GPU_PATH_GLOBAL;
    t.tile_log2 = 4;
    consider(t);
  }
  // Stage 2: each threshold of the chosen path in turn, the others held.
  margin = 0.997f;
  if (any && best_t.path == UGU_GPU_PATH_TILED) {
    if (best_t.tile_log2 == 5) {  // small views on 16-pixel tiles
      const ugu_gpu_tuning s0 = best_t;
      for (int v : {0, 320 * 240, 1280 * 720}) {
        ugu_gpu_tuning t = s0;
        t.small_view_pixels = v;
        consider(t);
      }
    }
    const ugu_gpu_tuning s1 = best_t;
    for (int v : {6, 7}) {
      ugu_gpu_tuning t = s1;
      t.ctas_per_sm = v;
      consider(t);
    }
    const ugu_gpu_tuning s2 = best_t;
    for (int v : {1, 64}) {
      ugu_gpu_tuning t = s2;
      t.split_class = v;
      consider(t);
    }
    const ugu_gpu_tuning s3 = best_t;
    for (int v : {1, 2}) {
      ugu_gpu_tuning t = s3;
      t.bin_faces = v;
      consider(t);
    }
  } else if (any) {
    const ugu_gpu_tuning s1 = best_t;
    for (int v : {64, 1024}) {
      ugu_gpu_tuning t = s1;
      t.small_bbox_max = v;
      consider(t);
    }
    const ugu_gpu_tuning s2 = best_t;
    for (int v : {4 << 20, 16 << 20}) {
      ugu_gpu_tuning t = s2;
      t.group_pixels = v;
      consider(t);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!any) {
    const std::string why = ctx->last_error;
    ugu_gpu_set_tuning(ctx, &start);
    return set_error(ctx, UGU_GPU_ERR_CUDA, "no candidate tuning rendered: %s", why.c_str());
  }
  rc = ugu_gpu_set_tuning(ctx, &best_t);
  if (rc) return rc;
  ctx->tuned[key] = best_t;
  write_cached_tuning(key, best_t);
  if (chosen) *chosen = best_t;
  return UGU_GPU_OK;
}

int ugu_gpu_backward(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_view* views,
                     const float* const* targets, float* grad_texels,
                     float* grad_vertex_colors, float* grad_vertices, float* loss_out,
                     uint32_t flags) {
  Range range("ugu_gpu backward");
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  if (n <= 0 || !views || !targets)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad view or target list");
  if (!(flags & UGU_GPU_DEVICE_POINTERS))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "backward works on device pointers");
  cudaSetDevice(ctx->device);
  const ugu_gpu_option& o = ctx->opt;
  if (o.diffuse_color != 1 && o.diffuse_color != 2)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                     "backward needs texture or vertex colour as diffuse colour");
  if (o.diffuse_shading != 0)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                     "backward differentiates the unshaded colour (diffuse_shading = kNone)");
  int64_t max_px = 0, sum_v = 0, texels = 0, sum_px = 0;
  int max_v = 0;
  for (int i = 0; i < n; ++i) {
    ugu_gpu_view v = views[i];
    if (grad_texels && o.diffuse_color == 1 && v.mesh >= 0 && v.mesh < kMaxMeshes)
      texels = std::max(texels, (int64_t)ctx->meshes[v.mesh].tex0_w * ctx->meshes[v.mesh].tex0_h);
    if (!v.images.face_id || !targets[i])
      return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                       "view %d needs the forward's face_id image and a target", i);
    int rc = validate_view(ctx, v, true);
    if (rc) return rc;
    max_px = std::max(max_px, (int64_t)v.camera.width * v.camera.height);
    sum_px += (int64_t)v.camera.width * v.camera.height;
    const int nv = ctx->meshes[v.mesh].dev.num_vertices;
    max_v = std::max(max_v, nv);
    sum_v += nv;
  }
  Scratch& s = ctx->scratch;
  int rc = ensure_scratch(ctx, s, 0, (size_t)n, 1, 0);
  if (rc) return rc;
  if ((size_t)n > s.targets_cap) {
    cudaFree(s.d_targets);
    cudaFreeHost(s.h_targets);
    s.d_targets = nullptr;
    s.h_targets = nullptr;
    s.targets_cap = 0;
    CK(ctx, cudaMalloc(&s.d_targets, n * sizeof(float*)), "cudaMalloc(targets)");
    CK(ctx, cudaMallocHost(&s.h_targets, n * sizeof(float*)), "cudaMallocHost(targets)");
    s.targets_cap = n;
  }
  if (grad_vertices && (size_t)sum_v > s.proj64_cap) {
    cudaFree(s.proj64);
    s.proj64 = nullptr;
    s.proj64_cap = 0;
    CK(ctx, cudaMalloc(&s.proj64, (size_t)sum_v * 32),
       "cudaMalloc(projection table)");
    s.proj64_cap = (size_t)sum_v;
  }
  // texel gradients through an RGBA scratch: one 16-byte atomic per texel
  // instead of an 8- and a 4-byte one, then added into grad_texels.  The
  // scratch costs a clear and a pass over the texture, about what the
  // atomics of 1.5 pixels per texel save (measured), so it is used from 2.
  if (sum_px < 2 * texels) texels = 0;
  if (texels > 0 && (size_t)texels > s.grad4_cap) {
    cudaFree(s.grad4);
    s.grad4 = nullptr;
    s.grad4_cap = 0;
    CK(ctx, cudaMalloc(&s.grad4, (size_t)texels * 4 * sizeof(float)),
       "cudaMalloc(texel gradient scratch)");
    s.grad4_cap = (size_t)texels;
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  int64_t proj_off = 0;
  for (int i = 0; i < n; ++i) {
    DevView& d = s.h_views[i];
    std::memset(&d, 0, sizeof(d));
    fill_cam(d.cam, views[i].camera);
    d.mesh = views[i].mesh;
    d.face_id = views[i].images.face_id;
    d.proj_offset = proj_off;
    proj_off += ctx->meshes[views[i].mesh].dev.num_vertices;
    s.h_targets[i] = targets[i];
  }
  CK(ctx, cudaMemcpyAsync(s.d_views, s.h_views, n * sizeof(DevView), cudaMemcpyHostToDevice,
                          ctx->stream),
     "cudaMemcpyAsync(views)");
  CK(ctx, cudaMemcpyAsync(s.d_targets, s.h_targets, n * sizeof(float*), cudaMemcpyHostToDevice,
                          ctx->stream),
     "cudaMemcpyAsync(targets)");
  BackwardParams p{};
  p.meshes = ctx->d_meshes;
  p.views = s.d_views;
  p.num_views = n;
  p.diffuse_color = o.diffuse_color;
  p.interp = o.interp;
  p.targets = s.d_targets;
  p.grad_texels = grad_texels;
  p.grad_vertex_colors = grad_vertex_colors;
  p.grad_vertices = grad_vertices;
  p.loss = loss_out;
  p.bad_ids = &s.counters[0].pad;
  p.proj64 = s.proj64;
  if (texels > 0) {
    p.grad_texels4 = s.grad4;
    p.num_texels4 = texels;
    CK(ctx, cudaMemsetAsync(s.grad4, 0, (size_t)texels * 4 * sizeof(float), ctx->stream),
       "cudaMemsetAsync(texel gradient scratch)");
  }
  CK(ctx, cudaMemsetAsync(s.counters, 0, sizeof(DevCounters), ctx->stream),
     "cudaMemsetAsync(counters)");
  launch_backward(p, max_px, max_v, ctx->num_sms, ctx->stream);
  CK(ctx, cudaGetLastError(), "backward launch");
  ctx->launches += 1 + (grad_vertices ? 1 : 0) + (texels > 0 ? 1 : 0);
  CK(ctx, cudaMemcpyAsync(s.h_counters, s.counters, sizeof(DevCounters), cudaMemcpyDeviceToHost,
                          ctx->stream),
     "cudaMemcpyAsync(counters)");
  if (flags & UGU_GPU_ASYNC) return UGU_GPU_OK;
  CK(ctx, cudaStreamSynchronize(ctx->stream), "backward");
  if (s.h_counters[0].pad)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                     "%llu face_id pixels hold ids outside the mesh (not a forward's output)",
                     (unsigned long long)s.h_counters[0].pad);
  return UGU_GPU_OK;
}

int ugu_gpu_get_device_mesh(ugu_gpu_context* ctx, int32_t slot, ugu_gpu_device_mesh* out) {
  if (!ctx || !out) return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL argument");
  if (slot < 0 || slot >= kMaxMeshes || !ctx->meshes[slot].present)
    return set_error(ctx, UGU_GPU_ERR_NOT_PREPARED, "mesh has not been initialized");
  const MeshSlot& m = ctx->meshes[slot];
  const DevMesh& d = m.dev;
  out->num_vertices = d.num_vertices;
  out->num_faces = d.num_faces;
  out->num_normals = d.num_normals;
  out->num_uv = d.num_uv;
  out->num_materials = d.num_materials;
  out->vertices4 = reinterpret_cast<const float*>(d.vertices);
  out->vertex_indices4 = reinterpret_cast<const int32_t*>(d.vidx);
  out->face_normals4 = reinterpret_cast<const float*>(d.fnormals);
  out->normals4 = reinterpret_cast<const float*>(d.normals);
  out->normal_indices4 = reinterpret_cast<const int32_t*>(d.nidx);
  out->vertex_colors4 = reinterpret_cast<const float*>(d.vcolors);
  out->uv2 = reinterpret_cast<const float*>(d.uv);
  out->uv_indices4 = reinterpret_cast<const int32_t*>(d.uvidx);
  out->material_ids = d.mat_ids;
  out->materials = m.dev_tex.empty() ? nullptr : m.dev_tex.data();
  return UGU_GPU_OK;
}

int ugu_gpu_visualize(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_vis* items,
                      uint32_t flags) {
  Range range("ugu_gpu visualize");
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  if (n < 0 || (n > 0 && !items))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad item list");
  cudaSetDevice(ctx->device);
  const bool dev = (flags & UGU_GPU_DEVICE_POINTERS) != 0;
  for (int k = 0; k < n; ++k) {
    ugu_gpu_vis it = items[k];
    if (it.width < 0 || it.height < 0)
      return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "item %d: negative size", k);
    const size_t px = (size_t)it.width * (size_t)it.height;
    if (px == 0) continue;
    if (!dev) {
      // inputs and outputs staged in one device buffer, 256-byte aligned parts
      struct Part {
        const void* in;
        void* out;
        size_t bytes;
      };
      const Part parts[7] = {{it.depth, nullptr, 4 * px},
                             {it.normal, nullptr, 12 * px},
                             {it.face_id, nullptr, 4 * px},
                             {nullptr, it.vis_depth, px},
                             {nullptr, it.depth_u16, 2 * px},
                             {nullptr, it.vis_normal, 3 * px},
                             {nullptr, it.vis_face_id, 3 * px}};
      size_t total = 0;
      for (const Part& q : parts)
        if (q.in || q.out) total += align256(q.bytes);
      if (total > ctx->vis_cap) {
        cudaFree(ctx->vis_buf);
        ctx->vis_buf = nullptr;
        ctx->vis_cap = 0;
        CK(ctx, cudaMalloc(&ctx->vis_buf, total), "cudaMalloc(visualize staging)");
        ctx->vis_cap = total;
      }
      void* dptr[7] = {};
      size_t off = 0;
      for (int j = 0; j < 7; ++j) {
        if (!parts[j].in && !parts[j].out) continue;
        dptr[j] = ctx->vis_buf + off;
        off += align256(parts[j].bytes);
        if (parts[j].in)
          CK(ctx, cudaMemcpyAsync(dptr[j], parts[j].in, parts[j].bytes, cudaMemcpyHostToDevice,
                                  ctx->stream),
             "cudaMemcpyAsync(visualize input)");
      }
      it.depth = static_cast<const float*>(dptr[0]);
      it.normal = static_cast<const float*>(dptr[1]);
      it.face_id = static_cast<const int32_t*>(dptr[2]);
      it.vis_depth = static_cast<uint8_t*>(dptr[3]);
      it.depth_u16 = static_cast<uint16_t*>(dptr[4]);
      it.vis_normal = static_cast<uint8_t*>(dptr[5]);
      it.vis_face_id = static_cast<uint8_t*>(dptr[6]);
      launch_vis(it, ctx->stream);
      CK(ctx, cudaGetLastError(), "visualize launch");
      for (int j = 3; j < 7; ++j)
        if (parts[j].out)
          CK(ctx, cudaMemcpyAsync(parts[j].out, dptr[j], parts[j].bytes, cudaMemcpyDeviceToHost,
                                  ctx->stream),
             "cudaMemcpyAsync(visualize output)");
      // the staging buffer is reused by the next item
      CK(ctx, cudaStreamSynchronize(ctx->stream), "visualize");
    } else {
      launch_vis(it, ctx->stream);
      CK(ctx, cudaGetLastError(), "visualize launch");
    }
    ++ctx->launches;
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream), "visualize");
  return UGU_GPU_OK;
}

int ugu_gpu_render_gbuffer(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_gbuffer* views,
                           uint32_t flags) {
  Range range("ugu_gpu gbuffer");
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  if (n < 0 || (n > 0 && !views))
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad view list");
  cudaSetDevice(ctx->device);
  int rc = check_option(ctx, ctx->opt);
  if (rc) return rc;
  for (int k = 0; k < n; ++k) {
    const ugu_gpu_gbuffer& v = views[k];
    if (v.mesh < 0 || v.mesh >= kMaxMeshes || !ctx->meshes[v.mesh].present)
      return set_error(ctx, UGU_GPU_ERR_NOT_PREPARED, "mesh has not been initialized");
    const MeshSlot& m = ctx->meshes[v.mesh];
    if (ctx->opt.shading_normal == 0 && !m.has_fnormals)
      return set_error(ctx, UGU_GPU_ERR_NO_FACE_NORMALS_FOR_SHADING,
                       "specified face normal as shading normal but face normal is empty.");
    if (ctx->opt.shading_normal == 1 && !m.has_normals)
      return set_error(ctx, UGU_GPU_ERR_NO_VERTEX_NORMALS,
                       "specified vertex normal as shading normal but vertex normal is empty.");
    if (!v.face_id || v.camera.width < 0 || v.camera.height < 0)
      return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "view %d: no face_id or bad size", k);
  }
  if (!ctx->gbuf_bad) {
    CK(ctx, cudaMalloc(&ctx->gbuf_bad, sizeof(unsigned long long)), "cudaMalloc(counter)");
    CK(ctx, cudaMallocHost(&ctx->h_gbuf_bad, sizeof(unsigned long long)),
       "cudaMallocHost(counter)");
  }
  CK(ctx, cudaMemsetAsync(ctx->gbuf_bad, 0, sizeof(unsigned long long), ctx->stream),
     "cudaMemsetAsync(counter)");
  const bool dev = (flags & UGU_GPU_DEVICE_POINTERS) != 0;
  for (int k = 0; k < n; ++k) {
    const ugu_gpu_gbuffer& v = views[k];
    const size_t px = (size_t)v.camera.width * (size_t)v.camera.height;
    if (px == 0) continue;
    GbufParams p{};
    fill_cam(p.cam, v.camera);
    p.mesh = ctx->d_meshes + v.mesh;
    p.shading_normal = ctx->opt.shading_normal;
    p.bad_ids = ctx->gbuf_bad;
    float* const outs[6] = {v.pos_wld, v.pos_cam, v.normal_wld, v.normal_cam, v.bary, v.uv};
    float** dst[6] = {&p.pos_wld, &p.pos_cam, &p.normal_wld, &p.normal_cam, &p.bary, &p.uv};
    if (dev) {
      p.face_id = v.face_id;
      for (int j = 0; j < 6; ++j) *dst[j] = outs[j];
      p.stencil = v.stencil;
      launch_gbuffer(p, ctx->stream);
      CK(ctx, cudaGetLastError(), "G-buffer launch");
    } else {
      size_t total = align256(4 * px) + align256(px);
      for (int j = 0; j < 6; ++j)
        if (outs[j]) total += align256(12 * px);
      if (total > ctx->vis_cap) {
        CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        cudaFree(ctx->vis_buf);
        ctx->vis_buf = nullptr;
        ctx->vis_cap = 0;
        CK(ctx, cudaMalloc(&ctx->vis_buf, total), "cudaMalloc(G-buffer staging)");
        ctx->vis_cap = total;
      }
      uint8_t* q = ctx->vis_buf;
      p.face_id = reinterpret_cast<const int32_t*>(q);
      CK(ctx, cudaMemcpyAsync(q, v.face_id, 4 * px, cudaMemcpyHostToDevice, ctx->stream),
         "cudaMemcpyAsync(face_id)");
      q += align256(4 * px);
      p.stencil = v.stencil ? q : nullptr;
      q += align256(px);
      for (int j = 0; j < 6; ++j) {
        *dst[j] = nullptr;
        if (!outs[j]) continue;
        *dst[j] = reinterpret_cast<float*>(q);
        q += align256(12 * px);
      }
      launch_gbuffer(p, ctx->stream);
      CK(ctx, cudaGetLastError(), "G-buffer launch");
      for (int j = 0; j < 6; ++j)
        if (outs[j])
          CK(ctx, cudaMemcpyAsync(outs[j], *dst[j], 12 * px, cudaMemcpyDeviceToHost, ctx->stream),
             "cudaMemcpyAsync(G-buffer)");
      if (v.stencil)
        CK(ctx, cudaMemcpyAsync(v.stencil, p.stencil, px, cudaMemcpyDeviceToHost, ctx->stream),
           "cudaMemcpyAsync(stencil)");
      // the staging buffer is reused by the next view
      CK(ctx, cudaStreamSynchronize(ctx->stream), "G-buffer");
    }
    ++ctx->launches;
  }
  CK(ctx, cudaMemcpyAsync(ctx->h_gbuf_bad, ctx->gbuf_bad, sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, ctx->stream),
     "cudaMemcpyAsync(counter)");
  CK(ctx, cudaStreamSynchronize(ctx->stream), "G-buffer");
  if (*ctx->h_gbuf_bad)
    return set_error(ctx, UGU_GPU_ERR_INDEX_OUT_OF_RANGE,
                     "%llu face ids outside [-1, num_faces)", *ctx->h_gbuf_bad);
  return UGU_GPU_OK;
}

int ugu_gpu_test_visibility(ugu_gpu_context* ctx, int32_t mesh, const float* normals, int32_t n,
                            const ugu_gpu_keyframe* keyframes,
                            const ugu_gpu_visibility_option* option, int32_t facewise,
                            const ugu_gpu_visibility_out* out, uint32_t flags) {
  Range range("ugu_gpu visibility");
  if (!ctx) return set_error(nullptr, UGU_GPU_ERR_INVALID_ARGUMENT, "NULL context");
  cudaSetDevice(ctx->device);
  if (n <= 0 || !keyframes || !option || !out)
    return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "bad keyframe list, option or output");
  if (mesh < 0 || mesh >= kMaxMeshes || !ctx->meshes[mesh].present)
    return set_error(ctx, UGU_GPU_ERR_NOT_PREPARED, "mesh has not been initialized");
  MeshSlot& ms = ctx->meshes[mesh];
  const int V = ms.dev.num_vertices, F = ms.dev.num_faces;
  if (V == 0 || F == 0 || !normals)  // PrepareData (:319-323)
    return set_error(ctx, UGU_GPU_ERR_NOT_PREPARED, "mesh is empty");
  const bool dev = (flags & UGU_GPU_DEVICE_POINTERS) != 0;
  for (int k = 0; k < n; ++k) {  // ValidateAndInitBeforeTest (:349-378)
    const ugu_gpu_keyframe& kf = keyframes[k];
    if (!kf.color || kf.camera.width <= 0 || kf.camera.height <= 0)
      return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT, "keyframe color is empty");
    if (option->use_mask && !kf.mask)
      return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                       "use_mask is true but keyframe mask is empty");
    if (option->use_depth && !kf.depth)
      return set_error(ctx, UGU_GPU_ERR_INVALID_ARGUMENT,
                       "use_depth is true but keyframe depth is empty");
  }
  int rc = ensure_vis_bvh(ctx, mesh);
  if (rc) return rc;
  const int64_t items = facewise ? 3 * (int64_t)F : (int64_t)V;
  // one device buffer: normals, keyframe table, staged images, staged outputs
  size_t img_bytes = 0;
  if (!dev)
    for (int k = 0; k < n; ++k) {
      const size_t px = (size_t)keyframes[k].camera.width * keyframes[k].camera.height;
      img_bytes += align256(3 * px) + (keyframes[k].depth ? align256(4 * px) : 0) +
                   (keyframes[k].mask ? align256(px) : 0);
    }
  const size_t ki = (size_t)n * (size_t)items;
  const size_t out_bytes = dev ? 0 : align256(ki) + align256(8 * ki) + 3 * align256(4 * ki) +
                                         align256(12 * ki);
  const size_t total = align256(16 * (size_t)V) + align256(sizeof(DevKeyframe) * n) + img_bytes +
                       out_bytes;
  CK(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (total > ctx->vis_cap) {
    cudaFree(ctx->vis_buf);
    ctx->vis_buf = nullptr;
    ctx->vis_cap = 0;
    CK(ctx, cudaMalloc(&ctx->vis_buf, total), "cudaMalloc(visibility buffers)");
    ctx->vis_cap = total;
  }
  uint8_t* q = ctx->vis_buf;
  auto take = [&](size_t bytes) {
    uint8_t* r = q;
    q += align256(bytes);
    return r;
  };
  std::vector<float4> n4((size_t)V);
  for (int i = 0; i < V; ++i)
    n4[i] = make_float4(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2], 0.0f);
  float4* d_normals = reinterpret_cast<float4*>(take(16 * (size_t)V));
  CK(ctx, cudaMemcpyAsync(d_normals, n4.data(), 16 * (size_t)V, cudaMemcpyHostToDevice,
                          ctx->stream),
     "cudaMemcpyAsync(normals)");
  DevKeyframe* d_kfs = reinterpret_cast<DevKeyframe*>(take(sizeof(DevKeyframe) * n));
  std::vector<DevKeyframe> hk((size_t)n);
  for (int k = 0; k < n; ++k) {
    const ugu_gpu_keyframe& kf = keyframes[k];
    DevKeyframe& d = hk[k];
    std::memset(&d, 0, sizeof(d));
    fill_cam(d.cam, kf.camera);
    std::memcpy(d.L, kf.w2c_linear, sizeof(d.L));
    d.id = kf.id;
    const size_t px = (size_t)kf.camera.width * kf.camera.height;
    if (dev) {
      d.color = kf.color;
      d.depth = kf.depth;
      d.mask = kf.mask;
      continue;
    }
    uint8_t* c = take(3 * px);
    CK(ctx, cudaMemcpyAsync(c, kf.color, 3 * px, cudaMemcpyHostToDevice, ctx->stream),
       "cudaMemcpyAsync(keyframe color)");
    d.color = c;
    if (kf.depth) {
      uint8_t* dd = take(4 * px);
      CK(ctx, cudaMemcpyAsync(dd, kf.depth, 4 * px, cudaMemcpyHostToDevice, ctx->stream),
         "cudaMemcpyAsync(keyframe depth)");
      d.depth = reinterpret_cast<const float*>(dd);
    }
    if (kf.mask) {
      uint8_t* mm = take(px);
      CK(ctx, cudaMemcpyAsync(mm, kf.mask, px, cudaMemcpyHostToDevice, ctx->stream),
         "cudaMemcpyAsync(keyframe mask)");
      d.mask = mm;
    }
  }
  CK(ctx, cudaMemcpyAsync(d_kfs, hk.data(), sizeof(DevKeyframe) * n, cudaMemcpyHostToDevice,
                          ctx->stream),
     "cudaMemcpyAsync(keyframes)");
  VisParams p{};
  p.mesh = ctx->d_meshes + mesh;
  p.normals = d_normals;
  p.kfs = d_kfs;
  p.num_kf = n;
  p.facewise = facewise ? 1 : 0;
  p.items = (int32_t)items;
  p.backface_th = option->backface_culling_angle_rad_th;
  p.max_viewing_angle = option->max_viewing_angle;
  p.max_distance = option->max_distance_from_camera_to_vertex;
  p.max_depth_difference = option->max_depth_difference;
  p.eps = option->eps;
  p.use_mask = option->use_mask ? 1 : 0;
  p.use_depth = option->use_depth ? 1 : 0;
  p.interp = option->interp;
  if (dev) {
    p.visible = out->visible;
    p.projected = out->projected_pos;
    p.viewing_angle = out->viewing_angle;
    p.distance = out->distance;
    p.color = out->color;
    p.intensity = out->intensity;
  } else {
    p.visible = out->visible ? take(ki) : nullptr;
    p.projected = out->projected_pos ? reinterpret_cast<float*>(take(8 * ki)) : nullptr;
    p.viewing_angle = out->viewing_angle ? reinterpret_cast<float*>(take(4 * ki)) : nullptr;
    p.distance = out->distance ? reinterpret_cast<float*>(take(4 * ki)) : nullptr;
    p.color = out->color ? reinterpret_cast<float*>(take(12 * ki)) : nullptr;
    p.intensity = out->intensity ? reinterpret_cast<float*>(take(4 * ki)) : nullptr;
  }
  launch_visibility(p, ctx->stream);
  CK(ctx, cudaGetLastError(), "visibility launch");
  ++ctx->launches;
  if (!dev) {
    auto back = [&](void* dst, const void* src, size_t bytes) -> int {
      if (!dst) return UGU_GPU_OK;
      CK(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream),
         "cudaMemcpyAsync(visibility)");
      return UGU_GPU_OK;
    };
    if ((rc = back(out->visible, p.visible, ki))) return rc;
    if ((rc = back(out->projected_pos, p.projected, 8 * ki))) return rc;
    if ((rc = back(out->viewing_angle, p.viewing_angle, 4 * ki))) return rc;
    if ((rc = back(out->distance, p.distance, 4 * ki))) return rc;
    if ((rc = back(out->color, p.color, 12 * ki))) return rc;
    if ((rc = back(out->intensity, p.intensity, 4 * ki))) return rc;
  }
  CK(ctx, cudaStreamSynchronize(ctx->stream), "visibility");
  return UGU_GPU_OK;
}

int ugu_gpu_get_stats(const ugu_gpu_context* ctx, ugu_gpu_stats* st) {
  if (!ctx || !st) return UGU_GPU_ERR_INVALID_ARGUMENT;
  st->launches = ctx->launches;
  st->special_candidates = ctx->special;
  st->large_face_tiles = ctx->large_items;
  uint64_t b = 0;
  for (const MeshSlot& m : ctx->meshes) b += m.bytes;
  const Scratch& s = ctx->scratch;
  b += s.keys_cap * 8 + s.items_cap * sizeof(TileItem) + s.d_out_cap;
  st->device_bytes = b;
  st->tile_kernel_ms = ctx->tile_ms;
  st->tile_kernel_launches = ctx->tile_launches;
  return UGU_GPU_OK;
}

}  // extern "C"
