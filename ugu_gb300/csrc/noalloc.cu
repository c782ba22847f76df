// noalloc.cu -- ugu_gpu_render_noalloc: one render that allocates nothing.
//
// Some callers cannot call cudaMalloc: a plug-in whose host application owns
// every byte of device memory and hands it only finished buffers; code that
// runs under a fixed device-memory budget managed by another allocator,
// where an extra allocation would fail or fragment the pool; a frame loop
// that must not take the implicit device synchronisation that cudaMalloc and
// cudaFree can cause.  For them this entry point renders one view with the
// same kernels as the global-z-buffer path (raster.cu, unchanged), taking its
// scratch -- the view and mesh descriptors, the 64-bit z-buffer, the counters
// and the large-face tile list -- from one file-scope __device__ array.
//
// Limits: at most kMaxPixels pixels per view, kMaxMaterials materials and
// kMaxItems (face, tile) items for faces whose bbox exceeds 256 pixels (past
// that the call returns UGU_GPU_ERR_CAPACITY and the images are not valid).
// Every GPU that loads this library holds the array (about 20 MB) until the
// process exits.  All calls share it: two calls whose work overlaps on the GPU
// (different streams, or different host threads) race on it and must be
// serialised by the caller.  Each call clears the part it uses first.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstring>
#include <mutex>

#include "internal.cuh"
#include "ugu_gpu.h"

namespace ugu_gpu {
void set_thread_error(const char* msg);  // capi.cu
}

namespace {

using namespace ugu_gpu;

constexpr int64_t kMaxPixels = UGU_GPU_NOALLOC_MAX_PIXELS;
constexpr int kMaxMaterials = UGU_GPU_NOALLOC_MAX_MATERIALS;
constexpr int64_t kMaxItems = UGU_GPU_NOALLOC_MAX_ITEMS;
constexpr size_t kHeadBytes = 4096;

struct Head {
  DevMesh mesh;
  DevView view;
  DevCounters counters;
  DevTexture textures[kMaxMaterials];
};
static_assert(sizeof(Head) <= kHeadBytes, "descriptor block too large");

constexpr size_t kKeyOffset = kHeadBytes;
constexpr size_t kItemOffset = kKeyOffset + (size_t)kMaxPixels * sizeof(unsigned long long);
constexpr size_t kScratchBytes = kItemOffset + (size_t)kMaxItems * sizeof(TileItem);

// The scratch.  In host code `g_noalloc_scratch` only names a host-side
// stand-in; kernels get the device address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};

int fail(int code, const char* msg) {
  set_thread_error(msg);
  return code;
}

// Device address of the scratch on the current device, looked up once per
// device (the first call on a device does this set-up) and kept for the life
// of the process: a cudaDeviceReset on that device while the library is in
// use would leave the kept address stale.
int scratch_address(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(UGU_GPU_ERR_CUDA, cudaGetErrorString(e));
    g_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_addr[dev];
  return UGU_GPU_OK;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// The checks of ValidateAndInitBeforeRender (util_private.cc:19-67), in
// order, on the caller's descriptor.
int validate(const ugu_gpu_device_mesh& m, const ugu_gpu_option& o, const ugu_gpu_camera& c,
             const ugu_gpu_images& im) {
  if (o.diffuse_color < 0 || o.diffuse_color > 2 || o.interp < 0 || o.interp > 1 ||
      o.shading_normal < 0 || o.shading_normal > 1 || o.diffuse_shading < 0 ||
      o.diffuse_shading > 2)
    return fail(UGU_GPU_ERR_INVALID_ARGUMENT, "option enum out of range");
  if (o.backface_culling && !m.face_normals4)
    return fail(UGU_GPU_ERR_NO_FACE_NORMALS, "specified back-face culling but face normal is empty.");
  if (o.diffuse_color == 1 && m.num_materials == 0)
    return fail(UGU_GPU_ERR_NO_TEXTURE, "specified texture as diffuse color but texture is empty.");
  if (o.diffuse_color == 1)
    for (int i = 0; i < m.num_materials; ++i)
      if (m.materials[i].width < 1 || m.materials[i].height < 1 ||
          (!m.materials[i].rgba8 && !m.materials[i].rgb_f32))
        return fail(UGU_GPU_ERR_EMPTY_TEXTURE, "specified texture as diffuse color but a texture is empty.");
  if (o.diffuse_color == 2 && !m.vertex_colors4)
    return fail(UGU_GPU_ERR_NO_VERTEX_COLORS, "specified vertex color as diffuse color but vertex color is empty.");
  if (o.shading_normal == 0 && !m.face_normals4)
    return fail(UGU_GPU_ERR_NO_FACE_NORMALS_FOR_SHADING, "specified face normal as shading normal but face normal is empty.");
  if (o.shading_normal == 1 && (!m.normals4 || (m.num_faces > 0 && !m.normal_indices4)))
    return fail(UGU_GPU_ERR_NO_VERTEX_NORMALS, "specified vertex normal as shading normal but vertex normal is empty.");
  if (!im.color && !im.depth && !im.normal && !im.mask && !im.face_id && !im.color_f32)
    return fail(UGU_GPU_ERR_NO_OUTPUT, "all arguments are nullptr. nothing to do");
  // rasterizer.cc:199 reads the face normal at every pixel of every face's
  // box; a mesh without faces reads none (nor uv, uv indices, material ids)
  if (m.num_faces > 0 && !m.face_normals4)
    return fail(UGU_GPU_ERR_NO_FACE_NORMALS, "face normals are required: the z pass reads them");
  if (m.num_faces > 0 && o.diffuse_color == 1 && (!m.uv2 || !m.uv_indices4 || !m.material_ids))
    return fail(UGU_GPU_ERR_NO_TEXTURE, "texture colour needs uv, uv_indices and material_ids");
  if (m.num_vertices < 0 || m.num_faces < 0 || (m.num_faces > 0 && (!m.vertices4 || !m.vertex_indices4)))
    return fail(UGU_GPU_ERR_INVALID_ARGUMENT, "vertices or faces missing");
  if (m.num_materials < 0 || m.num_materials > kMaxMaterials || (m.num_materials && !m.materials))
    return fail(UGU_GPU_ERR_CAPACITY, "more materials than the no-allocation limit");
  if (c.width <= 0 || c.height <= 0 || (int64_t)c.width * c.height > kMaxPixels)
    return fail(UGU_GPU_ERR_CAPACITY, "image larger than UGU_GPU_NOALLOC_MAX_PIXELS");
  const void* v16[] = {m.vertices4, m.vertex_indices4, m.face_normals4, m.normals4,
                       m.normal_indices4, m.vertex_colors4, m.uv_indices4};
  for (const void* p : v16)
    if (p && !aligned16(p)) return fail(UGU_GPU_ERR_INVALID_ARGUMENT, "4-wide arrays must be 16-byte aligned");
  return UGU_GPU_OK;
}

}  // namespace

extern "C" UGU_GPU_API int ugu_gpu_render_noalloc(const ugu_gpu_device_mesh* mesh,
                                                  const ugu_gpu_option* opt,
                                                  const ugu_gpu_camera* cam,
                                                  const ugu_gpu_images* images, void* stream) {
  if (!mesh || !opt || !images) return fail(UGU_GPU_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!cam) return fail(UGU_GPU_ERR_NO_CAMERA, "camera has not been set");
  int rc = validate(*mesh, *opt, *cam, *images);
  if (rc) return rc;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(UGU_GPU_ERR_NO_DEVICE, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(UGU_GPU_ERR_INVALID_ARGUMENT, "device index");
  unsigned char* base = nullptr;
  if ((rc = scratch_address(dev, &base))) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  Head h;
  std::memset(&h, 0, sizeof(h));
  const ugu_gpu_device_mesh& m = *mesh;
  h.mesh.num_vertices = m.num_vertices;
  h.mesh.num_faces = m.num_faces;
  h.mesh.num_normals = m.num_normals;
  h.mesh.num_uv = m.num_uv;
  h.mesh.num_materials = m.num_materials;
  h.mesh.vertices = reinterpret_cast<const float4*>(m.vertices4);
  h.mesh.vidx = reinterpret_cast<const int4*>(m.vertex_indices4);
  h.mesh.fnormals = reinterpret_cast<const float4*>(m.face_normals4);
  h.mesh.normals = reinterpret_cast<const float4*>(m.normals4);
  h.mesh.nidx = reinterpret_cast<const int4*>(m.normal_indices4);
  h.mesh.vcolors = reinterpret_cast<const float4*>(m.vertex_colors4);
  h.mesh.uv = reinterpret_cast<const float2*>(m.uv2);
  h.mesh.uvidx = reinterpret_cast<const int4*>(m.uv_indices4);
  h.mesh.mat_ids = m.material_ids;
  Head* d_head = reinterpret_cast<Head*>(base);
  h.mesh.textures = d_head->textures;
  for (int i = 0; i < m.num_materials; ++i) {
    h.textures[i].width = m.materials[i].width;
    h.textures[i].height = m.materials[i].height;
    h.textures[i].rgba8 = m.materials[i].rgba8;
    h.textures[i].rgbf = m.materials[i].rgb_f32;
  }
  Cam& c = h.view.cam;
  c.width = cam->width;
  c.height = cam->height;
  c.fx = cam->fx;
  c.fy = cam->fy;
  c.cx = cam->cx;
  c.cy = cam->cy;
  std::memcpy(c.R, cam->w2c_R, sizeof(c.R));
  std::memcpy(c.t, cam->w2c_t, sizeof(c.t));
  std::memcpy(c.C, cam->c2w_R, sizeof(c.C));
  h.view.mesh = 0;
  h.view.color = images->color;
  h.view.depth = images->depth;
  h.view.normal = images->normal;
  h.view.mask = images->mask;
  h.view.face_id = images->face_id;
  h.view.color_f32 = images->color_f32;

  const int64_t npx = (int64_t)cam->width * cam->height;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(base + kKeyOffset);
  // Clear what must start empty: the z-buffer part this view uses and the
  // counters; the descriptors are overwritten whole.
  if ((e = cudaMemcpyAsync(d_head, &h, sizeof(Head), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(keys, 0xff, (size_t)npx * sizeof(unsigned long long), s)) != cudaSuccess)
    return fail(UGU_GPU_ERR_CUDA, cudaGetErrorString(e));

  RenderParams p{};
  p.meshes = &d_head->mesh;
  p.views = &d_head->view;
  p.num_views = 1;
  p.shade.diffuse_color = opt->diffuse_color;
  p.shade.interp = opt->interp;
  p.shade.shading_normal = opt->shading_normal;
  p.shade.diffuse_shading = opt->diffuse_shading;
  const float sigma_2 = opt->oren_nayar_sigma * opt->oren_nayar_sigma;  // pixel_shader.h:143-148
  p.shade.on_A = 1.0f - (0.5f * sigma_2 / (sigma_2 + 0.33f));
  p.shade.on_B = 0.45f * sigma_2 / (sigma_2 + 0.09f);
  p.backface_culling = opt->backface_culling ? 1 : 0;
  p.keys = keys;
  p.counters = &d_head->counters;
  p.items = reinterpret_cast<TileItem*>(base + kItemOffset);
  p.item_capacity = kMaxItems;
  p.tile_log2 = 4;
  p.small_bbox_max = 256;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  launch_raster(p, m.num_faces, sms, s);
  launch_tiles(p, sms * 8, s);
  launch_resolve(p, npx, s);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(UGU_GPU_ERR_CUDA, cudaGetErrorString(e));
  DevCounters hc;
  if ((e = cudaMemcpyAsync(&hc, &d_head->counters, sizeof(hc), cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(UGU_GPU_ERR_CUDA, cudaGetErrorString(e));
  if (hc.overflow) return fail(UGU_GPU_ERR_CAPACITY, "large-face tile items exceeded the no-allocation list");
  if (hc.special)
    return fail(UGU_GPU_ERR_DEGENERATE_DEPTH, "covered samples had depth < FLT_MIN or NaN");
  return UGU_GPU_OK;
}
