// internal.cuh -- device-side data layout shared by the kernels and the C ABI.
//
// HBM layout of a mesh slot (uploaded once by ugu_gpu_set_mesh):
//   vertices       V x float4 (x, y, z, 0)      16-byte vector loads
//   vertex_indices F x int4   (i0, i1, i2, 0)
//   face_normals   F x float4
//   normals        N x float4,  normal_indices F x int4
//   vertex_colors  V x float4
//   uv             T x float2,  uv_indices     F x int4
//   material_ids   F x int32
//   textures       per material: RGBA8 texels (uint32, alpha 0) and/or RGB f32
// Per view: a Cam (floats exactly as the host computed them) and output
// pointers.  Z-buffer: one 64-bit key per pixel of the current view group.
#pragma once

#include <vector>

#include <cstdint>

#include "exact.cuh"
#include "ugu_gpu.h"

namespace ugu_gpu {

struct DevTexture {
  int32_t width, height;
  const uint32_t* rgba8;  // texel i at rgba8[i]: r | g << 8 | b << 16
  const float* rgbf;      // texel i at rgbf[3 i .. 3 i + 2]
};

struct DevMesh {
  int32_t num_vertices, num_faces, num_normals, num_uv, num_materials;
  const float4* vertices;
  const int4* vidx;
  const float4* fnormals;
  const float4* normals;
  const int4* nidx;
  const float4* vcolors;
  const float2* uv;
  const int4* uvidx;
  const int32_t* mat_ids;
  const DevTexture* textures;
  // Tiled path only (results never depend on them): the faces in 3D Morton
  // order of their centroids (the binning order), the vertices in Morton
  // order of their positions (the order of the projected-vertex table), the
  // vertex indices as ranks in that order, per face and per Morton face, and
  // the face normals per Morton face.
  const int32_t* order;
  const int32_t* vorder;
  const int4* vidx_ranked;
  const int4* vidx_morton;
  const float4* fnormals_morton;
  // Raytracer only (built on first use): the naive BVH flattened in
  // depth-first order, 2 float4 per node, and its leaf entries in that
  // order, 3 float4 per entry (an entry's index is its rank in the
  // reference's traversal order).  NULL until built.
  const float4* bvh_nodes;
  const float4* bvh_tris;
  int32_t bvh_depth;    // deepest node (root = 0)
  int32_t bvh_entries;
  // the visibility tester's tree (leaves of up to 5 faces), built on first use
  const float4* vis_nodes;
  const float4* vis_tris;
};

struct DevView {
  Cam cam;
  int32_t mesh;
  int32_t tiles_x;     // tiled path: tiles per row
  int64_t key_offset;  // global path: first z-buffer key of this view within its group
  int64_t proj_offset; // tiled path: first projected vertex of this view
  int32_t tile_base;   // tiled path: first global tile of this view
  float split_z;       // tiled path: faces wholly deeper than this are drawn last
  int32_t tile_log2;   // tiled path: this view's tile edge is 1 << tile_log2 pixels
  int32_t pad_;
  uint8_t* color;
  float* depth;
  float* normal;
  uint8_t* mask;
  int32_t* face_id;
  float* color_f32;
};

// Bits of the sticky status word (RenderParams::sticky, TileParams::sticky).
constexpr unsigned long long kStickyOverflow = 1ull;
constexpr unsigned long long kStickySpecial = 2ull;

// Counters shared by the kernels of one render (device memory).
struct DevCounters {
  unsigned long long special;     // covered samples with unorderable depth
  unsigned long long tile_items;  // (face, tile) items appended this group
  unsigned long long overflow;    // items dropped for lack of capacity
  unsigned long long pad;
};

// The option fields the pixel shaders read (RendererCpuOption,
// renderer.h:17-38) and the Oren-Nayar constants (pixel_shader.h:143-148).
struct ShadeOpts {
  int32_t diffuse_color, interp, shading_normal, diffuse_shading;
  float on_A, on_B;
};

struct Shaded {
  uint8_t c[3];
  float cf[3];
  float n[3];
};

struct TileItem {
  int32_t view;  // view index within the group
  int32_t face;
  int32_t tx, ty;  // tile coordinates
};

struct RenderParams {
  const DevMesh* meshes;
  const DevView* views;  // views of this group
  int32_t num_views;
  ShadeOpts shade;
  int32_t backface_culling;
  unsigned long long* keys;
  DevCounters* counters;
  TileItem* items;
  int64_t item_capacity;
  int32_t tile_log2;
  int32_t small_bbox_max;
  // sticky status of the context, or NULL: bit 0 a list overflowed (the
  // render's images are not valid), bit 1 a covered sample had an
  // unorderable depth; kept until ugu_gpu_synchronize reads and clears it
  unsigned long long* sticky;
};

// Counters of one tiled render (memset before every launch).
struct TileCounters {
  unsigned int next_tile;             // work-queue head of k_tile
  unsigned int invalid;                // entries outside their arrays (a bug)
  unsigned long long special;         // covered samples with unorderable depth
  unsigned long long dropped;         // entries did not fit (0: none)
  unsigned long long total_entries;   // (face, tile) entries of this render
};

// Tiled-path buffers.  k_count counts every tile's (face, tile) entries,
// k_scan_sum and k_scan_apply turn the counts into offsets and k_place places
// the entries:
// per global tile t, those of the faces drawn first in [tile_off[t],
// tile_lo[t]) and those of the faces drawn last in [tile_lo[t],
// tile_off[t + 1]).  An entry is (the face's number in the binning order
// DevMesh::order, bit pattern of a lower bound of every depth the face can
// produce).
struct TileParams {
  const DevMesh* meshes;
  const DevView* views;
  int32_t num_views;
  ShadeOpts shade;
  int32_t backface_culling;
  int32_t total_tiles;
  int32_t max_vertices;
  int32_t split_class;  // draw classes of at most this many entries are shared over the warps
  int32_t bin_faces;    // binning: faces per thread (1, 2 or 4)
  int64_t entry_cap;    // entries the entry buffer holds
  float4* proj;         // projected vertices (x, y, camera z, 0) of every view
  int32_t* tile_count;  // entries per tile (k_count adds; k_scan_apply reads and zeroes)
  int32_t* tile_off;    // total_tiles + 1 offsets into entries
  int32_t* tile_lo;     // first-drawn cursor / boundary per tile
  int32_t* tile_hi;     // last-drawn cursor per tile
  int2* entries;        // entries in tile order
  long long* chunk_sums;  // entries of each chunk of 4,096 tiles (scan_chunks(total_tiles))
  TileCounters* counters;
  unsigned long long* sticky;  // as RenderParams::sticky
};

struct BackwardParams {
  const DevMesh* meshes;
  const DevView* views;  // face_id: the forward's visibility (device)
  int32_t num_views;
  int32_t diffuse_color, interp;
  const float* const* targets;  // device array of per-view H*W*3 targets
  float* grad_texels;           // material 0, H*W*3 (or NULL)
  // texel gradients gathered first as RGBA (one 16-byte atomic per texel)
  // and then added into grad_texels, or NULL to scatter into it directly
  float* grad_texels4;
  int64_t num_texels4;
  float* grad_vertex_colors;    // V*3 (or NULL)
  float* grad_vertices;         // V*3 (or NULL)
  float* loss;                  // one per view (or NULL)
  unsigned long long* bad_ids;  // counts face ids outside [-1, num_faces)
  void* proj64;                 // per view (DevView::proj_offset), 32 bytes per vertex: screen
                                // x, y as hi + lo floats, and 1/z
};

// Image helpers of ugu_gpu_visualize (vis.cu): one item, device pointers.
void launch_vis(const ugu_gpu_vis& item, cudaStream_t s);

// G-buffer pass (vis.cu): one view, device pointers.
struct GbufParams {
  Cam cam;
  const DevMesh* mesh;  // device copy of the view's mesh slot
  int32_t shading_normal;
  const int32_t* face_id;
  float *pos_wld, *pos_cam, *normal_wld, *normal_cam, *bary, *uv;
  uint8_t* stencil;
  unsigned long long* bad_ids;  // face ids outside [-1, num_faces)
};
void launch_gbuffer(const GbufParams& p, cudaStream_t s);

// Visibility test (ray.cu): one thread per (keyframe, vertex) or, facewise,
// per (keyframe, face corner).
struct DevKeyframe {
  Cam cam;           // R, t: w2c rotation / translation; C, T: c2w
  float L[9];        // w2c().linear().cast<float>(), row-major
  int32_t id;
  const uint8_t* color;  // H*W*3
  const float* depth;    // H*W or NULL
  const uint8_t* mask;   // H*W or NULL
};
struct VisParams {
  const DevMesh* mesh;      // vertices, faces and the visibility tree
  const float4* normals;    // per vertex (the tester's normals)
  const DevKeyframe* kfs;
  int32_t num_kf;
  int32_t facewise;         // items = faces * 3 corners, else vertices
  int32_t items;
  float backface_th, max_viewing_angle, max_distance, max_depth_difference, eps;
  int32_t use_mask, use_depth, interp;
  uint8_t* visible;         // [kf][item]
  float* projected;         // [kf][item][2]
  float* viewing_angle;     // [kf][item]
  float* distance;          // [kf][item]
  float* color;             // [kf][item][3]
  float* intensity;         // [kf][item]
};
void launch_visibility(const VisParams& p, cudaStream_t s);

// TextureMapping on the mesh's own uv (texmap.cu).
struct TexMapParams {
  const float2* uv;
  const int4* uvidx;
  const float* face_target; // per face: its triangle in texel coordinates, 6 floats, or NULL
                            // (then it comes from uv and uvidx)
  int num_faces;
  const int32_t* face_kf;   // per face: its keyframe (an index of kf), or -1
  const float* face_tri;    // per face: projected triangle in that keyframe, 6 floats
  const DevKeyframe* kf;    // colour images (cam.width x cam.height RGB8)
  int tex_w, tex_h, hk;     // texture size; half the padding kernel
  int32_t* owner;           // per texel: the last face covering it, or -1
  uint8_t *tex0, *mask0;    // before padding
  uint8_t *tex, *mask;      // results
};
void launch_texture_mapping(const TexMapParams& p, cudaStream_t s);

// Raytracer (ray.cu): the views of one group, one thread per pixel.
struct RayParams {
  const DevMesh* meshes;
  const DevView* views;
  int32_t num_views;
  ShadeOpts shade;
  int32_t backface_culling;
  float depth_scale;
};

// Deepest BVH node the traversal stack holds (a median split of 2^60 faces).
constexpr int kMaxBvhDepth = 60;

// Host copy of a mesh's BVH (bvh.cu): 2 float4 per node, 3 per leaf entry.
struct HostBvh {
  std::vector<float4> nodes, tris;
  int depth = 0;
};
// Builds ugu::BvhNaive's tree for the mesh; false when it is deeper than
// kMaxBvhDepth or the mesh has no face.
bool build_bvh(const float* vertices, const int32_t* faces, int num_faces, HostBvh& out,
               int leaf_faces = 4);
// One block per kRayTileW x kRayTileH pixels; max_tiles = the most tiles of
// any view of the group.
constexpr int kRayTileW = 16, kRayTileH = 8;
void launch_ray(const RayParams& p, int64_t max_tiles, cudaStream_t s);

// Host-side launcher (backward.cu): the hi + lo projection table (when
// position gradients are asked for), then the per-pixel backward.
void launch_backward(const BackwardParams& p, int64_t max_pixels, int max_vertices, int num_sms,
                     cudaStream_t s);

// Host-side launchers of the tiled path.  launch_bin (bin.cu) enqueues
// projection, counting, the offset scan and the placing of the entries
// (launch_size all but the placing, to learn a render's entry count);
// launch_tile (tile.cu) the per-tile raster and resolve.
void launch_bin(const TileParams& p, int max_faces, cudaStream_t s);
void launch_size(const TileParams& p, int max_faces, cudaStream_t s);
void launch_tile(const TileParams& p, int grid, cudaStream_t s);
int tile_kernel_blocks_per_sm();
constexpr int kBinKernels = 5;
// Chunks of the tile-count scan for `tiles` tiles (TileParams::chunk_sums).
int64_t scan_chunks(int64_t tiles);

// Host-side launchers (raster.cu).
void launch_raster(const RenderParams& p, int max_faces, int num_sms, cudaStream_t s);
void launch_tiles(const RenderParams& p, int grid, cudaStream_t s);
void launch_resolve(const RenderParams& p, int64_t max_pixels, cudaStream_t s);
int raster_launches_per_group();

}  // namespace ugu_gpu
