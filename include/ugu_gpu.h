/*
 * ugu_gpu.h -- C ABI of the GB300 rasterizer (libugugpu.so).
 *
 * This is the boundary a ugu build binds to replace the CPU rasterizer
 * (ugu::Rasterizer, include/ugu/renderer/cpu/rasterizer.h:14-53) behind the
 * ugu::RendererCpu interface (include/ugu/renderer/cpu/renderer.h:42-76).
 * Plain pointers and sizes only; every entry point returns a status code
 * (0 = success) and leaves a message in ugu_gpu_last_error().
 *
 * Image layouts are ugu::Image's (include/ugu/image.h:347-427): row-major,
 * channels interleaved.  color: H*W*3 uint8 RGB; depth: H*W float;
 * normal: H*W*3 float (camera frame); mask: H*W uint8 (0/255);
 * face_id: H*W int32 (-1 = none).
 */
#ifndef UGU_GPU_H_
#define UGU_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UGU_GPU_ABI_VERSION 4

#if defined(__GNUC__)
#define UGU_GPU_API __attribute__((visibility("default")))
#else
#define UGU_GPU_API
#endif

typedef struct ugu_gpu_context ugu_gpu_context;
typedef struct ugu_gpu_plan ugu_gpu_plan;

/* Status codes.  3..10 are the failure cases of ugu's
 * ValidateAndInitBeforeRender (src/renderer/cpu/util_private.cc:19-67) and
 * Rasterizer::Impl::PrepareMesh (src/renderer/cpu/rasterizer.cc:90-99), which
 * the reference reports as `false` + LOGE. */
enum {
  UGU_GPU_OK = 0,
  UGU_GPU_ERR_INVALID_ARGUMENT = 1,
  UGU_GPU_ERR_NOT_PREPARED = 2,          /* mesh slot empty ("mesh has not been initialized") */
  UGU_GPU_ERR_NO_FACE_NORMALS = 3,       /* culling without face normals */
  UGU_GPU_ERR_NO_TEXTURE = 4,            /* kTexture without materials */
  UGU_GPU_ERR_EMPTY_TEXTURE = 5,         /* a material's texture is empty */
  UGU_GPU_ERR_NO_VERTEX_COLORS = 6,      /* kVertex without vertex colours */
  UGU_GPU_ERR_NO_FACE_NORMALS_FOR_SHADING = 7,
  UGU_GPU_ERR_NO_VERTEX_NORMALS = 8,
  UGU_GPU_ERR_NO_OUTPUT = 9,             /* every output pointer is NULL */
  UGU_GPU_ERR_NO_CAMERA = 10,
  UGU_GPU_ERR_INDEX_OUT_OF_RANGE = 11,   /* a face refers past its array */
  UGU_GPU_ERR_CUDA = 12,
  UGU_GPU_ERR_OUT_OF_MEMORY = 13,
  UGU_GPU_ERR_DEVICE_TIMEOUT = 14,       /* a bounded device-side wait ran out */
  UGU_GPU_ERR_CAPACITY = 15,             /* a device work list hit its capacity */
  UGU_GPU_ERR_NO_DEVICE = 16,
  UGU_GPU_ERR_DEGENERATE_DEPTH = 17      /* a covered sample with depth < FLT_MIN or NaN */
};

/* ugu::RendererCpuOption (include/ugu/renderer/cpu/renderer.h:17-38) with the
 * enums of include/ugu/renderer/base.h:11-32 and ugu::ColorInterpolation
 * (include/ugu/common.h:50-53). */
typedef struct {
  int32_t diffuse_color;   /* 0 kNone (white), 1 kTexture, 2 kVertex */
  int32_t interp;          /* 0 kNn, 1 kBilinear */
  int32_t shading_normal;  /* 0 kFace, 1 kVertex */
  int32_t diffuse_shading; /* 0 kNone, 1 kLambertian, 2 kOrenNayar */
  float depth_scale;       /* raytracer: multiplies the output depth (raytracer.cc:185);
                              the rasterizer ignores it, as ugu::Rasterizer does */
  int32_t backface_culling;
  float oren_nayar_sigma;
} ugu_gpu_option;

typedef struct {
  int32_t width, height;
  const uint8_t* rgb8;   /* H*W*3 (ugu::Image3b), or NULL */
  const float* rgb_f32;  /* H*W*3 float texels (differentiable path), or NULL */
} ugu_gpu_texture;

/* ugu::Mesh's SoA fields (include/ugu/mesh.h:83-98).  Optional arrays may be
 * NULL.  Indices are validated against their arrays on upload. */
typedef struct {
  int32_t num_vertices;
  const float* vertices;        /* V*3 */
  int32_t num_faces;
  const int32_t* vertex_indices;/* F*3 */
  const float* face_normals;    /* F*3 or NULL */
  int32_t num_normals;
  const float* normals;         /* N*3 or NULL */
  const int32_t* normal_indices;/* F*3 or NULL */
  const float* vertex_colors;   /* V*3 or NULL */
  int32_t num_uv;
  const float* uv;              /* T*2 or NULL */
  const int32_t* uv_indices;    /* F*3 or NULL */
  const int32_t* material_ids;  /* F or NULL */
  int32_t num_materials;
  const ugu_gpu_texture* materials;
} ugu_gpu_mesh;

/* The float camera parameters ugu::Rasterizer::Impl::Render reads from a
 * PinholeCamera (rasterizer.cc:118-119; camera.h:317-331, 380-387, 438-448),
 * computed on the host exactly as the reference does:
 *   w2c_R = camera->w2c().rotation().cast<float>()      (row-major)
 *   w2c_t = camera->w2c().translation().cast<float>()
 *   c2w_R = camera->c2w().matrix().block<3,3>(0,0).cast<float>() (row-major)
 *   c2w_t = camera->c2w().matrix().block<3,1>(0,3).cast<float>() (camera.h:322:
 *           the raytracer's ray origin, org_ray_w)
 *   fx, fy = focal_length(); cx, cy = principal_point(). */
typedef struct {
  int32_t width, height;
  float fx, fy, cx, cy;
  float w2c_R[9];
  float w2c_t[3];
  float c2w_R[9];
  float c2w_t[3];
} ugu_gpu_camera;

/* Output images of one view; NULL skips an output (Render's nullptr rule,
 * renderer.h:60-63).  color_f32 (H*W*3 float, unquantised colour) is an
 * extension used by the differentiable path. */
typedef struct {
  uint8_t* color;
  float* depth;
  float* normal;
  uint8_t* mask;
  int32_t* face_id;
  float* color_f32;
} ugu_gpu_images;

typedef struct {
  int32_t mesh; /* mesh slot set by ugu_gpu_set_mesh */
  ugu_gpu_camera camera;
  ugu_gpu_images images;
} ugu_gpu_view;

/* Flags for ugu_gpu_render_views / ugu_gpu_plan_create. */
enum {
  UGU_GPU_DEVICE_POINTERS = 1u << 0, /* images are device pointers (else host) */
  UGU_GPU_PER_VIEW = 1u << 1,        /* one launch sequence per view (baseline) */
  UGU_GPU_ASYNC = 1u << 2,           /* do not synchronise (device pointers only); on the
                                        tiled path the first such render of a view list
                                        runs a sizing pass first (synchronous, as
                                        ugu_gpu_plan_create does); its status comes from
                                        the next ugu_gpu_synchronize */
  UGU_GPU_TIME_KERNELS = 1u << 3,    /* time the per-tile raster kernel with CUDA events
                                        (ugu_gpu_stats.tile_kernel_ms); not with ASYNC */
  UGU_GPU_RAYTRACE = 1u << 4         /* render with ugu::Raytracer's semantics
                                        (src/renderer/cpu/raytracer.cc:127-224: naive BVH,
                                        nearest double-precision ray hit) instead of
                                        ugu::Rasterizer's */
};

/* The image helpers ugu's examples apply to a render
 * (examples/ex02_renderer.cc:146-154), in one device pass per item:
 *   vis_depth   = Depth2Gray(depth, min_d, max_d)   src/util/image_util.cc:392-411
 *   vis_normal  = Normal2Color(normal, gl_coord)    image_util.cc:413-446 (RGB order)
 *   vis_face_id = FaceId2RandomColor(face_id)       image_util.cc:448-487 (RGB order)
 *   depth_u16   = ConvertTo<uint16_t>(depth)        include/ugu/image_proc.h:453-...
 * An output is written when it and its input are non-NULL.  Depth2Gray's
 * defaults are min_d = 200, max_d = 1500. */
typedef struct {
  int32_t width, height;
  const float* depth;      /* H*W */
  const float* normal;     /* H*W*3 */
  const int32_t* face_id;  /* H*W */
  uint8_t* vis_depth;      /* H*W */
  uint16_t* depth_u16;     /* H*W */
  uint8_t* vis_normal;     /* H*W*3 */
  uint8_t* vis_face_id;    /* H*W*3 */
  float min_d, max_d;
  int32_t gl_coord;
} ugu_gpu_vis;

/* G-buffer channels of a render, the layout of ugu::GBuffer
 * (include/ugu/renderer/base.h:34-77) as RendererGl reads it back
 * (src/renderer/gl/renderer.cc:541-646), computed from the rasterizer's own
 * interpolation at each pixel of the face a render reported (face_id, an
 * input).  With w the pixel's perspective-correct weights (rasterizer.cc:
 * 208-224) and (u, v) = (w1, w2):
 *   pos_wld    = w0 P0 + w1 P1 + w2 P2           pos_cam    = w2c_t + w2c_R pos_wld
 *   normal_wld = normalize(shading normal)       normal_cam = w2c_R normal_wld
 *   bary       = (u, v, 1 - u - v)               uv = (t, s, 1 - t - s), the
 *                                                  texture coordinate (zeros without uv)
 *   stencil    = 255 where face_id >= 0.
 * Pixels with face_id < 0 get zeros.  Any output may be NULL. */
typedef struct {
  int32_t mesh;
  ugu_gpu_camera camera;
  const int32_t* face_id;  /* H*W, input */
  float* pos_wld;          /* H*W*3 */
  float* pos_cam;          /* H*W*3 */
  float* normal_wld;       /* H*W*3 */
  float* normal_cam;       /* H*W*3 */
  float* bary;             /* H*W*3 */
  float* uv;               /* H*W*3 */
  uint8_t* stencil;        /* H*W */
} ugu_gpu_gbuffer;

/* ugu::VisibilityTester (include/ugu/texturing/visibility_tester.h:216-265,
 * src/texturing/visibility_tester.cc): the per-keyframe vertex test
 * TestVertex (:416-529) for every (keyframe, vertex), or facewise
 * (:606-668) for every (keyframe, face corner) with the vertex moved 1e-3 of
 * the way to its face's centre.  The ray casts go through the tester's own
 * naive BVH (leaves of up to 5 faces, :285-294) over the mesh slot's
 * vertices and faces.  Keyframe images are host or device buffers per the
 * UGU_GPU_DEVICE_POINTERS flag, like the outputs. */
typedef struct {
  int32_t id;                 /* Keyframe::id */
  ugu_gpu_camera camera;      /* pinhole; c2w_R / c2w_t give the rays */
  float w2c_linear[9];        /* camera->w2c().cast<float>() linear part, row-major
                                 (TestVertex transforms with it, :422) */
  const uint8_t* color;       /* H*W*3 RGB8 */
  const float* depth;         /* H*W, needed with use_depth */
  const uint8_t* mask;        /* H*W, needed with use_mask */
} ugu_gpu_keyframe;

/* VisibilityTesterOption (visibility_tester.h:38-58). */
typedef struct {
  float backface_culling_angle_rad_th;
  int32_t use_mask, use_depth;
  int32_t interp;  /* 0 kNn, 1 kBilinear */
  float max_viewing_angle;
  float max_distance_from_camera_to_vertex;
  float max_depth_difference;
  float eps;
} ugu_gpu_visibility_option;

/* Per (keyframe, item) results, keyframe-major: item = vertex, or 3 *
 * face + corner when facewise.  VertexInfoPerKeyframe's fields
 * (visibility_tester.h:60-72); meaningful where visible is 1. */
typedef struct {
  uint8_t* visible;
  float* projected_pos;  /* 2 floats */
  float* viewing_angle;
  float* distance;       /* along the ray; FLT_MAX when the ray hit nothing */
  float* color;          /* 3 floats */
  float* intensity;
} ugu_gpu_visibility_out;

/* TextureMappingOption (include/ugu/texturing/texture_mapper.h:22-30)
 * fields of the kSimpleProjection / kUseOriginalMeshUv path. */
typedef struct {
  int32_t tex_w, tex_h;     /* texture size (1024 x 1024) */
  int32_t padding_kernel;   /* PaddingSimple's window (3) */
} ugu_gpu_texture_option;

/* GPU tunables (no reference counterpart; chosen by ugu_gpu_autotune).  A
 * new context starts on the tiled path with tile_log2 5, split_class 256,
 * bin_faces 4 and small_view_pixels 307200 (640 x 480). */
typedef struct {
  int32_t path;             /* UGU_GPU_PATH_TILED (default) or UGU_GPU_PATH_GLOBAL */
  int32_t tile_log2;        /* screen tile edge = 1 << tile_log2 pixels (4 or 5) */
  int32_t entry_capacity;   /* tiled: initial (face, tile) entry buffer, 0 = automatic;
                               grown to what a render reports it needs */
  int32_t small_bbox_max;   /* global: faces with larger bboxes are split by tile */
  int32_t group_pixels;     /* global: pixels of z-buffer kept live per view group */
  int32_t ctas_per_sm;      /* persistent-kernel blocks per SM (0 = occupancy limit) */
  int32_t split_class;      /* tiled: a draw class of at most this many (face, tile)
                               entries is shared out evenly over a tile's warps
                               (0 = 64; 1 = never) */
  int32_t bin_faces;        /* tiled binning: faces per thread of the counting and
                               placing passes (1, 2 or 4; 0 = 2) */
  int32_t small_view_pixels; /* tiled: views of at most this many pixels use 16-pixel
                               tiles whatever tile_log2 says (0 = none) */
} ugu_gpu_tuning;

enum {
  UGU_GPU_PATH_TILED = 0,  /* bin faces to tiles, rasterise + resolve each tile on chip */
  UGU_GPU_PATH_GLOBAL = 1  /* global 64-bit z-buffer per view group, then resolve */
};

typedef struct {
  uint64_t launches;            /* kernels launched by this context so far */
  uint64_t special_candidates;  /* covered samples with depth < FLT_MIN or NaN */
  uint64_t large_face_tiles;    /* (face, tile) items of the last render */
  uint64_t device_bytes;        /* scratch + mesh bytes held on the device */
  double tile_kernel_ms;        /* summed device time of timed tile-kernel launches */
  uint64_t tile_kernel_launches; /* launches timed (UGU_GPU_TIME_KERNELS renders) */
} ugu_gpu_stats;

/* --- texture mapping ---------------------------------------------------- */
/* TextureMapping (src/texturing/texture_mapper.cc:1009-1017) with
 * kSimpleProjection and kUseOriginalMeshUv (:294-345): a tex_h x tex_w RGB8
 * texture and its mask (255 where written) on the uv of mesh slot `mesh`.
 * face_kf[f] is the id of face f's best keyframe, chosen on the host from
 * the VisibilityInfo (:924-970), -1 for none; like the reference, the id
 * indexes `keyframes` (only their camera width/height and colour are read).
 * face_tri[6 f] is the face's projected triangle in that keyframe.  Faces
 * are drawn in order (a later face overwrites an earlier one) and then
 * padded (PaddingSimple, :148-201).  With UGU_GPU_DEVICE_POINTERS the
 * images, face arrays and outputs are device pointers; otherwise host. */
UGU_GPU_API int ugu_gpu_texture_mapping(ugu_gpu_context* ctx, int32_t mesh, int32_t n,
                                        const ugu_gpu_keyframe* keyframes,
                                        const int32_t* face_kf, const float* face_tri,
                                        const ugu_gpu_texture_option* option,
                                        uint8_t* texture, uint8_t* mask, uint32_t flags);

/* TextureMapping with kGenerateSimpleTriangles
 * (GenerateSimpleTrianglesTextureAndUv, texture_mapper.cc:347-440): as
 * ugu_gpu_texture_mapping, but face f is drawn into the triangle
 * face_target[6 f .. 6 f + 5] (texel coordinates) of the caller's layout
 * instead of its uv triangle; the layout and the output uv are the host's
 * (the reference pads with a 3-texel window: padding_kernel 3). */
UGU_GPU_API int ugu_gpu_texture_mapping_targets(ugu_gpu_context* ctx, int32_t num_faces,
                                                const float* face_target, int32_t n,
                                                const ugu_gpu_keyframe* keyframes,
                                                const int32_t* face_kf, const float* face_tri,
                                                const ugu_gpu_texture_option* option,
                                                uint8_t* texture, uint8_t* mask, uint32_t flags);

/* MakeTiledImage (texture_mapper.cc:29-60), the texture of
 * kGenerateSimpleTile: keyframe image i copied to tile (i % x_tiles,
 * i / x_tiles) of an RGB8 texture x_tiles images wide and n / x_tiles
 * high.  Every image must have the first one's size and the n images must
 * fill whole rows of tiles (the reference writes past its texture
 * otherwise); UGU_GPU_ERR_INVALID_ARGUMENT else.  Images and texture are
 * device pointers with UGU_GPU_DEVICE_POINTERS, else host. */
UGU_GPU_API int ugu_gpu_tile_images(ugu_gpu_context* ctx, int32_t n,
                                    const ugu_gpu_keyframe* keyframes, int32_t x_tiles,
                                    uint8_t* texture, uint32_t flags);

/* --- context ------------------------------------------------------------ */
UGU_GPU_API int ugu_gpu_create(int32_t device, ugu_gpu_context** out);
UGU_GPU_API int ugu_gpu_destroy(ugu_gpu_context* ctx);
UGU_GPU_API const char* ugu_gpu_last_error(const ugu_gpu_context* ctx);
UGU_GPU_API int ugu_gpu_abi_version(void);

/* Rasterizer::set_option (rasterizer.cc:73-75).  Like RendererCpuOption::
 * CopyTo (renderer.h:30-37) the host class passes the sigma it holds. */
UGU_GPU_API int ugu_gpu_set_option(ugu_gpu_context* ctx, const ugu_gpu_option* opt);

/* Rasterizer::set_mesh + PrepareMesh (rasterizer.cc:77-99): validates and
 * uploads the mesh into `slot` (0 <= slot < 16).  A NULL mesh empties it. */
UGU_GPU_API int ugu_gpu_set_mesh(ugu_gpu_context* ctx, int32_t slot, const ugu_gpu_mesh* mesh);

/* Rasterizer::Render (rasterizer.cc:105-307) for one view, host buffers,
 * synchronous: outputs are valid on return. */
UGU_GPU_API int ugu_gpu_render(ugu_gpu_context* ctx, int32_t mesh, const ugu_gpu_camera* cam,
                   const ugu_gpu_images* images);

/* Many views (several meshes, uneven resolutions) in one batched launch
 * sequence; see the UGU_GPU_* flags. */
UGU_GPU_API int ugu_gpu_render_views(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_view* views,
                         uint32_t flags);

/* Capture the batched render of `views` (device pointers) into a CUDA graph;
 * ugu_gpu_plan_launch replays it on the context's stream. */
UGU_GPU_API int ugu_gpu_plan_create(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_view* views,
                        uint32_t flags, ugu_gpu_plan** out);
UGU_GPU_API int ugu_gpu_plan_launch(ugu_gpu_plan* plan);
/* Also done by ugu_gpu_destroy for the plans of the context still alive:
 * a plan must not be used or destroyed after its context. */
UGU_GPU_API int ugu_gpu_plan_destroy(ugu_gpu_plan* plan);

/* Backward of the per-pixel L2 loss sum_p |C(p) - T(p)|^2 over pixels with
 * face_id > 0, where C is the unquantised colour of the forward (float
 * texels of material 0, bilinear; or vertex colours), visibility held fixed
 * at the forward's face_id images (views[i].images.face_id, device memory).
 * targets[i] is an H*W*3 float device image.  Gradients are accumulated (+=)
 * into the device buffers grad_texels (material 0, H*W*3), grad_vertex_colors
 * (V*3) and grad_vertices (V*3), any of which may be NULL.  loss_out (device,
 * one float per view) receives the per-view loss when non-NULL. */
UGU_GPU_API int ugu_gpu_backward(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_view* views,
                     const float* const* targets, float* grad_texels,
                     float* grad_vertex_colors, float* grad_vertices, float* loss_out,
                     uint32_t flags);

UGU_GPU_API int ugu_gpu_set_tuning(ugu_gpu_context* ctx, const ugu_gpu_tuning* tuning);
UGU_GPU_API int ugu_gpu_get_tuning(const ugu_gpu_context* ctx, ugu_gpu_tuning* tuning);
/* Times candidate tunings on the given views (device pointers) and keeps the
 * fastest: the path and tile size, then the size below which views use
 * 16-pixel tiles, the persistent grid's blocks per SM and the draw and
 * binning settings (split_class, bin_faces), or
 * the global path's small_bbox_max and group_pixels; every candidate gives
 * the same images.  The result is cached per workload shape (view sizes,
 * meshes, options), so a repeated call returns at once; when the
 * environment variable UGU_GPU_TUNING_CACHE names a file, results are also
 * read from and appended to it. */
UGU_GPU_API int ugu_gpu_autotune(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_view* views,
                     ugu_gpu_tuning* chosen);

UGU_GPU_API int ugu_gpu_get_stats(const ugu_gpu_context* ctx, ugu_gpu_stats* stats);

/* The helpers of ugu_gpu_vis for n items; UGU_GPU_DEVICE_POINTERS for device
 * buffers (else host buffers, staged through the device); synchronous. */
UGU_GPU_API int ugu_gpu_visualize(ugu_gpu_context* ctx, int32_t n, const ugu_gpu_vis* items,
                                  uint32_t flags);

/* The G-buffer channels of n views (ugu_gpu_gbuffer) with the context's
 * option (shading normal); UGU_GPU_DEVICE_POINTERS for device buffers (else
 * host, staged); synchronous.  A face id outside [-1, num_faces) is an
 * error (UGU_GPU_ERR_INDEX_OUT_OF_RANGE), its pixel left at zeros. */
UGU_GPU_API int ugu_gpu_render_gbuffer(ugu_gpu_context* ctx, int32_t n,
                                       const ugu_gpu_gbuffer* views, uint32_t flags);

/* VisibilityTester::Test (visibility_tester.cc:670-731) for the mesh in
 * `mesh` with per-vertex `normals` (V*3, the tester's own normals, host
 * memory) against n keyframes; facewise selects TestFacewiseVertices.  The
 * statistics (CalcStat) are left to the caller.  Synchronous. */
UGU_GPU_API int ugu_gpu_test_visibility(ugu_gpu_context* ctx, int32_t mesh, const float* normals,
                                        int32_t n, const ugu_gpu_keyframe* keyframes,
                                        const ugu_gpu_visibility_option* option,
                                        int32_t facewise, const ugu_gpu_visibility_out* out,
                                        uint32_t flags);
/* Waits for the context's stream, then reports what the asynchronous renders
 * and plan replays since the last call left: UGU_GPU_ERR_CAPACITY when a
 * (face, tile) list overflowed (those images are not valid; render again,
 * the lists have grown), UGU_GPU_ERR_DEGENERATE_DEPTH for a covered sample
 * with depth < FLT_MIN or NaN. */
UGU_GPU_API int ugu_gpu_synchronize(ugu_gpu_context* ctx);
/* Use a caller-owned cudaStream_t (NULL restores the context's own stream). */
UGU_GPU_API int ugu_gpu_set_stream(ugu_gpu_context* ctx, void* stream);

/* --- rendering without allocating ---------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: a plug-in whose host application owns all device memory and hands
 * out only finished buffers; code held to a fixed device-memory budget by
 * another allocator, where one more cudaMalloc would fail or fragment its
 * pool; a frame loop that cannot take the device synchronisation cudaMalloc
 * and cudaFree may cause.  ugu_gpu_render_noalloc renders one view with the
 * global-z-buffer kernels, allocates nothing (no cudaMalloc, no cudaFree, no
 * allocating library call) and needs no context: the mesh and the output
 * images are the caller's device buffers, and the scratch (z-buffer,
 * descriptors, counters, large-face tile list) is a static device array of
 * about 20 MB that every GPU loading this library keeps until the process
 * exits.
 *
 * Limits: width * height <= UGU_GPU_NOALLOC_MAX_PIXELS, at most
 * UGU_GPU_NOALLOC_MAX_MATERIALS materials; larger requests return
 * UGU_GPU_ERR_CAPACITY before any work.  Faces whose screen box exceeds 256
 * pixels are drawn as (face, 16x16 tile) items, at most
 * UGU_GPU_NOALLOC_MAX_ITEMS per call (about 32 full-screen faces at
 * 1920x1080); past that the call returns UGU_GPU_ERR_CAPACITY after the
 * kernels ran, and the images are then not valid.  The mesh arrays must be
 * in the 4-wide layout below (16-byte aligned) with in-range indices:
 * device-resident indices are not checked.  Face normals are required
 * whenever the mesh has faces: the reference's z pass reads them at every
 * pixel of every face (rasterizer.cc:199).  The first call on a device
 * looks up the array's device address for that device and keeps it for the
 * life of the process; do not cudaDeviceReset a device while this library
 * is in use there (the kept address would be stale).  All calls share the array and it keeps
 * the last call's contents (each call clears what it needs first), so
 * calls whose GPU work overlaps -- on different streams or from different
 * host threads -- race and must be serialised by the caller.  Runs on the
 * current device and on `stream` (NULL = default stream) and is
 * synchronous: it returns when the images are written.  Errors are
 * reported in ugu_gpu_last_error(NULL). */
#define UGU_GPU_NOALLOC_MAX_PIXELS 2097152 /* e.g. 1920 x 1080 */
#define UGU_GPU_NOALLOC_MAX_MATERIALS 16
#define UGU_GPU_NOALLOC_MAX_ITEMS 262144

typedef struct {
  int32_t width, height;
  const uint32_t* rgba8; /* device, H*W texels r | g << 8 | b << 16, or NULL */
  const float* rgb_f32;  /* device, H*W*3, or NULL */
} ugu_gpu_device_texture;

typedef struct {
  int32_t num_vertices, num_faces, num_normals, num_uv, num_materials;
  const float* vertices4;          /* device, V*4: x, y, z, unused */
  const int32_t* vertex_indices4;  /* device, F*4: i0, i1, i2, unused */
  const float* face_normals4;      /* device, F*4 */
  const float* normals4;           /* device, N*4, or NULL */
  const int32_t* normal_indices4;  /* device, F*4, or NULL */
  const float* vertex_colors4;     /* device, V*4, or NULL */
  const float* uv2;                /* device, T*2, or NULL */
  const int32_t* uv_indices4;      /* device, F*4, or NULL */
  const int32_t* material_ids;     /* device, F, or NULL */
  const ugu_gpu_device_texture* materials; /* host array of num_materials */
} ugu_gpu_device_mesh;

/* Device arrays of a mesh slot in the layout above (pointers owned by the
 * context, valid until the slot is set again).  Lets a caller update the
 * uploaded parameters in place, e.g. a gradient step on the float texels.
 * Values (positions, normals, colours, uvs, texels) may change in place;
 * the index arrays may not (the slot keeps derived copies of them): upload
 * new connectivity with ugu_gpu_set_mesh.  No counterpart in the
 * reference. */
UGU_GPU_API int ugu_gpu_get_device_mesh(ugu_gpu_context* ctx, int32_t slot,
                                        ugu_gpu_device_mesh* out);

UGU_GPU_API int ugu_gpu_render_noalloc(const ugu_gpu_device_mesh* mesh,
                                       const ugu_gpu_option* opt,
                                       const ugu_gpu_camera* cam,
                                       const ugu_gpu_images* images, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* UGU_GPU_H_ */
