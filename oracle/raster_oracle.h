/*
 * raster_oracle.h -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C, single-threaded restatement of ugu's CPU rasterizer forward path
 * (ugu::Rasterizer::Impl::Render, src/renderer/cpu/rasterizer.cc:105-307, and
 * the pixel shaders in include/ugu/renderer/cpu/pixel_shader.h:215-422), plus an
 * FP64 recomputation of the interpolated outputs and an FP64 analytic gradient
 * of the per-pixel L2 colour loss.  It is the checker for the GPU kernels:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 * Nothing in the product links or calls this code.
 *
 * Floating-point contract (shared with the CUDA kernels): IEEE binary32, no
 * contraction (built with -ffp-contract=off), correctly rounded / and sqrt, and
 * every 3-term sum of a dot product or matrix-vector row associated as
 * a0 + (a1 + a2) -- the order of Eigen's unrolled size-3 reduction on x86-64.
 */
#ifndef UGU_RASTER_ORACLE_H_
#define UGU_RASTER_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int32_t width;
  int32_t height;
  const uint8_t* data; /* HWC, RGB8, row-major (ugu::Image3b layout) */
} oracle_texture;

typedef struct {
  int32_t num_vertices;
  const float* vertices; /* V x 3 */
  int32_t num_faces;
  const int32_t* vertex_indices; /* F x 3 */
  int32_t num_face_normals;
  const float* face_normals; /* F x 3 */
  int32_t num_normals;
  const float* normals; /* N x 3 */
  int32_t num_normal_indices;
  const int32_t* normal_indices; /* F x 3 */
  int32_t num_vertex_colors;
  const float* vertex_colors; /* V x 3 */
  int32_t num_uv;
  const float* uv; /* T x 2 */
  int32_t num_uv_indices;
  const int32_t* uv_indices; /* F x 3 */
  int32_t num_material_ids;
  const int32_t* material_ids; /* F */
  int32_t num_materials;
  const oracle_texture* textures; /* one diffuse texture per material */
  /* Float RGB textures (differentiable path only; no reference counterpart). */
  const float* const* textures_f32; /* per material: H x W x 3 float, or NULL */
} oracle_mesh;

typedef struct {
  int32_t width;
  int32_t height;
  float fx, fy, cx, cy;
  float w2c_R[9]; /* row-major, = camera->w2c().rotation().cast<float>() */
  float w2c_t[3]; /* = camera->w2c().translation().cast<float>() */
  float c2w_R[9]; /* row-major, = c2w block<3,3> cast to float */
  float c2w_t[3]; /* = c2w block<3,1>(0,3) cast to float (camera.h:322), the
                     raytracer's ray origin */
} oracle_camera;

typedef struct {
  int32_t diffuse_color;   /* 0 none, 1 texture, 2 vertex */
  int32_t interp;          /* 0 nearest, 1 bilinear */
  int32_t shading_normal;  /* 0 face, 1 vertex */
  int32_t diffuse_shading; /* 0 none, 1 Lambertian, 2 Oren-Nayar */
  int32_t backface_culling;
  float oren_nayar_sigma;
} oracle_option;

typedef struct {
  int64_t bbox_pixels;       /* pixel tests in the z pass */
  int64_t covered;           /* candidates that passed the edge test */
  int64_t special_candidates;/* candidates with z < FLT_MIN or NaN */
  int64_t texel_clamps;      /* texel reads that left the texture allocation */
} oracle_stats;

/* Return codes mirror ValidateAndInitBeforeRender's failure cases
 * (src/renderer/cpu/util_private.cc:19-67). */
enum {
  ORACLE_OK = 0,
  ORACLE_ERR_NO_FACE_NORMALS_FOR_CULLING = 3,
  ORACLE_ERR_NO_TEXTURE = 4,
  ORACLE_ERR_EMPTY_TEXTURE = 5,
  ORACLE_ERR_NO_VERTEX_COLORS = 6,
  ORACLE_ERR_NO_FACE_NORMALS_FOR_SHADING = 7,
  ORACLE_ERR_NO_VERTEX_NORMALS = 8,
  ORACLE_ERR_NO_OUTPUT = 9,
  ORACLE_ERR_ALLOC = 20
};

/* The forward render.  Any output may be NULL.  color: H*W*3 u8, depth: H*W
 * f32, normal: H*W*3 f32, mask: H*W u8, face_id: H*W i32.  If color_f32 is
 * non-NULL (float-texture / float-vertex-colour path, no reference
 * counterpart) the unquantised RGB colour is written there too. */
int oracle_render(const oracle_mesh* mesh, const oracle_camera* cam,
                  const oracle_option* opt, uint8_t* color, float* depth,
                  float* normal, uint8_t* mask, int32_t* face_id,
                  float* color_f32, oracle_stats* stats);

/* ugu::Raytracer::Impl::Render (src/renderer/cpu/raytracer.cc:127-224):
 * one ray per pixel through the naive BVH (ray_oracle.cc), nearest hit,
 * back faces culled after the search, depth scaled by depth_scale.
 * sort_dependent (H*W, or NULL) marks the pixels whose reported face the
 * reference's std::sort decides among equal distances (ray_oracle.cc). */
int oracle_raytrace(const oracle_mesh* mesh, const oracle_camera* cam,
                    const oracle_option* opt, float depth_scale, uint8_t* color,
                    float* depth, float* normal, uint8_t* mask, int32_t* face_id,
                    float* color_f32, uint8_t* sort_dependent);

/* The G-buffer channels (include/ugu_gpu.h, ugu_gpu_gbuffer) of the faces a
 * render reported: the rasterizer's perspective-correct weights at each
 * pixel (rasterizer.cc:201-224) applied to positions, the shading normal
 * (normalised) and the texture coordinates; the layout of ugu::GBuffer
 * (include/ugu/renderer/base.h:34-77) as src/renderer/gl/renderer.cc:541-646
 * fills it.  Returns the number of face ids outside [-1, F). */
int64_t oracle_gbuffer(const oracle_mesh* mesh, const oracle_camera* cam,
                       const oracle_option* opt, const int32_t* face_id, float* pos_wld,
                       float* pos_cam, float* normal_wld, float* normal_cam, float* bary,
                       float* uv, uint8_t* stencil);

/* ugu::Keyframe (visibility_tester.h:196-212) and VisibilityTesterOption
 * (:38-58) as the visibility test reads them; L = w2c().cast<float>()'s
 * linear part, row-major. */
typedef struct {
  int32_t id;
  oracle_camera cam;
  float L[9];
  const uint8_t* color;
  const float* depth;
  const uint8_t* mask;
} oracle_keyframe;

typedef struct {
  float backface_th;
  int32_t use_mask, use_depth, interp;
  float max_viewing_angle, max_distance, max_depth_difference, eps;
} oracle_vis_option;

void oracle_test_visibility(const float* V, int32_t nv, const int32_t* F, int32_t nf,
                            const float* N, int32_t n_kf, const oracle_keyframe* kfs,
                            const oracle_vis_option* o, int32_t facewise, uint8_t* visible,
                            float* proj, float* angle, float* dist, float* color,
                            float* intensity);

/* ray_oracle.cc: ugu::BvhNaive over the mesh (NULL when it has no face) and
 * its nearest hit along a ray (1 and t, u, v, face, or 0). */
void* oracle_bvh_build(const float* vertices, int32_t num_faces, const int32_t* faces);
void oracle_bvh_free(void* bvh);
int oracle_bvh_nearest(const void* bvh, const float* org, const float* dir, float* t,
                       float* u, float* v, int32_t* fid, int32_t* sort_dependent);

/* The camera ray the reference tabulates (camera.h:438-448, 482-513). */
void oracle_ray_w(const oracle_camera* cam, int32_t x, int32_t y, float out[3]);

/* FP64 recomputation of depth, camera-frame normal and pre-quantisation colour
 * for every pixel whose final face id is >= 0 (depth) / > 0 (normal, colour),
 * given the FP32 face_id image.  Outputs are double arrays (may be NULL). */
void oracle_interp_f64(const oracle_mesh* mesh, const oracle_camera* cam,
                       const oracle_option* opt, const int32_t* face_id,
                       double* depth, double* normal, double* color);

/* One parameter moved by `delta` (in double) inside the FP64 path, for
 * finite differences: kind 1 = texel of material 0 (flat index into
 * H*W*3), 2 = vertex colour (V*3), 3 = vertex position (V*3). */
typedef struct {
  int32_t kind;
  int64_t index;
  double delta;
} oracle_perturb;

/* FP64 analytic gradient of L = sum over pixels with face_id > 0 of
 * |C(p) - T(p)|^2 where C is the float colour of the differentiable path
 * (float RGB texture, bilinear; or float vertex colours), visibility held
 * fixed at the given face_id image.  Gradients are ACCUMULATED (+=) into the
 * double buffers (any may be NULL): grad_tex (material 0, H*W*3),
 * grad_vcolor (V*3), grad_vpos (V*3).  Returns the loss. */
double oracle_backward_f64(const oracle_mesh* mesh, const oracle_camera* cam,
                           const oracle_option* opt, const int32_t* face_id,
                           const float* target, double* grad_tex,
                           double* grad_vcolor, double* grad_vpos,
                           const oracle_perturb* perturb);

/* Mesh::CalcFaceNormal / Mesh::CalcNormal (src/mesh.cc:297-349). */
void oracle_calc_normals(int32_t num_vertices, const float* vertices,
                         int32_t num_faces, const int32_t* vertex_indices,
                         float* face_normals, float* normals);

#ifdef __cplusplus
}
#endif

#endif /* UGU_RASTER_ORACLE_H_ */
