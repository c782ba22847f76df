/*
 * raster_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * CPU restatement of ugu's software rasterizer, used to check the CUDA
 * kernels.  Each function names the reference lines it restates.  Build with
 * -O2 -ffp-contract=off (no FMA contraction) so every float operation rounds
 * exactly once, in the order written here.
 *
 * Where the reference's behaviour is undefined in C++ the oracle picks the
 * behaviour the GB300 host (aarch64) and CUDA's cvt instructions both give:
 *   - float -> int32 casts saturate and map NaN to 0 (rasterizer.cc:185-188,
 *     pixel_shader.h:286-287, 329-330);
 *   - float -> uint8 casts keep the low byte of that saturated int32
 *     (pixel_shader.h:254, 296, 357, 386, 420);
 *   - texel reads use the reference's linear address y*cols + x
 *     (image.h:416-427) and are clamped to the texture allocation only when
 *     that address falls outside it (the reference reads out of bounds there).
 */
#include "raster_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Eigen's unrolled size-3 reduction (dot, squaredNorm, one row of a 3x3
 * matrix-vector product) as compiled on x86-64: a0 + (a1 + a2). */
#define SUM3(a0, a1, a2) ((a0) + ((a1) + (a2)))

static int32_t f2i_sat(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f < -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}

static uint8_t f2u8(float f) { return (uint8_t)(uint32_t)f2i_sat(f); }

/* rasterizer.cc:25-28 */
static float edge_fn(float ax, float ay, float bx, float by, float cx,
                     float cy) {
  return (cx - ax) * (by - ay) - (cy - ay) * (bx - ax);
}

/* std::min({a,b,c}) / std::max({a,b,c}) as min_element / max_element
 * evaluate them (first element kept on ties, NaN handling included). */
static float min3_std(float a, float b, float c) {
  float m = a;
  if (b < m) m = b;
  if (c < m) m = c;
  return m;
}
static float max3_std(float a, float b, float c) {
  float m = a;
  if (m < b) m = b;
  if (m < c) m = c;
  return m;
}

/* 3x3 row-major matrix times vector, one SUM3 per row. */
static void matvec3(const float* M, const float* v, float* out) {
  float r0 = SUM3(M[0] * v[0], M[1] * v[1], M[2] * v[2]);
  float r1 = SUM3(M[3] * v[0], M[4] * v[1], M[5] * v[2]);
  float r2 = SUM3(M[6] * v[0], M[7] * v[1], M[8] * v[2]);
  out[0] = r0;
  out[1] = r1;
  out[2] = r2;
}

static float dot3(const float* a, const float* b) {
  return SUM3(a[0] * b[0], a[1] * b[1], a[2] * b[2]);
}

/* PinholeCamera::ray_c(float,float) + ray_w(float,float)
 * (camera.h:438-448): d = ((x-cx)/fx, (y-cy)/fy, 1); d.normalize();
 * ray_w = c2w_R_f * d.  The reference tabulates it per pixel
 * (InitRayTable, camera.h:482-513); the value is the same. */
void oracle_ray_w(const oracle_camera* cam, int32_t x, int32_t y,
                  float out[3]) {
  float d[3];
  d[0] = ((float)x - cam->cx) / cam->fx;
  d[1] = ((float)y - cam->cy) / cam->fy;
  d[2] = 1.0f;
  float n2 = SUM3(d[0] * d[0], d[1] * d[1], d[2] * d[2]);
  if (n2 > 0.0f) {
    float s = sqrtf(n2);
    d[0] = d[0] / s;
    d[1] = d[1] / s;
    d[2] = d[2] / s;
  }
  matvec3(cam->c2w_R, d, out);
}

/* Linear texel address of at<Vec3b>(y, x) (image.h:416-427), clamped to the
 * allocation only when it falls outside it. */
static int64_t texel_index(int64_t y, int64_t x, int32_t cols, int32_t rows,
                           oracle_stats* st) {
  int64_t i = y * (int64_t)cols + x;
  int64_t n = (int64_t)cols * (int64_t)rows;
  if (i < 0 || i >= n) {
    if (st) st->texel_clamps++;
    i = i < 0 ? 0 : n - 1;
  }
  return i;
}

static int validate(const oracle_mesh* m, const oracle_option* o,
                    const void* color, const void* depth, const void* normal,
                    const void* mask, const void* face_id,
                    const void* color_f32) {
  /* util_private.cc:27-67, in the same order. */
  if (o->backface_culling && m->num_face_normals == 0)
    return ORACLE_ERR_NO_FACE_NORMALS_FOR_CULLING;
  if (o->diffuse_color == 1 && m->num_materials == 0)
    return ORACLE_ERR_NO_TEXTURE;
  if (o->diffuse_color == 1) {
    for (int i = 0; i < m->num_materials; i++) {
      const oracle_texture* t = &m->textures[i];
      int has_f32 = m->textures_f32 && m->textures_f32[i];
      if ((t->width < 1 || t->height < 1) || (!t->data && !has_f32))
        return ORACLE_ERR_EMPTY_TEXTURE;
    }
  }
  if (o->diffuse_color == 2 && m->num_vertex_colors == 0)
    return ORACLE_ERR_NO_VERTEX_COLORS;
  if (o->shading_normal == 0 && m->num_face_normals == 0)
    return ORACLE_ERR_NO_FACE_NORMALS_FOR_SHADING;
  if (o->shading_normal == 1 && m->num_normals == 0)
    return ORACLE_ERR_NO_VERTEX_NORMALS;
  if (!color && !depth && !normal && !mask && !face_id && !color_f32)
    return ORACLE_ERR_NO_OUTPUT;
  return ORACLE_OK;
}

/* Barycentric colour/uv weights of the pixel shaders use (1 - u - v), u, v
 * with u = w1, v = w2 (pixel_shader.h:248-250, 277-279, 320-322). */
static void shade_color(const oracle_mesh* m, const oracle_option* o, int fid,
                        float u, float v, const float* ray_w,
                        const float* shading_normal_w, float on_A, float on_B,
                        uint8_t* c, float* cf, oracle_stats* st) {
  float s = 1.0f - u - v;
  float col[3] = {255.0f, 255.0f, 255.0f};
  if (o->diffuse_color == 2) {
    /* DiffuseVertexColorColorizer::Process, pixel_shader.h:234-256 */
    const int32_t* f = &m->vertex_indices[3 * fid];
    const float* c0 = &m->vertex_colors[3 * f[0]];
    const float* c1 = &m->vertex_colors[3 * f[1]];
    const float* c2 = &m->vertex_colors[3 * f[2]];
    for (int k = 0; k < 3; k++) col[k] = (s * c0[k] + u * c1[k]) + v * c2[k];
    for (int k = 0; k < 3; k++) c[k] = f2u8(col[k]);
  } else if (o->diffuse_color == 1) {
    int mid = m->material_ids[fid];
    const oracle_texture* t = &m->textures[mid];
    const float* tf = m->textures_f32 ? m->textures_f32[mid] : NULL;
    const int32_t* f = &m->uv_indices[3 * fid];
    const float* a = &m->uv[2 * f[0]];
    const float* b = &m->uv[2 * f[1]];
    const float* cc = &m->uv[2 * f[2]];
    float uv0 = (s * a[0] + u * b[0]) + v * cc[0];
    float uv1 = (s * a[1] + u * b[1]) + v * cc[1];
    float fx = uv0 * (float)(t->width - 1);
    float fy = (1.0f - uv1) * (float)(t->height - 1);
    if (o->interp == 0) {
      /* DiffuseTextureNnColorizer::Process, pixel_shader.h:260-298 */
      int32_t tx = f2i_sat(roundf(fx));
      int32_t ty = f2i_sat(roundf(fy));
      int64_t i = texel_index(ty, tx, t->width, t->height, st);
      for (int k = 0; k < 3; k++)
        col[k] = tf ? tf[3 * i + k] : (float)t->data[3 * i + k];
      for (int k = 0; k < 3; k++) c[k] = f2u8(col[k]);
    } else {
      /* DiffuseTextureBilinearColorizer::Process, pixel_shader.h:302-359 */
      int32_t x0 = f2i_sat(floorf(fx));
      int32_t y0 = f2i_sat(floorf(fy));
      int64_t x1 = (int64_t)x0 + 1;
      int64_t y1 = (int64_t)y0 + 1;
      float lu = fx - (float)x0;
      float lv = fy - (float)y0;
      int64_t i00 = texel_index(y0, x0, t->width, t->height, st);
      int64_t i10 = texel_index(y0, x1, t->width, t->height, st);
      int64_t i01 = texel_index(y1, x0, t->width, t->height, st);
      int64_t i11 = texel_index(y1, x1, t->width, t->height, st);
      for (int k = 0; k < 3; k++) {
        float t00, t10, t01, t11;
        if (tf) {
          t00 = tf[3 * i00 + k];
          t10 = tf[3 * i10 + k];
          t01 = tf[3 * i01 + k];
          t11 = tf[3 * i11 + k];
        } else {
          t00 = (float)t->data[3 * i00 + k];
          t10 = (float)t->data[3 * i10 + k];
          t01 = (float)t->data[3 * i01 + k];
          t11 = (float)t->data[3 * i11 + k];
        }
        col[k] = (((1.0f - lu) * (1.0f - lv) * t00 + lu * (1.0f - lv) * t10) +
                  (1.0f - lu) * lv * t01) +
                 lu * lv * t11;
      }
      for (int k = 0; k < 3; k++) c[k] = f2u8(col[k]);
    }
  } else {
    /* DiffuseDefaultColorizer::Process, pixel_shader.h:222-230 */
    c[0] = c[1] = c[2] = 255;
  }
  if (cf) {
    cf[0] = col[0];
    cf[1] = col[1];
    cf[2] = col[2];
  }

  if (o->diffuse_shading == 1) {
    /* DiffuseLambertianShader::Process, pixel_shader.h:370-388 */
    float coeff = -dot3(ray_w, shading_normal_w);
    if (coeff < 0.0f) coeff = 0.0f;
    for (int k = 0; k < 3; k++) c[k] = f2u8(coeff * (float)c[k]);
  } else if (o->diffuse_shading == 2) {
    /* DiffuseOrenNayarShader::Process, pixel_shader.h:392-422; the light
     * direction is the view ray (rasterizer.cc:293). */
    const float* n = shading_normal_w;
    const float* l = ray_w;
    float dot_light = -dot3(l, n);
    float theta_i = acosf(dot_light);
    float dot_ray = -dot3(ray_w, n);
    float theta_r = acosf(dot_ray);
    float bl[3], br[3];
    for (int k = 0; k < 3; k++) bl[k] = (-n[k]) * dot_light - l[k];
    for (int k = 0; k < 3; k++) br[k] = (-n[k]) * dot_light - ray_w[k];
    float pdc = dot3(bl, br);
    float phi_diff_cos = (0.0f < pdc) ? pdc : 0.0f;
    float alpha = (theta_i < theta_r) ? theta_r : theta_i;
    float beta = (theta_r < theta_i) ? theta_r : theta_i;
    float dl = (0.0f < dot_light) ? dot_light : 0.0f;
    float coeff = dl * (on_A + (on_B * phi_diff_cos * sinf(alpha) * tanf(beta)));
    for (int k = 0; k < 3; k++) c[k] = f2u8(coeff * (float)c[k]);
  }
}

/* Projected vertex of Loop A (rasterizer.cc:131-136): camera-frame position
 * w2c_R * v + w2c_t, then PinholeCamera::Project (camera.h:380-387):
 * x = fx / z * x + cx, y = fy / z * y + cy, keep z. */
static void project_vertex(const oracle_camera* cam, const float* v,
                           float* out) {
  float c[3];
  matvec3(cam->w2c_R, v, c);
  c[0] = c[0] + cam->w2c_t[0];
  c[1] = c[1] + cam->w2c_t[1];
  c[2] = c[2] + cam->w2c_t[2];
  out[0] = cam->fx / c[2] * c[0] + cam->cx;
  out[1] = cam->fy / c[2] * c[1] + cam->cy;
  out[2] = c[2];
}

int oracle_render(const oracle_mesh* m, const oracle_camera* cam,
                  const oracle_option* o, uint8_t* color, float* depth,
                  float* normal, uint8_t* mask, int32_t* face_id,
                  float* color_f32, oracle_stats* st) {
  int rc = validate(m, o, color, depth, normal, mask, face_id, color_f32);
  if (rc) return rc;
  const int W = cam->width, H = cam->height;
  const size_t npx = (size_t)W * (size_t)H;

  /* ValidateAndInitBeforeRender's Init calls (util_private.cc:72-87) and
   * rasterizer.cc:138-159. */
  float* dep = depth ? depth : (float*)malloc(npx * sizeof(float));
  int32_t* fidimg = face_id ? face_id : (int32_t*)malloc(npx * sizeof(int32_t));
  uint8_t* bfimg = (uint8_t*)calloc(npx ? npx : 1, 1);
  float* wimg = (float*)calloc(npx ? 3 * npx : 1, sizeof(float));
  float* img = (float*)malloc(((size_t)m->num_vertices + 1) * 3 * sizeof(float));
  if (!dep || !fidimg || !bfimg || !wimg || !img) {
    if (!depth) free(dep);
    if (!face_id) free(fidimg);
    free(bfimg);
    free(wimg);
    free(img);
    return ORACLE_ERR_ALLOC;
  }
  for (size_t i = 0; i < npx; i++) {
    dep[i] = 0.0f;
    fidimg[i] = -1;
  }
  if (color) memset(color, 0, 3 * npx);
  if (normal) memset(normal, 0, 3 * npx * sizeof(float));
  if (mask) memset(mask, 0, npx);
  if (color_f32) memset(color_f32, 0, 3 * npx * sizeof(float));

  /* Oren-Nayar constants (pixel_shader.h:143-148). */
  float sigma_2 = o->oren_nayar_sigma * o->oren_nayar_sigma;
  float on_A = 1.0f - (0.5f * sigma_2 / (sigma_2 + 0.33f));
  float on_B = 0.45f * sigma_2 / (sigma_2 + 0.09f);

  /* Loop A (rasterizer.cc:131-136).  camera_normals there is a dead store. */
  for (int i = 0; i < m->num_vertices; i++)
    project_vertex(cam, &m->vertices[3 * i], &img[3 * i]);

  /* Loop B: z-buffer pass in ascending face order (rasterizer.cc:162-241). */
  const float flt_min = FLT_MIN;
  for (int i = 0; i < m->num_faces; i++) {
    const int32_t* f = &m->vertex_indices[3 * i];
    const float* v0 = &img[3 * f[0]];
    const float* v1 = &img[3 * f[1]];
    const float* v2 = &img[3 * f[2]];
    if (v0[2] < 0.0f || v1[2] < 0.0f || v2[2] < 0.0f) continue;
    float xmin = min3_std(v0[0], v1[0], v2[0]);
    float ymin = min3_std(v0[1], v1[1], v2[1]);
    float xmax = max3_std(v0[0], v1[0], v2[0]);
    float ymax = max3_std(v0[1], v1[1], v2[1]);
    if (xmin > (float)(W - 1) || xmax < 0.0f || ymin > (float)(H - 1) ||
        ymax < 0.0f)
      continue;
    int32_t x0 = f2i_sat(ceilf(xmin));
    if (x0 < 0) x0 = 0;
    int32_t x1 = f2i_sat(floorf(xmax));
    if (x1 > W - 1) x1 = W - 1;
    int32_t y0 = f2i_sat(ceilf(ymin));
    if (y0 < 0) y0 = 0;
    int32_t y1 = f2i_sat(floorf(ymax));
    if (y1 > H - 1) y1 = H - 1;
    float area = edge_fn(v0[0], v0[1], v1[0], v1[1], v2[0], v2[1]);
    if (fabsf(area) < flt_min) continue;
    const float* fn = &m->face_normals[3 * i];
    for (int32_t y = y0; y <= y1; ++y) {
      for (int32_t x = x0; x <= x1; ++x) {
        float ray[3];
        oracle_ray_w(cam, x, y, ray);
        int backface = dot3(fn, ray) > 0.0f;
        float px = (float)x, py = (float)y;
        float w0 = edge_fn(v1[0], v1[1], v2[0], v2[1], px, py);
        float w1 = edge_fn(v2[0], v2[1], v0[0], v0[1], px, py);
        float w2 = edge_fn(v0[0], v0[1], v1[0], v1[1], px, py);
        if (st) st->bbox_pixels++;
        if ((!backface && (w0 >= 0 && w1 >= 0 && w2 >= 0)) ||
            (backface && (w0 <= 0 && w1 <= 0 && w2 <= 0))) {
          w0 = w0 / area;
          w1 = w1 / area;
          w2 = w2 / area;
          w0 = w0 / v0[2];
          w1 = w1 / v1[2];
          w2 = w2 / v2[2];
          float z = 1.0f / (w0 + w1 + w2);
          w0 = w0 * z;
          w1 = w1 * z;
          w2 = w2 * z;
          if (st) {
            st->covered++;
            if (!(z >= flt_min)) st->special_candidates++;
          }
          size_t p = (size_t)y * (size_t)W + (size_t)x;
          float d = dep[p];
          if (d < flt_min || z < d) {
            dep[p] = z;
            fidimg[p] = i;
            wimg[3 * p + 0] = w0;
            wimg[3 * p + 1] = w1;
            wimg[3 * p + 2] = w2;
            bfimg[p] = backface ? 255 : 0;
          }
        }
      }
    }
  }

  /* Loop C: resolve (rasterizer.cc:244-301). */
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      size_t p = (size_t)y * (size_t)W + (size_t)x;
      int fid = fidimg[p];
      if (o->backface_culling && bfimg[p] == 255) {
        dep[p] = 0.0f;
        fidimg[p] = -1;
        continue;
      }
      if (fid > 0) {
        float ray[3];
        oracle_ray_w(cam, x, y, ray);
        float w0 = wimg[3 * p + 0], w1 = wimg[3 * p + 1], w2 = wimg[3 * p + 2];
        if (mask) mask[p] = 255;
        float sn[3] = {0.0f, 0.0f, 0.0f};
        if (o->shading_normal == 0) {
          sn[0] = m->face_normals[3 * fid + 0];
          sn[1] = m->face_normals[3 * fid + 1];
          sn[2] = m->face_normals[3 * fid + 2];
        } else if (o->shading_normal == 1) {
          const int32_t* ni = &m->normal_indices[3 * fid];
          const float* n0 = &m->normals[3 * ni[0]];
          const float* n1 = &m->normals[3 * ni[1]];
          const float* n2 = &m->normals[3 * ni[2]];
          for (int k = 0; k < 3; k++) sn[k] = (w0 * n0[k] + w1 * n1[k]) + w2 * n2[k];
        }
        if (normal) matvec3(cam->w2c_R, sn, &normal[3 * p]);
        if (color || color_f32) {
          uint8_t c[3];
          shade_color(m, o, fid, w1, w2, ray, sn, on_A, on_B, c,
                      color_f32 ? &color_f32[3 * p] : NULL, st);
          if (color) {
            color[3 * p + 0] = c[0];
            color[3 * p + 1] = c[1];
            color[3 * p + 2] = c[2];
          }
        }
      }
    }
  }

  if (!depth) free(dep);
  if (!face_id) free(fidimg);
  free(bfimg);
  free(wimg);
  free(img);
  return ORACLE_OK;
}

/* ------------------------------------------------------------------------ */
/* FP64 recomputation (no reference counterpart: the error yardstick).       */
int64_t oracle_gbuffer(const oracle_mesh* m, const oracle_camera* cam,
                       const oracle_option* o, const int32_t* face_id, float* pos_wld,
                       float* pos_cam, float* normal_wld, float* normal_cam, float* bary,
                       float* uv, uint8_t* stencil) {
  const int W = cam->width, H = cam->height;
  int64_t bad = 0;
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      const size_t p = (size_t)y * (size_t)W + (size_t)x;
      const int fid = face_id[p];
      float pw[3] = {0, 0, 0}, pc[3] = {0, 0, 0}, nw[3] = {0, 0, 0}, nc[3] = {0, 0, 0};
      float b3[3] = {0, 0, 0}, t3[3] = {0, 0, 0};
      uint8_t st = 0;
      if (fid < -1 || fid >= m->num_faces) {
        bad++;
      } else if (fid >= 0) {
        st = 255;
        const int32_t* f = &m->vertex_indices[3 * fid];
        float v0[3], v1[3], v2[3];
        project_vertex(cam, &m->vertices[3 * f[0]], v0);
        project_vertex(cam, &m->vertices[3 * f[1]], v1);
        project_vertex(cam, &m->vertices[3 * f[2]], v2);
        const float area = edge_fn(v0[0], v0[1], v1[0], v1[1], v2[0], v2[1]);
        const float px = (float)x, py = (float)y;
        float w0 = edge_fn(v1[0], v1[1], v2[0], v2[1], px, py);
        float w1 = edge_fn(v2[0], v2[1], v0[0], v0[1], px, py);
        float w2 = edge_fn(v0[0], v0[1], v1[0], v1[1], px, py);
        w0 = w0 / area;
        w1 = w1 / area;
        w2 = w2 / area;
        w0 = w0 / v0[2];
        w1 = w1 / v1[2];
        w2 = w2 / v2[2];
        const float z = 1.0f / (w0 + w1 + w2);
        w0 = w0 * z;
        w1 = w1 * z;
        w2 = w2 * z;
        b3[0] = w1;
        b3[1] = w2;
        b3[2] = 1.f - w1 - w2;
        const float* P0 = &m->vertices[3 * f[0]];
        const float* P1 = &m->vertices[3 * f[1]];
        const float* P2 = &m->vertices[3 * f[2]];
        for (int k = 0; k < 3; k++) pw[k] = (w0 * P0[k] + w1 * P1[k]) + w2 * P2[k];
        /* w2c_t + (w2c_R * wld) */
        matvec3(cam->w2c_R, pw, pc);
        for (int k = 0; k < 3; k++) pc[k] = cam->w2c_t[k] + pc[k];
        float sn[3];
        if (o->shading_normal == 0) {
          for (int k = 0; k < 3; k++) sn[k] = m->face_normals[3 * fid + k];
        } else {
          const int32_t* ni = &m->normal_indices[3 * fid];
          const float* n0 = &m->normals[3 * ni[0]];
          const float* n1 = &m->normals[3 * ni[1]];
          const float* n2 = &m->normals[3 * ni[2]];
          for (int k = 0; k < 3; k++) sn[k] = (w0 * n0[k] + w1 * n1[k]) + w2 * n2[k];
        }
        const float n2s = dot3(sn, sn);
        if (n2s > 0.0f) {
          const float r = sqrtf(n2s);
          for (int k = 0; k < 3; k++) nw[k] = sn[k] / r;
        } else {
          for (int k = 0; k < 3; k++) nw[k] = sn[k];
        }
        matvec3(cam->w2c_R, nw, nc);
        if (m->num_uv > 0 && m->num_uv_indices > 0) {
          const float s0 = 1.0f - w1 - w2;
          const int32_t* ti = &m->uv_indices[3 * fid];
          const float* a = &m->uv[2 * ti[0]];
          const float* b = &m->uv[2 * ti[1]];
          const float* d = &m->uv[2 * ti[2]];
          t3[0] = (s0 * a[0] + w1 * b[0]) + w2 * d[0];
          t3[1] = (s0 * a[1] + w1 * b[1]) + w2 * d[1];
          t3[2] = 1.f - t3[0] - t3[1];
        }
      }
      for (int k = 0; k < 3; k++) {
        if (pos_wld) pos_wld[3 * p + k] = pw[k];
        if (pos_cam) pos_cam[3 * p + k] = pc[k];
        if (normal_wld) normal_wld[3 * p + k] = nw[k];
        if (normal_cam) normal_cam[3 * p + k] = nc[k];
        if (bary) bary[3 * p + k] = b3[k];
        if (uv) uv[3 * p + k] = t3[k];
      }
      if (stencil) stencil[p] = st;
    }
  }
  return bad;
}

/* ugu::Raytracer::Impl::Render (raytracer.cc:127-224), same validation and
 * output initialisation as the rasterizer (util_private.cc:12-90). */
int oracle_raytrace(const oracle_mesh* m, const oracle_camera* cam,
                    const oracle_option* o, float depth_scale, uint8_t* color,
                    float* depth, float* normal, uint8_t* mask, int32_t* face_id,
                    float* color_f32, uint8_t* sort_dependent) {
  int rc = validate(m, o, color, depth, normal, mask, face_id, color_f32);
  if (rc) return rc;
  const int W = cam->width, H = cam->height;
  const size_t npx = (size_t)W * (size_t)H;
  if (depth) for (size_t i = 0; i < npx; i++) depth[i] = 0.0f;
  if (face_id) for (size_t i = 0; i < npx; i++) face_id[i] = -1;
  if (color) memset(color, 0, 3 * npx);
  if (normal) memset(normal, 0, 3 * npx * sizeof(float));
  if (mask) memset(mask, 0, npx);
  if (color_f32) memset(color_f32, 0, 3 * npx * sizeof(float));
  if (sort_dependent) memset(sort_dependent, 0, npx);
  void* bvh = oracle_bvh_build(m->vertices, m->num_faces, m->vertex_indices);
  if (!bvh) return ORACLE_ERR_ALLOC;
  float sigma_2 = o->oren_nayar_sigma * o->oren_nayar_sigma;
  float on_A = 1.0f - (0.5f * sigma_2 / (sigma_2 + 0.33f));
  float on_B = 0.45f * sigma_2 / (sigma_2 + 0.09f);
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      size_t p = (size_t)y * (size_t)W + (size_t)x;
      float ray[3];
      oracle_ray_w(cam, x, y, ray);
      float t, u, v;
      int32_t fid, sd = 0;
      int hit = oracle_bvh_nearest(bvh, cam->c2w_t, ray, &t, &u, &v, &fid, &sd);
      if (sort_dependent) sort_dependent[p] = (uint8_t)sd;
      if (!hit) continue;
      /* back face: the face normal points along the ray (:166-171) */
      if (o->backface_culling && dot3(&m->face_normals[3 * fid], ray) > 0.0f) continue;
      if (face_id) face_id[p] = fid;
      if (mask) mask[p] = 255;
      if (depth) {
        float hw[3], hc2;
        for (int k = 0; k < 3; k++) hw[k] = cam->c2w_t[k] + ray[k] * t;
        hc2 = SUM3(cam->w2c_R[6] * hw[0], cam->w2c_R[7] * hw[1], cam->w2c_R[8] * hw[2]) +
              cam->w2c_t[2];
        depth[p] = hc2 * depth_scale;
      }
      float sn[3] = {0.0f, 0.0f, 0.0f};
      if (o->shading_normal == 0) {
        for (int k = 0; k < 3; k++) sn[k] = m->face_normals[3 * fid + k];
      } else if (o->shading_normal == 1) {
        /* (1.0f - u - v) * n0 + u * n1 + v * n2 (:196-199) */
        const int32_t* ni = &m->normal_indices[3 * fid];
        const float* n0 = &m->normals[3 * ni[0]];
        const float* n1 = &m->normals[3 * ni[1]];
        const float* n2 = &m->normals[3 * ni[2]];
        float s = 1.0f - u - v;
        for (int k = 0; k < 3; k++) sn[k] = (s * n0[k] + u * n1[k]) + v * n2[k];
      }
      if (normal) matvec3(cam->w2c_R, sn, &normal[3 * p]);
      if (color || color_f32) {
        uint8_t c[3];
        shade_color(m, o, fid, u, v, ray, sn, on_A, on_B, c,
                    color_f32 ? &color_f32[3 * p] : NULL, NULL);
        if (color) {
          color[3 * p + 0] = c[0];
          color[3 * p + 1] = c[1];
          color[3 * p + 2] = c[2];
        }
      }
    }
  }
  oracle_bvh_free(bvh);
  return ORACLE_OK;
}

/* ------------------------------------------------------------------------ */

typedef struct {
  double X[3], Y[3], Z[3]; /* projected vertices */
  double cx[3], cy[3];     /* camera-frame x, y (for the position gradient) */
  double A;                /* screen-space area */
  double e[3];             /* edge functions at the pixel */
  double b[3];             /* screen barycentrics e/A */
  double q[3];             /* b / Z */
  double s;                /* sum q */
  double w[3];             /* perspective-correct weights q / s */
} face_px64;

static double edge64(double ax, double ay, double bx, double by, double cx,
                     double cy) {
  return (cx - ax) * (by - ay) - (cy - ay) * (bx - ax);
}

static void setup64(const double* P, const int32_t* f, const oracle_camera* cam,
                    int x, int y, face_px64* r) {
  for (int k = 0; k < 3; k++) {
    const double* v = &P[3 * f[k]];
    double c[3];
    for (int j = 0; j < 3; j++)
      c[j] = (double)cam->w2c_R[3 * j + 0] * v[0] +
             (double)cam->w2c_R[3 * j + 1] * v[1] +
             (double)cam->w2c_R[3 * j + 2] * v[2] + (double)cam->w2c_t[j];
    r->cx[k] = c[0];
    r->cy[k] = c[1];
    r->Z[k] = c[2];
    r->X[k] = (double)cam->fx * c[0] / c[2] + (double)cam->cx;
    r->Y[k] = (double)cam->fy * c[1] / c[2] + (double)cam->cy;
  }
  double px = x, py = y;
  r->A = edge64(r->X[0], r->Y[0], r->X[1], r->Y[1], r->X[2], r->Y[2]);
  r->e[0] = edge64(r->X[1], r->Y[1], r->X[2], r->Y[2], px, py);
  r->e[1] = edge64(r->X[2], r->Y[2], r->X[0], r->Y[0], px, py);
  r->e[2] = edge64(r->X[0], r->Y[0], r->X[1], r->Y[1], px, py);
  r->s = 0.0;
  for (int k = 0; k < 3; k++) {
    r->b[k] = r->e[k] / r->A;
    r->q[k] = r->b[k] / r->Z[k];
    r->s += r->q[k];
  }
  for (int k = 0; k < 3; k++) r->w[k] = r->q[k] / r->s;
}

/* The parameter moved for finite differences (NULL = none); set by
 * oracle_backward_f64 for the duration of one call. */
static _Thread_local const oracle_perturb* g_pert = NULL;

static double pert(int kind, int64_t index) {
  return (g_pert && g_pert->kind == kind && g_pert->index == index) ? g_pert->delta : 0.0;
}

static double* positions64(const oracle_mesh* m) {
  double* P = (double*)malloc(((size_t)m->num_vertices + 1) * 3 * sizeof(double));
  if (!P) return NULL;
  for (int i = 0; i < 3 * m->num_vertices; i++) P[i] = m->vertices[i] + pert(3, i);
  return P;
}

static double texel64(const oracle_mesh* m, int mid, int64_t idx, int k) {
  const float* tf = m->textures_f32 ? m->textures_f32[mid] : NULL;
  double d = mid == 0 ? pert(1, 3 * idx + k) : 0.0;
  if (tf) return tf[3 * idx + k] + d;
  return (double)m->textures[mid].data[3 * idx + k] + d;
}

/* Colour of the differentiable path in double, plus its derivatives with
 * respect to u and v (per channel). */
static void color64(const oracle_mesh* m, const oracle_option* o, int fid,
                    double u, double v, double* col, double* dcdu,
                    double* dcdv, int64_t* tix, double* tw) {
  double s = 1.0 - u - v;
  if (o->diffuse_color == 2) {
    const int32_t* f = &m->vertex_indices[3 * fid];
    for (int k = 0; k < 3; k++) {
      double c0 = m->vertex_colors[3 * f[0] + k] + pert(2, 3 * f[0] + k);
      double c1 = m->vertex_colors[3 * f[1] + k] + pert(2, 3 * f[1] + k);
      double c2 = m->vertex_colors[3 * f[2] + k] + pert(2, 3 * f[2] + k);
      col[k] = s * c0 + u * c1 + v * c2;
      if (dcdu) dcdu[k] = c1 - c0;
      if (dcdv) dcdv[k] = c2 - c0;
    }
  } else if (o->diffuse_color == 1) {
    int mid = m->material_ids[fid];
    const oracle_texture* t = &m->textures[mid];
    const int32_t* f = &m->uv_indices[3 * fid];
    const float* a = &m->uv[2 * f[0]];
    const float* b = &m->uv[2 * f[1]];
    const float* c = &m->uv[2 * f[2]];
    double uvx = s * a[0] + u * b[0] + v * c[0];
    double uvy = s * a[1] + u * b[1] + v * c[1];
    double fx = uvx * (t->width - 1);
    double fy = (1.0 - uvy) * (t->height - 1);
    double x0 = floor(fx), y0 = floor(fy);
    double lu = fx - x0, lv = fy - y0;
    int64_t i00 = texel_index((int64_t)y0, (int64_t)x0, t->width, t->height, NULL);
    int64_t i10 = texel_index((int64_t)y0, (int64_t)x0 + 1, t->width, t->height, NULL);
    int64_t i01 = texel_index((int64_t)y0 + 1, (int64_t)x0, t->width, t->height, NULL);
    int64_t i11 = texel_index((int64_t)y0 + 1, (int64_t)x0 + 1, t->width, t->height, NULL);
    double dfx_du = (b[0] - (double)a[0]) * (t->width - 1);
    double dfx_dv = (c[0] - (double)a[0]) * (t->width - 1);
    double dfy_du = -(b[1] - (double)a[1]) * (t->height - 1);
    double dfy_dv = -(c[1] - (double)a[1]) * (t->height - 1);
    for (int k = 0; k < 3; k++) {
      double t00 = texel64(m, mid, i00, k), t10 = texel64(m, mid, i10, k);
      double t01 = texel64(m, mid, i01, k), t11 = texel64(m, mid, i11, k);
      col[k] = (1 - lu) * (1 - lv) * t00 + lu * (1 - lv) * t10 +
               (1 - lu) * lv * t01 + lu * lv * t11;
      double dlu = (1 - lv) * (t10 - t00) + lv * (t11 - t01);
      double dlv = (1 - lu) * (t01 - t00) + lu * (t11 - t10);
      if (dcdu) dcdu[k] = dlu * dfx_du + dlv * dfy_du;
      if (dcdv) dcdv[k] = dlu * dfx_dv + dlv * dfy_dv;
    }
    if (tix) {
      tix[0] = i00; tix[1] = i10; tix[2] = i01; tix[3] = i11;
      tw[0] = (1 - lu) * (1 - lv);
      tw[1] = lu * (1 - lv);
      tw[2] = (1 - lu) * lv;
      tw[3] = lu * lv;
    }
  } else {
    col[0] = col[1] = col[2] = 255.0;
    if (dcdu) dcdu[0] = dcdu[1] = dcdu[2] = 0.0;
    if (dcdv) dcdv[0] = dcdv[1] = dcdv[2] = 0.0;
  }
}

void oracle_interp_f64(const oracle_mesh* m, const oracle_camera* cam,
                       const oracle_option* o, const int32_t* face_id,
                       double* depth, double* normal, double* color) {
  const int W = cam->width, H = cam->height;
  double* P = positions64(m);
  if (!P) return;
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      size_t p = (size_t)y * W + x;
      int fid = face_id[p];
      if (depth) depth[p] = 0.0;
      if (normal) normal[3 * p] = normal[3 * p + 1] = normal[3 * p + 2] = 0.0;
      if (color) color[3 * p] = color[3 * p + 1] = color[3 * p + 2] = 0.0;
      if (fid < 0) continue;
      face_px64 r;
      setup64(P, &m->vertex_indices[3 * fid], cam, x, y, &r);
      if (depth) depth[p] = 1.0 / r.s;
      if (fid == 0) continue;
      if (normal) {
        double sn[3];
        if (o->shading_normal == 0) {
          for (int k = 0; k < 3; k++) sn[k] = m->face_normals[3 * fid + k];
        } else {
          const int32_t* ni = &m->normal_indices[3 * fid];
          for (int k = 0; k < 3; k++)
            sn[k] = r.w[0] * m->normals[3 * ni[0] + k] +
                    r.w[1] * m->normals[3 * ni[1] + k] +
                    r.w[2] * m->normals[3 * ni[2] + k];
        }
        for (int j = 0; j < 3; j++)
          normal[3 * p + j] = cam->w2c_R[3 * j] * sn[0] +
                              (double)cam->w2c_R[3 * j + 1] * sn[1] +
                              (double)cam->w2c_R[3 * j + 2] * sn[2];
      }
      if (color) color64(m, o, fid, r.w[1], r.w[2], &color[3 * p], NULL, NULL, NULL, NULL);
    }
  }
  free(P);
}

/* Derivative of E(a, b, c) = (c.x-a.x)(b.y-a.y) - (c.y-a.y)(b.x-a.x) with
 * respect to the coordinates of a, b and c, scaled by g and accumulated. */
static void edge_grad(double g, double ax, double ay, double bx, double by,
                      double cx, double cy, double* gax, double* gay,
                      double* gbx, double* gby, double* gcx, double* gcy) {
  if (gax) *gax += g * (cy - by);
  if (gay) *gay += g * (bx - cx);
  if (gbx) *gbx += g * (-(cy - ay));
  if (gby) *gby += g * (cx - ax);
  if (gcx) *gcx += g * (by - ay);
  if (gcy) *gcy += g * (-(bx - ax));
}

double oracle_backward_f64(const oracle_mesh* m, const oracle_camera* cam,
                           const oracle_option* o, const int32_t* face_id,
                           const float* target, double* grad_tex,
                           double* grad_vcolor, double* grad_vpos,
                           const oracle_perturb* perturb) {
  const int W = cam->width, H = cam->height;
  g_pert = perturb;
  double* P = positions64(m);
  if (!P) {
    g_pert = NULL;
    return NAN;
  }
  double loss = 0.0;
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      size_t p = (size_t)y * W + x;
      int fid = face_id[p];
      if (fid <= 0) continue;
      const int32_t* f = &m->vertex_indices[3 * fid];
      face_px64 r;
      setup64(P, f, cam, x, y, &r);
      double col[3], dcdu[3], dcdv[3], tw[4];
      int64_t tix[4];
      color64(m, o, fid, r.w[1], r.w[2], col, dcdu, dcdv, tix, tw);
      double gC[3];
      for (int k = 0; k < 3; k++) {
        double d = col[k] - (double)target[3 * p + k];
        loss += d * d;
        gC[k] = 2.0 * d;
      }
      double u = r.w[1], v = r.w[2];
      if (o->diffuse_color == 2 && grad_vcolor) {
        for (int k = 0; k < 3; k++) {
          grad_vcolor[3 * f[0] + k] += gC[k] * (1.0 - u - v);
          grad_vcolor[3 * f[1] + k] += gC[k] * u;
          grad_vcolor[3 * f[2] + k] += gC[k] * v;
        }
      }
      if (o->diffuse_color == 1 && grad_tex && m->material_ids[fid] == 0) {
        for (int j = 0; j < 4; j++)
          for (int k = 0; k < 3; k++) grad_tex[3 * tix[j] + k] += gC[k] * tw[j];
      }
      if (!grad_vpos) continue;
      /* dL/du, dL/dv, then back through w = q / s, q = b / Z, b = e / A. */
      double gw[3] = {0.0, 0.0, 0.0};
      for (int k = 0; k < 3; k++) {
        gw[1] += gC[k] * dcdu[k];
        gw[2] += gC[k] * dcdv[k];
      }
      double gdotw = gw[0] * r.w[0] + gw[1] * r.w[1] + gw[2] * r.w[2];
      double gX[3] = {0, 0, 0}, gY[3] = {0, 0, 0}, gZ[3] = {0, 0, 0};
      double gb[3];
      for (int k = 0; k < 3; k++) {
        double gq = (gw[k] - gdotw) / r.s;
        gb[k] = gq / r.Z[k];
        gZ[k] += -gq * r.q[k] / r.Z[k];
      }
      double gA = 0.0;
      double px = x, py = y;
      for (int k = 0; k < 3; k++) gA += -gb[k] * r.b[k] / r.A;
      /* e0 = E(v1, v2, p), e1 = E(v2, v0, p), e2 = E(v0, v1, p). */
      edge_grad(gb[0] / r.A, r.X[1], r.Y[1], r.X[2], r.Y[2], px, py, &gX[1], &gY[1], &gX[2], &gY[2], NULL, NULL);
      edge_grad(gb[1] / r.A, r.X[2], r.Y[2], r.X[0], r.Y[0], px, py, &gX[2], &gY[2], &gX[0], &gY[0], NULL, NULL);
      edge_grad(gb[2] / r.A, r.X[0], r.Y[0], r.X[1], r.Y[1], px, py, &gX[0], &gY[0], &gX[1], &gY[1], NULL, NULL);
      edge_grad(gA, r.X[0], r.Y[0], r.X[1], r.Y[1], r.X[2], r.Y[2], &gX[0], &gY[0], &gX[1], &gY[1], &gX[2], &gY[2]);
      for (int k = 0; k < 3; k++) {
        double z = r.Z[k];
        double gcx = gX[k] * cam->fx / z;
        double gcy = gY[k] * cam->fy / z;
        double gcz = -gX[k] * cam->fx * r.cx[k] / (z * z) -
                     gY[k] * cam->fy * r.cy[k] / (z * z) + gZ[k];
        for (int j = 0; j < 3; j++)
          grad_vpos[3 * f[k] + j] += cam->w2c_R[0 * 3 + j] * gcx +
                                     (double)cam->w2c_R[1 * 3 + j] * gcy +
                                     (double)cam->w2c_R[2 * 3 + j] * gcz;
      }
    }
  }
  free(P);
  g_pert = NULL;
  return loss;
}

/* ------------------------------------------------------------------------ */
/* Mesh normals (src/mesh.cc:297-349).                                       */
/* ------------------------------------------------------------------------ */

static void normalize3(float* v) {
  float n2 = SUM3(v[0] * v[0], v[1] * v[1], v[2] * v[2]);
  if (n2 > 0.0f) {
    float s = sqrtf(n2);
    v[0] = v[0] / s;
    v[1] = v[1] / s;
    v[2] = v[2] / s;
  }
}

void oracle_calc_normals(int32_t nv, const float* V, int32_t nf,
                         const int32_t* F, float* FN, float* N) {
  /* CalcFaceNormal: normalize(normalize(v1-v0) x normalize(v2-v0)). */
  for (int i = 0; i < nf; i++) {
    const float* a = &V[3 * F[3 * i]];
    const float* b = &V[3 * F[3 * i + 1]];
    const float* c = &V[3 * F[3 * i + 2]];
    float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    normalize3(e1);
    normalize3(e2);
    float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                  e1[0] * e2[1] - e1[1] * e2[0]};
    normalize3(n);
    FN[3 * i] = n[0];
    FN[3 * i + 1] = n[1];
    FN[3 * i + 2] = n[2];
  }
  if (!N) return;
  /* CalcNormal: per-vertex sum of incident face normals in face order,
   * divided by the count, normalised; unreferenced vertices get 0. */
  int32_t* cnt = (int32_t*)calloc((size_t)nv + 1, sizeof(int32_t));
  if (!cnt) return;
  for (int i = 0; i < 3 * nv; i++) N[i] = 0.0f;
  for (int i = 0; i < nf; i++)
    for (int j = 0; j < 3; j++) {
      int idx = F[3 * i + j];
      N[3 * idx] = N[3 * idx] + FN[3 * i];
      N[3 * idx + 1] = N[3 * idx + 1] + FN[3 * i + 1];
      N[3 * idx + 2] = N[3 * idx + 2] + FN[3 * i + 2];
      cnt[idx]++;
    }
  for (int i = 0; i < nv; i++) {
    if (cnt[i] > 0) {
      float c = (float)cnt[i];
      N[3 * i] = N[3 * i] / c;
      N[3 * i + 1] = N[3 * i + 1] / c;
      N[3 * i + 2] = N[3 * i + 2] / c;
      normalize3(&N[3 * i]);
    } else {
      N[3 * i] = N[3 * i + 1] = N[3 * i + 2] = 0.0f;
    }
  }
  free(cnt);
}
