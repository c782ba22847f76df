// ref_driver.cc -- TEST INFRASTRUCTURE ONLY.
//
// C entry points around the reference's own ugu::Rasterizer and
// ugu::Raytracer (src/renderer/cpu/rasterizer.cc and raytracer.cc, compiled
// unmodified from the reference checkout against the Eigen-compatible shim),
// used to pin the oracle's restatements and to generate golden fixtures.
// Each builds a ugu::Mesh and a ugu::PinholeCamera from plain arrays, calls
// Render, and copies the images out together with the camera floats Render
// derived.
#include <chrono>
#include <cstring>
#include <memory>
#include <vector>

#include "ugu/discrete/bin_packer_2d.h"
#include "ugu/image_proc.h"
#include "ugu/util/image_util.h"
#include "ugu/renderer/cpu/rasterizer.h"
#include "ugu/renderer/cpu/raytracer.h"

namespace ugu {
// The camera classes' vtables name these camera_util functions
// (src/util/camera_util.cc, not compiled here); the rasterizer never calls
// them, so they are stubs.
Eigen::Matrix4f GetProjectionMatrixOpenGlForPinhole(int, int, float, float, float, float,
                                                   float, float) {
  return Eigen::Matrix4f::Identity();
}
Eigen::Matrix4f GetProjectionMatrixOpenGlForOrtho(float, float, float, float, float, float) {
  return Eigen::Matrix4f::Identity();
}
void UndistortPixelOpencv(float*, float*, float, float, float, float, float, float, float,
                          float, float, float, float, float) {}
}  // namespace ugu

extern "C" {

struct ref_mesh {
  int num_vertices;
  const float* vertices;
  int num_faces;
  const int* vertex_indices;
  const float* face_normals;  // F*3 or NULL
  int num_normals;
  const float* normals;
  const int* normal_indices;
  const float* vertex_colors;  // V*3 or NULL
  int num_uv;
  const float* uv;
  const int* uv_indices;
  const int* material_ids;  // F or NULL
  int num_materials;
  const int* tex_wh;            // 2 per material
  const unsigned char* const* tex;  // per material RGB8
};

struct ref_option {
  int diffuse_color, interp, shading_normal, diffuse_shading, backface_culling;
  float oren_nayar_sigma;
  float depth_scale;
};

}  // extern "C"

// c2w: 4x4 row-major double.  cam_out: w2c_R[9], w2c_t[3], c2w_R[9] (row-major
// floats) as Render and the ray table use them.  times_ms, when not NULL:
// Render is called twice on the same camera and the wall times of both calls
// are stored, the first with the camera's ray table still to be built
// (PinholeCamera::InitRayTable, camera.h:100-101), the second with it built.
template <typename Renderer>
static int render_with(const ref_mesh* m, int width, int height, float fx, float fy, float cx,
                       float cy, const double* c2w, const ref_option* o, unsigned char* color,
                       float* depth, float* normal, unsigned char* mask, int* face_id,
                       float* cam_out, double* times_ms = nullptr) {
  ugu::set_log_level(ugu::LogLevel::kError);
  auto mesh = std::make_shared<ugu::Mesh>();
  std::vector<Eigen::Vector3f> v(m->num_vertices);
  for (int i = 0; i < m->num_vertices; ++i)
    v[i] = Eigen::Vector3f(m->vertices[3 * i], m->vertices[3 * i + 1], m->vertices[3 * i + 2]);
  mesh->set_vertices(v);
  std::vector<Eigen::Vector3i> f(m->num_faces);
  for (int i = 0; i < m->num_faces; ++i)
    f[i] = Eigen::Vector3i(m->vertex_indices[3 * i], m->vertex_indices[3 * i + 1],
                           m->vertex_indices[3 * i + 2]);
  mesh->set_vertex_indices(f);
  auto vec3 = [](const float* a, int n) {
    std::vector<Eigen::Vector3f> r(n);
    for (int i = 0; i < n; ++i) r[i] = Eigen::Vector3f(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
    return r;
  };
  auto idx3 = [](const int* a, int n) {
    std::vector<Eigen::Vector3i> r(n);
    for (int i = 0; i < n; ++i) r[i] = Eigen::Vector3i(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
    return r;
  };
  if (m->face_normals) mesh->set_face_normals(vec3(m->face_normals, m->num_faces));
  if (m->normals) {
    mesh->set_normals(vec3(m->normals, m->num_normals));
    mesh->set_normal_indices(idx3(m->normal_indices, m->num_faces));
  }
  if (m->vertex_colors) mesh->set_vertex_colors(vec3(m->vertex_colors, m->num_vertices));
  if (m->uv) {
    std::vector<Eigen::Vector2f> uv(m->num_uv);
    for (int i = 0; i < m->num_uv; ++i) uv[i] = Eigen::Vector2f(m->uv[2 * i], m->uv[2 * i + 1]);
    mesh->set_uv(uv);
    mesh->set_uv_indices(idx3(m->uv_indices, m->num_faces));
  }
  if (m->material_ids)
    mesh->set_material_ids(std::vector<int>(m->material_ids, m->material_ids + m->num_faces));
  std::vector<ugu::ObjMaterial> mats(m->num_materials);
  for (int i = 0; i < m->num_materials; ++i) {
    int w = m->tex_wh[2 * i], h = m->tex_wh[2 * i + 1];
    mats[i].diffuse_tex = ugu::Image3b::zeros(h, w);
    std::memcpy(mats[i].diffuse_tex.data, m->tex[i], (size_t)w * h * 3);
  }
  mesh->set_materials(mats);

  Eigen::Matrix4d M;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) M(r, c) = c2w[4 * r + c];
  Eigen::Affine3d pose(M);
  auto cam = std::make_shared<ugu::PinholeCamera>(width, height, pose, Eigen::Vector2f(cx, cy),
                                                  Eigen::Vector2f(fx, fy));
  ugu::RendererCpuOption opt;
  opt.diffuse_color = static_cast<ugu::DiffuseColor>(o->diffuse_color);
  opt.interp = static_cast<ugu::ColorInterpolation>(o->interp);
  opt.shading_normal = static_cast<ugu::ShadingNormal>(o->shading_normal);
  opt.diffuse_shading = static_cast<ugu::DiffuseShading>(o->diffuse_shading);
  opt.backface_culling = o->backface_culling != 0;
  opt.oren_nayar_sigma = o->oren_nayar_sigma;
  opt.depth_scale = o->depth_scale;

  Renderer r(opt);
  r.set_mesh(mesh);
  if (!r.PrepareMesh()) return 100;
  r.set_camera(cam);
  ugu::Image3b c_img;
  ugu::Image1f d_img;
  ugu::Image3f n_img;
  ugu::Image1b m_img;
  ugu::Image1i f_img;
  bool ok = true;
  for (int k = 0; k < (times_ms ? 2 : 1) && ok; ++k) {
    const auto t0 = std::chrono::steady_clock::now();
    ok = r.Render(color ? &c_img : nullptr, depth ? &d_img : nullptr,
                  normal ? &n_img : nullptr, mask ? &m_img : nullptr,
                  face_id ? &f_img : nullptr);
    const auto t1 = std::chrono::steady_clock::now();
    if (times_ms) times_ms[k] = std::chrono::duration<double, std::milli>(t1 - t0).count();
  }
  if (!ok) return 1;
  const size_t px = (size_t)width * height;
  if (color) std::memcpy(color, c_img.data, px * 3);
  if (depth) std::memcpy(depth, d_img.data, px * 4);
  if (normal) std::memcpy(normal, n_img.data, px * 12);
  if (mask) std::memcpy(mask, m_img.data, px);
  if (face_id) std::memcpy(face_id, f_img.data, px * 4);
  if (cam_out) {
    Eigen::Matrix3f R = cam->w2c().rotation().cast<float>();
    Eigen::Vector3f t = cam->w2c().translation().cast<float>();
    Eigen::Matrix3f C = cam->c2w().matrix().block<3, 3>(0, 0).cast<float>();
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        cam_out[3 * a + b] = R(a, b);
        cam_out[12 + 3 * a + b] = C(a, b);
      }
    for (int a = 0; a < 3; ++a) cam_out[9 + a] = t[a];
  }
  return 0;
}

extern "C" {

int ref_render(const ref_mesh* m, int width, int height, float fx, float fy, float cx,
               float cy, const double* c2w, const ref_option* o, unsigned char* color,
               float* depth, float* normal, unsigned char* mask, int* face_id,
               float* cam_out) {
  return render_with<ugu::Rasterizer>(m, width, height, fx, fy, cx, cy, c2w, o, color, depth,
                                      normal, mask, face_id, cam_out);
}

// ref_render, timed: times_ms[0] the first Render on a fresh camera,
// times_ms[1] a second Render on the same camera.
int ref_render_timed(const ref_mesh* m, int width, int height, float fx, float fy, float cx,
                     float cy, const double* c2w, const ref_option* o, unsigned char* color,
                     float* depth, float* normal, unsigned char* mask, int* face_id,
                     double* times_ms) {
  return render_with<ugu::Rasterizer>(m, width, height, fx, fy, cx, cy, c2w, o, color, depth,
                                      normal, mask, face_id, nullptr, times_ms);
}

int ref_raytrace(const ref_mesh* m, int width, int height, float fx, float fy, float cx,
                 float cy, const double* c2w, const ref_option* o, unsigned char* color,
                 float* depth, float* normal, unsigned char* mask, int* face_id,
                 float* cam_out) {
  return render_with<ugu::Raytracer>(m, width, height, fx, fy, cx, cy, c2w, o, color, depth,
                                     normal, mask, face_id, cam_out);
}

// ugu::BinPacking2D (src/discrete/bin_packer_2d.cc) on n integer rects
// (x, y, width, height each): packed receives n rects, free_rects the
// available rects left (at most free_cap; *n_free says how many there are).
// Returns 1 when every rect was packed, 0 otherwise.
int ref_bin_packing_2d(const int* rects, int n, int x_min, int x_max, int y_min, int y_max,
                       int* packed, int* free_rects, int free_cap, int* n_free) {
  std::vector<ugu::Rect> in;
  for (int i = 0; i < n; ++i)
    in.emplace_back(rects[4 * i], rects[4 * i + 1], rects[4 * i + 2], rects[4 * i + 3]);
  std::vector<ugu::Rect> out, avail;
  const bool ok = ugu::BinPacking2D(in, &out, &avail, x_min, x_max, y_min, y_max);
  for (size_t i = 0; i < out.size() && (int)i < n; ++i) {
    packed[4 * i] = out[i].x;
    packed[4 * i + 1] = out[i].y;
    packed[4 * i + 2] = out[i].width;
    packed[4 * i + 3] = out[i].height;
  }
  *n_free = (int)avail.size();
  for (size_t i = 0; i < avail.size() && (int)i < free_cap; ++i) {
    free_rects[4 * i] = avail[i].x;
    free_rects[4 * i + 1] = avail[i].y;
    free_rects[4 * i + 2] = avail[i].width;
    free_rects[4 * i + 3] = avail[i].height;
  }
  return ok ? 1 : 0;
}

// The image helpers after a render (src/util/image_util.cc: Depth2Gray,
// Normal2Color, FaceId2RandomColor; include/ugu/image_proc.h: ConvertTo to
// 16 bits) on W x H images; an input or output may be NULL.
int ref_visualize(int width, int height, const float* depth, const float* normal,
                  const int* face_id, unsigned char* vis_depth, unsigned short* depth_u16,
                  unsigned char* vis_normal, unsigned char* vis_face_id, float min_d,
                  float max_d, int gl_coord) {
  const size_t px = (size_t)width * height;
  if (depth) {
    ugu::Image1f d = ugu::Image1f::zeros(height, width);
    std::memcpy(d.data, depth, px * 4);
    if (vis_depth) {
      ugu::Image1b g;
      ugu::Depth2Gray(d, &g, min_d, max_d);
      std::memcpy(vis_depth, g.data, px);
    }
    if (depth_u16) {
      ugu::Image1w w;
      ugu::ConvertTo(d, &w);
      std::memcpy(depth_u16, w.data, px * 2);
    }
  }
  if (normal && vis_normal) {
    ugu::Image3f n = ugu::Image3f::zeros(height, width);
    std::memcpy(n.data, normal, px * 12);
    ugu::Image3b c;
    ugu::Normal2Color(n, &c, gl_coord != 0);
    std::memcpy(vis_normal, c.data, px * 3);
  }
  if (face_id && vis_face_id) {
    ugu::Image1i f = ugu::Image1i::zeros(height, width);
    std::memcpy(f.data, face_id, px * 4);
    ugu::Image3b c;
    ugu::FaceId2RandomColor(f, &c);
    std::memcpy(vis_face_id, c.data, px * 3);
  }
  return 0;
}

}  // extern "C"
