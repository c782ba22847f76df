// ref_visibility.cc -- TEST INFRASTRUCTURE ONLY.
//
// C entry points around the reference's own ugu::VisibilityTester and
// ugu::TextureMapping (src/texturing/visibility_tester.cc and
// texture_mapper.cc, compiled unmodified against the Eigen-compatible shim),
// on plain arrays: the VisibilityInfo of Test(keyframes, info, facewise)
// copied out field by field, and the texture, uv, uv indices and material
// ids TextureMapping leaves on the mesh, so that the oracle's restatements
// and the host mirror can be compared with them.
#include <cstring>
#include <memory>
#include <vector>

#include "ugu/texturing/texture_mapper.h"
#include "ugu/texturing/visibility_tester.h"
#include "ugu/util/math_util.h"

namespace ugu {
// src/util/math_util.cc:44-56 (that file needs Eigen's dynamic matrices and
// SVD, which the shim lacks): the per-channel Median of math_util.h.
Eigen::Vector3f MedianColor(const std::vector<Eigen::Vector3f>& colors) {
  Eigen::Vector3f m;
  std::vector<std::vector<float>> ch(3);
  for (const auto& c : colors)
    for (int i = 0; i < 3; ++i) ch[i].push_back(c[i]);
  for (int i = 0; i < 3; ++i) m[i] = Median(ch[i]);
  return m;
}
}  // namespace ugu

extern "C" {

struct ref_keyframe {
  int id, width, height;
  float fx, fy, cx, cy;
  double c2w[16];              // row-major 4x4
  const unsigned char* color;  // H*W*3
  const float* depth;          // H*W, or NULL
  const unsigned char* mask;   // H*W, or NULL
};

struct ref_vis_option {
  float backface_culling_angle_rad_th;
  int use_mask, use_depth, interp, calc_stat_vertex_info, collect_face_info,
      calc_stat_face_info;
  float max_viewing_angle, max_distance_from_camera_to_vertex, max_depth_difference, eps;
  float invalid_color[3];
};

}  // extern "C"

namespace {

// VisibilityTester(option).set_data(...), PrepareData, then
// Test(keyframes, info, facewise); 0, 1 when Test returns false, 2 when
// PrepareData does.
int run_visibility(const float* vertices, int nv, const float* normals, const int* indices,
                   int nf, const ref_keyframe* kfs, int nkf, const ref_vis_option* o,
                   int facewise, std::vector<std::shared_ptr<ugu::Keyframe>>* out_keyframes,
                   ugu::VisibilityInfo* out_info) {
  ugu::set_log_level(ugu::LogLevel::kError);
  std::vector<Eigen::Vector3f> v(nv), n(nv);
  for (int i = 0; i < nv; ++i) {
    v[i] = Eigen::Vector3f(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]);
    n[i] = Eigen::Vector3f(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
  }
  std::vector<Eigen::Vector3i> f(nf);
  for (int i = 0; i < nf; ++i)
    f[i] = Eigen::Vector3i(indices[3 * i], indices[3 * i + 1], indices[3 * i + 2]);

  ugu::VisibilityTesterOption opt;
  opt.backface_culling_angle_rad_th = o->backface_culling_angle_rad_th;
  opt.use_mask = o->use_mask != 0;
  opt.use_depth = o->use_depth != 0;
  opt.interp = static_cast<ugu::ColorInterpolation>(o->interp);
  opt.calc_stat_vertex_info = o->calc_stat_vertex_info != 0;
  opt.collect_face_info = o->collect_face_info != 0;
  opt.calc_stat_face_info = o->calc_stat_face_info != 0;
  opt.max_viewing_angle = o->max_viewing_angle;
  opt.max_distance_from_camera_to_vertex = o->max_distance_from_camera_to_vertex;
  opt.max_depth_difference = o->max_depth_difference;
  opt.eps = o->eps;
  opt.invalid_color =
      Eigen::Vector3f(o->invalid_color[0], o->invalid_color[1], o->invalid_color[2]);

  ugu::VisibilityTester tester(opt);
  tester.set_data(v, n, f);
  if (!tester.PrepareData()) return 2;

  std::vector<std::shared_ptr<ugu::Keyframe>> keyframes;
  for (int k = 0; k < nkf; ++k) {
    const ref_keyframe& s = kfs[k];
    auto kf = ugu::Keyframe::Create();
    kf->id = s.id;
    kf->color = ugu::Image3b::zeros(s.height, s.width);
    std::memcpy(kf->color.data, s.color, (size_t)s.width * s.height * 3);
    if (s.depth) {
      kf->depth = ugu::Image1f::zeros(s.height, s.width);
      std::memcpy(kf->depth.data, s.depth, (size_t)s.width * s.height * 4);
    }
    if (s.mask) {
      kf->mask = ugu::Image1b::zeros(s.height, s.width);
      std::memcpy(kf->mask.data, s.mask, (size_t)s.width * s.height);
    }
    Eigen::Matrix4d M;
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) M(r, c) = s.c2w[4 * r + c];
    kf->camera = std::make_shared<ugu::PinholeCamera>(
        s.width, s.height, Eigen::Affine3d(M), Eigen::Vector2f(s.cx, s.cy),
        Eigen::Vector2f(s.fx, s.fy));
    keyframes.push_back(kf);
  }

  out_info->vertex_info_list.resize(nv);
  out_info->face_info_list.resize(nf);
  if (!tester.Test(keyframes, out_info, facewise != 0)) return 1;
  *out_keyframes = keyframes;
  return 0;
}

}  // namespace


extern "C" {

// Per-vertex outputs (K = nkf): vcount[V]; vrec_id[V*K]; vrec[V*K*9] = color
// (3), intensity, projected_pos (2), viewing_angle, distance, 0; vstat_i[V*5]
// = min_viewing_angle index, id, min_distance index, id, mode_frequency;
// vstat[V*43] = mean_color, median_color, min_viewing_angle_color,
// mean_viewing_angle_color, median_viewing_angle_color, min_distance_color,
// mean_distance_color, median_distance_color, median_intensity_color,
// min_intensity_color, mode, mode_viewing_angle_color (3 each), then
// min_intensity, median_intensity, mean_viewing_angle, median_viewing_angle,
// mean_distance, median_distance, mode_frequency_viewing_angle_color.
// Per-face outputs: fcount[F]; frec_id[F*K*2] = kf_id, face_id; frec[F*K*9] =
// area, viewing_angle, distance, projected_tri (6); fstat_i[F*6] = max_area
// index, id, min_viewing_angle index, id, min_distance index, id; fstat[F*3]
// = max_area, min_viewing_angle, min_distance.  Statistics of a vertex or
// face without records are left as they are.  Returns 0, or 1 when Test
// returns false.
int ref_visibility(const float* vertices, int nv, const float* normals, const int* indices,
                   int nf, const ref_keyframe* kfs, int nkf, const ref_vis_option* o,
                   int facewise, int* vcount, int* vrec_id, float* vrec, int* vstat_i,
                   float* vstat, int* fcount, int* frec_id, float* frec, int* fstat_i,
                   float* fstat) {
  std::vector<std::shared_ptr<ugu::Keyframe>> keyframes;
  ugu::VisibilityInfo info;
  const int rc = run_visibility(vertices, nv, normals, indices, nf, kfs, nkf, o, facewise,
                                &keyframes, &info);
  if (rc) return rc;

  auto put3 = [](float* d, const Eigen::Vector3f& a) {
    d[0] = a[0];
    d[1] = a[1];
    d[2] = a[2];
  };
  for (int i = 0; i < nv; ++i) {
    const ugu::VertexInfo& vi = info.vertex_info_list[i];
    const int c = (int)vi.visible_keyframes.size();
    vcount[i] = c;
    for (int j = 0; j < c && j < nkf; ++j) {
      const ugu::VertexInfoPerKeyframe& r = vi.visible_keyframes[j];
      float* d = vrec + ((size_t)i * nkf + j) * 9;
      vrec_id[(size_t)i * nkf + j] = r.kf_id;
      put3(d, r.color);
      d[3] = r.intensity;
      d[4] = r.projected_pos[0];
      d[5] = r.projected_pos[1];
      d[6] = r.viewing_angle;
      d[7] = r.distance;
      d[8] = 0.0f;
    }
    if (c == 0) continue;
    int* si = vstat_i + (size_t)i * 5;
    si[0] = vi.min_viewing_angle_index;
    si[1] = vi.min_viewing_angle_id;
    si[2] = vi.min_distance_index;
    si[3] = vi.min_distance_id;
    si[4] = vi.mode_frequency;
    float* s = vstat + (size_t)i * 43;
    const Eigen::Vector3f* cols[12] = {&vi.mean_color,
                                       &vi.median_color,
                                       &vi.min_viewing_angle_color,
                                       &vi.mean_viewing_angle_color,
                                       &vi.median_viewing_angle_color,
                                       &vi.min_distance_color,
                                       &vi.mean_distance_color,
                                       &vi.median_distance_color,
                                       &vi.median_intensity_color,
                                       &vi.min_intensity_color,
                                       &vi.mode,
                                       &vi.mode_viewing_angle_color};
    for (int k = 0; k < 12; ++k) put3(s + 3 * k, *cols[k]);
    s[36] = vi.min_intensity;
    s[37] = vi.median_intensity;
    s[38] = vi.mean_viewing_angle;
    s[39] = vi.median_viewing_angle;
    s[40] = vi.mean_distance;
    s[41] = vi.median_distance;
    s[42] = vi.mode_frequency_viewing_angle_color;
  }
  for (int i = 0; i < nf; ++i) {
    const ugu::FaceInfo& fi = info.face_info_list[i];
    const int c = (int)fi.visible_keyframes.size();
    fcount[i] = c;
    for (int j = 0; j < c && j < nkf; ++j) {
      const ugu::FaceInfoPerKeyframe& r = fi.visible_keyframes[j];
      const size_t at = (size_t)i * nkf + j;
      frec_id[2 * at] = r.kf_id;
      frec_id[2 * at + 1] = r.face_id;
      float* d = frec + at * 9;
      d[0] = r.area;
      d[1] = r.viewing_angle;
      d[2] = r.distance;
      for (int k = 0; k < 3; ++k) {
        d[3 + 2 * k] = r.projected_tri[k][0];
        d[4 + 2 * k] = r.projected_tri[k][1];
      }
    }
    if (c == 0) continue;
    int* si = fstat_i + (size_t)i * 6;
    si[0] = fi.max_area_index;
    si[1] = fi.max_area_id;
    si[2] = fi.min_viewing_angle_index;
    si[3] = fi.min_viewing_angle_id;
    si[4] = fi.min_distance_index;
    si[5] = fi.min_distance_id;
    float* s = fstat + (size_t)i * 3;
    s[0] = fi.max_area;
    s[1] = fi.min_viewing_angle;
    s[2] = fi.min_distance;
  }
  return 0;
}

// TextureMapping (src/texturing/texture_mapper.cc:1009-1017) after the
// visibility test above, on a ugu::Mesh of the vertices and faces (and the
// mesh's own uv and uv indices when uv is not NULL), with
// TextureMappingOption {criteria, kSimpleProjection, uv_type, tex_w, tex_h,
// padding_kernel}.  Copies out the first material's texture (tex_wh = its
// width and height; at most tex_cap bytes), the mesh's uv (*n_uv of them, at
// most uv_cap), its uv indices (F*3) and material ids (F).  Returns 0; 1 or
// 2 as run_visibility; 4 when TextureMapping returns false; 3 when the
// texture or the uv do not fit (tex_wh and *n_uv then say how large they
// are).
int ref_texture_mapping(const float* vertices, int nv, const float* normals, const int* indices,
                        int nf, const float* uv, int nuv, const int* uv_indices,
                        const ref_keyframe* kfs, int nkf, const ref_vis_option* o, int facewise,
                        int criteria, int uv_type, int tex_w, int tex_h, int padding_kernel,
                        unsigned char* tex, long long tex_cap, int* tex_wh, float* uv_out,
                        int uv_cap, int* n_uv, int* uvi_out, int* mat_ids) {
  std::vector<std::shared_ptr<ugu::Keyframe>> keyframes;
  ugu::VisibilityInfo info;
  int rc = run_visibility(vertices, nv, normals, indices, nf, kfs, nkf, o, facewise,
                          &keyframes, &info);
  if (rc) return rc;
  ugu::Mesh mesh;
  std::vector<Eigen::Vector3f> v(nv);
  for (int i = 0; i < nv; ++i)
    v[i] = Eigen::Vector3f(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]);
  std::vector<Eigen::Vector3i> f(nf);
  for (int i = 0; i < nf; ++i)
    f[i] = Eigen::Vector3i(indices[3 * i], indices[3 * i + 1], indices[3 * i + 2]);
  mesh.set_vertices(v);
  mesh.set_vertex_indices(f);
  if (uv) {
    std::vector<Eigen::Vector2f> u(nuv);
    for (int i = 0; i < nuv; ++i) u[i] = Eigen::Vector2f(uv[2 * i], uv[2 * i + 1]);
    std::vector<Eigen::Vector3i> ui(nf);
    for (int i = 0; i < nf; ++i)
      ui[i] = Eigen::Vector3i(uv_indices[3 * i], uv_indices[3 * i + 1], uv_indices[3 * i + 2]);
    mesh.set_uv(u);
    mesh.set_uv_indices(ui);
  }
  ugu::TextureMappingOption opt;
  opt.criteria = static_cast<ugu::ViewSelectionCriteria>(criteria);
  opt.type = ugu::TextureMappingType::kSimpleProjection;
  opt.uv_type = static_cast<ugu::TexturingOutputUvType>(uv_type);
  opt.tex_w = tex_w;
  opt.tex_h = tex_h;
  opt.padding_kernel = padding_kernel;
  if (!ugu::TextureMapping(keyframes, info, &mesh, opt)) return 4;

  const ugu::Image3b& t = mesh.materials()[0].diffuse_tex;
  tex_wh[0] = t.cols;
  tex_wh[1] = t.rows;
  *n_uv = (int)mesh.uv().size();
  const long long bytes = (long long)t.cols * t.rows * 3;
  if (bytes > tex_cap || *n_uv > uv_cap) return 3;
  for (int y = 0; y < t.rows; ++y)
    std::memcpy(tex + (size_t)y * t.cols * 3, t.data + t.step[0] * y, (size_t)t.cols * 3);
  for (int i = 0; i < *n_uv; ++i) {
    uv_out[2 * i] = mesh.uv()[i][0];
    uv_out[2 * i + 1] = mesh.uv()[i][1];
  }
  const auto& ui = mesh.uv_indices();
  for (int i = 0; i < nf && i < (int)ui.size(); ++i)
    for (int k = 0; k < 3; ++k) uvi_out[3 * i + k] = ui[i][k];
  const auto& mi = mesh.material_ids();
  for (int i = 0; i < nf && i < (int)mi.size(); ++i) mat_ids[i] = mi[i];
  return 0;
}

}  // extern "C"
