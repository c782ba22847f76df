// fake_ugu_gpu.cc -- TEST DOUBLE of include/ugu_gpu.h backed by the oracle.
// Lets the C++ drop-in class (ugu_gb300/host/rasterizer_gpu.cc) be checked on
// a machine without a GPU: every render runs the oracle's CPU restatement.
#include <cstring>
#include <string>
#include <vector>

#include "raster_oracle.h"
#include "ugu_gpu.h"

struct ugu_gpu_context {
  ugu_gpu_option opt{};
  std::string err;
  bool has_mesh = false;
  std::vector<float> v, fn, n, vc, uv;
  std::vector<int32_t> f, ni, ui, mi;
  std::vector<std::vector<uint8_t>> tex;
  std::vector<oracle_texture> otex;
  int32_t nv = 0, nf = 0, nn = 0, nuv = 0;
};

static std::string g_err;

extern "C" {
int ugu_gpu_abi_version(void) { return UGU_GPU_ABI_VERSION; }
const char* ugu_gpu_last_error(const ugu_gpu_context* c) { return c ? c->err.c_str() : g_err.c_str(); }
int ugu_gpu_create(int32_t, ugu_gpu_context** out) {
  *out = new ugu_gpu_context();
  return 0;
}
int ugu_gpu_destroy(ugu_gpu_context* c) {
  delete c;
  return 0;
}
int ugu_gpu_set_option(ugu_gpu_context* c, const ugu_gpu_option* o) {
  c->opt = *o;
  return 0;
}
int ugu_gpu_set_mesh(ugu_gpu_context* c, int32_t, const ugu_gpu_mesh* m) {
  c->nv = m->num_vertices;
  c->nf = m->num_faces;
  c->v.assign(m->vertices, m->vertices + 3 * c->nv);
  c->f.assign(m->vertex_indices, m->vertex_indices + 3 * c->nf);
  c->fn.clear();
  if (m->face_normals) c->fn.assign(m->face_normals, m->face_normals + 3 * c->nf);
  c->nn = m->normals ? m->num_normals : 0;
  c->n.clear();
  c->ni.clear();
  if (m->normals) {
    c->n.assign(m->normals, m->normals + 3 * c->nn);
    c->ni.assign(m->normal_indices, m->normal_indices + 3 * c->nf);
  }
  c->vc.clear();
  if (m->vertex_colors) c->vc.assign(m->vertex_colors, m->vertex_colors + 3 * c->nv);
  c->nuv = m->uv ? m->num_uv : 0;
  c->uv.clear();
  c->ui.clear();
  if (m->uv) {
    c->uv.assign(m->uv, m->uv + 2 * c->nuv);
    c->ui.assign(m->uv_indices, m->uv_indices + 3 * c->nf);
  }
  c->mi.clear();
  if (m->material_ids) c->mi.assign(m->material_ids, m->material_ids + c->nf);
  c->tex.clear();
  c->otex.clear();
  for (int i = 0; i < m->num_materials; ++i) {
    const ugu_gpu_texture& t = m->materials[i];
    c->tex.emplace_back(t.rgb8, t.rgb8 + (size_t)3 * t.width * t.height);
  }
  for (int i = 0; i < m->num_materials; ++i)
    c->otex.push_back({m->materials[i].width, m->materials[i].height, c->tex[i].data()});
  c->has_mesh = true;
  return 0;
}
static int fake_render(ugu_gpu_context* c, const ugu_gpu_camera* cam, const ugu_gpu_images* im,
                       bool ray) {
  oracle_mesh m;
  std::memset(&m, 0, sizeof(m));
  m.num_vertices = c->nv;
  m.vertices = c->v.data();
  m.num_faces = c->nf;
  m.vertex_indices = c->f.data();
  m.num_face_normals = c->fn.empty() ? 0 : c->nf;
  m.face_normals = c->fn.data();
  m.num_normals = c->nn;
  m.normals = c->n.data();
  m.num_normal_indices = c->ni.empty() ? 0 : c->nf;
  m.normal_indices = c->ni.data();
  m.num_vertex_colors = c->vc.empty() ? 0 : c->nv;
  m.vertex_colors = c->vc.data();
  m.num_uv = c->nuv;
  m.uv = c->uv.data();
  m.num_uv_indices = c->ui.empty() ? 0 : c->nf;
  m.uv_indices = c->ui.data();
  m.num_material_ids = c->mi.empty() ? 0 : c->nf;
  m.material_ids = c->mi.data();
  m.num_materials = (int32_t)c->otex.size();
  m.textures = c->otex.data();
  oracle_camera oc;
  oc.width = cam->width;
  oc.height = cam->height;
  oc.fx = cam->fx;
  oc.fy = cam->fy;
  oc.cx = cam->cx;
  oc.cy = cam->cy;
  std::memcpy(oc.w2c_R, cam->w2c_R, sizeof(oc.w2c_R));
  std::memcpy(oc.w2c_t, cam->w2c_t, sizeof(oc.w2c_t));
  std::memcpy(oc.c2w_R, cam->c2w_R, sizeof(oc.c2w_R));
  std::memcpy(oc.c2w_t, cam->c2w_t, sizeof(oc.c2w_t));
  oracle_option o{c->opt.diffuse_color, c->opt.interp, c->opt.shading_normal,
                  c->opt.diffuse_shading, c->opt.backface_culling, c->opt.oren_nayar_sigma};
  int rc = ray ? oracle_raytrace(&m, &oc, &o, c->opt.depth_scale, im->color, im->depth,
                                 im->normal, im->mask, im->face_id, im->color_f32, nullptr)
               : oracle_render(&m, &oc, &o, im->color, im->depth, im->normal, im->mask,
                               im->face_id, im->color_f32, nullptr);
  if (rc) c->err = "oracle validation failed";
  return rc;
}
int ugu_gpu_render(ugu_gpu_context* c, int32_t, const ugu_gpu_camera* cam,
                   const ugu_gpu_images* im) {
  return fake_render(c, cam, im, false);
}
int ugu_gpu_render_views(ugu_gpu_context* c, int32_t n, const ugu_gpu_view* v, uint32_t flags) {
  for (int i = 0; i < n; ++i) {
    int rc = fake_render(c, &v[i].camera, &v[i].images, (flags & UGU_GPU_RAYTRACE) != 0);
    if (rc) return rc;
  }
  return 0;
}
}
