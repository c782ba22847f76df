// drop_in_check.cc -- renders one scene with the reference's ugu::Rasterizer
// (ugu::Raytracer) and with ugu::RasterizerGpu (ugu::RaytracerGpu,
// ugu_gb300/host) and counts differing bytes.  Built by
// tests/test_drop_in_cpu.py against the reference headers.
#include <cstring>
#include <memory>

#include "rasterizer_gpu.h"
#include "ugu/renderer/cpu/rasterizer.h"
#include "ugu/renderer/cpu/raytracer.h"

namespace ugu {
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

template <typename T>
static long diff(const ugu::Image<T>& a, const ugu::Image<T>& b) {
  if (a.rows != b.rows || a.cols != b.cols) return -1;
  const size_t n = (size_t)a.rows * a.step[0];
  long d = 0;
  for (size_t i = 0; i < n; ++i) d += a.data[i] != b.data[i];
  return d;
}

template <typename Ref, typename Gpu>
static int check(int nv, const float* v, int nf, const int* f, const float* fn, const float* vn,
                 const float* vc, int nuv, const float* uv, const int* uvi, int tw, int th,
                 const unsigned char* tex, int W, int H, float fx, float fy, float cx, float cy,
                 const double* c2w, int dc, int interp, int sn, int shading, int cull,
                 float depth_scale, long* out6) {
  ugu::set_log_level(ugu::LogLevel::kError);
  auto mesh = std::make_shared<ugu::Mesh>();
  std::vector<Eigen::Vector3f> V(nv), N(nv), C(nv), FN(nf);
  std::vector<Eigen::Vector3i> F(nf), UI(nf);
  std::vector<Eigen::Vector2f> UV(nuv);
  for (int i = 0; i < nv; ++i) {
    V[i] = Eigen::Vector3f(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    N[i] = Eigen::Vector3f(vn[3 * i], vn[3 * i + 1], vn[3 * i + 2]);
    C[i] = Eigen::Vector3f(vc[3 * i], vc[3 * i + 1], vc[3 * i + 2]);
  }
  for (int i = 0; i < nf; ++i) {
    F[i] = Eigen::Vector3i(f[3 * i], f[3 * i + 1], f[3 * i + 2]);
    FN[i] = Eigen::Vector3f(fn[3 * i], fn[3 * i + 1], fn[3 * i + 2]);
    UI[i] = Eigen::Vector3i(uvi[3 * i], uvi[3 * i + 1], uvi[3 * i + 2]);
  }
  for (int i = 0; i < nuv; ++i) UV[i] = Eigen::Vector2f(uv[2 * i], uv[2 * i + 1]);
  mesh->set_vertices(V);
  mesh->set_vertex_indices(F);
  mesh->set_face_normals(FN);
  mesh->set_normals(N);
  mesh->set_normal_indices(F);
  mesh->set_vertex_colors(C);
  mesh->set_uv(UV);
  mesh->set_uv_indices(UI);
  mesh->set_material_ids(std::vector<int>(nf, 0));
  std::vector<ugu::ObjMaterial> mats(1);
  mats[0].diffuse_tex = ugu::Image3b::zeros(th, tw);
  std::memcpy(mats[0].diffuse_tex.data, tex, (size_t)tw * th * 3);
  mesh->set_materials(mats);
  Eigen::Matrix4d M;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) M(r, c) = c2w[4 * r + c];
  auto cam = std::make_shared<ugu::PinholeCamera>(W, H, Eigen::Affine3d(M),
                                                  Eigen::Vector2f(cx, cy), Eigen::Vector2f(fx, fy));
  ugu::RendererCpuOption opt;
  opt.diffuse_color = static_cast<ugu::DiffuseColor>(dc);
  opt.interp = static_cast<ugu::ColorInterpolation>(interp);
  opt.shading_normal = static_cast<ugu::ShadingNormal>(sn);
  opt.diffuse_shading = static_cast<ugu::DiffuseShading>(shading);
  opt.backface_culling = cull != 0;
  opt.depth_scale = depth_scale;

  Ref ref(opt);
  Gpu gpu(opt);
  std::shared_ptr<ugu::RendererCpu> r0(&ref, [](ugu::RendererCpu*) {});
  std::shared_ptr<ugu::RendererCpu> r1(&gpu, [](ugu::RendererCpu*) {});
  ugu::Image3b c[2];
  ugu::Image1f d[2];
  ugu::Image3f n[2];
  ugu::Image1b m[2];
  ugu::Image1i id[2];
  ugu::Image1w dw[2];
  int k = 0;
  for (auto& r : {r0, r1}) {  // both through the RendererCpu interface
    r->set_mesh(mesh);
    if (!r->PrepareMesh()) return 100 + k;
    r->set_camera(cam);
    if (!r->Render(&c[k], &d[k], &n[k], &m[k], &id[k])) return 200 + k;
    if (!r->RenderDepthW(&dw[k])) return 300 + k;
    ++k;
  }
  out6[0] = diff(c[0], c[1]);
  out6[1] = diff(d[0], d[1]);
  out6[2] = diff(n[0], n[1]);
  out6[3] = diff(m[0], m[1]);
  out6[4] = diff(id[0], id[1]);
  out6[5] = diff(dw[0], dw[1]);
  return 0;
}

extern "C" int drop_in_check(int nv, const float* v, int nf, const int* f, const float* fn,
                             const float* vn, const float* vc, int nuv, const float* uv,
                             const int* uvi, int tw, int th, const unsigned char* tex, int W,
                             int H, float fx, float fy, float cx, float cy, const double* c2w,
                             int dc, int interp, int sn, int shading, int cull, long* out6) {
  return check<ugu::Rasterizer, ugu::RasterizerGpu>(nv, v, nf, f, fn, vn, vc, nuv, uv, uvi, tw,
                                                    th, tex, W, H, fx, fy, cx, cy, c2w, dc,
                                                    interp, sn, shading, cull, 1.0f, out6);
}

extern "C" int drop_in_check_ray(int nv, const float* v, int nf, const int* f, const float* fn,
                                 const float* vn, const float* vc, int nuv, const float* uv,
                                 const int* uvi, int tw, int th, const unsigned char* tex, int W,
                                 int H, float fx, float fy, float cx, float cy, const double* c2w,
                                 int dc, int interp, int sn, int shading, int cull,
                                 float depth_scale, long* out6) {
  return check<ugu::Raytracer, ugu::RaytracerGpu>(nv, v, nf, f, fn, vn, vc, nuv, uv, uvi, tw,
                                                  th, tex, W, H, fx, fy, cx, cy, c2w, dc, interp,
                                                  sn, shading, cull, depth_scale, out6);
}

// Error paths that need no backend: no camera, mesh not prepared.
extern "C" int drop_in_errors() {
  ugu::set_log_level(ugu::LogLevel::kNone);
  ugu::RasterizerGpu gpu;
  ugu::Image1i id;
  if (gpu.RenderFaceId(&id)) return 1;  // camera has not been set
  gpu.set_camera(std::make_shared<ugu::PinholeCamera>(8, 8, 60.0f));
  if (gpu.RenderFaceId(&id)) return 2;  // mesh has not been initialized
  if (gpu.PrepareMesh()) return 3;      // mesh has not been set
  ugu::Image1w dw;
  if (gpu.RenderW(nullptr, nullptr, nullptr, nullptr, nullptr)) return 4;
  ugu::RaytracerGpu ray;
  if (ray.PrepareMesh()) return 5;  // mesh has not been set
  ray.set_mesh(std::make_shared<ugu::Mesh>());
  if (ray.PrepareMesh()) return 6;  // mesh is empty
  return 0;
}
