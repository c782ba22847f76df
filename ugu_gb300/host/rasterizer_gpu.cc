/*
 * rasterizer_gpu.cc -- ugu::RasterizerGpu over the C ABI of libugugpu.so.
 * See rasterizer_gpu.h.  The method bodies follow ugu::Rasterizer's
 * (src/renderer/cpu/rasterizer.cc:68-404) with the two render loops replaced
 * by one call into the GPU library.
 */
#include "rasterizer_gpu.h"

#include <cstring>

#include "ugu/camera.h"
#include "ugu/image_proc.h"
#include "ugu_gpu.h"

namespace ugu {

namespace {

// The float camera parameters Rasterizer::Impl::Render reads, computed by
// the same Eigen expressions (rasterizer.cc:118-119, camera.h:321, 380-387).
bool FillCamera(const Camera& cam, ugu_gpu_camera* out) {
  const auto* pin = dynamic_cast<const PinholeCamera*>(&cam);
  if (pin == nullptr || dynamic_cast<const OpenCvCamera*>(&cam) != nullptr) return false;
  out->width = cam.width();
  out->height = cam.height();
  out->fx = pin->focal_length()[0];
  out->fy = pin->focal_length()[1];
  out->cx = pin->principal_point()[0];
  out->cy = pin->principal_point()[1];
  const Eigen::Matrix3f w2c_R = cam.w2c().rotation().cast<float>();
  const Eigen::Vector3f w2c_t = cam.w2c().translation().cast<float>();
  const Eigen::Matrix3f c2w_R = cam.c2w().matrix().block<3, 3>(0, 0).cast<float>();
  const Eigen::Vector3f c2w_t = cam.c2w().matrix().block<3, 1>(0, 3).cast<float>();
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) {
      out->w2c_R[3 * r + c] = w2c_R(r, c);
      out->c2w_R[3 * r + c] = c2w_R(r, c);
    }
    out->w2c_t[r] = w2c_t[r];
    out->c2w_t[r] = c2w_t[r];
  }
  return true;
}

template <typename T>
void Resize(Image<T>* img, int w, int h) {
  if (img->cols != w || img->rows != h) *img = Image<T>::zeros(h, w);
}

}  // namespace

class RasterizerGpu::Impl {
 public:
  bool mesh_initialized_{false};
  std::shared_ptr<const Camera> camera_{nullptr};
  std::shared_ptr<const Mesh> mesh_{nullptr};
  RendererCpuOption option_;
  ugu_gpu_context* ctx_{nullptr};
  int device_{0};
  uint32_t flags_{0};  // UGU_GPU_RAYTRACE for RaytracerGpu

  explicit Impl(int device) : device_(device) {}
  ~Impl() { ugu_gpu_destroy(ctx_); }

  bool EnsureContext() {
    if (ctx_) return true;
    int rc = ugu_gpu_create(device_, &ctx_);
    if (rc != UGU_GPU_OK) {
      LOGE("GPU rasterizer unavailable: %s\n", ugu_gpu_last_error(nullptr));
      ctx_ = nullptr;
      return false;
    }
    return true;
  }

  bool PushOption() const {
    ugu_gpu_option o;
    o.diffuse_color = static_cast<int32_t>(option_.diffuse_color);
    o.interp = static_cast<int32_t>(option_.interp);
    o.shading_normal = static_cast<int32_t>(option_.shading_normal);
    o.diffuse_shading = static_cast<int32_t>(option_.diffuse_shading);
    o.depth_scale = option_.depth_scale;
    o.backface_culling = option_.backface_culling ? 1 : 0;
    o.oren_nayar_sigma = option_.oren_nayar_sigma;
    if (ugu_gpu_set_option(ctx_, &o) != UGU_GPU_OK) {
      LOGE("%s\n", ugu_gpu_last_error(ctx_));
      return false;
    }
    return true;
  }

  bool Upload() {
    if (!EnsureContext()) return false;
    const Mesh& m = *mesh_;
    ugu_gpu_mesh d;
    std::memset(&d, 0, sizeof(d));
    // std::vector<Eigen::Vector3f> stores x, y, z contiguously (no padding).
    static_assert(sizeof(Eigen::Vector3f) == 12 && sizeof(Eigen::Vector3i) == 12 &&
                      sizeof(Eigen::Vector2f) == 8,
                  "packed Eigen vectors expected");
    d.num_vertices = static_cast<int32_t>(m.vertices().size());
    d.vertices = reinterpret_cast<const float*>(m.vertices().data());
    d.num_faces = static_cast<int32_t>(m.vertex_indices().size());
    d.vertex_indices = reinterpret_cast<const int32_t*>(m.vertex_indices().data());
    if (m.face_normals().size() == m.vertex_indices().size() && !m.face_normals().empty())
      d.face_normals = reinterpret_cast<const float*>(m.face_normals().data());
    if (!m.normals().empty() && m.normal_indices().size() == m.vertex_indices().size()) {
      d.num_normals = static_cast<int32_t>(m.normals().size());
      d.normals = reinterpret_cast<const float*>(m.normals().data());
      d.normal_indices = reinterpret_cast<const int32_t*>(m.normal_indices().data());
    }
    if (m.vertex_colors().size() == m.vertices().size() && !m.vertex_colors().empty())
      d.vertex_colors = reinterpret_cast<const float*>(m.vertex_colors().data());
    if (!m.uv().empty() && m.uv_indices().size() == m.vertex_indices().size()) {
      d.num_uv = static_cast<int32_t>(m.uv().size());
      d.uv = reinterpret_cast<const float*>(m.uv().data());
      d.uv_indices = reinterpret_cast<const int32_t*>(m.uv_indices().data());
    }
    if (m.material_ids().size() == m.vertex_indices().size() && !m.material_ids().empty())
      d.material_ids = m.material_ids().data();
    std::vector<ugu_gpu_texture> tex(m.materials().size());
    for (size_t i = 0; i < tex.size(); ++i) {
      const Image3b& t = m.materials()[i].diffuse_tex;
      tex[i].width = t.empty() ? 0 : t.cols;
      tex[i].height = t.empty() ? 0 : t.rows;
      tex[i].rgb8 = t.empty() ? nullptr : t.data;
      tex[i].rgb_f32 = nullptr;
    }
    d.num_materials = static_cast<int32_t>(tex.size());
    d.materials = tex.empty() ? nullptr : tex.data();
    if (ugu_gpu_set_mesh(ctx_, 0, &d) != UGU_GPU_OK) {
      LOGE("%s\n", ugu_gpu_last_error(ctx_));
      return false;
    }
    return true;
  }

  bool Render(Image3b* color, Image1f* depth, Image3f* normal, Image1b* mask,
              Image1i* face_id) const {
    // ValidateAndInitBeforeRender (util_private.cc:19-26) before the GPU
    // checks the remaining preconditions in the same order.
    if (camera_ == nullptr) {
      LOGE("camera has not been set\n");
      return false;
    }
    if (!mesh_initialized_) {
      LOGE("mesh has not been initialized\n");
      return false;
    }
    ugu_gpu_camera cam;
    if (!FillCamera(*camera_, &cam)) {
      LOGE("RasterizerGpu supports ugu::PinholeCamera only\n");
      return false;
    }
    if (!PushOption()) return false;
    const int w = camera_->width(), h = camera_->height();
    if (color) Resize(color, w, h);
    if (depth) Resize(depth, w, h);
    if (normal) Resize(normal, w, h);
    if (mask) Resize(mask, w, h);
    if (face_id) Resize(face_id, w, h);
    ugu_gpu_images im;
    im.color = color ? color->data : nullptr;
    im.depth = depth ? reinterpret_cast<float*>(depth->data) : nullptr;
    im.normal = normal ? reinterpret_cast<float*>(normal->data) : nullptr;
    im.mask = mask ? mask->data : nullptr;
    im.face_id = face_id ? reinterpret_cast<int32_t*>(face_id->data) : nullptr;
    im.color_f32 = nullptr;
    ugu_gpu_view v;
    v.mesh = 0;
    v.camera = cam;
    v.images = im;
    const int rc = ugu_gpu_render_views(ctx_, 1, &v, flags_);
    if (rc != UGU_GPU_OK) {
      LOGE("%s\n", ugu_gpu_last_error(ctx_));
      return false;
    }
    return true;
  }
};

RasterizerGpu::RasterizerGpu() : pimpl_(new Impl(0)) {}

void RasterizerGpu::set_render_flags(uint32_t flags) { pimpl_->flags_ = flags; }

bool RasterizerGpu::has_mesh() const { return pimpl_->mesh_ != nullptr; }

bool RasterizerGpu::has_mesh_data() const {
  return pimpl_->mesh_ != nullptr && !pimpl_->mesh_->vertices().empty() &&
         !pimpl_->mesh_->vertex_indices().empty();
}
RasterizerGpu::~RasterizerGpu() {}
RasterizerGpu::RasterizerGpu(const RendererCpuOption& option, int device)
    : pimpl_(new Impl(device)) {
  set_option(option);
}

void RasterizerGpu::set_option(const RendererCpuOption& option) {
  option.CopyTo(&pimpl_->option_);  // rasterizer.cc:73-75
}

void RasterizerGpu::set_mesh(std::shared_ptr<const Mesh> mesh) {  // rasterizer.cc:77-88
  pimpl_->mesh_initialized_ = false;
  pimpl_->mesh_ = mesh;
  if (mesh->face_normals().empty()) {
    LOGW("face normal is empty. culling and shading may not work\n");
  }
  if (mesh->normals().empty()) {
    LOGW("vertex normal is empty. shading may not work\n");
  }
}

bool RasterizerGpu::PrepareMesh() {  // rasterizer.cc:90-99, plus the upload
  if (pimpl_->mesh_ == nullptr) {
    LOGE("mesh has not been set\n");
    return false;
  }
  if (!pimpl_->Upload()) return false;
  pimpl_->mesh_initialized_ = true;
  return true;
}

void RasterizerGpu::set_camera(std::shared_ptr<const Camera> camera) {
  pimpl_->camera_ = camera;
}

bool RasterizerGpu::Render(Image3b* color, Image1f* depth, Image3f* normal, Image1b* mask,
                           Image1i* face_id) const {
  return pimpl_->Render(color, depth, normal, mask, face_id);
}

bool RasterizerGpu::RenderColor(Image3b* color) const {
  return Render(color, nullptr, nullptr, nullptr, nullptr);
}
bool RasterizerGpu::RenderDepth(Image1f* depth) const {
  return Render(nullptr, depth, nullptr, nullptr, nullptr);
}
bool RasterizerGpu::RenderNormal(Image3f* normal) const {
  return Render(nullptr, nullptr, normal, nullptr, nullptr);
}
bool RasterizerGpu::RenderMask(Image1b* mask) const {
  return Render(nullptr, nullptr, nullptr, mask, nullptr);
}
bool RasterizerGpu::RenderFaceId(Image1i* face_id) const {
  return Render(nullptr, nullptr, nullptr, nullptr, face_id);
}

bool RasterizerGpu::RenderW(Image3b* color, Image1w* depth, Image3f* normal, Image1b* mask,
                            Image1i* face_id) const {  // rasterizer.cc:329-344
  if (depth == nullptr) {
    LOGE("depth is nullptr");
    return false;
  }
  Image1f f_depth;
  bool org_ret = Render(color, &f_depth, normal, mask, face_id);
  if (org_ret) {
    ConvertTo(f_depth, depth);
  }
  return org_ret;
}

bool RasterizerGpu::RenderDepthW(Image1w* depth) const {
  return RenderW(nullptr, depth, nullptr, nullptr, nullptr);
}

bool RasterizerGpu::RenderViews(const std::vector<std::shared_ptr<const Camera>>& cameras,
                                std::vector<Image3b>* colors, std::vector<Image1f>* depths,
                                std::vector<Image3f>* normals, std::vector<Image1b>* masks,
                                std::vector<Image1i>* face_ids) const {
  Impl& p = *pimpl_;
  if (!p.mesh_initialized_) {
    LOGE("mesh has not been initialized\n");
    return false;
  }
  if (!p.PushOption()) return false;
  const size_t n = cameras.size();
  if (colors) colors->resize(n);
  if (depths) depths->resize(n);
  if (normals) normals->resize(n);
  if (masks) masks->resize(n);
  if (face_ids) face_ids->resize(n);
  std::vector<ugu_gpu_view> views(n);
  for (size_t i = 0; i < n; ++i) {
    if (!cameras[i] || !FillCamera(*cameras[i], &views[i].camera)) {
      LOGE("camera %d is missing or not a ugu::PinholeCamera\n", static_cast<int>(i));
      return false;
    }
    const int w = cameras[i]->width(), h = cameras[i]->height();
    views[i].mesh = 0;
    ugu_gpu_images& im = views[i].images;
    std::memset(&im, 0, sizeof(im));
    if (colors) Resize(&(*colors)[i], w, h), im.color = (*colors)[i].data;
    if (depths)
      Resize(&(*depths)[i], w, h), im.depth = reinterpret_cast<float*>((*depths)[i].data);
    if (normals)
      Resize(&(*normals)[i], w, h), im.normal = reinterpret_cast<float*>((*normals)[i].data);
    if (masks) Resize(&(*masks)[i], w, h), im.mask = (*masks)[i].data;
    if (face_ids)
      Resize(&(*face_ids)[i], w, h),
          im.face_id = reinterpret_cast<int32_t*>((*face_ids)[i].data);
  }
  const int rc = ugu_gpu_render_views(p.ctx_, static_cast<int32_t>(n), views.data(), p.flags_);
  if (rc != UGU_GPU_OK) {
    LOGE("%s\n", ugu_gpu_last_error(p.ctx_));
    return false;
  }
  return true;
}

RaytracerGpu::RaytracerGpu() : RasterizerGpu() { set_render_flags(UGU_GPU_RAYTRACE); }

RaytracerGpu::RaytracerGpu(const RendererCpuOption& option, int device)
    : RasterizerGpu(option, device) {
  set_render_flags(UGU_GPU_RAYTRACE);
}

// raytracer.cc:90-110: "mesh has not been set" (reported by the base), then
// "mesh is empty"; the BVH itself is built on the device side at the first
// render.
bool RaytracerGpu::PrepareMesh() {
  if (has_mesh() && !has_mesh_data()) {
    LOGE("mesh is empty\n");
    return false;
  }
  return RasterizerGpu::PrepareMesh();
}

}  // namespace ugu
