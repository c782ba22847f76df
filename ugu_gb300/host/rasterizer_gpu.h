/*
 * rasterizer_gpu.h -- ugu::RasterizerGpu, a drop-in for ugu::Rasterizer
 * (include/ugu/renderer/cpu/rasterizer.h:14-53) behind the same
 * ugu::RendererCpu interface (include/ugu/renderer/cpu/renderer.h:42-76).
 *
 * Compile it inside a ugu build (it includes ugu's headers) and link
 * libugugpu.so.  Behaviour matches ugu::Rasterizer: the same option copy
 * (RendererCpuOption::CopyTo keeps oren_nayar_sigma at its default), the same
 * validation messages through LOGE with a `false` return, outputs (re)sized
 * by the renderer, nullptr outputs skipped.  The images are computed on the
 * GPU by the kernels behind include/ugu_gpu.h and copied back before Render
 * returns.  Only PinholeCamera is supported (OpenCvCamera's distortion and
 * OrthoCamera are rejected with an error).
 *
 * ugu::RaytracerGpu is the same drop-in for ugu::Raytracer
 * (include/ugu/renderer/cpu/raytracer.h:14-53): its renders cast one ray per
 * pixel through the reference's naive BVH (UGU_GPU_RAYTRACE).
 */
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "ugu/renderer/cpu/renderer.h"

namespace ugu {

class RasterizerGpu : public RendererCpu {
  class Impl;
  std::unique_ptr<Impl> pimpl_;

 public:
  RasterizerGpu();
  ~RasterizerGpu() override;

  explicit RasterizerGpu(const RendererCpuOption& option, int device = 0);
  void set_option(const RendererCpuOption& option) override;

  void set_mesh(std::shared_ptr<const Mesh> mesh) override;

  // Should call after set_mesh() and before Render(); uploads the mesh.
  // Don't modify mesh outside after calling PrepareMesh()
  bool PrepareMesh() override;

  void set_camera(std::shared_ptr<const Camera> camera) override;

  bool Render(Image3b* color, Image1f* depth, Image3f* normal, Image1b* mask,
              Image1i* face_id) const override;

  bool RenderColor(Image3b* color) const override;
  bool RenderDepth(Image1f* depth) const override;
  bool RenderNormal(Image3f* normal) const override;
  bool RenderMask(Image1b* mask) const override;
  bool RenderFaceId(Image1i* face_id) const override;

  bool RenderW(Image3b* color, Image1w* depth, Image3f* normal, Image1b* mask,
               Image1i* face_id) const override;
  bool RenderDepthW(Image1w* depth) const override;

  // Extension: many cameras of the prepared mesh in one batched launch.
  // Output vectors may be nullptr; they are resized to cameras.size().
  bool RenderViews(const std::vector<std::shared_ptr<const Camera>>& cameras,
                   std::vector<Image3b>* colors, std::vector<Image1f>* depths,
                   std::vector<Image3f>* normals, std::vector<Image1b>* masks,
                   std::vector<Image1i>* face_ids) const;

 protected:
  // UGU_GPU_* flags added to every render (RaytracerGpu: UGU_GPU_RAYTRACE).
  void set_render_flags(uint32_t flags);
  bool has_mesh() const;       // a mesh was set
  bool has_mesh_data() const;  // ... with vertices and faces
};

class RaytracerGpu : public RasterizerGpu {
 public:
  RaytracerGpu();
  explicit RaytracerGpu(const RendererCpuOption& option, int device = 0);

  // raytracer.cc:90-110: fails on a missing or empty mesh.
  bool PrepareMesh() override;
};

}  // namespace ugu
