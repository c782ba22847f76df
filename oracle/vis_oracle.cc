/* vis_oracle.cc -- TEST INFRASTRUCTURE ONLY.
 *
 * The image helpers ugu's examples apply to a render, restated per pixel
 * with the same standard-library calls the reference makes:
 *   Depth2Gray          src/util/image_util.cc:392-411
 *   Normal2Color        src/util/image_util.cc:413-446 (RGB order, no OpenCV)
 *   FaceId2RandomColor  src/util/image_util.cc:448-487 (std::mt19937(fid),
 *                       three draws mod 256, RGB order)
 *   ConvertTo<uint16_t> include/ugu/image_proc.h:453-475 with scale 1
 * (src/util/image_util.cc itself needs Eigen's dynamic matrices, which the
 * Eigen-compatible shim does not provide, so it is not built here.)  The
 * double-to-integer casts, undefined by C++ outside the target range, take
 * the low bits of the truncated int32 value, as the GPU does.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>

namespace {

int32_t trunc_i32(double v) {
  if (!(v == v)) return 0;
  if (v >= 2147483647.0) return 2147483647;
  if (v <= -2147483648.0) return (int32_t)-2147483647 - 1;
  return (int32_t)v;
}

}  // namespace

extern "C" void oracle_visualize(int32_t width, int32_t height, const float* depth,
                                 const float* normal, const int32_t* face_id, uint8_t* vis_depth,
                                 uint16_t* depth_u16, uint8_t* vis_normal, uint8_t* vis_face_id,
                                 float min_d, float max_d, int32_t gl_coord) {
  const size_t n = (size_t)width * (size_t)height;
  const float inv_denom = 1.0f / (max_d - min_d);
  for (size_t i = 0; i < n; ++i) {
    if (depth && vis_depth) {
      float norm_color = (depth[i] - min_d) * inv_denom;
      norm_color = std::min(std::max(norm_color, 0.0f), 1.0f);
      vis_depth[i] = (uint8_t)(uint32_t)trunc_i32(norm_color * 255);
    }
    if (depth && depth_u16) depth_u16[i] = (uint16_t)(uint32_t)trunc_i32(1.0f * (double)depth[i]);
    if (normal && vis_normal) {
      float nv[3] = {normal[3 * i], normal[3 * i + 1], normal[3 * i + 2]};
      if (gl_coord) {
        nv[0] *= -1.f;
        nv[2] *= -1.f;
      }
      vis_normal[3 * i + 0] = (uint8_t)(uint32_t)trunc_i32(std::round((nv[0] + 1.0) * 0.5 * 255));
      vis_normal[3 * i + 1] = (uint8_t)(uint32_t)trunc_i32(std::round((nv[1] + 1.0) * 0.5 * 255));
      vis_normal[3 * i + 2] = (uint8_t)(uint32_t)trunc_i32(std::round(-nv[2] * 127.0) + 128);
    }
    if (face_id && vis_face_id) {
      const int fid = face_id[i];
      uint8_t c[3] = {0, 0, 0};
      if (fid >= 0) {
        std::mt19937 mt(fid);
        c[0] = static_cast<uint8_t>(mt() % 256);
        c[1] = static_cast<uint8_t>(mt() % 256);
        c[2] = static_cast<uint8_t>(mt() % 256);
      }
      vis_face_id[3 * i + 0] = c[0];
      vis_face_id[3 * i + 1] = c[1];
      vis_face_id[3 * i + 2] = c[2];
    }
  }
}
