/* vis_oracle.cc -- TEST INFRASTRUCTURE ONLY.
 *
 * The image helpers ugu's examples apply to a render, restated per pixel
 * with the same standard-library calls the reference makes:
 *   Depth2Gray          src/util/image_util.cc:392-411
 *   Normal2Color        src/util/image_util.cc:413-446 (RGB order, no OpenCV)
 *   FaceId2RandomColor  src/util/image_util.cc:448-487 (std::mt19937(fid),
 *                       three draws mod 256, RGB order)
 *   ConvertTo<uint16_t> include/ugu/image_proc.h:453-475 with scale 1
 * Pinned, where the cast is defined, to src/util/image_util.cc itself,
 * built into oracle/_ref against the Eigen-compatible shim
 * (tests/test_vis.py).  The double-to-integer casts, undefined by C++
 * outside the target range, take the low bits of the truncated int32 value,
 * as the GPU does.  The texture mapping restatements below are pinned to
 * the reference's own texture_mapper.cc and bin_packer_2d.cc the same way
 * (tests/test_texture_mapping.py).
 */
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <deque>
#include <map>
#include <random>
#include <utility>
#include <vector>

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

/* TextureMapping with kSimpleProjection and kUseOriginalMeshUv
 * (src/texturing/texture_mapper.cc:924-1006 and :294-345): faces in order,
 * each one's uv triangle rasterized into a tex_w x tex_h texture
 * (RasterizeTriangle, :234-292) with texels sampled from its keyframe's
 * colour image at the same barycentric point of the face's projected
 * triangle (BilinearInterpolation, include/ugu/util/image_util.h:156-192);
 * a later face overwrites an earlier one.  Then PaddingSimple (:148-201).
 * face_kf[f] is the id of the face's best keyframe (-1: none); like the
 * reference, the id indexes the keyframe list.  Returns 0, or -1 when an id
 * is outside the list.  Pixel reads outside an image's allocation are
 * clamped to it. */
namespace {

constexpr float FLT_MIN_ = 1.17549435e-38f;  // std::numeric_limits<float>::min()

float edge(float ax, float ay, float bx, float by, float cx, float cy) {
  return (cx - ax) * (by - ay) - (cy - ay) * (bx - ax);
}

uint8_t f2u8(float v) { return (uint8_t)(uint32_t)trunc_i32((double)v); }

void bilinear3(float x, float y, const uint8_t* img, int32_t cols, int32_t rows, uint8_t out[3]) {
  int32_t x0 = trunc_i32((double)std::floor(x)), y0 = trunc_i32((double)std::floor(y));
  int32_t x1 = x0 + 1, y1 = y0 + 1;
  if (x0 < 0) x0 = 0;
  if (y0 < 0) y0 = 0;
  if (cols <= x1) x1 = cols - 1;
  if (rows <= y1) y1 = rows - 1;
  const float lu = x - (float)x0, lv = y - (float)y0;
  const int64_t n = (int64_t)cols * rows;
  auto px = [&](int32_t yy, int32_t xx) {
    int64_t i = (int64_t)yy * cols + xx;
    i = i < 0 ? 0 : (i >= n ? n - 1 : i);
    return img + 3 * i;
  };
  const uint8_t *a = px(y0, x0), *b = px(y0, x1), *c = px(y1, x0), *d = px(y1, x1);
  for (int k = 0; k < 3; ++k) {
    const float v = (1.0f - lu) * (1.0f - lv) * (float)a[k] + lu * (1.0f - lv) * (float)b[k] +
                    (1.0f - lu) * lv * (float)c[k] + lu * lv * (float)d[k];
    out[k] = f2u8(v);
  }
}

}  // namespace

// RasterizeTriangle (texture_mapper.cc:234-292) for every face in order:
// face f's target triangle (texel coordinates, tx/ty) sampled from its
// keyframe's image at the same barycentric point of face_tri[f].
static int draw_faces(int32_t num_faces, const float* target, int32_t num_kf,
                      const int32_t* kf_w, const int32_t* kf_h, const uint8_t* const* kf_color,
                      const int32_t* face_kf, const float* face_tri, int32_t tex_w,
                      int32_t tex_h, uint8_t* texture, uint8_t* mask) {
  for (int32_t f = 0; f < num_faces; ++f) {
    const int32_t k = face_kf[f];
    if (k < 0) continue;
    if (k >= num_kf) return -1;
    float tx[3], ty[3];
    for (int j = 0; j < 3; ++j) {
      tx[j] = target[6 * (size_t)f + 2 * j];
      ty[j] = target[6 * (size_t)f + 2 * j + 1];
    }
    const float* s = face_tri + 6 * (size_t)f;
    float area = edge(tx[0], ty[0], tx[1], ty[1], tx[2], ty[2]);
    if (std::fabs(area) < FLT_MIN_) area = area > 0 ? FLT_MIN_ : -FLT_MIN_;
    const float inv_area = 1.0f / area;
    auto clampi = [](int32_t v, int32_t hi) { return std::max(0, std::min(v, hi)); };
    const int32_t xmin = clampi(trunc_i32((double)(std::min({tx[0], tx[1], tx[2]}) - 1)), tex_w - 1);
    const int32_t xmax = clampi(trunc_i32((double)(std::max({tx[0], tx[1], tx[2]}) + 1)), tex_w - 1);
    const int32_t ymin = clampi(trunc_i32((double)(std::min({ty[0], ty[1], ty[2]}) - 1)), tex_h - 1);
    const int32_t ymax = clampi(trunc_i32((double)(std::max({ty[0], ty[1], ty[2]}) + 1)), tex_h - 1);
    for (int32_t y = ymin; y <= ymax; ++y)
      for (int32_t x = xmin; x <= xmax; ++x) {
        const float px = (float)x, py = (float)y;
        float w0 = edge(tx[1], ty[1], tx[2], ty[2], px, py);
        float w1 = edge(tx[2], ty[2], tx[0], ty[0], px, py);
        float w2 = edge(tx[0], ty[0], tx[1], ty[1], px, py);
        w0 *= inv_area;
        w1 *= inv_area;
        w2 *= inv_area;
        if (w0 < 0 || w1 < 0 || w2 < 0) continue;
        const float sx = w0 * s[0] + w1 * s[2] + w2 * s[4];
        const float sy = w0 * s[1] + w1 * s[3] + w2 * s[5];
        bilinear3(sx, sy, kf_color[k], kf_w[k], kf_h[k], texture + 3 * ((size_t)y * tex_w + x));
        mask[(size_t)y * tex_w + x] = 255;
      }
  }
  return 0;
}

// PaddingSimple (texture_mapper.cc:148-201): each empty texel away from
// the border takes the float mean of the valid texels of its kernel
// window, read before any fill.
static void pad_simple(int32_t tex_w, int32_t tex_h, int32_t padding_kernel, uint8_t* texture,
                       uint8_t* mask);

// GenerateTextureOnOriginalUv (texture_mapper.cc:294-345): the target
// triangles from the mesh's uv.
extern "C" int oracle_texture_mapping(int32_t num_faces, const float* uv, const int32_t* uv_idx,
                                      int32_t num_kf, const int32_t* kf_w, const int32_t* kf_h,
                                      const uint8_t* const* kf_color, const int32_t* face_kf,
                                      const float* face_tri, int32_t tex_w, int32_t tex_h,
                                      int32_t padding_kernel, uint8_t* texture, uint8_t* mask) {
  const size_t n = (size_t)tex_w * tex_h;
  std::fill(texture, texture + 3 * n, 0);
  std::fill(mask, mask + n, 0);
  std::vector<float> target(6 * (size_t)std::max(num_faces, 0));
  for (int32_t f = 0; f < num_faces; ++f)
    for (int j = 0; j < 3; ++j) {
      const float* t = uv + 2 * (size_t)uv_idx[3 * (size_t)f + j];
      target[6 * (size_t)f + 2 * j] = t[0] * (float)tex_w - 0.5f;
      target[6 * (size_t)f + 2 * j + 1] = (1.0f - t[1]) * (float)tex_h - 0.5f;
    }
  if (draw_faces(num_faces, target.data(), num_kf, kf_w, kf_h, kf_color, face_kf, face_tri,
                 tex_w, tex_h, texture, mask))
    return -1;
  pad_simple(tex_w, tex_h, padding_kernel, texture, mask);
  return 0;
}

// GenerateSimpleTrianglesTextureAndUv's layout (texture_mapper.cc:347-440):
// the faces' target triangles (texel coordinates) and uv, zeros for faces
// without a keyframe; -1 where the reference returns false.
extern "C" int oracle_simple_triangles_layout(int32_t num_faces, const int32_t* face_kf,
                                              int32_t tex_w, int32_t tex_h, float* target,
                                              float* uv) {
  const int padding_tri = 2;
  const int rect_num = (num_faces + 1) / 2;
  std::fill(target, target + 6 * (size_t)num_faces, 0.0f);
  std::fill(uv, uv + 6 * (size_t)num_faces, 0.0f);
  if (rect_num == 0) return 0;
  const int pix_per_rect = tex_h * tex_w / rect_num;
  if (pix_per_rect < 6) return -1;
  const int max_rect_edge_len = 100;
  int sq_len = std::min(static_cast<int>(std::sqrt(pix_per_rect)), max_rect_edge_len);
  int max_rect_num = (tex_w / (sq_len + 2 + padding_tri)) * (tex_h / (sq_len + 1 + padding_tri));
  while (max_rect_num < rect_num) {
    sq_len--;
    if (sq_len < 3) return -1;
    max_rect_num = (tex_w / (sq_len + 2 + padding_tri)) * (tex_h / (sq_len + 1 + padding_tri));
  }
  const int rect_w = sq_len + 2, rect_h = sq_len + 1;
  const int rect_w_num = tex_w / (rect_w + padding_tri);
  for (int i = 0; i < num_faces; ++i) {
    if (face_kf[i] < 0) continue;
    const int rect_id = i / 2, rect_x = rect_id % rect_w_num, rect_y = rect_id / rect_w_num;
    float tx[3], ty[3];
    if (i % 2 == 0) {
      const int x0 = (rect_w + padding_tri) * rect_x + 2, x1 = x0 + sq_len - 1;
      const int y0 = (rect_h + padding_tri) * rect_y, y1 = y0 + sq_len - 1;
      tx[0] = (float)x0; ty[0] = (float)y0;
      tx[1] = (float)x1; ty[1] = (float)y0;
      tx[2] = (float)x1; ty[2] = (float)y1;
    } else {
      const int x0 = (rect_w + padding_tri) * rect_x, x1 = x0 + sq_len - 1;
      const int y0 = (rect_h + padding_tri) * rect_y + 1, y1 = y0 + sq_len - 1;
      tx[0] = (float)x0; ty[0] = (float)y0;
      tx[1] = (float)x0; ty[1] = (float)y1;
      tx[2] = (float)x1; ty[2] = (float)y1;
    }
    for (int j = 0; j < 3; ++j) {
      target[6 * (size_t)i + 2 * j] = tx[j];
      target[6 * (size_t)i + 2 * j + 1] = ty[j];
      uv[6 * (size_t)i + 2 * j] = (tx[j] + 0.5f) / tex_w;
      uv[6 * (size_t)i + 2 * j + 1] = 1.0f - ((ty[j] + 0.5f) / tex_h);
    }
  }
  return 0;
}

// kGenerateSimpleTriangles end to end: the layout, the faces drawn into it,
// a 3-texel padding (:430).
extern "C" int oracle_simple_triangles(int32_t num_faces, int32_t num_kf, const int32_t* kf_w,
                                       const int32_t* kf_h, const uint8_t* const* kf_color,
                                       const int32_t* face_kf, const float* face_tri,
                                       int32_t tex_w, int32_t tex_h, uint8_t* texture,
                                       uint8_t* mask, float* uv) {
  const size_t n = (size_t)tex_w * tex_h;
  std::fill(texture, texture + 3 * n, 0);
  std::fill(mask, mask + n, 0);
  std::vector<float> target(6 * (size_t)std::max(num_faces, 0));
  if (oracle_simple_triangles_layout(num_faces, face_kf, tex_w, tex_h, target.data(), uv))
    return -1;
  if (draw_faces(num_faces, target.data(), num_kf, kf_w, kf_h, kf_color, face_kf, face_tri,
                 tex_w, tex_h, texture, mask))
    return -1;
  pad_simple(tex_w, tex_h, 3, texture, mask);
  return 0;
}

// GenerateSimpleTileTextureAndUv (texture_mapper.cc:62-141) with
// MakeTiledImage (:29-60): the keyframe images tiled (int)sqrt(n) wide, and
// the faces' uv on their keyframe's tile (an unknown keyframe id maps to
// tile 0); -1 where the images differ in size or do not fill whole rows.
extern "C" int oracle_simple_tile(int32_t num_kf, const int32_t* kf_id, const int32_t* kf_w,
                                  const int32_t* kf_h, const uint8_t* const* kf_color,
                                  int32_t num_faces, const int32_t* face_kf,
                                  const float* face_tri, int32_t* tiles, uint8_t* texture,
                                  float* uv) {
  if (num_kf <= 0) return -1;
  const int default_x = static_cast<int>(std::sqrt(num_kf));
  const int x_tile_num = num_kf < default_x ? num_kf : default_x;
  const int y_tile_num = num_kf / x_tile_num;
  const int org_w = kf_w[0], org_h = kf_h[0];
  for (int i = 0; i < num_kf; ++i)
    if (kf_w[i] != org_w || kf_h[i] != org_h) return -1;
  if (num_kf % x_tile_num) return -1;
  tiles[0] = x_tile_num;
  tiles[1] = y_tile_num;
  const int tex_w = x_tile_num * org_w, tex_h = y_tile_num * org_h;
  if (texture)
    for (int i = 0; i < num_kf; ++i) {
      const int tpx = (i % x_tile_num) * org_w, tpy = (i / x_tile_num) * org_h;
      for (int j = 0; j < org_h; ++j)
        std::copy(kf_color[i] + (size_t)org_w * 3 * j, kf_color[i] + (size_t)org_w * 3 * (j + 1),
                  texture + ((size_t)(tpy + j) * tex_w + tpx) * 3);
    }
  for (int f = 0; f < num_faces; ++f) {
    float* u = uv + 6 * (size_t)f;
    if (face_kf[f] < 0) {
      std::fill(u, u + 6, 0.0f);
      continue;
    }
    int index = 0;  // the first position of the id (emplace keeps it)
    for (int i = 0; i < num_kf; ++i)
      if (kf_id[i] == face_kf[f]) {
        index = i;
        break;
      }
    const int tpx = (index % x_tile_num) * org_w, tpy = (index / x_tile_num) * org_h;
    for (int j = 0; j < 3; ++j) {
      const float x = face_tri[6 * (size_t)f + 2 * j] + tpx;
      const float y = face_tri[6 * (size_t)f + 2 * j + 1] + tpy;
      u[2 * j] = (x + 0.5f) / tex_w;
      u[2 * j + 1] = 1.0f - ((y + 0.5f) / tex_h);
    }
  }
  return 0;
}

static void pad_simple(int32_t tex_w, int32_t tex_h, int32_t padding_kernel, uint8_t* texture,
                       uint8_t* mask) {
  const size_t n = (size_t)tex_w * tex_h;
  std::vector<uint8_t> org_t(texture, texture + 3 * n), org_m(mask, mask + n);
  const int32_t hk = padding_kernel / 2;
  for (int32_t j = hk; j < tex_h - hk; ++j)
    for (int32_t i = hk; i < tex_w - hk; ++i) {
      if (org_m[(size_t)j * tex_w + i] == 255) continue;
      float sum[3] = {0, 0, 0};
      int cnt = 0;
      for (int32_t jj = -hk; jj <= hk; ++jj)
        for (int32_t ii = -hk; ii <= hk; ++ii) {
          const size_t q = (size_t)(j + jj) * tex_w + (i + ii);
          if (org_m[q] != 255) continue;
          for (int c = 0; c < 3; ++c) sum[c] += (float)org_t[3 * q + c];
          ++cnt;
        }
      if (!cnt) continue;
      const size_t p = (size_t)j * tex_w + i;
      mask[p] = 255;
      for (int c = 0; c < 3; ++c) texture[3 * p + c] = f2u8(sum[c] / (float)cnt);
    }
}

// GenerateSimpleChartsTextureAndUv with GenerateAtlas (texture_mapper.cc:
// 476-922), BinPacking2D (src/discrete/bin_packer_2d.cc:14-113), the
// FaceAdjacency edge lookups (include/ugu/face_adjacency.h:49-151, 194-209)
// and PaddingBorderSimple (texture_mapper.cc:203-231).  Charts of equal
// patch area keep their chart order (std::stable_sort; libstdc++'s
// std::sort leaves it unspecified).  Called with texture == NULL it only
// reports the texture size (dims[0], dims[1]) and the uv count (dims[2]).
// Returns 0, -1 when nothing packs within 8192, -2 for a patch outside its
// keyframe image, -3 for an edge sum that names no face (the reference then
// reads past its arrays).
namespace {

struct ORect {
  int x, y, w, h;
};

bool bin_packing(const std::vector<ORect>& rects, std::vector<ORect>* packed,
                 std::vector<ORect>* avail, int x_min, int x_max, int y_min, int y_max) {
  avail->assign(1, ORect{x_min, y_min, x_max, y_max});
  packed->clear();
  for (const ORect& r : rects) {
    for (;;) {
      int best = -1, best_diff = 2147483647;
      for (int i = 0; i < (int)avail->size(); ++i) {
        const ORect& a = (*avail)[i];
        if (r.h <= a.h && r.w <= a.w && a.w * a.h - r.w * r.h < best_diff) {
          best_diff = a.w * a.h - r.w * r.h;
          best = i;
        }
      }
      if (best < 0 || (*avail)[best].w * (*avail)[best].h < r.w * r.h) return false;
      const ORect b = (*avail)[best];
      if (b.w == r.w && b.h == r.h) {
        packed->push_back(b);
        avail->erase(avail->begin() + best);
        break;
      }
      ORect c1, c2;
      if (b.h - r.h > b.w - r.w) {
        c1 = ORect{b.x, b.y, b.w, r.h};
        c2 = ORect{b.x, b.y + r.h, b.w, b.h - r.h};
      } else {
        c1 = ORect{b.x, b.y, r.w, b.h};
        c2 = ORect{b.x + r.w, b.y, b.w - r.w, b.h};
      }
      avail->erase(avail->begin() + best);
      avail->push_back(c2);
      avail->push_back(c1);
    }
  }
  return true;
}

struct OChart {
  int w = 0, h = 0;
  std::vector<uint8_t> patch;
  std::vector<std::pair<float, float>> pos;       // per chart vertex, vertex-id order
  std::vector<std::pair<int, std::array<int, 3>>> face_idx;
};

}  // namespace

extern "C" int oracle_simple_charts(int32_t num_faces, const int32_t* vidx, const int32_t* face_kf,
                                    const float* face_tri, int32_t num_kf, const int32_t* kf_w,
                                    const int32_t* kf_h, const uint8_t* const* kf_color,
                                    int32_t tex_w, int32_t tex_h, int32_t* dims,
                                    uint8_t* texture, float* uv, int32_t* uv_indices) {
  const int F = num_faces;
  std::map<std::pair<int, int>, long long> edges;
  for (int f = 0; f < F; ++f) {
    const int* v = vidx + 3 * (size_t)f;
    edges[{v[0], v[1]}] += f + 1;
    edges[{v[1], v[2]}] += f + 1;
    edges[{v[2], v[0]}] += f + 1;
  }
  auto lookup = [&](int a, int b) -> long long {
    auto it = edges.find({a, b});
    return it == edges.end() ? 0 : it->second;
  };
  std::vector<char> selected(F, 0);
  std::vector<OChart> valid;
  std::vector<int> invalid_faces;
  for (int seed = 0; seed < F; ++seed) {
    if (selected[seed]) continue;
    const int kf = face_kf[seed];
    std::vector<int> faces{seed};
    selected[seed] = 1;
    std::deque<int> queue{seed};
    while (!queue.empty()) {
      const int fid = queue.front();
      queue.pop_front();
      const int* v = vidx + 3 * (size_t)fid;
      std::vector<long long> adj;
      for (auto e : {std::make_pair(v[1], v[0]), std::make_pair(v[2], v[1]),
                     std::make_pair(v[0], v[2])}) {
        const long long m = lookup(e.first, e.second);
        if (m > 0) adj.push_back(m - 1);
      }
      for (auto e : {std::make_pair(v[0], v[1]), std::make_pair(v[1], v[2]),
                     std::make_pair(v[2], v[0])}) {
        auto it = edges.find(e);
        if (it != edges.end()) it->second = 0;
      }
      for (long long g : adj)
        if (g >= F) return -3;
      std::vector<int> add;
      for (long long g : adj)
        if (face_kf[g] == kf && !selected[g]) add.push_back((int)g);
      for (int g : add) {
        queue.push_back(g);
        faces.push_back(g);
        selected[g] = 1;
      }
    }
    if (kf < 0) {
      invalid_faces.insert(invalid_faces.end(), faces.begin(), faces.end());
      continue;
    }
    if (kf >= num_kf) return -2;
    float xminf = 1e30f, xmaxf = -1e30f, yminf = 1e30f, ymaxf = -1e30f;
    for (int f : faces)
      for (int j = 0; j < 3; ++j) {
        xminf = std::min(xminf, face_tri[6 * (size_t)f + 2 * j]);
        xmaxf = std::max(xmaxf, face_tri[6 * (size_t)f + 2 * j]);
        yminf = std::min(yminf, face_tri[6 * (size_t)f + 2 * j + 1]);
        ymaxf = std::max(ymaxf, face_tri[6 * (size_t)f + 2 * j + 1]);
      }
    const int xmin = (int)std::floor(xminf), ymin = (int)std::floor(yminf);
    const int xmax = (int)std::ceil(xmaxf), ymax = (int)std::ceil(ymaxf);
    if (xmin < 0 || ymin < 0 || xmax >= kf_w[kf] || ymax >= kf_h[kf]) return -2;
    const int pad = 1;
    OChart c;
    c.w = xmax - xmin + 1 + 2 * pad;
    c.h = ymax - ymin + 1 + 2 * pad;
    c.patch.assign((size_t)c.w * c.h * 3, 0);
    for (int y = ymin; y <= ymax; ++y)
      std::copy(kf_color[kf] + ((size_t)kf_w[kf] * y + xmin) * 3,
                kf_color[kf] + ((size_t)kf_w[kf] * y + xmax + 1) * 3,
                c.patch.begin() + ((size_t)c.w * (y - ymin + pad) + pad) * 3);
    auto px = [&](int y, int x) { return c.patch.begin() + ((size_t)c.w * y + x) * 3; };
    for (int y = 0; y < pad; ++y)
      for (int x = 0; x < c.w; ++x) std::copy(px(pad, x), px(pad, x) + 3, px(y, x));
    for (int y = c.h - pad; y < c.h; ++y)
      for (int x = 0; x < c.w; ++x) std::copy(px(c.h - pad - 1, x), px(c.h - pad - 1, x) + 3, px(y, x));
    for (int y = 0; y < c.h; ++y)
      for (int x = 0; x < pad; ++x) std::copy(px(y, pad), px(y, pad) + 3, px(y, x));
    for (int y = 0; y < c.h; ++y)
      for (int x = c.w - pad; x < c.w; ++x) std::copy(px(y, c.w - pad - 1), px(y, c.w - pad - 1) + 3, px(y, x));
    std::map<int, std::pair<float, float>> vpos;
    for (int f : faces)
      for (int j = 0; j < 3; ++j) {
        const float lx = face_tri[6 * (size_t)f + 2 * j] - xmin + pad;
        const float ly = face_tri[6 * (size_t)f + 2 * j + 1] - ymin + pad;
        vpos.insert({vidx[3 * (size_t)f + j], {lx, ly}});
      }
    std::map<int, int> renum;
    for (const auto& kv : vpos) {
      renum[kv.first] = (int)c.pos.size();
      c.pos.push_back(kv.second);
    }
    for (int f : faces)
      c.face_idx.push_back({f, {renum[vidx[3 * (size_t)f]], renum[vidx[3 * (size_t)f + 1]],
                                renum[vidx[3 * (size_t)f + 2]]}});
    valid.push_back(std::move(c));
  }
  std::stable_sort(valid.begin(), valid.end(),
                   [](const OChart& a, const OChart& b) { return a.w * a.h > b.w * b.h; });
  std::vector<ORect> rects, packed, avail;
  for (const OChart& c : valid) rects.push_back(ORect{0, 0, c.w, c.h});
  int cur_w = tex_w, cur_h = tex_h, tries = 0;
  const float ratio = std::sqrt(2.0f);
  while (!bin_packing(rects, &packed, &avail, 1, cur_w - 1, 1, cur_h - 1)) {
    ++tries;
    cur_w = (int)(tex_w * std::pow(ratio, tries));
    cur_h = (int)(tex_h * std::pow(ratio, tries));
    if (8192 < cur_w || 8192 < cur_h) return -1;
  }
  int nuv = 3;
  for (const OChart& c : valid) nuv += (int)c.pos.size();
  dims[0] = cur_w;
  dims[1] = cur_h;
  dims[2] = nuv;
  if (!texture) return 0;
  std::fill(texture, texture + (size_t)cur_w * cur_h * 3, 0);
  const float cols = (float)cur_w, rows = (float)cur_h;
  int off = 0;
  for (size_t k = 0; k < valid.size(); ++k) {
    const OChart& c = valid[k];
    const ORect& r = packed[k];
    for (int y = 0; y < c.h; ++y)
      std::copy(c.patch.begin() + (size_t)c.w * y * 3, c.patch.begin() + (size_t)c.w * (y + 1) * 3,
                texture + ((size_t)cur_w * (y + r.y) + r.x) * 3);
    for (size_t i = 0; i < c.pos.size(); ++i) {
      uv[2 * (off + i)] = (c.pos[i].first + r.x + 0.5f) / cols;
      uv[2 * (off + i) + 1] = 1.0f - ((c.pos[i].second + r.y + 0.5f) / rows);
    }
    for (const auto& fi : c.face_idx)
      for (int j = 0; j < 3; ++j) uv_indices[3 * (size_t)fi.first + j] = off + fi.second[j];
    off += (int)c.pos.size();
  }
  float iu = 0.0f, iv = 0.0f;
  if (!avail.empty()) {
    iu = (avail[0].x + 0.5f) / cols;
    iv = 1.0f - ((avail[0].y + 0.5f) / rows);
  }
  for (int j = 0; j < 3; ++j) {
    uv[2 * (off + j)] = iu;
    uv[2 * (off + j) + 1] = iv;
  }
  for (int f : invalid_faces)
    for (int j = 0; j < 3; ++j) uv_indices[3 * (size_t)f + j] = off + j;
  return 0;
}
