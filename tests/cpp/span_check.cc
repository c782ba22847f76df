// Host check of ugu_gb300/csrc/span.cuh: for seeded faces of many shapes,
// every pixel of a face's box-in-tile that the rasterizer's exact edge test
// finds covered (either back-face sign, rasterizer.cc:201-207) lies in the
// face's spans, and the candidate numbers 0..count-1 decode to exactly the
// span pixels, each once.  Built with -ffp-contract=off so that the float
// arithmetic is the kernel's.
//
// usage: span_check <faces> <seed>; prints "ok <faces> <box pixels>
// <candidate pixels> <covered pixels of span faces> <span faces> <their box
// pixels> <their candidate pixels>" or the first failure.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "span.cuh"

using namespace ugu_gpu;

namespace {

float edge_fn(float ax, float ay, float bx, float by, float cx, float cy) {
  return (cx - ax) * (by - ay) - (cy - ay) * (bx - ax);
}

struct Rng {  // splitmix64
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  double uni() { return (double)(next() >> 11) * 0x1p-53; }
  float range(double a, double b) { return (float)(a + (b - a) * uni()); }
};

constexpr int kImg = 2048, kTile = 32;

// One face of kind k (0..6) in image coordinates.
void make_face(Rng& r, int kind, float v[6]) {
  const float cx = r.range(-8, kImg + 8), cy = r.range(-8, kImg + 8);
  switch (kind) {
    case 0: {  // small, 0.3 .. 12 pixels across
      const double s = 0.3 + 12 * r.uni() * r.uni();
      for (int i = 0; i < 3; ++i) {
        v[2 * i] = cx + (float)(s * (r.uni() - 0.5));
        v[2 * i + 1] = cy + (float)(s * (r.uni() - 0.5));
      }
      break;
    }
    case 1: {  // sliver: a long edge and a third vertex close to it
      const double len = 1 + 40 * r.uni(), ang = 6.283185307179586 * r.uni();
      const double dx = len * std::cos(ang), dy = len * std::sin(ang);
      const double t = r.uni(), off = std::pow(10.0, -6 + 6 * r.uni()) * (r.uni() < 0.5 ? -1 : 1);
      v[0] = cx, v[1] = cy;
      v[2] = (float)(cx + dx), v[3] = (float)(cy + dy);
      v[4] = (float)(cx + t * dx - off * dy / len), v[5] = (float)(cy + t * dy + off * dx / len);
      break;
    }
    case 2: {  // vertices on integer and half-integer pixel lines: exact zeros
      for (int i = 0; i < 3; ++i) {
        v[2 * i] = std::floor(cx) + 0.5f * (float)(int)(r.next() % 13) - 3.0f;
        v[2 * i + 1] = std::floor(cy) + 0.5f * (float)(int)(r.next() % 13) - 3.0f;
      }
      break;
    }
    case 3: {  // one vertex far from the others
      for (int i = 0; i < 3; ++i) {
        v[2 * i] = cx + r.range(-4, 4);
        v[2 * i + 1] = cy + r.range(-4, 4);
      }
      const int j = (int)(r.next() % 3);
      v[2 * j] += r.range(-300, 300);
      v[2 * j + 1] += r.range(-300, 300);
      break;
    }
    case 4: {  // medium faces, up to 8 or up to 16 rows
      const double h = r.uni() < 0.5 ? 4.5 : 9.0;
      for (int i = 0; i < 3; ++i) {
        v[2 * i] = cx + r.range(-20, 20);
        v[2 * i + 1] = cy + r.range(-h, h);
      }
      break;
    }
    case 5: {  // nearly horizontal or vertical edges
      v[0] = cx, v[1] = cy;
      v[2] = cx + r.range(-10, 10), v[3] = cy + r.range(-1e-4, 1e-4);
      v[4] = cx + r.range(-1e-4, 1e-4), v[5] = cy + r.range(-6, 6);
      if (r.uni() < 0.5) std::swap(v[2], v[3]), std::swap(v[4], v[5]);
      break;
    }
    default: {  // area near the threshold: collinear plus a nudge of a few ulps
      const float dx = r.range(-12, 12), dy = r.range(-6, 6), t = r.range(0, 1);
      v[0] = cx, v[1] = cy;
      v[2] = cx + dx, v[3] = cy + dy;
      v[4] = cx + t * dx, v[5] = cy + t * dy;
      const int n = (int)(r.next() % 64) - 32;
      v[4] = std::nextafter(v[4], n > 0 ? 1e9f : -1e9f);
      for (int i = 0; i < std::abs(n) / 8; ++i) v[5] = std::nextafter(v[5], 1e9f);
      break;
    }
  }
}

}  // namespace

int main(int argc, char** argv) {
  const long faces = argc > 1 ? std::atol(argv[1]) : 200000;
  Rng rng{argc > 2 ? (uint64_t)std::atoll(argv[2]) : 1ull};
  long long box_px = 0, span_px = 0, cov_px = 0, span_faces = 0, span_box = 0, span_cand = 0;
  std::vector<uint8_t> in_span(kTile * kTile);
  for (long f = 0; f < faces; ++f) {
    float v[6];
    make_face(rng, (int)(f % 7), v);
    const float xmin = std::fmin(std::fmin(v[0], v[2]), v[4]);
    const float xmax = std::fmax(std::fmax(v[0], v[2]), v[4]);
    const float ymin = std::fmin(std::fmin(v[1], v[3]), v[5]);
    const float ymax = std::fmax(std::fmax(v[1], v[3]), v[5]);
    if (xmin > (float)(kImg - 1) || xmax < 0.0f || ymin > (float)(kImg - 1) || ymax < 0.0f)
      continue;
    const int x0 = std::max(0, (int)std::ceil(xmin)), x1 = std::min(kImg - 1, (int)std::floor(xmax));
    const int y0 = std::max(0, (int)std::ceil(ymin)), y1 = std::min(kImg - 1, (int)std::floor(ymax));
    const float area = edge_fn(v[0], v[1], v[2], v[3], v[4], v[5]);
    if (std::fabs(area) < 1.17549435e-38f || x1 < x0 || y1 < y0) continue;
    for (int ty = y0 / kTile; ty <= y1 / kTile; ++ty)
      for (int tx = x0 / kTile; tx <= x1 / kTile; ++tx) {
        const int tx0 = tx * kTile, ty0 = ty * kTile;
        const int bx0 = std::max(x0, tx0), bx1 = std::min(x1, tx0 + kTile - 1);
        const int by0 = std::max(y0, ty0), by1 = std::min(y1, ty0 + kTile - 1);
        if (bx1 < bx0 || by1 < by0) continue;
        FaceSpans s;
        const bool use = face_spans(v[0], v[1], v[2], v[3], v[4], v[5], area, bx0, bx1, by0, by1,
                                    tx0, s);
        const int bw = bx1 - bx0 + 1, bh = by1 - by0 + 1;
        box_px += (long long)bw * bh;
        std::fill(in_span.begin(), in_span.end(), 0);
        if (use) {
          ++span_faces;
          span_px += s.count;
          span_box += (long long)bw * bh;
          span_cand += s.count;
          if (s.count > kSpanMax || !(s.start[1] & kSpanFlag) ||
              ((s.start[1] & kSpanTall) != 0) != (bh > 8)) {
            std::printf("FAIL bad count or flag: face %ld count %d\n", f, s.count);
            return 1;
          }
          for (int k = 0; k < s.count; ++k) {
            int dx, row;
            span_pixel(s, k, dx, row);
            const int x = tx0 + dx, y = by0 + row;
            if (row < 0 || row >= bh || x < bx0 || x > bx1) {
              std::printf("FAIL decode outside the box: face %ld k %d x %d row %d\n", f, k, x, row);
              return 1;
            }
            uint8_t& m = in_span[(y - ty0) * kTile + (x - tx0)];
            if (m) {
              std::printf("FAIL pixel decoded twice: face %ld k %d\n", f, k);
              return 1;
            }
            m = 1;
          }
        } else {
          span_px += (long long)bw * bh;
          continue;  // the whole box is tested: nothing to check
        }
        for (int y = by0; y <= by1; ++y)
          for (int x = bx0; x <= bx1; ++x) {
            const float px = (float)x, py = (float)y;
            const float w0 = edge_fn(v[2], v[3], v[4], v[5], px, py);
            const float w1 = edge_fn(v[4], v[5], v[0], v[1], px, py);
            const float w2 = edge_fn(v[0], v[1], v[2], v[3], px, py);
            const bool cov = (w0 >= 0 && w1 >= 0 && w2 >= 0) || (w0 <= 0 && w1 <= 0 && w2 <= 0);
            cov_px += cov;
            if (use && cov && !in_span[(y - ty0) * kTile + (x - tx0)]) {
              std::printf(
                  "FAIL covered pixel outside the spans: face %ld kind %ld pixel (%d, %d) "
                  "v = %.9g %.9g %.9g %.9g %.9g %.9g w = %.9g %.9g %.9g\n",
                  f, f % 7, x, y, v[0], v[1], v[2], v[3], v[4], v[5], w0, w1, w2);
              return 1;
            }
          }
      }
  }
  std::printf("ok %ld %lld %lld %lld %lld %lld %lld\n", faces, box_px, span_px, cov_px, span_faces,
              span_box, span_cand);
  return 0;
}
