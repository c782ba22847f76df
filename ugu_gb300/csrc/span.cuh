// span.cuh -- conservative per-row pixel spans of one face inside one tile.
//
// Loop B (rasterizer.cc:196-207) tests every pixel of a face's bounding box,
// and for the small faces of a dense mesh most of those pixels lie outside
// the triangle.  This computes, per box row, an interval of x that contains
// every pixel the exact test can find covered (with either back-face sign);
// the exact test then runs on those pixels only, so the result is the same.
//
// Why the interval is safe.  The edge value the rasterizer computes at pixel
// (x, y) for the edge a -> b is w = fl(fl(fl(x - ax) * dy) - fl(fl(y - ay) * dx))
// with the float differences dy = fl(by - ay), dx = fl(bx - ax).  It differs
// from the real linear form E(x, y) = (x - ax) dy - (y - ay) dx by at most
// 6.01 u (|x - ax| |dy| + |y - ay| |dx|) <= 6.01 u * 2 W H (u = 2^-24; W, H
// the face's box extents plus one), below err = 2^-20 W H.  The three exact
// forms sum to the face's exact doubled area up to the differences' roundings
// (6 u W H), and the computed area lies within 8 u W H of that.  So when
// |area| > 2^-17 W H, all three w <= 0 is impossible for area > 0 (and all
// three w >= 0 for area < 0): a covered pixel has g E_i >= -err for every
// edge, g = sign(area).  Each such inequality is a bound x >= T(y) or
// x <= T(y), T(y) = c0 + c1 y, evaluated here (through one reciprocal of dy)
// with a margin of 2^-17 times the magnitudes involved, more than 16 times
// its rounding error.
//
// Faces with more than kSpanRows rows in the tile, more than kSpanMax
// candidate pixels, extents above 4096 pixels, or |area| at or below the
// threshold keep the whole box.  Spans of up to 8 rows take 16 bytes, of
// up to 16 rows 32.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define UGU_SPAN_HD __host__ __device__ __forceinline__
#else
#define UGU_SPAN_HD inline
#endif

namespace ugu_gpu {

constexpr int kSpanRows = 16;  // rows of a face's box in one tile
constexpr int kSpanMax = 127;  // candidate pixels (byte-wise compares need <= 127)

// Byte r of the 16-byte cum (word w = bytes 4w .. 4w + 3): pixels in rows
// before r, 127 for rows past the last.  Byte r of start: tile-local x of
// row r's first candidate.  Bit 31 of start[1] marks a face that uses spans,
// bit 30 one with more than 8 rows (words 2 and 3 in use; for other faces
// they hold 127s and zeros and need not be stored).
struct FaceSpans {
  uint32_t cum[4], start[4];
  int count;
};

constexpr uint32_t kSpanFlag = 0x80000000u;
constexpr uint32_t kSpanTall = 0x40000000u;

// One edge's bound x >= T(y) (lower) or x <= T(y), T(y) = c0 + c1 y +/- mu.
struct SpanEdge {
  float c0, c1, mu;
  int kind;  // +1 lower bound, -1 upper bound, 0 none
};

UGU_SPAN_HD SpanEdge span_edge(float ax, float ay, float bx, float by, float g, float err,
                               float ymag) {
  SpanEdge e;
  const float dy = by - ay, dx = bx - ax;
  if (!(fabsf(dy) >= 0x1p-12f)) {  // nearly horizontal: no bound on x
    e.c0 = e.c1 = e.mu = 0.0f;
    e.kind = 0;
    return e;
  }
  const float rdy = 1.0f / dy;
  e.c1 = dx * rdy;
  const float es = (g * err) * rdy;  // err / (g dy)
  e.c0 = (ax - ay * e.c1) - es;
  e.mu = 0x1p-17f * (fabsf(ax) + (fabsf(ay) + ymag) * fabsf(e.c1) + fabsf(es) + fabsf(e.c0)) +
         0x1p-17f;
  e.kind = g * dy > 0.0f ? 1 : -1;
  return e;
}

// Spans of the face (v0, v1, v2) over the box-in-tile [bx0, bx1] x [by0, by1]
// of the tile at (tx0, ty0).  Returns false when the face keeps its box.
UGU_SPAN_HD bool face_spans(float v0x, float v0y, float v1x, float v1y, float v2x, float v2y,
                            float area, int bx0, int bx1, int by0, int by1, int tx0,
                            FaceSpans& o) {
  const int rows = by1 - by0 + 1;
  if (rows > kSpanRows) return false;
  const float xmin = fminf(fminf(v0x, v1x), v2x), xmax = fmaxf(fmaxf(v0x, v1x), v2x);
  const float ymin = fminf(fminf(v0y, v1y), v2y), ymax = fmaxf(fmaxf(v0y, v1y), v2y);
  const float W = (xmax - xmin) + 1.0f, H = (ymax - ymin) + 1.0f;
  if (!(W <= 4096.0f && H <= 4096.0f)) return false;
  const float WH = W * H;
  if (!(fabsf(area) > 0x1p-17f * WH)) return false;
  const float g = area > 0.0f ? 1.0f : -1.0f;
  const float err = 0x1p-20f * WH;
  const float ymag = fmaxf(fabsf(ymin), fabsf(ymax)) + 1.0f;
  SpanEdge e[3];
  e[0] = span_edge(v1x, v1y, v2x, v2y, g, err, ymag);
  e[1] = span_edge(v2x, v2y, v0x, v0y, g, err, ymag);
  e[2] = span_edge(v0x, v0y, v1x, v1y, g, err, ymag);
  uint32_t c0 = 0x7f7f7f7fu, c1 = 0x7f7f7f7fu, c2 = 0x7f7f7f7fu, c3 = 0x7f7f7f7fu;
  uint32_t s0 = 0u, s1 = 0u, s2 = 0u, s3 = 0u;
  int count = 0;
  // candidate interval of box row r: its width, and its first x relative to the tile
  auto row_span = [&](int r, int& w, int& sx) {
    const float y = (float)(by0 + r);
    float lo = (float)bx0, hi = (float)bx1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float t = fmaf(y, e[k].c1, e[k].c0);
      if (e[k].kind > 0) lo = fmaxf(lo, ceilf(t - e[k].mu));
      if (e[k].kind < 0) hi = fminf(hi, floorf(t + e[k].mu));
    }
    w = hi >= lo ? (int)(hi - lo) + 1 : 0;
    sx = w ? (int)lo - tx0 : 0;
  };
  const int rows_lo = rows < 8 ? rows : 8;
  for (int r = 0; r < rows_lo; ++r) {
    int w, sx;
    row_span(r, w, sx);
    const int sh = 8 * (r & 3);
    const uint32_t cm = ~(0xffu << sh), cv = (uint32_t)count << sh, sv = (uint32_t)sx << sh;
    if (r < 4) {
      c0 = (c0 & cm) | cv;
      s0 |= sv;
    } else {
      c1 = (c1 & cm) | cv;
      s1 |= sv;
    }
    count += w;
    if (count > kSpanMax) return false;
  }
  for (int r = 8; r < rows; ++r) {
    int w, sx;
    row_span(r, w, sx);
    const int sh = 8 * (r & 3);
    const uint32_t cm = ~(0xffu << sh), cv = (uint32_t)count << sh, sv = (uint32_t)sx << sh;
    if (r < 12) {
      c2 = (c2 & cm) | cv;
      s2 |= sv;
    } else {
      c3 = (c3 & cm) | cv;
      s3 |= sv;
    }
    count += w;
    if (count > kSpanMax) return false;
  }
  o.cum[0] = c0;
  o.cum[1] = c1;
  o.cum[2] = c2;
  o.cum[3] = c3;
  o.start[0] = s0;
  o.start[1] = s1 | kSpanFlag | (rows > 8 ? kSpanTall : 0u);
  o.start[2] = s2;
  o.start[3] = s3;
  o.count = count;
  return true;
}

// Tile-local x offset and box row of candidate number k < count of a span
// face: the row is the last one whose byte in cum is <= k (bytes compared
// four at a time: k + 128 - c keeps bit 7 set exactly when k >= c, for
// k, c <= 127).  Words 2 and 3 are read only for a face flagged tall.
UGU_SPAN_HD uint32_t span_ge(uint32_t kk, uint32_t c) { return (kk - c) & 0x80808080u; }

UGU_SPAN_HD int span_popc(uint32_t v) {
#ifdef __CUDA_ARCH__
  return __popc(v);
#else
  return __builtin_popcount(v);
#endif
}

// Byte n (0..7) of the 8 bytes lo | hi << 32.
UGU_SPAN_HD uint32_t span_byte(uint32_t lo, uint32_t hi, int n) {
#ifdef __CUDA_ARCH__
  return __byte_perm(lo, hi, (uint32_t)n) & 0xffu;
#else
  return (uint32_t)((((uint64_t)hi << 32) | lo) >> (8 * n)) & 0xffu;
#endif
}

UGU_SPAN_HD void span_pixel(const FaceSpans& s, int k, int& dx, int& row) {
  const uint32_t kk = ((uint32_t)k * 0x01010101u) | 0x80808080u;
  int n = span_popc(span_ge(kk, s.cum[0])) + span_popc(span_ge(kk, s.cum[1]));
  const bool tall = (s.start[1] & kSpanTall) != 0u;
  if (tall) n += span_popc(span_ge(kk, s.cum[2])) + span_popc(span_ge(kk, s.cum[3]));
  row = n - 1;
  uint32_t c, x0;
  if (row < 8) {
    c = span_byte(s.cum[0], s.cum[1], row);
    x0 = span_byte(s.start[0], s.start[1], row);
  } else {
    c = span_byte(s.cum[2], s.cum[3], row - 8);
    x0 = span_byte(s.start[2], s.start[3], row - 8);
  }
  dx = (int)(x0 & 0x1fu) + k - (int)c;
}

}  // namespace ugu_gpu
