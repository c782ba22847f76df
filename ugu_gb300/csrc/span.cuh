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
// threshold keep the whole box.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define UGU_SPAN_HD __host__ __device__ __forceinline__
#else
#define UGU_SPAN_HD inline
#endif

namespace ugu_gpu {

constexpr int kSpanRows = 8;   // rows of a face's box in one tile
constexpr int kSpanMax = 127;  // candidate pixels (byte-wise compares need <= 127)

// Byte r of cum (lo = bytes 0..3, hi = bytes 4..7): pixels in rows before r,
// 127 for rows past the last.  Byte r of start: tile-local x of row r's first
// candidate.  Bit 31 of start_hi marks a face that uses spans.
struct FaceSpans {
  uint32_t cum_lo, cum_hi, start_lo, start_hi;
  int count;
};

constexpr uint32_t kSpanFlag = 0x80000000u;

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
  uint32_t cum_lo = 0x7f7f7f7fu, cum_hi = 0x7f7f7f7fu, start_lo = 0u, start_hi = 0u;
  int count = 0;
  for (int r = 0; r < rows; ++r) {
    const float y = (float)(by0 + r);
    float lo = (float)bx0, hi = (float)bx1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float t = fmaf(y, e[k].c1, e[k].c0);
      if (e[k].kind > 0) lo = fmaxf(lo, ceilf(t - e[k].mu));
      if (e[k].kind < 0) hi = fminf(hi, floorf(t + e[k].mu));
    }
    const int w = hi >= lo ? (int)(hi - lo) + 1 : 0;
    const int sx = w ? (int)lo - tx0 : 0;
    const int sh = 8 * (r & 3);
    if (r < 4) {
      cum_lo = (cum_lo & ~(0xffu << sh)) | ((uint32_t)count << sh);
      start_lo |= (uint32_t)sx << sh;
    } else {
      cum_hi = (cum_hi & ~(0xffu << sh)) | ((uint32_t)count << sh);
      start_hi |= (uint32_t)sx << sh;
    }
    count += w;
    if (count > kSpanMax) return false;
  }
  o.cum_lo = cum_lo;
  o.cum_hi = cum_hi;
  o.start_lo = start_lo;
  o.start_hi = start_hi | kSpanFlag;
  o.count = count;
  return true;
}

// Tile-local (x, y) offsets of candidate number k < count of a span face
// whose box-in-tile starts at row y0: the row is the last one whose byte in
// cum is <= k (bytes compared four at a time: k + 128 - c keeps bit 7 set
// exactly when k >= c, for k, c <= 127).
UGU_SPAN_HD void span_pixel(const FaceSpans& s, int k, int& dx, int& row) {
  const uint32_t kk = ((uint32_t)k * 0x01010101u) | 0x80808080u;
  const uint32_t a = (kk - s.cum_lo) & 0x80808080u;
  const uint32_t b = (kk - s.cum_hi) & 0x80808080u;
#ifdef __CUDA_ARCH__
  row = __popc(a) + __popc(b) - 1;
  const uint32_t c = __byte_perm(s.cum_lo, s.cum_hi, (uint32_t)row) & 0xffu;
  const uint32_t x0 = __byte_perm(s.start_lo, s.start_hi, (uint32_t)row) & 0x1fu;
#else
  row = __builtin_popcount(a) + __builtin_popcount(b) - 1;
  const uint64_t cum = (uint64_t)s.cum_lo | ((uint64_t)s.cum_hi << 32);
  const uint64_t st = (uint64_t)s.start_lo | ((uint64_t)s.start_hi << 32);
  const uint32_t c = (uint32_t)(cum >> (8 * row)) & 0xffu;
  const uint32_t x0 = (uint32_t)(st >> (8 * row)) & 0x1fu;
#endif
  dx = (int)x0 + k - (int)c;
}

}  // namespace ugu_gpu
