// tile.cu -- the tiled forward path's tile kernel: persistent blocks that
// rasterise and resolve each screen tile in shared memory, from the
// (face, tile) entry lists the binning kernels (bin.cu) built.
//
//   k_tile   persistent blocks pull (view, tile) items from a work queue.
//            For one tile, each warp on its own: take the next 32 listed
//            faces (a quarter of a small draw class), set them up in the
//            warp's slots of shared memory with
//            their candidate pixels (the box-in-tile, or conservative row
//            spans for small faces, span.cuh), split them into (face, pixel)
//            pairs with a warp prefix scan of their candidate counts, test
//            every pair's coverage (Loop B's pixel test) and run the covered
//            ones' z-test into the block's shared-memory z-buffer of
//            64-bit (depth bits << 32 | face id << 1 | back-face bit) keys
//            with atomicMin, then run Loop C (rasterizer.cc:244-301) for the
//            tile's pixels: depth, face id, mask and the shading.
//
// A face whose depth lower bound lies behind the view's split depth (the
// camera depth of the mesh's bounding-box centre) is drawn last, and skipped
// when that bound lies behind the deepest key of a fully covered tile: such
// a face can never win the z-test there, so the result is unchanged.
#include <cuda_runtime.h>

#include "internal.cuh"
#include "shade.cuh"
#include "span.cuh"
#include "tilecommon.cuh"

namespace ugu_gpu {

namespace {

using tiled::copy_words;
using tiled::kU64;
using tiled::setup_proj;

#ifndef UGU_TILE_THREADS
#define UGU_TILE_THREADS 128
#endif
#ifndef UGU_TILE_BLOCKS
#define UGU_TILE_BLOCKS 8
#endif
constexpr int kTileThreads = UGU_TILE_THREADS;  // one tile per block
constexpr int kWarps = kTileThreads / 32;
constexpr int kChunk = kTileThreads;  // window slots: 32 faces per warp
static_assert(kChunk <= 256, "a covered pair packs its face slot in 8 bits");
constexpr int kMaxTile = 32;     // tile edge <= 32 pixels

__device__ __forceinline__ int find_view_by_tile(const TileParams& p, int t) {
  int lo = 0, hi = p.num_views - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (p.views[mid].tile_base <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Faces of one tile set up in shared memory: warp w owns slots
// [32 w, 32 w + 32) and holds up to 32 of its entries there at a time.
struct Region {
  float4 r0[kChunk];  // v0.x v0.y v1.x v1.y
  float4 r1[kChunk];  // v2.x v2.y area box (pack_box)
  float4 r2[kChunk];  // v0.z v1.z v2.z fid-bits
  float4 r3[kChunk];  // back-face sign surrogate: sa sb sc tolerance
  float4 r5[kChunk];  // depth pre-test: z1 z2, z0 z2, z0 z1, |area| z0 z1 z2 (1 - 2^-16)
  uint4 r4[kChunk];   // row spans (FaceSpans words cum 0, 1, start 0, 1), or 0
  uint4 r6[kChunk];   // FaceSpans words cum 2, 3, start 2, 3 of a face flagged tall
};

// A face's bbox-in-tile in 32 bits: tile-local x0 and y0, width - 1 (5 bits
// each) and m = ceil(2^16 / width) (17 bits), so that row = (k * m) >> 16
// for every pixel number k < width * height <= 1024 of the box.  m comes
// from a table of the 32 widths in shared memory (box_recip).
__device__ __forceinline__ unsigned box_recip_of(int w) {
  return (65536u + (unsigned)w - 1u) / (unsigned)w;
}
__device__ __forceinline__ float pack_box(int x0, int y0, int w, unsigned m) {
  return __uint_as_float((unsigned)x0 | ((unsigned)y0 << 5) | ((unsigned)(w - 1) << 10) |
                         (m << 15));
}


struct TileSmem {
  unsigned long long keys[kMaxTile * kMaxTile];
  Region reg;
  DevView view;
  DevMesh mesh;
  DevTexture tex0;  // the view's mesh's first material, for the resolve
  int item;
  unsigned zmax_bits;
  int cursor[2];  // next entry of each draw class: warps take 32 at a time
  unsigned box_recip[kMaxTile];  // ceil(2^16 / w) for box widths w = 1 .. 32
};
// Eight blocks (with the 1 KB each block reserves) within the 196 KB
// shared-memory carve-out, which leaves 60 KB of L1 for the setup and
// shading gathers; past 196 KB the carve-out becomes 228 KB with 28 KB of
// L1, which costs the gathers a few percent.
static_assert(UGU_TILE_THREADS != 128 || UGU_TILE_BLOCKS != 8 ||
                  8 * (sizeof(TileSmem) + 1024) <= 196 * 1024,
              "k_tile's shared memory no longer fits the 196 KB carve-out");

// The reference's back-face test fn . ray_w(x, y) > 0 (rasterizer.cc:199),
// for the rare pixels the surrogate cannot decide; kept out of line so the
// pixel loop keeps its registers.
__device__ __noinline__ bool backface_exact(const DevMesh& m, const Cam& c, int fid, int x,
                                            int y) {
  const float4 fn = __ldg(&m.fnormals[fid]);
  const float3 r = ray_w(c, x, y);
  return dot3(fn.x, fn.y, fn.z, r.x, r.y, r.z) > 0.0f;
}

// The z-test of one covered candidate (rasterizer.cc:208-237): Loop B's
// depth, then an atomicMin of its key into the tile's shared z-buffer.
__device__ __forceinline__ void depth_test(TileSmem& sm, const Region& R, const TileParams& p,
                                           const float4 q, int tlog) {
  const int packed = __float_as_int(q.w);
  const int j = packed & 255, lx = (packed >> 8) & 31, ly = (packed >> 13) & 31;
  const bool bf = (packed >> 18) & 1;
  unsigned long long* kp = &sm.keys[(ly << tlog) + lx];
  const unsigned long long cur = *(volatile unsigned long long*)kp;
  const float4 r1 = R.r1[j];
  // Depth pre-test: z' = |A| z0 z1 z2 / |w0 z1 z2 + w1 z0 z2 + w2 z0 z1| is
  // the depth Loop B computes up to 14 rounding errors of its own and of
  // this expression (all terms share one sign on a covered pixel), so
  // z' (1 - 2^-16) > current depth proves the candidate loses.
  const float4 r5 = R.r5[j];
  const float s2 = fmaf(q.x, r5.x, fmaf(q.y, r5.y, q.z * r5.z));
  if (r5.w > key_depth(cur) * fabsf(s2) && (s2 > 0.0f) == (r1.z > 0.0f)) return;
  const float4 r2 = R.r2[j];
  FaceSetup s;
  s.v0.z = r2.x;
  s.v1.z = r2.y;
  s.v2.z = r2.z;
  s.area = r1.z;
  Bary b;
  b.w0 = q.x;
  b.w1 = q.y;
  b.w2 = q.z;
  const float z = perspective(s, b);
  if (!orderable_depth(z)) {
    atomicAdd(&p.counters->special, 1ull);
    if (p.sticky) atomicOr(p.sticky, kStickySpecial);
    return;
  }
  const unsigned long long key = make_key(z, __float_as_int(r2.w), bf);
  if (key < *(volatile unsigned long long*)kp) atomicMin(kp, key);
}

// Loop B (rasterizer.cc:196-237) over the m <= 32 faces the warp set up in
// its own slots of the window: flatten their (face, pixel) pairs with a
// prefix scan and test one pair per lane: back-face sign, edge functions,
// coverage.  A covered pair takes the depth test at once: with row spans
// most lanes' pairs are covered, so batching them buys nothing.  `box_cnt`
// is the lane's face's bbox-in-tile pixel count (0 for an empty slot).
__device__ __forceinline__ void raster_pass(TileSmem& sm, Region& R, const TileParams& p,
                                            const Cam& c, int m, int tx0, int ty0, int tlog,
                                            int box_cnt) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  {
    const int base = warp * 32;
    const int j = base + lane;
    int cnt = lane < m ? box_cnt : 0;
    // the candidate pixels of the lane's face: its row spans when the face is
    // small enough (span.cuh), else the whole box-in-tile
    if (cnt > 0) {
      const float4 a = R.r0[j], b = R.r1[j];
      const unsigned box = __float_as_uint(b.w);
      // bh = cnt / bw through the box's reciprocal m = ceil(2^16 / bw):
      // exact, since bh (bw - 1) < 2^16 for boxes of at most 32 x 32
      const int bw = (int)((box >> 10) & 31u) + 1, bh = (cnt * (int)(box >> 15)) >> 16;
      const int bx0 = tx0 + (int)(box & 31u), by0 = ty0 + (int)((box >> 5) & 31u);
      FaceSpans sp;
      if (face_spans(a.x, a.y, a.z, a.w, b.x, b.y, b.z, bx0, bx0 + bw - 1, by0, by0 + bh - 1,
                     tx0, sp)) {
        cnt = sp.count;
        R.r4[j] = make_uint4(sp.cum[0], sp.cum[1], sp.start[0], sp.start[1]);
        if (sp.start[1] & kSpanTall)
          R.r6[j] = make_uint4(sp.cum[2], sp.cum[3], sp.start[2], sp.start[3]);
      }
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int pre = incl - cnt;  // the lane's face: its first pair number
    __syncwarp();                // the spans written above, for every lane
    for (int kb = 0; kb < total; kb += 32) {
      const int k = kb + lane;
      // the face of pair k: the last lane whose first pair number is <= k
      int q = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1)
        if (__shfl_sync(0xffffffffu, pre, q + step) <= k) q += step;
      const int pre_q = __shfl_sync(0xffffffffu, pre, q);
      bool cov = false;
      float4 ent;
      if (k < total) {
        const int jj = base + q;
        const int local = k - pre_q;
        const float4 r0 = R.r0[jj];
        const float4 r1 = R.r1[jj];
        const float4 r3 = R.r3[jj];
        const uint4 r4 = R.r4[jj];
        const unsigned box = __float_as_uint(r1.w);
        int x, y;
        if (r4.w & kSpanFlag) {  // candidate `local` of the face's row spans
          FaceSpans sp = {{r4.x, r4.y, 0x7f7f7f7fu, 0x7f7f7f7fu}, {r4.z, r4.w, 0u, 0u}, 0};
          if (r4.w & kSpanTall) {
            const uint4 r6 = R.r6[jj];
            sp.cum[2] = r6.x;
            sp.cum[3] = r6.y;
            sp.start[2] = r6.z;
            sp.start[3] = r6.w;
          }
          int dx, row;
          span_pixel(sp, local, dx, row);
          x = tx0 + dx;
          y = ty0 + (int)((box >> 5) & 31u) + row;
        } else {  // pixel `local` of the box, row-major
          const int bw = (int)((box >> 10) & 31u) + 1;
          const int yy = (local * (int)(box >> 15)) >> 16;
          x = tx0 + (int)(box & 31u) + local - yy * bw;
          y = ty0 + (int)((box >> 5) & 31u) + yy;
        }
        // sign of face_normal . ray_w: the affine surrogate decides unless
        // it is within its error bound of zero; then the reference's ray.
        const float sv = fmaf(r3.x, (float)x, fmaf(r3.y, (float)y, r3.z));
        bool bf;
        if (sv > r3.w)
          bf = true;
        else if (sv < -r3.w)
          bf = false;
        else
          bf = backface_exact(sm.mesh, c, __float_as_int(R.r2[jj].w), x, y);
        FaceSetup s;
        s.v0.x = r0.x;
        s.v0.y = r0.y;
        s.v1.x = r0.z;
        s.v1.y = r0.w;
        s.v2.x = r1.x;
        s.v2.y = r1.y;
        const Bary b = edges_at(s, x, y);
        cov = covered(b, bf);
        ent = make_float4(b.w0, b.w1, b.w2,
                          __int_as_float((jj & 255) | ((x - tx0) << 8) | ((y - ty0) << 13) |
                                         (bf ? 1 << 18 : 0)));
      }
      if (cov) depth_test(sm, R, p, ent, tlog);
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kTileThreads, UGU_TILE_BLOCKS) k_tile(TileParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem& sm = *reinterpret_cast<TileSmem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (p.counters->dropped) return;  // entries were not written: the host retries
  int v_begin = 0, v_end = 0;  // global tiles of the view in shared memory
  Region& R = sm.reg;
  if (tid < kMaxTile) sm.box_recip[tid] = box_recip_of(tid + 1);  // read after the next barrier
  for (;;) {
    if (tid == 0) sm.item = (int)atomicAdd(&p.counters->next_tile, 1u);
    __syncthreads();
    const int item = sm.item;
    if (item >= p.total_tiles) break;
    if (item < v_begin || item >= v_end) {
      const int v = find_view_by_tile(p, item);
      copy_words(sm.view, p.views[v]);
      __syncthreads();
      copy_words(sm.mesh, p.meshes[sm.view.mesh]);
      if (tid == 0) {
        const DevMesh& gm = p.meshes[sm.view.mesh];
        sm.tex0 = gm.num_materials > 0 ? gm.textures[0] : DevTexture{0, 0, nullptr, nullptr};
      }
      v_begin = p.views[v].tile_base;
      v_end = v + 1 < p.num_views ? p.views[v + 1].tile_base : p.total_tiles;
    }
    const Cam& c = sm.view.cam;
    const int tlog = sm.view.tile_log2;  // this view's tile edge: 16 or 32 pixels
    const int T = 1 << tlog;
    const int local = item - sm.view.tile_base;
    const int tyi = local / sm.view.tiles_x;
    const int txi = local - tyi * sm.view.tiles_x;
    const int tx0 = txi << tlog, ty0 = tyi << tlog;
    const int tw = min(T, c.width - tx0), th = min(T, c.height - ty0);
    for (int i = tid; i < T * T; i += kTileThreads) sm.keys[i] = kEmptyKey;
    // entries drawn first: [e0, e1); drawn last: [e1, e2)
    const int e0 = p.tile_off[item], e1 = p.tile_lo[item], e2 = p.tile_off[item + 1];
    const float4* proj = p.proj + sm.view.proj_offset;
    if (tid == 0) {
      sm.cursor[0] = e0;
      sm.cursor[1] = e1;
    }
    __syncthreads();

    // Per-view constants of the back-face surrogate and its error bound.
    // The surrogate's coefficients use 1/fx and 1/fy: one rounding more
    // than a division, far inside the bound's 64-ulp margins.
    const float rfx = 1.0f / c.fx, rfy = 1.0f / c.fy;
    const float Dx = (c.width + fabsf(c.cx)) / c.fx;
    const float Dy = (c.height + fabsf(c.cy)) / c.fy;
    const float Dmax = 1.0f + fmaxf(fabsf(c.cx), fabsf(c.width - 1 - c.cx)) / c.fx +
                       fmaxf(fabsf(c.cy), fabsf(c.height - 1 - c.cy)) / c.fy;

    for (int phase = 0; phase < 2; ++phase) {
      float zmax = __int_as_float(0x7f800000);
      if (phase == 1) {
        if (e2 == e1) break;
        // deepest key of the tile (+inf while any pixel is still empty),
        // once every warp has drawn its faces of the first class
        if (tid == 0) sm.zmax_bits = 0u;
        __syncthreads();
        float zm = 0.0f;
        for (int i = tid; i < T * T; i += kTileThreads) {
          const int ly = i >> tlog, lx = i & (T - 1);
          if (lx >= tw || ly >= th) continue;
          const unsigned long long k = sm.keys[i];
          zm = fmaxf(zm, k == kEmptyKey ? __int_as_float(0x7f800000) : key_depth(k));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) zm = fmaxf(zm, __shfl_xor_sync(0xffffffffu, zm, o));
        if ((tid & 31) == 0) atomicMax(&sm.zmax_bits, __float_as_uint(zm));
        __syncthreads();
        zmax = __uint_as_float(sm.zmax_bits);
      }
      const int eb = phase ? e1 : e0, ee = phase ? e2 : e1;
      // Each warp takes the class's next entries (32, or a quarter of a
      // class of at most p.split_class entries, so that few large faces still
      // keep every warp busy), sets them up in its own 32 slots of the window
      // and draws them; warps meet only at the class boundary, so one warp's
      // large faces hold up no other warp.
      const int grab =
          ee - eb <= p.split_class ? min(32, max(1, (ee - eb + kWarps - 1) / kWarps)) : 32;
      for (;;) {
        int cs = 0;
        if (lane == 0) cs = atomicAdd(&sm.cursor[phase], grab);
        cs = __shfl_sync(0xffffffffu, cs, 0);
        if (cs >= ee) break;
        const int m = min(grab, ee - cs);
        const int j = warp * 32 + lane;
        int box_cnt = 0;    // the slot's bbox-in-tile pixels, 0 when the face is skipped
        if (lane < m) do {  // `continue` leaves the slot empty
          const int2 e = p.entries[cs + lane];
          const float zlb = __int_as_float(e.y);
          if ((unsigned)e.x >= (unsigned)sm.mesh.num_faces) {  // never for the binning's entries
            atomicAdd(&p.counters->invalid, 1u);
            continue;
          }
          if (zlb > zmax) continue;  // behind every key of a covered tile: cannot win
          const int f = __ldg(&sm.mesh.order[e.x]);  // the entry holds the binning number
          FaceSetup s;
          setup_proj(proj, sm.mesh.vidx_morton, e.x, c, s);  // succeeded in k_count: same arithmetic
          const int bx0 = max(s.x0, tx0), bx1 = min(s.x1, tx0 + tw - 1);
          const int by0 = max(s.y0, ty0), by1 = min(s.y1, ty0 + th - 1);
          const int bw = bx1 - bx0 + 1, bh = by1 - by0 + 1;
          if (bw <= 0 || bh <= 0) continue;
          // back-face surrogate: s(x, y) = (C^T n) . ((x-cx)/fx, (y-cy)/fy, 1)
          const float4 fn = __ldg(&sm.mesh.fnormals_morton[e.x]);
          const float* C = c.C;
          const float g0 = C[0] * fn.x + C[3] * fn.y + C[6] * fn.z;
          const float g1 = C[1] * fn.x + C[4] * fn.y + C[7] * fn.z;
          const float g2 = C[2] * fn.x + C[5] * fn.y + C[8] * fn.z;
          const float G = (fabsf(C[0]) + fabsf(C[1]) + fabsf(C[2])) * fabsf(fn.x) +
                          (fabsf(C[3]) + fabsf(C[4]) + fabsf(C[5])) * fabsf(fn.y) +
                          (fabsf(C[6]) + fabsf(C[7]) + fabsf(C[8])) * fabsf(fn.z);
          const float sa = g0 * rfx, sb = g1 * rfy;
          const float sc = g2 - sa * c.cx - sb * c.cy;
          const float tol = kU64 * (G * (1.0f + Dx + Dy) + fabsf(sa) * (c.width + fabsf(c.cx)) +
                                    fabsf(sb) * (c.height + fabsf(c.cy)) + fabsf(g2)) +
                            2.0f * kU64 * G * Dmax;
          // depth pre-test factors, only where every product stays normal
          const float z0 = s.v0.z, z1 = s.v1.z, z2 = s.v2.z;
          const float zlo = 9.5367431640625e-07f, zhi = 1048576.0f;  // 2^-20, 2^20
          const bool pre_ok = z0 >= zlo && z0 <= zhi && z1 >= zlo && z1 <= zhi && z2 >= zlo &&
                              z2 <= zhi && fabsf(s.area) >= 8.673617379884035e-19f;  // 2^-60
          const float aP = pre_ok ? fabsf(s.area) * (z0 * z1 * z2) * 0.99998474f
                                  : __int_as_float(0x7fc00000);
          R.r0[j] = make_float4(s.v0.x, s.v0.y, s.v1.x, s.v1.y);
          R.r1[j] = make_float4(s.v2.x, s.v2.y, s.area, pack_box(bx0 - tx0, by0 - ty0, bw,
                                                                 sm.box_recip[bw - 1]));
          R.r2[j] = make_float4(z0, z1, z2, __int_as_float(f));
          R.r3[j] = make_float4(sa, sb, sc, tol);
          R.r5[j] = make_float4(z1 * z2, z0 * z2, z0 * z1, aP);
          R.r4[j] = make_uint4(0u, 0u, 0u, 0u);  // the whole box, unless raster_pass narrows it
          box_cnt = bw * bh;
        } while (0);
        __syncwarp();
        raster_pass(sm, R, p, c, m, tx0, ty0, tlog, box_cnt);
        __syncwarp();
      }
    }
    __syncthreads();  // every face drawn

    // Loop C (rasterizer.cc:244-301) for the tile's pixels.
    const DevView& V = sm.view;
    const int W = c.width;
    for (int i = tid; i < T * T; i += kTileThreads) {
      const int ly = i >> tlog, lx = i & (T - 1);
      if (lx >= tw || ly >= th) continue;
      const int64_t pix = (int64_t)(ty0 + ly) * W + tx0 + lx;
      const unsigned long long key = sm.keys[i];
      float depth = 0.0f;
      int32_t fid = -1;
      uint8_t mask = 0;
      if (key != kEmptyKey && !(p.backface_culling && key_backface(key))) {
        depth = key_depth(key);
        fid = key_face(key);
        if (fid > 0) mask = 255;  // rasterizer.cc:254: face 0 is never shaded
      }
      if (V.depth) V.depth[pix] = depth;
      if (V.face_id) V.face_id[pix] = fid;
      if (V.mask) V.mask[pix] = mask;
      // Loop C's shading (rasterizer.cc:254-299)
      if (V.color || V.normal || V.color_f32) {
        Shaded sh;
        sh.c[0] = sh.c[1] = sh.c[2] = 0;
        sh.cf[0] = sh.cf[1] = sh.cf[2] = 0.0f;
        sh.n[0] = sh.n[1] = sh.n[2] = 0.0f;
        if (fid > 0)
          shade_tile_pixel(p.shade, sm.mesh, sm.tex0, c, proj, fid, tx0 + lx, ty0 + ly, depth, sh);
        if (V.color) {
          V.color[3 * pix + 0] = sh.c[0];
          V.color[3 * pix + 1] = sh.c[1];
          V.color[3 * pix + 2] = sh.c[2];
        }
        if (V.normal) {
          V.normal[3 * pix + 0] = sh.n[0];
          V.normal[3 * pix + 1] = sh.n[1];
          V.normal[3 * pix + 2] = sh.n[2];
        }
        if (V.color_f32) {
          V.color_f32[3 * pix + 0] = sh.cf[0];
          V.color_f32[3 * pix + 1] = sh.cf[1];
          V.color_f32[3 * pix + 2] = sh.cf[2];
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace

void launch_tile(const TileParams& p, int grid, cudaStream_t s) {
  k_tile<<<grid, kTileThreads, sizeof(TileSmem), s>>>(p);
}


int tile_kernel_blocks_per_sm() {
  static int blocks = 0;
  if (!blocks) {
    cudaFuncSetAttribute(k_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(TileSmem));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_tile, kTileThreads,
                                                  sizeof(TileSmem));
    if (blocks < 1) blocks = 1;
  }
  return blocks;
}

}  // namespace ugu_gpu
