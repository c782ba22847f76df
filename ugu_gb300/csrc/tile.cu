// tile.cu -- the tiled forward path: bin faces to (view, tile) lists, then one
// persistent kernel that rasterises and resolves each tile in shared memory.
//
//   k_proj   Loop A (rasterizer.cc:131-136): every vertex of every view through
//            PinholeCamera::Project once, into a table of float4 (x, y, z).
//   k_bin    one pass over every (view, face): the per-face culls of Loop B
//            (rasterizer.cc:163-193) from the table and the screen tiles the
//            face's bbox touches.  A block sorts its (face, tile) entries by
//            tile in shared memory and stages them as runs, one per
//            (tile, draw class), counting the entries of every tile.
//   k_scan   exclusive scan of the per-tile counts into entry offsets, so the
//            entry buffer holds exactly the render's (face, tile) pairs.
//   k_gather copies every run into its tile's range: faces drawn first from
//            the front, faces drawn last from the back.
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

namespace ugu_gpu {

namespace {

constexpr int kBinThreads = 256;
constexpr int kScanThreads = 1024;
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
constexpr int kBinFaces = 2;     // faces per binning thread
constexpr int kAgg = 256;        // distinct tiles a binning block aggregates
constexpr int kAggProbes = 8;
constexpr int kScanItems = 8;    // tile counts per scan thread and round
constexpr float kU64 = 3.814697265625e-06f;  // 2^-18 = 64 ulp(1)

__device__ __forceinline__ int find_view_by_tile(const TileParams& p, int t) {
  int lo = 0, hi = p.num_views - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (p.views[mid].tile_base <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Loop B's per-face setup (rasterizer.cc:163-193) from projected vertices.
__device__ __forceinline__ bool setup_proj(const float4* proj, const int4* vidx, int f,
                                           const Cam& c, FaceSetup& s) {
  const int4 vi = __ldg(&vidx[f]);
  const float4 a = __ldg(&proj[vi.x]);
  const float4 b = __ldg(&proj[vi.y]);
  const float4 d = __ldg(&proj[vi.z]);
  return face_setup(c, make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z),
                    make_float3(d.x, d.y, d.z), s);
}

// A lower bound of the depth Loop B computes for the face at any covered
// pixel: the three edge functions carry rounding errors of at most
// delta = 2^-18 * bboxW * bboxH, so the interpolation weights' sum exceeds
// the area by at most delta and the depth is at least
// zmin * |A| / (|A| + delta), less a margin for this expression's own
// roundings.  -1 when no bound is proven.
__device__ __forceinline__ float depth_lower_bound(const FaceSetup& s) {
  const float zmin = fminf(fminf(s.v0.z, s.v1.z), s.v2.z);
  const float BW = fmaxf(fmaxf(s.v0.x, s.v1.x), s.v2.x) -
                   fminf(fminf(s.v0.x, s.v1.x), s.v2.x) + 1.0f;
  const float BH = fmaxf(fmaxf(s.v0.y, s.v1.y), s.v2.y) -
                   fminf(fminf(s.v0.y, s.v1.y), s.v2.y) + 1.0f;
  const float delta = kU64 * BW * BH;
  const float aa = fabsf(s.area);
  return (aa > 2.0f * delta && zmin > 0.0f) ? zmin * (aa / (aa + delta)) * 0.99998474f : -1.0f;
}

template <typename T>
__device__ __forceinline__ void copy_words(T& dst, const T& src) {
  const int* a = reinterpret_cast<const int*>(&src);
  int* b = reinterpret_cast<int*>(&dst);
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += blockDim.x) b[i] = a[i];
}

// Loop A for every vertex of one view (blockIdx.y), stored by vertex rank.
__global__ void __launch_bounds__(kBinThreads) k_proj(TileParams p) {
  __shared__ Cam sc;
  __shared__ int mesh, nv;
  __shared__ long long off;
  copy_words(sc, p.views[blockIdx.y].cam);
  if (threadIdx.x == 0) {
    mesh = p.views[blockIdx.y].mesh;
    off = p.views[blockIdx.y].proj_offset;
    nv = p.meshes[mesh].num_vertices;
  }
  __syncthreads();
  const int i = blockIdx.x * kBinThreads + threadIdx.x;
  if (i >= nv) return;
  const int* vorder = p.meshes[mesh].vorder;  // the table is in vertex-rank order
  const float4 a = __ldg(&p.meshes[mesh].vertices[vorder ? __ldg(&vorder[i]) : i]);
  const float3 q = project(sc, a.x, a.y, a.z);
  p.proj[off + i] = make_float4(q.x, q.y, q.z, 0.0f);
}

struct BinSmem {
  DevView view;
  DevMesh mesh;
  int tile[kAgg];
  int cnt[2 * kAgg];  // per (slot, class): entries, then their block-local offset
  int cur[2 * kAgg];  // per (slot, class): next entry of a many-tile face
  int warp_sum[kBinThreads / 32][2];
  int nspill;         // entries whose tile found no slot: one run each
  int spill_cur;
  unsigned long long base;      // the block's first staged entry
  unsigned long long run_base;  // the block's first run
  int ok;
};

__device__ __forceinline__ int agg_slot(BinSmem& sb, int t) {
  unsigned h = ((unsigned)t * 2654435761u) >> 24;  // 8 bits
  for (int probe = 0; probe < kAggProbes; ++probe) {
    const int seen = *(volatile int*)&sb.tile[h];
    if (seen == t) return (int)h;
    if (seen == -1) {
      const int cur = atomicCAS(&sb.tile[h], -1, t);
      if (cur == -1 || cur == t) return (int)h;
    }
    h = (h + 1) & (kAgg - 1);
  }
  return -1;
}

// The screen tiles of one face: the per-face culls of Loop B from the
// projected-vertex table, then the tile range of its pixel bbox.
struct FaceBins {
  int i, n, tx0, ty0, ntx, cls;  // i: the face's number in the binning order
  float zlb;
};

// Face number i of the binning order (DevMesh::order).
__device__ __forceinline__ FaceBins bin_face(const TileParams& p, const BinSmem& sb, int i) {
  FaceBins b{i, 0, 0, 0, 1, 0, -1.0f};
  if (i >= sb.mesh.num_faces) return b;
  FaceSetup s;
  if (!setup_proj(p.proj + sb.view.proj_offset, sb.mesh.vidx_morton, i, sb.view.cam, s) ||
      s.x1 < s.x0 || s.y1 < s.y0)
    return b;
  const int ts = p.tile_log2;
  b.tx0 = s.x0 >> ts;
  b.ty0 = s.y0 >> ts;
  b.ntx = (s.x1 >> ts) - b.tx0 + 1;
  b.n = b.ntx * ((s.y1 >> ts) - b.ty0 + 1);
  b.zlb = depth_lower_bound(s);
  b.cls = b.zlb > sb.view.split_z ? 1 : 0;
  return b;
}

// Slot of tile t in the block's table, or -1 (no insertion).
__device__ __forceinline__ int find_slot(const BinSmem& sb, int t) {
  unsigned h = ((unsigned)t * 2654435761u) >> 24;
  for (int probe = 0; probe < kAggProbes; ++probe) {
    const int seen = sb.tile[h];
    if (seen == t) return (int)h;
    if (seen == -1) return -1;
    h = (h + 1) & (kAgg - 1);
  }
  return -1;
}

// One block per (kBinThreads * kBinFaces faces, view), one pass over the
// faces.  The block sorts its (face, tile) entries by (tile, class) in
// shared memory, claims a range of the staging buffer and of the run list
// with one global atomic each, and writes each (tile, class) group as one
// run.  Faces touching at most kAggPerFace tiles (a tuning field,
// TileParams::agg_per_face: 1, 2 or 4) take their ranks with one
// shared atomic per warp and key; faces touching more take positions from
// per-group cursors after the fast ones; entries whose tile finds no slot
// in the table (at most kAggProbes probes) become runs of one.
#ifndef UGU_BIN_BLOCKS
#define UGU_BIN_BLOCKS 6
#endif
template <int kAggPerFace>
__global__ void __launch_bounds__(kBinThreads, UGU_BIN_BLOCKS) k_bin(TileParams p) {
  __shared__ BinSmem sb;
  copy_words(sb.view, p.views[blockIdx.y]);
  for (int i = threadIdx.x; i < kAgg; i += kBinThreads) {
    sb.tile[i] = -1;
    sb.cnt[2 * i] = sb.cnt[2 * i + 1] = 0;
  }
  if (threadIdx.x == 0) sb.nspill = sb.spill_cur = 0;
  __syncthreads();
  copy_words(sb.mesh, p.meshes[sb.view.mesh]);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  const int tbase = sb.view.tile_base, tiles_x = sb.view.tiles_x;
  const int f0 = blockIdx.x * (kBinThreads * kBinFaces) + threadIdx.x;
  FaceBins fb[kBinFaces];
#pragma unroll
  for (int u = 0; u < kBinFaces; ++u) fb[u] = bin_face(p, sb, f0 + u * kBinThreads);
  auto tile_of = [&](const FaceBins& b, int k) {
    return tbase + (b.ty0 + k / b.ntx) * tiles_x + b.tx0 + k % b.ntx;
  };
  // fast entries: ranks within their (slot, class) group
  int pk[kBinFaces][kAggPerFace];  // (slot, class) | rank << 9, or -1: a spilled entry
#pragma unroll
  for (int u = 0; u < kBinFaces; ++u) {
#pragma unroll
    for (int k = 0; k < kAggPerFace; ++k) {
      pk[u][k] = -1;
      const bool act = fb[u].n <= kAggPerFace && k < fb[u].n;
      const int t = act ? tile_of(fb[u], k) : 0;
      const unsigned am = __ballot_sync(0xffffffffu, act);
      if (act) {
        const unsigned peers = __match_any_sync(am, 2 * t + fb[u].cls);
        const int leader = __ffs(peers) - 1;
        int slot = 0, base = 0;
        if (lane == leader) {
          slot = agg_slot(sb, t);
          if (slot >= 0)
            base = atomicAdd(&sb.cnt[2 * slot + fb[u].cls], __popc(peers));
          else
            atomicAdd(&sb.nspill, __popc(peers));
        }
        slot = __shfl_sync(peers, slot, leader);
        base = __shfl_sync(peers, base, leader);
        if (slot >= 0)
          pk[u][k] = (2 * slot + fb[u].cls) | ((base + __popc(peers & below)) << 9);
      }
    }
  }
  __syncthreads();
  // many-tile faces: counted after the fast entries of every group, whose
  // counts the cursors keep (copied before any many-tile count is added)
  for (int i = threadIdx.x; i < 2 * kAgg; i += kBinThreads) sb.cur[i] = sb.cnt[i];
  __syncthreads();
#pragma unroll
  for (int u = 0; u < kBinFaces; ++u) {
    if (fb[u].n <= kAggPerFace) continue;
    for (int k = 0; k < fb[u].n; ++k) {
      const int slot = agg_slot(sb, tile_of(fb[u], k));
      if (slot >= 0)
        atomicAdd(&sb.cnt[2 * slot + fb[u].cls], 1);
      else
        atomicAdd(&sb.nspill, 1);
    }
  }
  __syncthreads();
  // block-wide exclusive scan of the (slot, class) counts and of the
  // nonempty groups (the runs); thread i owns slot i
  static_assert(kAgg == kBinThreads, "one aggregation slot per thread");
  const int i = threadIdx.x;
  const int c0 = sb.cnt[2 * i], c1 = sb.cnt[2 * i + 1];
  const int own_e = c0 + c1, own_r = (c0 > 0) + (c1 > 0);
  int xe = own_e, xr = own_r;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int ye = __shfl_up_sync(0xffffffffu, xe, o);
    const int yr = __shfl_up_sync(0xffffffffu, xr, o);
    if (lane >= o) {
      xe += ye;
      xr += yr;
    }
  }
  if (lane == 31) {
    sb.warp_sum[warp][0] = xe;
    sb.warp_sum[warp][1] = xr;
  }
  __syncthreads();
  int pe = 0, pr = 0, te = 0, tr = 0;
  for (int w = 0; w < kBinThreads / 32; ++w) {
    if (w < warp) {
      pe += sb.warp_sum[w][0];
      pr += sb.warp_sum[w][1];
    }
    te += sb.warp_sum[w][0];
    tr += sb.warp_sum[w][1];
  }
  // spilled entries follow the grouped ones, in the staging buffer and in
  // the run list alike
  const int ns = sb.nspill;
  const int off0 = pe + xe - own_e;  // block-local offset of (slot i, class 0)
  if (threadIdx.x == 0) {
    const unsigned long long ne = (unsigned long long)(te + ns), nr = (unsigned long long)(tr + ns);
    const unsigned long long b = ne ? atomicAdd(&p.counters->total_entries, ne) : 0;
    const unsigned long long r = nr ? atomicAdd(&p.counters->total_runs, nr) : 0;
    const bool ok = b + ne <= (unsigned long long)p.entry_cap &&
                    r + nr <= (unsigned long long)p.run_cap;
    if (!ok) {
      atomicExch(&p.counters->dropped, 1ull);
      if (p.sticky) atomicOr(p.sticky, kStickyOverflow);
    }
    sb.base = b;
    sb.run_base = r;
    sb.ok = ok;
  }
  __syncthreads();
  const bool ok = sb.ok;
  if (!ok) return;  // the render is retried with the counts this one reported
  sb.cur[2 * i] += off0;
  sb.cur[2 * i + 1] += off0 + c0;
  sb.cnt[2 * i] = off0;
  sb.cnt[2 * i + 1] = off0 + c0;
  if (own_r) {
    const int t = sb.tile[i];
    unsigned long long r = sb.run_base + (pr + xr - own_r);
    if (c0) p.runs[r++] = make_int4(t, 0, (int)(sb.base + off0), c0);
    if (c1) p.runs[r] = make_int4(t, 1, (int)(sb.base + off0 + c0), c1);
    atomicAdd(&p.tile_count[t], own_e);
  }
  __syncthreads();
  auto spill = [&](int t, int cls, int2 e) {
    const int k = atomicAdd(&sb.spill_cur, 1);
    const unsigned long long pos = sb.base + te + k;
    p.staged[pos] = e;
    p.runs[sb.run_base + tr + k] = make_int4(t, cls, (int)pos, 1);
    atomicAdd(&p.tile_count[t], 1);
  };
#pragma unroll
  for (int u = 0; u < kBinFaces; ++u) {
    const FaceBins& b = fb[u];
    const int2 e = make_int2(b.i, __float_as_int(b.zlb));
    if (b.n <= kAggPerFace) {
#pragma unroll
      for (int k = 0; k < kAggPerFace; ++k) {
        if (k >= b.n) continue;
        const int q = pk[u][k];
        if (q >= 0)
          p.staged[sb.base + sb.cnt[q & 511] + (q >> 9)] = e;
        else
          spill(tile_of(b, k), b.cls, e);
      }
    } else {
      for (int k = 0; k < b.n; ++k) {
        const int t = tile_of(b, k);
        const int slot = find_slot(sb, t);
        if (slot >= 0)
          p.staged[sb.base + atomicAdd(&sb.cur[2 * slot + b.cls], 1)] = e;
        else
          spill(t, b.cls, e);
      }
    }
  }
}

// Copies every run of staged entries into its tile's range (k_scan placed
// the cursors): faces drawn first from the front, faces drawn last from the
// back.  One warp per run.
__global__ void __launch_bounds__(256) k_gather(TileParams p) {
  if (p.counters->dropped) return;  // entries were not staged: the host retries
  const unsigned long long nr = p.counters->total_runs;
  const int lane = threadIdx.x & 31;
  const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x / 32);
  for (unsigned long long r = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); r < nr;
       r += warps) {
    const int4 run = p.runs[r];  // (tile, class, first staged entry, count)
    if (run.x < 0 || run.x >= p.total_tiles || run.z < 0 || run.w < 0 ||
        (int64_t)run.z + run.w > p.entry_cap) {  // never for k_bin's runs: reported, skipped
      if (lane == 0) atomicAdd(&p.counters->invalid, 1u);
      continue;
    }
    int dst = 0;
    if (lane == 0)
      dst = run.y ? atomicSub(&p.tile_hi[run.x], run.w) - run.w
                  : atomicAdd(&p.tile_lo[run.x], run.w);
    dst = __shfl_sync(0xffffffffu, dst, 0);
    for (int k = lane; k < run.w; k += 32) p.entries[dst + k] = p.staged[run.z + k];
  }
}

// Exclusive scan of the per-tile counts (one block, kScanItems consecutive
// tiles per thread and round, staged through shared memory so that global
// accesses coalesce); zeroes the counts for the next render and flags a
// render whose entries exceed the buffer.
__global__ void __launch_bounds__(kScanThreads) k_scan(TileParams p) {
  __shared__ int stage[kScanThreads * kScanItems];
  __shared__ long long warp_sum[kScanThreads / 32];
  const int T = p.total_tiles;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int kRound = kScanThreads * kScanItems;
  long long carry = 0;
  for (int r0 = 0; r0 < T; r0 += kRound) {
    for (int i = tid; i < kRound; i += kScanThreads) {
      const int t = r0 + i;
      stage[i] = t < T ? p.tile_count[t] : 0;
      if (t < T) p.tile_count[t] = 0;
    }
    __syncthreads();
    int v[kScanItems];
    long long own = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      v[k] = stage[tid * kScanItems + k];
      own += v[k];
    }
    long long x = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      long long w = warp_sum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_sum[lane] = w;
    }
    __syncthreads();
    long long run = carry + x - own + (warp ? warp_sum[warp - 1] : 0);
    const long long round_total = warp_sum[kScanThreads / 32 - 1];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      stage[tid * kScanItems + k] = (int)run;  // offsets stay below the entry capacity
      run += v[k];
    }
    __syncthreads();
    for (int i = tid; i < kRound; i += kScanThreads) {
      const int t = r0 + i;
      if (t >= T) break;
      const int off = stage[i];
      const int nxt = i + 1 < kRound ? stage[i + 1] : (int)(carry + round_total);
      p.tile_off[t] = off;
      p.tile_lo[t] = off;
      p.tile_hi[t] = nxt;
    }
    carry += round_total;
    __syncthreads();
  }
  if (tid == 0) {
    p.tile_off[T] = (int)carry;  // k_bin's cursor keeps the render's entry count
    if (carry > p.entry_cap) {
      p.counters->dropped = 1ull;
      if (p.sticky) atomicOr(p.sticky, kStickyOverflow);
    }
  }
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
// for every pixel number k < width * height <= 1024 of the box.
__device__ __forceinline__ float pack_box(int x0, int y0, int w) {
  const unsigned m = (65536u + (unsigned)w - 1u) / (unsigned)w;
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
      const int bw = (int)((box >> 10) & 31u) + 1, bh = cnt / bw;
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
  const int tlog = p.tile_log2;
  const int T = 1 << tlog;
  if (p.counters->dropped) return;  // entries were not written: the host retries
  int v_begin = 0, v_end = 0;  // global tiles of the view in shared memory
  Region& R = sm.reg;
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
          if ((unsigned)e.x >= (unsigned)sm.mesh.num_faces) {  // never for k_bin's entries
            atomicAdd(&p.counters->invalid, 1u);
            continue;
          }
          if (zlb > zmax) continue;  // behind every key of a covered tile: cannot win
          const int f = __ldg(&sm.mesh.order[e.x]);  // the entry holds the binning number
          FaceSetup s;
          setup_proj(proj, sm.mesh.vidx_morton, e.x, c, s);  // succeeded in k_bin: same arithmetic
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
          R.r1[j] = make_float4(s.v2.x, s.v2.y, s.area, pack_box(bx0 - tx0, by0 - ty0, bw));
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

void launch_size(const TileParams& p, int max_faces, cudaStream_t s) {
  constexpr int kPerBlock = kBinThreads * kBinFaces;
  // a mesh without vertices or faces bins nothing (a grid of zero blocks is
  // a launch error); the scan, gather and tile kernels then write empty images
  if (p.max_vertices > 0)
    k_proj<<<dim3((p.max_vertices + kBinThreads - 1) / kBinThreads, p.num_views), kBinThreads,
             0, s>>>(p);
  if (max_faces > 0) {
    const dim3 grid((max_faces + kPerBlock - 1) / kPerBlock, p.num_views);
    if (p.agg_per_face == 1)
      k_bin<1><<<grid, kBinThreads, 0, s>>>(p);
    else if (p.agg_per_face == 4)
      k_bin<4><<<grid, kBinThreads, 0, s>>>(p);
    else
      k_bin<2><<<grid, kBinThreads, 0, s>>>(p);
  }
  k_scan<<<1, kScanThreads, 0, s>>>(p);
}

void launch_bin(const TileParams& p, int max_faces, int gather_blocks, cudaStream_t s) {
  launch_size(p, max_faces, s);
  k_gather<<<gather_blocks, 256, 0, s>>>(p);
}

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

int bin_kernel_blocks_per_sm() {
  static int blocks = 0;
  if (!blocks) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_bin<2>, kBinThreads, 0);
    if (blocks < 1) blocks = 1;
  }
  return blocks;
}

}  // namespace ugu_gpu
