// bin.cu -- the tiled forward path's binning: every face of every view to
// the screen tiles it may cover, as (face, tile) entry lists per tile that
// the tile kernel (tile.cu) reads.
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
#include <cuda_runtime.h>

#include "internal.cuh"
#include "tilecommon.cuh"

namespace ugu_gpu {

namespace {

using tiled::copy_words;
using tiled::kU64;
using tiled::setup_proj;

constexpr int kBinThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kBinFaces = 2;     // faces per binning thread
constexpr int kAgg = 256;        // distinct tiles a binning block aggregates
constexpr int kAggProbes = 8;
constexpr int kScanItems = 8;    // tile counts per scan thread and round

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
  const int ts = sb.view.tile_log2;
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

int bin_kernel_blocks_per_sm() {
  static int blocks = 0;
  if (!blocks) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_bin<2>, kBinThreads, 0);
    if (blocks < 1) blocks = 1;
  }
  return blocks;
}

}  // namespace ugu_gpu
