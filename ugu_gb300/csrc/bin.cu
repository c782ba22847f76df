// bin.cu -- the tiled forward path's binning: every face of every view to
// the screen tiles it may cover, as (face, tile) entry lists per tile that
// the tile kernel (tile.cu) reads.  A counting sort in two passes over the
// faces, with no staging buffer:
//
//   k_proj   Loop A (rasterizer.cc:131-136): every vertex of every view through
//            PinholeCamera::Project once, into a table of float4 (x, y, z).
//   k_count  one pass over every (view, face): the per-face culls of Loop B
//            (rasterizer.cc:163-193) from the table and the screen tiles the
//            face's bbox touches; a warp's entries of one tile are added to
//            the tile's count with one atomic.
//   k_scan_sum, k_scan_apply
//            exclusive scan of the per-tile counts into entry offsets, so the
//            entry buffer holds exactly the render's (face, tile) pairs: each
//            chunk of 4,096 tiles summed, then scanned from the sums before it.
//   k_place  the same pass again: each entry goes straight to its place in
//            its tile's range, faces drawn first from the front and faces
//            drawn last from the back, one atomic per warp, tile and class.
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.cuh"
#include "tilecommon.cuh"

namespace ugu_gpu {

namespace {

using tiled::copy_words;
using tiled::kU64;

constexpr int kBinThreads = 256;
constexpr int kScanThreads = 256;
constexpr int kScanWarps = kScanThreads / 32;
constexpr int kScanItems = 16;  // tile counts per scan thread
constexpr int kScanChunk = kScanThreads * kScanItems;

// A lower bound of the depth Loop B computes for the face at any covered
// pixel: the three edge functions carry rounding errors of at most
// delta = 2^-18 * bboxW * bboxH, so the interpolation weights' sum exceeds
// the area by at most delta and the depth is at least
// zmin * |A| / (|A| + delta), less a margin of 2^-16 for this expression's
// own roundings: four of 2^-24 each, and the fast quotient's (at most two
// ulp, 2^-22, for a divisor in [2^-126, 2^126]; |A| + delta >= 3 * 2^-18,
// and past 2^126 the fast quotient is 0, which is still a lower bound).
// -1 when no bound is proven.
__device__ __forceinline__ float depth_lower_bound(const FaceSetup& s) {
  const float zmin = fminf(fminf(s.v0.z, s.v1.z), s.v2.z);
  const float BW = fmaxf(fmaxf(s.v0.x, s.v1.x), s.v2.x) -
                   fminf(fminf(s.v0.x, s.v1.x), s.v2.x) + 1.0f;
  const float BH = fmaxf(fmaxf(s.v0.y, s.v1.y), s.v2.y) -
                   fminf(fminf(s.v0.y, s.v1.y), s.v2.y) + 1.0f;
  const float delta = kU64 * BW * BH;
  const float aa = fabsf(s.area);
  return (aa > 2.0f * delta && zmin > 0.0f) ? zmin * __fdividef(aa, aa + delta) * 0.99998474f
                                             : -1.0f;
}

// Loop A for every vertex of one view (blockIdx.y), stored by vertex rank;
// kProjVerts vertices per thread, so that the per-block set-up (the camera
// copied to shared memory) is paid for once per 1,024 vertices.
constexpr int kProjVerts = 4;
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
  const int* vorder = p.meshes[mesh].vorder;  // the table is in vertex-rank order
  const float4* vert = p.meshes[mesh].vertices;
#pragma unroll
  for (int k = 0; k < kProjVerts; ++k) {
    const int i = (blockIdx.x * kProjVerts + k) * kBinThreads + threadIdx.x;
    if (i >= nv) return;
    const float4 a = __ldg(&vert[vorder ? __ldg(&vorder[i]) : i]);
    const float3 q = project(sc, a.x, a.y, a.z);
    p.proj[off + i] = make_float4(q.x, q.y, q.z, 0.0f);
  }
}

// The view and its mesh, in shared memory for a binning block.
struct BinShared {
  DevView view;
  DevMesh mesh;
};

// Binning blocks run view-fastest: block b takes face block b / num_views of
// view b % num_views, so that the blocks resident together spread over all
// views' tiles rather than crowd one view's tile counters with atomics.
__device__ __forceinline__ int bin_block_view(const TileParams& p) {
  return (int)(blockIdx.x % (unsigned)p.num_views);
}
__device__ __forceinline__ int bin_block_faces(const TileParams& p) {
  return (int)(blockIdx.x / (unsigned)p.num_views);
}

__device__ __forceinline__ void load_bin_view(const TileParams& p, BinShared& sb) {
  copy_words(sb.view, p.views[bin_block_view(p)]);
  __syncthreads();
  copy_words(sb.mesh, p.meshes[sb.view.mesh]);
  __syncthreads();
}

// The screen tiles of one face: the per-face culls of Loop B from the
// projected-vertex table, then the tile range of its pixel bbox.
struct FaceBins {
  int i, n, tx0, ty0, ntx, cls;  // i: the face's number in the binning order
  float zlb;
};

// Loop B's per-face set-up (rasterizer.cc:163-193) as face_setup computes
// it, with one more cull first: a bbox holding no integer pixel (most faces
// of a finely tessellated mesh at these view sizes) is rejected before the
// area is formed.  Every face it keeps has face_setup's values; every face
// it rejects, face_setup rejects or gives an empty bbox.
__device__ __forceinline__ bool bin_setup(const float4* proj, const int4* vidx, int f,
                                          const Cam& c, FaceSetup& s) {
  const int4 vi = __ldg(&vidx[f]);
  const float4 a = __ldg(&proj[vi.x]);
  const float4 b = __ldg(&proj[vi.y]);
  const float4 d = __ldg(&proj[vi.z]);
  if (a.z < 0.0f || b.z < 0.0f || d.z < 0.0f) return false;
  const float xmin = min3_std(a.x, b.x, d.x), ymin = min3_std(a.y, b.y, d.y);
  const float xmax = max3_std(a.x, b.x, d.x), ymax = max3_std(a.y, b.y, d.y);
  if (xmin > (float)(c.width - 1) || xmax < 0.0f || ymin > (float)(c.height - 1) || ymax < 0.0f)
    return false;
  s.x0 = max(0, f2i_sat(ceilf(xmin)));
  s.x1 = min(c.width - 1, f2i_sat(floorf(xmax)));
  s.y0 = max(0, f2i_sat(ceilf(ymin)));
  s.y1 = min(c.height - 1, f2i_sat(floorf(ymax)));
  if (s.x1 < s.x0 || s.y1 < s.y0) return false;
  s.area = edge_fn(a.x, a.y, b.x, b.y, d.x, d.y);
  if (fabsf(s.area) < FLT_MIN) return false;
  s.v0 = make_float3(a.x, a.y, a.z);
  s.v1 = make_float3(b.x, b.y, b.z);
  s.v2 = make_float3(d.x, d.y, d.z);
  return true;
}

// Face number i of the binning order (DevMesh::order); n = 0 for a face
// that reaches no pixel.  Faces whose depth lower bound lies behind the
// split depth are drawn last (cls 1).
__device__ __forceinline__ FaceBins bin_face(const TileParams& p, const BinShared& sb, int i) {
  FaceBins b{i, 0, 0, 0, 1, 0, -1.0f};
  if (i >= sb.mesh.num_faces) return b;
  FaceSetup s;
  if (!bin_setup(p.proj + sb.view.proj_offset, sb.mesh.vidx_morton, i, sb.view.cam, s)) return b;
  const int ts = sb.view.tile_log2;
  b.tx0 = s.x0 >> ts;
  b.ty0 = s.y0 >> ts;
  b.ntx = (s.x1 >> ts) - b.tx0 + 1;
  b.n = b.ntx * ((s.y1 >> ts) - b.ty0 + 1);
  b.zlb = depth_lower_bound(s);
  b.cls = b.zlb > sb.view.split_z ? 1 : 0;
  return b;
}

// kPlace false: count every (face, tile) entry of kFaces faces per thread;
// true: write each entry to its place.  The lanes of a warp walk their
// faces' tiles together; lanes whose current tile (and, when placing, draw
// class) agree take one atomic between them, made by the lowest of them.
template <int kFaces, bool kPlace>
__device__ __forceinline__ void bin_pass(const TileParams& p) {
  __shared__ BinShared sb;
  if (kPlace && p.counters->dropped) return;  // entries do not fit: the host retries
  load_bin_view(p, sb);
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int f0 = bin_block_faces(p) * (kBinThreads * kFaces) + threadIdx.x;
#pragma unroll
  for (int u = 0; u < kFaces; ++u) {
    const FaceBins b = bin_face(p, sb, f0 + u * kBinThreads);
    const int nmax = __reduce_max_sync(0xffffffffu, b.n);
    const int2 e = make_int2(b.i, __float_as_int(b.zlb));
    // the face's tiles in row-major order over its tile range, walked
    // without a division per tile
    int cx = 0, row = sb.view.tile_base + b.ty0 * sb.view.tiles_x + b.tx0;
    for (int k = 0; k < nmax; ++k) {
      const bool act = k < b.n;
      const unsigned am = __ballot_sync(0xffffffffu, act);
      if (!act) continue;
      const int t = row + cx;
      if (++cx == b.ntx) {
        cx = 0;
        row += sb.view.tiles_x;
      }
      const unsigned peers = __match_any_sync(am, kPlace ? 2 * t + b.cls : t);
      const int leader = __ffs(peers) - 1, cnt = __popc(peers);
      if (!kPlace) {
        if (lane == leader) atomicAdd(&p.tile_count[t], cnt);
        continue;
      }
      int base = 0;
      if (lane == leader)
        base = b.cls ? atomicSub(&p.tile_hi[t], cnt) - cnt : atomicAdd(&p.tile_lo[t], cnt);
      base = __shfl_sync(peers, base, leader);
      const int pos = base + __popc(peers & below);
      if ((unsigned)pos < (unsigned)p.entry_cap)  // always: the counts match the places
        p.entries[pos] = e;
      else
        atomicAdd(&p.counters->invalid, 1u);
    }
  }
}

template <int kFaces>
__global__ void __launch_bounds__(kBinThreads) k_count(TileParams p) {
  bin_pass<kFaces, false>(p);
}

// Eight blocks per SM (32 registers, a few spilled) rather than the six that
// 40 registers allow: the placing atomics' latency wants the warps.
template <int kFaces>
__global__ void __launch_bounds__(kBinThreads, 8) k_place(TileParams p) {
  bin_pass<kFaces, true>(p);
}

// Exclusive scan of the per-tile counts in chunks of kScanChunk tiles, one
// block per chunk: k_scan_sum sums each chunk, k_scan_apply scans its chunk
// from the sum of the chunks before it.  A block's counts are staged through
// shared memory so that global accesses coalesce, kScanItems consecutive
// tiles per thread (the staging index skips one word in 33, so that a
// thread's run sits in different banks).  k_scan_apply zeroes the counts for
// the next render, and its last block flags a render whose entries exceed
// the buffer.
__device__ __forceinline__ int skew(int i) { return i + (i >> 5); }

// A block's sum of one value per thread (every thread gets it).
__device__ __forceinline__ long long block_sum(long long v, long long* warp_part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();  // warp_part may still be read from a previous use
  if (lane == 0) warp_part[warp] = v;
  __syncthreads();
  long long t = 0;
#pragma unroll
  for (int w = 0; w < kScanWarps; ++w) t += warp_part[w];
  return t;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sum(TileParams p) {
  __shared__ long long warp_part[kScanWarps];
  const int T = p.total_tiles, tid = threadIdx.x;
  const int r0 = blockIdx.x * kScanChunk;
  long long v = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int t = r0 + k * kScanThreads + tid;
    if (t < T) v += p.tile_count[t];
  }
  v = block_sum(v, warp_part);
  if (tid == 0) p.chunk_sums[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(TileParams p) {
  __shared__ int stage[kScanChunk + kScanChunk / 32];  // skew(kScanChunk) words
  __shared__ long long warp_part[kScanWarps];
  const int T = p.total_tiles;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = blockIdx.x * kScanChunk;
  // the entries of the chunks before this one
  long long carry = 0;
  for (int j = tid; j < (int)blockIdx.x; j += kScanThreads) carry += p.chunk_sums[j];
  carry = block_sum(carry, warp_part);
  {
    // every load issued before the first store, so that the thread waits
    // for one memory latency and not one per count
    int c[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      const int t = r0 + k * kScanThreads + tid;
      c[k] = t < T ? p.tile_count[t] : 0;
    }
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      const int t = r0 + k * kScanThreads + tid;
      stage[skew(k * kScanThreads + tid)] = c[k];
      if (t < T) p.tile_count[t] = 0;
    }
  }
  __syncthreads();
  int v[kScanItems];
  long long own = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = stage[skew(tid * kScanItems + k)];
    own += v[k];
  }
  long long x = own;  // inclusive scan of the threads' sums: warps, then the block
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();  // warp_part's sums above have been read
  if (lane == 31) warp_part[warp] = x;
  __syncthreads();
  long long before = 0, total = 0;
#pragma unroll
  for (int w = 0; w < kScanWarps; ++w) {
    const long long sw = warp_part[w];
    if (w < warp) before += sw;
    total += sw;
  }
  long long run = carry + before + x - own;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    stage[skew(tid * kScanItems + k)] = (int)run;  // offsets stay below the entry capacity
    run += v[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int i = k * kScanThreads + tid;
    const int t = r0 + i;
    if (t >= T) break;
    const int off = stage[skew(i)];
    const int nxt = i + 1 < kScanChunk ? stage[skew(i + 1)] : (int)(carry + total);
    p.tile_off[t] = off;
    p.tile_lo[t] = off;
    p.tile_hi[t] = nxt;
  }
  if (blockIdx.x == gridDim.x - 1 && tid == 0) {
    const long long all = carry + total;
    p.tile_off[T] = (int)all;
    p.counters->total_entries = (unsigned long long)all;  // the render's entry count
    if (all > p.entry_cap) {
      p.counters->dropped = 1ull;
      if (p.sticky) atomicOr(p.sticky, kStickyOverflow);
    }
  }
}

}  // namespace

template <int kFaces>
void launch_pass(const TileParams& p, dim3 grid, bool place, cudaStream_t s) {
  if (place)
    k_place<kFaces><<<grid, kBinThreads, 0, s>>>(p);
  else
    k_count<kFaces><<<grid, kBinThreads, 0, s>>>(p);
}

void launch_pass(const TileParams& p, int max_faces, bool place, cudaStream_t s) {
  const int faces = p.bin_faces == 1 || p.bin_faces == 4 ? p.bin_faces : 2;
  const dim3 grid((unsigned)(((int64_t)max_faces + kBinThreads * faces - 1) /
                             (kBinThreads * faces) * p.num_views));
  if (faces == 1)
    launch_pass<1>(p, grid, place, s);
  else if (faces == 4)
    launch_pass<4>(p, grid, place, s);
  else
    launch_pass<2>(p, grid, place, s);
}

void launch_size(const TileParams& p, int max_faces, cudaStream_t s) {
  // a mesh without vertices or faces bins nothing (a grid of zero blocks is
  // a launch error); the scan and tile kernels then write empty images
  if (p.max_vertices > 0)
    k_proj<<<dim3((p.max_vertices + kProjVerts * kBinThreads - 1) / (kProjVerts * kBinThreads),
                  p.num_views),
             kBinThreads, 0, s>>>(p);
  if (max_faces > 0) launch_pass(p, max_faces, false, s);
  const int chunks = std::max(1, (p.total_tiles + kScanChunk - 1) / kScanChunk);
  k_scan_sum<<<chunks, kScanThreads, 0, s>>>(p);
  k_scan_apply<<<chunks, kScanThreads, 0, s>>>(p);
}

int64_t scan_chunks(int64_t tiles) { return std::max<int64_t>(1, (tiles + kScanChunk - 1) / kScanChunk); }

void launch_bin(const TileParams& p, int max_faces, cudaStream_t s) {
  launch_size(p, max_faces, s);
  if (max_faces > 0) launch_pass(p, max_faces, true, s);
}

}  // namespace ugu_gpu
