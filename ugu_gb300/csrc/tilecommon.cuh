// tilecommon.cuh -- pieces shared by the tiled path's binning kernels
// (bin.cu) and its tile kernel (tile.cu).
#pragma once

#include "internal.cuh"

namespace ugu_gpu {
namespace tiled {

constexpr float kU64 = 3.814697265625e-06f;  // 2^-18 = 64 ulp(1)

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

template <typename T>
__device__ __forceinline__ void copy_words(T& dst, const T& src) {
  const int* a = reinterpret_cast<const int*>(&src);
  int* b = reinterpret_cast<int*>(&dst);
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += blockDim.x) b[i] = a[i];
}

}  // namespace tiled
}  // namespace ugu_gpu
