// backward.cu -- gradient of a per-pixel L2 colour loss through the resolve.
//
// No reference counterpart (ugu's rasterizer has no backward).  For each view
// the loss is L = sum over pixels p with face_id(p) > 0 of |C(p) - T(p)|^2,
// where C is the unquantised colour of the forward's colorizer
// (pixel_shader.h:234-359, float texels or vertex colours, no shading) and T
// the target image.  Visibility is held fixed: the kernel reads the
// forward's face_id image and recomputes that face's perspective-correct
// barycentrics at the pixel with the forward's exact arithmetic, so C here is
// bit-identical to the forward's colour.  Gradients:
//   texels        dL/dt = 2 (C - T) * bilinear weight (4 texels, material 0)
//   vertex colour dL/dc_k = 2 (C - T) * (1 - u - v, u, v)_k
//   vertex xyz    through u, v -> w = q / sum q, q_k = b_k / z_k,
//                 b_k = e_k / A (edge functions over the area), the pinhole
//                 projection and the camera rotation.
// Per-face contributions of a warp's pixels are summed in registers first:
// in one image row the pixels of one face form a contiguous run of lanes, so
// a segmented shuffle reduction leaves the run's total in its first lane,
// which issues the atomics (warp-aggregated scatter).
#include <cuda_runtime.h>

#include "internal.cuh"
#include "shade.cuh"

namespace ugu_gpu {

namespace {

constexpr int kThreads = 256;

// Sum v over the contiguous run of lanes that share the run id `key`; the
// run's first lane ends up with the total.  Lanes with key < 0 take no part.
__device__ __forceinline__ float run_sum(float v, int key, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float ov = __shfl_down_sync(0xffffffffu, v, o);
    const int ok = __shfl_down_sync(0xffffffffu, key, o);
    if (lane + o < 32 && ok == key) v += ov;
  }
  return v;
}

// Lane of the first pixel of this lane's run of equal keys (or -1): the run
// id used by run_sum.  Runs of the same face separated by another face's
// pixels get different ids, so every run is contiguous.
__device__ __forceinline__ int run_id(int key, int lane) {
  const int prev = __shfl_up_sync(0xffffffffu, key, 1);
  const bool head = key >= 0 && (lane == 0 || prev != key);
  const unsigned heads = __ballot_sync(0xffffffffu, head);
  if (key < 0) return -1;
  return 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
}

// One vertex of one view in double: screen x, y, camera z and 1 / z.
struct alignas(16) Proj64 {
  double x, y, z, iz;
};

// The pinhole projection of every vertex of one view (blockIdx.y) in
// double, from the float vertices and camera (camera.h:380-387).
__global__ void __launch_bounds__(kThreads) k_proj64(BackwardParams p) {
  const DevView& V = p.views[blockIdx.y];
  const DevMesh& M = p.meshes[V.mesh];
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= M.num_vertices) return;
  const Cam& c = V.cam;
  const float4 P = __ldg(&M.vertices[i]);
  double cc[3];
#pragma unroll
  for (int j = 0; j < 3; ++j)
    cc[j] = (double)c.R[3 * j] * P.x + (double)c.R[3 * j + 1] * P.y +
            (double)c.R[3 * j + 2] * P.z + (double)c.t[j];
  Proj64 o;
  o.iz = 1.0 / cc[2];
  o.x = (double)c.fx * cc[0] * o.iz + (double)c.cx;
  o.y = (double)c.fy * cc[1] * o.iz + (double)c.cy;
  o.z = cc[2];
  reinterpret_cast<Proj64*>(p.proj64)[V.proj_offset + i] = o;
}

__device__ __forceinline__ Proj64 load_proj64(const Proj64* t, int i) {
  const double2* q = reinterpret_cast<const double2*>(t + i);
  const double2 a = __ldg(q), b = __ldg(q + 1);
  Proj64 o;
  o.x = a.x;
  o.y = a.y;
  o.z = b.x;
  o.iz = b.y;
  return o;
}

// Vertex-position (and colour, texel) gradients of one pixel.  The
// quantities whose float rounding the sum over pixels would amplify are
// formed in double from the view's double projection table: the edge
// functions and the normalised perspective weights w = r / sum(r) with
// r_k = e_k / z_k (the area cancels in w, so it has no gradient), the
// texture coordinates with their texel cell and offsets, and the
// pixel-to-vertex differences the edge derivatives multiply.  The rest of
// the chain is float.
struct PixGrad {
  float loss;
  float gpos[9];
  float gcol[9];
  int64_t tix[4];
  float tg[4][3];  // per texel: dL/dt
  int ntex;
};

__device__ __forceinline__ void pixel_backward(const BackwardParams& p, const DevMesh& m,
                                               const Cam& c, const Proj64* tab, int fid, int x,
                                               int y, const float* target, PixGrad& o) {
  const int4 vi = __ldg(&m.vidx[fid]);
  const Proj64 P[3] = {load_proj64(tab, vi.x), load_proj64(tab, vi.y), load_proj64(tab, vi.z)};
  const double px = x, py = y;
  double dx[3], dy[3];  // pixel minus vertex
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dx[k] = px - P[k].x;
    dy[k] = py - P[k].y;
  }
  // e_k = edge(v_a, v_b, p) for (a, b) = (1, 2), (2, 0), (0, 1)
  const double e0 = dx[1] * (P[2].y - P[1].y) - dy[1] * (P[2].x - P[1].x);
  const double e1 = dx[2] * (P[0].y - P[2].y) - dy[2] * (P[0].x - P[2].x);
  const double e2 = dx[0] * (P[1].y - P[0].y) - dy[0] * (P[1].x - P[0].x);
  const double r[3] = {e0 * P[0].iz, e1 * P[1].iz, e2 * P[2].iz};
  const double iS = 1.0 / (r[0] + r[1] + r[2]);
  const double ud = r[1] * iS, vd = r[2] * iS, s0d = 1.0 - ud - vd;
  const float u = (float)ud, v = (float)vd, s0 = (float)s0d;
  float col[3], dcu[3], dcv[3];
  o.ntex = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    o.tix[j] = 0;
    o.tg[j][0] = o.tg[j][1] = o.tg[j][2] = 0.0f;
  }
  if (p.diffuse_color == 2) {
    const float4 c0 = __ldg(&m.vcolors[vi.x]);
    const float4 c1 = __ldg(&m.vcolors[vi.y]);
    const float4 c2 = __ldg(&m.vcolors[vi.z]);
    const float a0[3] = {c0.x, c0.y, c0.z}, a1[3] = {c1.x, c1.y, c1.z}, a2[3] = {c2.x, c2.y, c2.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      col[k] = (float)(s0d * a0[k] + ud * a1[k] + vd * a2[k]);
      dcu[k] = a1[k] - a0[k];
      dcv[k] = a2[k] - a0[k];
    }
  } else {
    const int mid = __ldg(&m.mat_ids[fid]);
    const DevTexture t = m.textures[mid];
    const int4 ti = __ldg(&m.uvidx[fid]);
    const float2 a = __ldg(&m.uv[ti.x]), b = __ldg(&m.uv[ti.y]), d = __ldg(&m.uv[ti.z]);
    const double uvx = s0d * a.x + ud * b.x + vd * d.x;
    const double uvy = s0d * a.y + ud * b.y + vd * d.y;
    const double fx = uvx * (t.width - 1), fy = (1.0 - uvy) * (t.height - 1);
    if (p.interp == 0) {
      const int64_t ix = texel_index((int64_t)llrint(fy), (int64_t)llrint(fx), t.width, t.height);
      fetch_texel(t, ix, col);
#pragma unroll
      for (int k = 0; k < 3; ++k) dcu[k] = dcv[k] = 0.0f;
      o.tix[0] = ix;
      o.tg[0][0] = o.tg[0][1] = o.tg[0][2] = 1.0f;  // weights; scaled by dL/dC below
      o.ntex = mid == 0 ? 1 : 0;
    } else {
      const double x0 = floor(fx), y0 = floor(fy);
      const float lu = (float)(fx - x0), lv = (float)(fy - y0);
      o.tix[0] = texel_index((int64_t)y0, (int64_t)x0, t.width, t.height);
      o.tix[1] = texel_index((int64_t)y0, (int64_t)x0 + 1, t.width, t.height);
      o.tix[2] = texel_index((int64_t)y0 + 1, (int64_t)x0, t.width, t.height);
      o.tix[3] = texel_index((int64_t)y0 + 1, (int64_t)x0 + 1, t.width, t.height);
      float t00[3], t10[3], t01[3], t11[3];
      fetch_texel(t, o.tix[0], t00);
      fetch_texel(t, o.tix[1], t10);
      fetch_texel(t, o.tix[2], t01);
      fetch_texel(t, o.tix[3], t11);
      const float dfx_du = (b.x - a.x) * (float)(t.width - 1);
      const float dfx_dv = (d.x - a.x) * (float)(t.width - 1);
      const float dfy_du = -(b.y - a.y) * (float)(t.height - 1);
      const float dfy_dv = -(d.y - a.y) * (float)(t.height - 1);
      const float w00 = (1.0f - lu) * (1.0f - lv), w10 = lu * (1.0f - lv);
      const float w01 = (1.0f - lu) * lv, w11 = lu * lv;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        col[k] = w00 * t00[k] + w10 * t10[k] + w01 * t01[k] + w11 * t11[k];
        const float dlu = (1.0f - lv) * (t10[k] - t00[k]) + lv * (t11[k] - t01[k]);
        const float dlv = (1.0f - lu) * (t01[k] - t00[k]) + lu * (t11[k] - t10[k]);
        dcu[k] = dlu * dfx_du + dlv * dfy_du;
        dcv[k] = dlu * dfx_dv + dlv * dfy_dv;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        o.tg[0][k] = w00;
        o.tg[1][k] = w10;
        o.tg[2][k] = w01;
        o.tg[3][k] = w11;
      }
      o.ntex = mid == 0 ? 4 : 0;
    }
  }
  float gC[3];
  o.loss = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float dd = col[k] - __ldg(&target[k]);
    o.loss += dd * dd;
    gC[k] = 2.0f * dd;
    o.gcol[k] = gC[k] * s0;
    o.gcol[3 + k] = gC[k] * u;
    o.gcol[6 + k] = gC[k] * v;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) o.tg[j][k] *= gC[k];
  // through w = r / S, r_k = e_k / z_k
  const float gw1 = gC[0] * dcu[0] + gC[1] * dcu[1] + gC[2] * dcu[2];
  const float gw2 = gC[0] * dcv[0] + gC[1] * dcv[1] + gC[2] * dcv[2];
  const float gdotw = gw1 * u + gw2 * v;
  const float fiS = (float)iS;
  const float gr[3] = {-gdotw * fiS, (gw1 - gdotw) * fiS, (gw2 - gdotw) * fiS};
  float ge[3], gZ[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float iz = (float)P[k].iz;
    ge[k] = gr[k] * iz;
    gZ[k] = -gr[k] * (float)r[k] * iz;
  }
  const float fdx[3] = {(float)dx[0], (float)dx[1], (float)dx[2]};
  const float fdy[3] = {(float)dy[0], (float)dy[1], (float)dy[2]};
  float gX[3] = {0.0f, 0.0f, 0.0f}, gY[3] = {0.0f, 0.0f, 0.0f};
  const int ea[3] = {1, 2, 0}, eb[3] = {2, 0, 1};
#pragma unroll
  for (int k = 0; k < 3; ++k) {  // e_k = dy_a dx_b - dx_a dy_b (d = pixel - vertex)
    const int ia = ea[k], ib = eb[k];
    gX[ia] += ge[k] * fdy[ib];
    gY[ia] -= ge[k] * fdx[ib];
    gX[ib] -= ge[k] * fdy[ia];
    gY[ib] += ge[k] * fdx[ia];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float iz = (float)P[k].iz;
    const float gcx = gX[k] * c.fx * iz;
    const float gcy = gY[k] * c.fy * iz;
    const float gcz = -(gX[k] * (float)(P[k].x - c.cx) + gY[k] * (float)(P[k].y - c.cy)) * iz + gZ[k];
#pragma unroll
    for (int j = 0; j < 3; ++j) o.gpos[3 * k + j] = c.R[j] * gcx + c.R[3 + j] * gcy + c.R[6 + j] * gcz;
  }
}

__global__ void __launch_bounds__(kThreads) k_backward(BackwardParams p) {
  __shared__ DevView sv;
  __shared__ DevMesh sm;
  __shared__ float s_loss[kThreads / 32];
  {
    const int* src = reinterpret_cast<const int*>(&p.views[blockIdx.y]);
    int* dst = reinterpret_cast<int*>(&sv);
    for (int i = threadIdx.x; i < (int)(sizeof(DevView) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    const int* msrc = reinterpret_cast<const int*>(&p.meshes[sv.mesh]);
    int* mdst = reinterpret_cast<int*>(&sm);
    for (int i = threadIdx.x; i < (int)(sizeof(DevMesh) / 4); i += blockDim.x) mdst[i] = msrc[i];
    __syncthreads();
  }
  const Cam& c = sv.cam;
  const int lane = threadIdx.x & 31;
  const int64_t npx = (int64_t)c.width * c.height;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int fid = -1;
  int x = 0, y = 0;
  if (i < npx) {
    fid = sv.face_id[i];
    x = (int)(i % c.width);
    y = (int)(i / c.width);
    if (fid < -1 || fid >= sm.num_faces) {  // not a forward's face id: reported, skipped
      atomicAdd(p.bad_ids, 1ull);
      fid = -1;
    }
  }
  // a run of one face never continues across an image row
  const int key = fid > 0 ? fid * 2 + (y & 1) : -1;

  float loss = 0.0f;
  float gv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // vertex xyz grads, 3 vertices
  float gc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // vertex colour grads
  int4 vi = make_int4(0, 0, 0, 0);
  if (fid > 0 && p.grad_vertices) {
    // Position gradients sum many contributions of both signs, which
    // amplifies rounding: see pixel_backward.
    vi = __ldg(&sm.vidx[fid]);
    PixGrad o;
    pixel_backward(p, sm, c, reinterpret_cast<const Proj64*>(p.proj64) + sv.proj_offset, fid, x,
                   y, &p.targets[blockIdx.y][3 * i], o);
    loss = o.loss;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      gv[k] = o.gpos[k];
      gc[k] = p.diffuse_color == 2 ? o.gcol[k] : 0.0f;
    }
    if (p.grad_texels && p.diffuse_color == 1)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < o.ntex)
#pragma unroll
          for (int k = 0; k < 3; ++k) atomicAdd(&p.grad_texels[3 * o.tix[j] + k], o.tg[j][k]);
  } else if (fid > 0) {
    // Texel and vertex-colour gradients only: the float colour equals the
    // forward's (same exact arithmetic), so the loss is the rendered one.
    vi = __ldg(&sm.vidx[fid]);
    FaceSetup s = project_face(sm, c, fid);
    Bary w = edges_at(s, x, y);
    perspective(s, w);
    const float u = w.w1, v = w.w2;
    const float s0 = fsub(fsub(1.0f, u), v);
    const float* tg = &p.targets[blockIdx.y][3 * i];
    if (p.diffuse_color == 2) {
      const float4 c0 = __ldg(&sm.vcolors[vi.x]);
      const float4 c1 = __ldg(&sm.vcolors[vi.y]);
      const float4 c2 = __ldg(&sm.vcolors[vi.z]);
      const float a0[3] = {c0.x, c0.y, c0.z}, a1[3] = {c1.x, c1.y, c1.z},
                  a2[3] = {c2.x, c2.y, c2.z};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float col = fadd(fadd(fmul(s0, a0[k]), fmul(u, a1[k])), fmul(v, a2[k]));
        const float dd = col - __ldg(&tg[k]);
        loss += dd * dd;
        gc[k] = 2.0f * dd * s0;
        gc[3 + k] = 2.0f * dd * u;
        gc[6 + k] = 2.0f * dd * v;
      }
    } else {
      const int mid = __ldg(&sm.mat_ids[fid]);
      const DevTexture t = sm.textures[mid];
      const int4 ti = __ldg(&sm.uvidx[fid]);
      const float2 a = __ldg(&sm.uv[ti.x]);
      const float2 b = __ldg(&sm.uv[ti.y]);
      const float2 d = __ldg(&sm.uv[ti.z]);
      const float uvx = fadd(fadd(fmul(s0, a.x), fmul(u, b.x)), fmul(v, d.x));
      const float uvy = fadd(fadd(fmul(s0, a.y), fmul(u, b.y)), fmul(v, d.y));
      const float fx = fmul(uvx, (float)(t.width - 1));
      const float fy = fmul(fsub(1.0f, uvy), (float)(t.height - 1));
      int64_t tix[4];
      float tw[4];
      int nt;
      float col[3];
      if (p.interp == 0) {  // nearest texel
        tix[0] = texel_index(f2i_sat(roundf(fy)), f2i_sat(roundf(fx)), t.width, t.height);
        tw[0] = 1.0f;
        nt = 1;
        fetch_texel(t, tix[0], col);
      } else {
        const int32_t x0 = f2i_sat(floorf(fx));
        const int32_t y0 = f2i_sat(floorf(fy));
        const float lu = fsub(fx, (float)x0);
        const float lv = fsub(fy, (float)y0);
        tix[0] = texel_index(y0, x0, t.width, t.height);
        tix[1] = texel_index(y0, (int64_t)x0 + 1, t.width, t.height);
        tix[2] = texel_index((int64_t)y0 + 1, x0, t.width, t.height);
        tix[3] = texel_index((int64_t)y0 + 1, (int64_t)x0 + 1, t.width, t.height);
        tw[0] = fmul(fsub(1.0f, lu), fsub(1.0f, lv));
        tw[1] = fmul(lu, fsub(1.0f, lv));
        tw[2] = fmul(fsub(1.0f, lu), lv);
        tw[3] = fmul(lu, lv);
        nt = 4;
        float t00[3], t10[3], t01[3], t11[3];
        fetch_texel(t, tix[0], t00);
        fetch_texel(t, tix[1], t10);
        fetch_texel(t, tix[2], t01);
        fetch_texel(t, tix[3], t11);
#pragma unroll
        for (int k = 0; k < 3; ++k)
          col[k] = fadd(fadd(fadd(fmul(tw[0], t00[k]), fmul(tw[1], t10[k])), fmul(tw[2], t01[k])),
                        fmul(tw[3], t11[k]));
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float dd = col[k] - __ldg(&tg[k]);
        loss += dd * dd;
        if (mid == 0 && p.grad_texels)
          for (int j = 0; j < nt; ++j) atomicAdd(&p.grad_texels[3 * tix[j] + k], 2.0f * dd * tw[j]);
      }
    }
  }

  // Warp-aggregated scatter of the per-face contributions.
  const int run = run_id(key, lane);
  const bool head = run == lane;
  const int vids[3] = {vi.x, vi.y, vi.z};
  if (p.grad_vertices) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const float t = run_sum(gv[k], run, lane);
      if (head) atomicAdd(&p.grad_vertices[3 * vids[k / 3] + (k % 3)], t);
    }
  }
  if (p.grad_vertex_colors && p.diffuse_color == 2) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const float t = run_sum(gc[k], run, lane);
      if (head) atomicAdd(&p.grad_vertex_colors[3 * vids[k / 3] + (k % 3)], t);
    }
  }
  if (p.loss) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0) s_loss[threadIdx.x >> 5] = loss;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.0f;
      for (int w = 0; w < kThreads / 32; ++w) t += s_loss[w];
      atomicAdd(&p.loss[blockIdx.y], t);
    }
  }
}

}  // namespace

void launch_backward(const BackwardParams& p, int64_t max_pixels, int max_vertices,
                     cudaStream_t s) {
  if (p.grad_vertices)
    k_proj64<<<dim3((max_vertices + kThreads - 1) / kThreads, p.num_views), kThreads, 0, s>>>(p);
  dim3 grid((unsigned)((max_pixels + kThreads - 1) / kThreads), p.num_views);
  k_backward<<<grid, kThreads, 0, s>>>(p);
}

}  // namespace ugu_gpu
