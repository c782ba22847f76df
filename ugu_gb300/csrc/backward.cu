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

// The per-pixel chain in double, from the float inputs (the FP64 restatement
// the gradients are checked against): colour, loss, dL/dC and the
// gradients of the three vertices' positions and colours; texel weights and
// indices for the texel scatter.
struct Pix64 {
  double loss;
  double gC[3];
  double gpos[9];
  double gcol[9];
  int64_t tix[4];
  double tw[4];
  int ntex;
};

__device__ __noinline__ void pixel_backward_f64(const BackwardParams& p, const DevMesh& m,
                                                const Cam& c, int fid, int x, int y,
                                                const float* target, Pix64& o) {
  const int4 vi = __ldg(&m.vidx[fid]);
  const int vid[3] = {vi.x, vi.y, vi.z};
  double X[3], Y[3], Z[3], CX[3], CY[3];
  for (int k = 0; k < 3; ++k) {
    const float4 P = __ldg(&m.vertices[vid[k]]);
    double cc[3];
    for (int j = 0; j < 3; ++j)
      cc[j] = (double)c.R[3 * j] * P.x + (double)c.R[3 * j + 1] * P.y +
              (double)c.R[3 * j + 2] * P.z + (double)c.t[j];
    CX[k] = cc[0];
    CY[k] = cc[1];
    Z[k] = cc[2];
    X[k] = (double)c.fx * cc[0] / cc[2] + (double)c.cx;
    Y[k] = (double)c.fy * cc[1] / cc[2] + (double)c.cy;
  }
  const double px = x, py = y;
  auto E = [](double ax, double ay, double bx, double by, double qx, double qy) {
    return (qx - ax) * (by - ay) - (qy - ay) * (bx - ax);
  };
  const double A = E(X[0], Y[0], X[1], Y[1], X[2], Y[2]);
  const double e[3] = {E(X[1], Y[1], X[2], Y[2], px, py), E(X[2], Y[2], X[0], Y[0], px, py),
                       E(X[0], Y[0], X[1], Y[1], px, py)};
  double b[3], q[3], ssum = 0.0;
  for (int k = 0; k < 3; ++k) {
    b[k] = e[k] / A;
    q[k] = b[k] / Z[k];
    ssum += q[k];
  }
  const double w[3] = {q[0] / ssum, q[1] / ssum, q[2] / ssum};
  const double u = w[1], v = w[2], s0 = 1.0 - u - v;
  double col[3], dcu[3], dcv[3];
  o.ntex = 0;
  if (p.diffuse_color == 2) {
    for (int k = 0; k < 3; ++k) {
      const double c0 = ((const float*)&m.vcolors[vid[0]])[k];
      const double c1 = ((const float*)&m.vcolors[vid[1]])[k];
      const double c2 = ((const float*)&m.vcolors[vid[2]])[k];
      col[k] = s0 * c0 + u * c1 + v * c2;
      dcu[k] = c1 - c0;
      dcv[k] = c2 - c0;
    }
  } else {
    const int mid = __ldg(&m.mat_ids[fid]);
    const DevTexture t = m.textures[mid];
    const int4 ti = __ldg(&m.uvidx[fid]);
    const float2 a = __ldg(&m.uv[ti.x]), bb = __ldg(&m.uv[ti.y]), d = __ldg(&m.uv[ti.z]);
    const double uvx = s0 * a.x + u * bb.x + v * d.x;
    const double uvy = s0 * a.y + u * bb.y + v * d.y;
    const double fx = uvx * (t.width - 1), fy = (1.0 - uvy) * (t.height - 1);
    if (p.interp == 0) {
      const int64_t ix = texel_index((int64_t)llround(fy), (int64_t)llround(fx), t.width, t.height);
      float tv[3];
      fetch_texel(t, ix, tv);
      for (int k = 0; k < 3; ++k) col[k] = tv[k], dcu[k] = dcv[k] = 0.0;
      o.tix[0] = ix;
      o.tw[0] = 1.0;
      o.ntex = mid == 0 ? 1 : 0;
    } else {
      const double x0 = floor(fx), y0 = floor(fy);
      const double lu = fx - x0, lv = fy - y0;
      const int64_t i00 = texel_index((int64_t)y0, (int64_t)x0, t.width, t.height);
      const int64_t i10 = texel_index((int64_t)y0, (int64_t)x0 + 1, t.width, t.height);
      const int64_t i01 = texel_index((int64_t)y0 + 1, (int64_t)x0, t.width, t.height);
      const int64_t i11 = texel_index((int64_t)y0 + 1, (int64_t)x0 + 1, t.width, t.height);
      float t00[3], t10[3], t01[3], t11[3];
      fetch_texel(t, i00, t00);
      fetch_texel(t, i10, t10);
      fetch_texel(t, i01, t01);
      fetch_texel(t, i11, t11);
      const double dfx_du = ((double)bb.x - a.x) * (t.width - 1);
      const double dfx_dv = ((double)d.x - a.x) * (t.width - 1);
      const double dfy_du = -((double)bb.y - a.y) * (t.height - 1);
      const double dfy_dv = -((double)d.y - a.y) * (t.height - 1);
      for (int k = 0; k < 3; ++k) {
        col[k] = (1 - lu) * (1 - lv) * t00[k] + lu * (1 - lv) * t10[k] +
                 (1 - lu) * lv * t01[k] + lu * lv * t11[k];
        const double dlu = (1 - lv) * ((double)t10[k] - t00[k]) + lv * ((double)t11[k] - t01[k]);
        const double dlv = (1 - lu) * ((double)t01[k] - t00[k]) + lu * ((double)t11[k] - t10[k]);
        dcu[k] = dlu * dfx_du + dlv * dfy_du;
        dcv[k] = dlu * dfx_dv + dlv * dfy_dv;
      }
      o.tix[0] = i00; o.tix[1] = i10; o.tix[2] = i01; o.tix[3] = i11;
      o.tw[0] = (1 - lu) * (1 - lv);
      o.tw[1] = lu * (1 - lv);
      o.tw[2] = (1 - lu) * lv;
      o.tw[3] = lu * lv;
      o.ntex = mid == 0 ? 4 : 0;
    }
  }
  o.loss = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double dd = col[k] - (double)target[k];
    o.loss += dd * dd;
    o.gC[k] = 2.0 * dd;
    o.gcol[k] = o.gC[k] * s0;
    o.gcol[3 + k] = o.gC[k] * u;
    o.gcol[6 + k] = o.gC[k] * v;
  }
  double gw[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < 3; ++k) {
    gw[1] += o.gC[k] * dcu[k];
    gw[2] += o.gC[k] * dcv[k];
  }
  const double gdotw = gw[1] * w[1] + gw[2] * w[2];
  double gX[3] = {0, 0, 0}, gY[3] = {0, 0, 0}, gZ[3] = {0, 0, 0}, gb[3];
  double gA = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double gq = (gw[k] - gdotw) / ssum;
    gb[k] = gq / Z[k];
    gZ[k] = -gq * q[k] / Z[k];
    gA -= gb[k] * b[k] / A;
  }
  const int ea[3] = {1, 2, 0}, eb[3] = {2, 0, 1};
  for (int k = 0; k < 3; ++k) {  // e_k = E(v_ea, v_eb, p)
    const double g = gb[k] / A;
    const int ia = ea[k], ib = eb[k];
    gX[ia] += g * (py - Y[ib]);
    gY[ia] += g * (X[ib] - px);
    gX[ib] -= g * (py - Y[ia]);
    gY[ib] += g * (px - X[ia]);
  }
  gX[0] += gA * (Y[2] - Y[1]);
  gY[0] += gA * (X[1] - X[2]);
  gX[1] -= gA * (Y[2] - Y[0]);
  gY[1] += gA * (X[2] - X[0]);
  gX[2] += gA * (Y[1] - Y[0]);
  gY[2] -= gA * (X[1] - X[0]);
  for (int k = 0; k < 3; ++k) {
    const double z = Z[k];
    const double gcx = gX[k] * c.fx / z;
    const double gcy = gY[k] * c.fy / z;
    const double gcz = -gX[k] * c.fx * CX[k] / (z * z) - gY[k] * c.fy * CY[k] / (z * z) + gZ[k];
    for (int j = 0; j < 3; ++j)
      o.gpos[3 * k + j] = (double)c.R[j] * gcx + (double)c.R[3 + j] * gcy + (double)c.R[6 + j] * gcz;
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
    // Position gradients sum many contributions of both signs; the float
    // chain's rounding (e.g. of the texel coordinates) would be amplified
    // by that cancellation, so this pixel's chain runs in double.
    vi = __ldg(&sm.vidx[fid]);
    Pix64 o;
    pixel_backward_f64(p, sm, c, fid, x, y, &p.targets[blockIdx.y][3 * i], o);
    loss = (float)o.loss;
    for (int k = 0; k < 9; ++k) {
      gv[k] = (float)o.gpos[k];
      gc[k] = p.diffuse_color == 2 ? (float)o.gcol[k] : 0.0f;
    }
    if (p.grad_texels && p.diffuse_color == 1)
      for (int j = 0; j < o.ntex; ++j)
        for (int k = 0; k < 3; ++k)
          atomicAdd(&p.grad_texels[3 * o.tix[j] + k], (float)(o.gC[k] * o.tw[j]));
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

void launch_backward(const BackwardParams& p, int64_t max_pixels, cudaStream_t s) {
  dim3 grid((unsigned)((max_pixels + kThreads - 1) / kThreads), p.num_views);
  k_backward<<<grid, kThreads, 0, s>>>(p);
}

}  // namespace ugu_gpu
