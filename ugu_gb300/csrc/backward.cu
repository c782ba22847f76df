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

#include <algorithm>

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

// Adds (g0, g1, g2) to the 3 consecutive floats of element `tix` (a texel's
// RGB, a vertex's xyz or colour): one 8-byte and one 4-byte atomic add when
// the buffer is 8-byte aligned (the pair starts at the element's even
// float), else three 4-byte ones.
__device__ __forceinline__ void add3(float* g, int64_t tix, float g0, float g1,
                                               float g2, bool aligned8) {
  float* t = g + 3 * tix;
  if (!aligned8) {
    atomicAdd(t, g0);
    atomicAdd(t + 1, g1);
    atomicAdd(t + 2, g2);
  } else if ((tix & 1) == 0) {
    atomicAdd(reinterpret_cast<float2*>(t), make_float2(g0, g1));
    atomicAdd(t + 2, g2);
  } else {
    atomicAdd(t, g0);
    atomicAdd(reinterpret_cast<float2*>(t + 1), make_float2(g1, g2));
  }
}

// A texel's RGB gradient: one 16-byte atomic into the RGBA scratch when
// there is one (every texel 16-byte aligned), else add3 into the H*W*3
// buffer.
__device__ __forceinline__ void add_texel(const BackwardParams& p, int64_t tix, float g0,
                                          float g1, float g2, bool aligned8) {
  if (p.grad_texels4)
    atomicAdd(reinterpret_cast<float4*>(p.grad_texels4) + tix, make_float4(g0, g1, g2, 0.0f));
  else
    add3(p.grad_texels, tix, g0, g1, g2, aligned8);
}

// One vertex of one view: its screen x and y, projected in double, as
// unevaluated sums hi + lo of two floats (about 48 significant bits), and
// 1 / z.  32 bytes per vertex.
struct alignas(16) ProjHL {
  float xh, yh, xl, yl;
  float iz, pad_[3];
};

// Error-free transformations (Knuth's TwoSum, and the FMA product error):
// a + b = s + e and a * b = p + e exactly.  The library is compiled without
// FMA contraction, so the separate roundings these rely on are kept.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Float-float arithmetic (Dekker 1971; Shewchuk 1997): a value is the
// unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2, about 48
// significant bits.  Sums use TwoSum, products the FMA product error; a
// quotient is refined from the float quotient of the high parts by two
// correction steps against the float-float remainder.
struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_norm(float s, float e) {  // s + e, renormalised
  FF r;
  two_sum(s, e, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  return ff_norm(s, e + (a.lo + b.lo));
}

__device__ __forceinline__ FF ff_prod(float a, float b) {  // exact
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ FF ff_mul(FF a, float b) {
  const float p = a.hi * b;
  return ff_norm(p, fmaf(a.lo, b, fmaf(a.hi, b, -p)));
}

__device__ __forceinline__ FF ff_sub_mul(FF r, FF b, float q) {  // r - b q
  const FF bq = ff_mul(b, q);
  return ff_add(r, {-bq.hi, -bq.lo});
}

__device__ __forceinline__ FF ff_div(FF a, FF b) {
  const float q1 = a.hi / b.hi;
  const FF r1 = ff_sub_mul(a, b, q1);
  const float q2 = r1.hi / b.hi;
  const FF r2 = ff_sub_mul(r1, b, q2);
  const float q3 = r2.hi / b.hi;
  const FF q = ff_norm(q1, q2);
  return ff_add(q, {q3, 0.0f});
}

// The pinhole projection of every vertex of one view (blockIdx.y)
// (camera.h:380-387) from the float vertices and camera, in float-float:
// the camera coordinates R p + t from exact products, then
// x = fx x_c / z_c + cx and y likewise, each split into hi + lo floats, and
// 1 / z_c.  Accurate to a few units of 2^-46 relative, which the hi + lo
// pair stores; GB300 issues float-float several times faster than FP64.
__global__ void __launch_bounds__(kThreads) k_proj64(BackwardParams p) {
  const DevView& V = p.views[blockIdx.y];
  const DevMesh& M = p.meshes[V.mesh];
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= M.num_vertices) return;
  const Cam& c = V.cam;
  const float4 P = __ldg(&M.vertices[i]);
  FF cc[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    FF acc = ff_prod(c.R[3 * j], P.x);
    acc = ff_add(acc, ff_prod(c.R[3 * j + 1], P.y));
    acc = ff_add(acc, ff_prod(c.R[3 * j + 2], P.z));
    cc[j] = ff_add(acc, {c.t[j], 0.0f});
  }
  const FF x = ff_add(ff_div(ff_mul(cc[0], c.fx), cc[2]), {c.cx, 0.0f});
  const FF y = ff_add(ff_div(ff_mul(cc[1], c.fy), cc[2]), {c.cy, 0.0f});
  const FF iz = ff_div({1.0f, 0.0f}, cc[2]);
  float4* dst = reinterpret_cast<float4*>(reinterpret_cast<ProjHL*>(p.proj64) + V.proj_offset + i);
  dst[0] = make_float4(x.hi, y.hi, x.lo, y.lo);
  dst[1] = make_float4(iz.hi + iz.lo, 0.0f, 0.0f, 0.0f);
}

// Texel coordinate base + t (t small: the offset of the pixel's texture
// coordinate from one vertex's, in texels) split into an integer cell and a
// fraction in [0, 1).  base = hi + lo is exact; the cell is found from hi's
// integer part first, so the fraction keeps float precision relative to a
// texel rather than to the coordinate.
__device__ __forceinline__ void texel_cell(float hi, float lo, float t, int64_t& cell,
                                           float& frac) {
  const float ih = floorf(hi);
  const float rem = (hi - ih) + (lo + t);  // hi - ih is exact for |hi| < 2^23
  const float ir = floorf(rem);
  cell = (int64_t)f2i_sat(ih) + (int64_t)f2i_sat(ir);
  frac = rem - ir;
}

// The same for rounding to the nearest texel (round half away from zero).
__device__ __forceinline__ int64_t texel_nearest(float hi, float lo, float t) {
  const float ih = floorf(hi);
  const float rem = (hi - ih) + (lo + t);
  return (int64_t)f2i_sat(ih) + (int64_t)f2i_sat(roundf(rem));
}

// Vertex-position (and colour, texel) gradients of one pixel, in float.
// The sum over pixels amplifies systematic rounding and the gradients of
// sliver faces are large, so three quantities keep more than float
// precision: the pixel-to-vertex differences (from the double projection's
// hi + lo parts, accurate relative to the difference rather than to the
// screen coordinate), the edge functions (accurate relative to themselves
// however thin the face), and the texture coordinate (a texel-exact base
// at one vertex plus a small offset, texel_cell).  The perspective weights
// are w = r / sum(r) with r_k = e_k / z_k (the area cancels in w, so it has
// no gradient).
struct PixGrad {
  float loss;
  float gpos[9];
  float gcol[9];
  int64_t tix[4];
  float tg[4][3];  // per texel: dL/dt
  int ntex;
};

__device__ __forceinline__ void pixel_backward(const BackwardParams& p, const DevMesh& m,
                                               const Cam& c, const ProjHL* tab, int fid, int x,
                                               int y, const float* target, PixGrad& o) {
  const int4 vi = __ldg(&m.vidx[fid]);
  const int vv[3] = {vi.x, vi.y, vi.z};
  float xh[3], yh[3], xl[3], yl[3], iz[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(tab + vv[k]));
    xh[k] = a.x;
    yh[k] = a.y;
    xl[k] = a.z;
    yl[k] = a.w;
    iz[k] = __ldg(&tab[vv[k]].iz);
  }
  // pixel minus vertex as unevaluated sums dh + dl (about 48 bits)
  const float px = (float)x, py = (float)y;
  float dxh[3], dxl[3], dyh[3], dyl[3], dx[3], dy[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float e;
    two_sum(px, -xh[k], dxh[k], e);
    dxl[k] = e - xl[k];
    two_sum(py, -yh[k], dyh[k], e);
    dyl[k] = e - yl[k];
    dx[k] = dxh[k] + dxl[k];
    dy[k] = dyh[k] + dyl[k];
  }
  // e_k = edge(v_a, v_b, p) = dy_a dx_b - dx_a dy_b for (a, b) = (1, 2),
  // (2, 0), (0, 1).  On a sliver face the two products nearly cancel, so
  // they are formed exactly (FMA product errors) and the lo parts enter
  // as first-order terms: e_k is then accurate relative to itself.
  const int ea[3] = {1, 2, 0}, eb[3] = {2, 0, 1};
  float r[3], rs = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int ia = ea[k], ib = eb[k];
    const float p1 = dyh[ia] * dxh[ib], q1 = fmaf(dyh[ia], dxh[ib], -p1);
    const float p2 = dxh[ia] * dyh[ib], q2 = fmaf(dxh[ia], dyh[ib], -p2);
    const float cross = (dyh[ia] * dxl[ib] + dyl[ia] * dxh[ib]) -
                        (dxh[ia] * dyl[ib] + dxl[ia] * dyh[ib]);
    const float e = (p1 - p2) + ((q1 - q2) + cross);
    r[k] = e * iz[k];
    rs += r[k];
  }
  const float iS = 1.0f / rs;
  const float u = r[1] * iS, v = r[2] * iS, s0 = (1.0f - u) - v;
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
      dcu[k] = a1[k] - a0[k];
      dcv[k] = a2[k] - a0[k];
      col[k] = a0[k] + (u * dcu[k] + v * dcv[k]);
    }
  } else {
    const int mid = __ldg(&m.mat_ids[fid]);
    const DevTexture t = m.textures[mid];
    const int4 ti = __ldg(&m.uvidx[fid]);
    const float2 a = __ldg(&m.uv[ti.x]), b = __ldg(&m.uv[ti.y]), d = __ldg(&m.uv[ti.z]);
    const float Wm = (float)(t.width - 1), Hm = (float)(t.height - 1);
    // fx = Wm * uvx, fy = Hm * (1 - uvy), uv = a + u (b - a) + v (d - a)
    const float dfx_du = (b.x - a.x) * Wm, dfx_dv = (d.x - a.x) * Wm;
    const float dfy_du = -(b.y - a.y) * Hm, dfy_dv = -(d.y - a.y) * Hm;
    const float ox = u * dfx_du + v * dfx_dv;
    const float oy = u * dfy_du + v * dfy_dv;
    const float bxh = Wm * a.x, bxl = fmaf(Wm, a.x, -bxh);  // Wm a.x, exactly
    const float pyh = Hm * a.y, pyl = fmaf(Hm, a.y, -pyh);  // Hm a.y, exactly
    float byh, bye;
    two_sum(Hm, -pyh, byh, bye);  // Hm - Hm a.y = byh + bye - pyl
    const float byl = bye - pyl;
    if (p.interp == 0) {
      const int64_t ix =
          texel_index(texel_nearest(byh, byl, oy), texel_nearest(bxh, bxl, ox), t.width, t.height);
      fetch_texel(t, ix, col);
#pragma unroll
      for (int k = 0; k < 3; ++k) dcu[k] = dcv[k] = 0.0f;
      o.tix[0] = ix;
      o.tg[0][0] = o.tg[0][1] = o.tg[0][2] = 1.0f;  // weights; scaled by dL/dC below
      o.ntex = mid == 0 ? 1 : 0;
    } else {
      int64_t x0, y0;
      float lu, lv;
      texel_cell(bxh, bxl, ox, x0, lu);
      texel_cell(byh, byl, oy, y0, lv);
      o.tix[0] = texel_index(y0, x0, t.width, t.height);
      o.tix[1] = texel_index(y0, x0 + 1, t.width, t.height);
      o.tix[2] = texel_index(y0 + 1, x0, t.width, t.height);
      o.tix[3] = texel_index(y0 + 1, x0 + 1, t.width, t.height);
      float t00[3], t10[3], t01[3], t11[3];
      fetch_texel(t, o.tix[0], t00);
      fetch_texel(t, o.tix[1], t10);
      fetch_texel(t, o.tix[2], t01);
      fetch_texel(t, o.tix[3], t11);
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
  const float gr[3] = {-gdotw * iS, (gw1 - gdotw) * iS, (gw2 - gdotw) * iS};
  float ge[3], gZ[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    ge[k] = gr[k] * iz[k];
    gZ[k] = -gr[k] * r[k] * iz[k];
  }
  float gX[3] = {0.0f, 0.0f, 0.0f}, gY[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int k = 0; k < 3; ++k) {  // e_k = dy_a dx_b - dx_a dy_b (d = pixel - vertex)
    const int ia = ea[k], ib = eb[k];
    gX[ia] += ge[k] * dy[ib];
    gY[ia] -= ge[k] * dx[ib];
    gX[ib] -= ge[k] * dy[ia];
    gY[ib] += ge[k] * dx[ia];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float gcx = gX[k] * c.fx * iz[k];
    const float gcy = gY[k] * c.fy * iz[k];
    const float sx = (xh[k] - c.cx) + xl[k], sy = (yh[k] - c.cy) + yl[k];
    const float gcz = -(gX[k] * sx + gY[k] * sy) * iz[k] + gZ[k];
#pragma unroll
    for (int j = 0; j < 3; ++j) o.gpos[3 * k + j] = c.R[j] * gcx + c.R[3 + j] * gcy + c.R[6 + j] * gcz;
  }
}

// One pixel of one view (the thread's pixel i of the view's image; i may
// lie past its end): its gradients, scattered, and its loss returned.  All
// lanes of the warp take part (the run reductions shuffle across them).
__device__ __forceinline__ float backward_pixel(const BackwardParams& p, const DevView& sv,
                                                const DevMesh& sm, int64_t i, int lane,
                                                bool aligned8) {
  const Cam& c = sv.cam;
  const int64_t npx = (int64_t)c.width * c.height;
  int fid = -1;
  int x = 0, y = 0;
  if (i < npx) {
    fid = sv.face_id[i];
    if (npx <= 0x7fffffff) {  // 32-bit division for every image below 2^31 pixels
      y = (int)((uint32_t)i / (uint32_t)c.width);
      x = (int)((uint32_t)i - (uint32_t)y * (uint32_t)c.width);
    } else {
      x = (int)(i % c.width);
      y = (int)(i / c.width);
    }
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
    pixel_backward(p, sm, c, reinterpret_cast<const ProjHL*>(p.proj64) + sv.proj_offset, fid, x,
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
          add_texel(p, o.tix[j], o.tg[j][0], o.tg[j][1], o.tg[j][2], aligned8);
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
      float gC[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float dd = col[k] - __ldg(&tg[k]);
        loss += dd * dd;
        gC[k] = 2.0f * dd;
      }
      if (mid == 0 && p.grad_texels)
        for (int j = 0; j < nt; ++j)
          add_texel(p, tix[j], gC[0] * tw[j], gC[1] * tw[j], gC[2] * tw[j], aligned8);
    }
  }

  // Warp-aggregated scatter of the per-face contributions.
  const int run = run_id(key, lane);
  const bool head = run == lane;
  const int vids[3] = {vi.x, vi.y, vi.z};
  if (p.grad_vertices) {
    const bool al = (reinterpret_cast<uintptr_t>(p.grad_vertices) & 7) == 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) gv[k] = run_sum(gv[k], run, lane);
    if (head)
#pragma unroll
      for (int k = 0; k < 3; ++k) add3(p.grad_vertices, vids[k], gv[3 * k], gv[3 * k + 1], gv[3 * k + 2], al);
  }
  if (p.grad_vertex_colors && p.diffuse_color == 2) {
    const bool al = (reinterpret_cast<uintptr_t>(p.grad_vertex_colors) & 7) == 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) gc[k] = run_sum(gc[k], run, lane);
    if (head)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        add3(p.grad_vertex_colors, vids[k], gc[3 * k], gc[3 * k + 1], gc[3 * k + 2], al);
  }
  return loss;
}

// 4 blocks of 256 per SM: at most 64 registers a thread
__global__ void __launch_bounds__(kThreads, 4) k_backward(BackwardParams p) {
  // blockIdx.y: the view; blockIdx.x: every gridDim.x-th chunk of kThreads
  // pixels of it, so the descriptor copies and the loss reduction below are
  // paid once per block
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
  const int lane = threadIdx.x & 31;
  const bool aligned8 = (reinterpret_cast<uintptr_t>(p.grad_texels) & 7) == 0;
  const int64_t npx = (int64_t)sv.cam.width * sv.cam.height;
  const int64_t nchunks = (npx + kThreads - 1) / kThreads;
  float loss = 0.0f;
  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x)
    loss += backward_pixel(p, sv, sm, ch * kThreads + threadIdx.x, lane, aligned8);
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

// grad_texels += the RGB of the RGBA scratch, one thread per texel.
__global__ void __launch_bounds__(kThreads) k_fold_texels(float* g3, const float4* g4, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (t >= n) return;
  const float4 v = g4[t];
  g3[3 * t + 0] += v.x;
  g3[3 * t + 1] += v.y;
  g3[3 * t + 2] += v.z;
}

}  // namespace

void launch_backward(const BackwardParams& p, int64_t max_pixels, int max_vertices, int num_sms,
                     cudaStream_t s) {
  if (p.grad_vertices)
    k_proj64<<<dim3((max_vertices + kThreads - 1) / kThreads, p.num_views), kThreads, 0, s>>>(p);
  // about 4 waves of 4 blocks per SM over all views
  const int64_t chunks = (max_pixels + kThreads - 1) / kThreads;
  const int64_t per_view = std::max<int64_t>(1, ((int64_t)num_sms * 16 + p.num_views - 1) / p.num_views);
  dim3 grid((unsigned)std::max<int64_t>(1, std::min(chunks, per_view)), p.num_views);
  k_backward<<<grid, kThreads, 0, s>>>(p);
  if (p.grad_texels4 && p.num_texels4 > 0)
    k_fold_texels<<<(unsigned)((p.num_texels4 + kThreads - 1) / kThreads), kThreads, 0, s>>>(
        p.grad_texels, reinterpret_cast<const float4*>(p.grad_texels4), p.num_texels4);
}

}  // namespace ugu_gpu
