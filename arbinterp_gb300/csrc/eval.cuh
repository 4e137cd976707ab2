// Device-side evaluation of one query: on-the-fly from the grid (3D/4D) or
// from the coefficient table, plus the output writers and the shared
// query prologue (cell index, out-of-volume rows, sentinel semantics).
#pragma once

#include <string.h>

#include "arb_common.cuh"

namespace arb {


struct KParams {
  double inv_h[4];
  float inv_hf[4];
  FastAxis ax[4];
};

// Output rows.  Strides are normalised on the host (normalize_out), so the
// kernels always see the row stride of each output.
__device__ __forceinline__ void st_v4(double *p, double a, double b, double c, double d) {
  asm volatile("st.global.v4.b64 [%0], {%1,%2,%3,%4};" ::"l"(p), "d"(a), "d"(b), "d"(c), "d"(d) : "memory");
}

// Interleaved rows (see arb_query_out): whole 32-byte sectors per store.
template <int DIM, int F>
__device__ __forceinline__ bool interleaved_rows(const arb_query_out &o) {
  if (F == 4)
    return o.comps && o.norms == o.comps + 3 && o.grads == o.comps + 4 && o.comps_stride == 8 &&
           o.norms_stride == 8 && o.grads_stride == 8 && !((uintptr_t)o.comps & 31);
  if (F == 1) {
    constexpr int R = DIM == 3 ? 4 : 8;
    return o.norms && o.grads == o.norms + 1 && o.norms_stride == R && o.grads_stride == R &&
           !((uintptr_t)o.norms & 31);
  }
  return o.comps && o.comps_stride == 4 && !((uintptr_t)o.comps & 31);
}

template <int DIM, int F>
__device__ __forceinline__ void write_rows_v4(const arb_query_out &o, int64_t i, const double *val,
                                              const double *grad) {
  if (F == 4) {
    double *r = o.comps + i * 8;
    st_v4(r, val[0], val[1], val[2], val[3]);
    st_v4(r + 4, grad[0], grad[1], grad[2], DIM == 4 ? grad[DIM - 1] : 0.0);
  } else if (F == 1) {
    double *r = o.norms + i * (DIM == 3 ? 4 : 8);
    st_v4(r, val[0], grad[0], grad[1], grad[2]);
    if (DIM == 4) st_v4(r + 4, grad[DIM - 1], 0.0, 0.0, 0.0);
  } else {
    st_v4(o.comps + i * 4, val[0], val[1], val[2], 0.0);
  }
}

template <int DIM, int F>
__device__ __forceinline__ void write_const(const arb_query_out &o, int64_t i, double v) {
  if (interleaved_rows<DIM, F>(o)) {
    const double vv[4] = {v, v, v, v}, gg[4] = {v, v, v, v};
    write_rows_v4<DIM, F>(o, i, vv, gg);
    return;
  }
  if (F >= 3 && o.comps) {
    o.comps[i * o.comps_stride + 0] = v;
    o.comps[i * o.comps_stride + 1] = v;
    o.comps[i * o.comps_stride + 2] = v;
  }
  if (F != 3) {
    if (o.norms) o.norms[i * o.norms_stride] = v;
    if (o.grads) {
#pragma unroll
      for (int a = 0; a < DIM; ++a) o.grads[i * o.grads_stride + a] = v;
    }
  }
}

template <int DIM, int F>
__device__ __forceinline__ void write_vals(const arb_query_out &o, int64_t i, const double *val,
                                           const double *grad) {
  if (interleaved_rows<DIM, F>(o)) {
    write_rows_v4<DIM, F>(o, i, val, grad);
    return;
  }
  if (F >= 3 && o.comps) {
    o.comps[i * o.comps_stride + 0] = val[0];
    o.comps[i * o.comps_stride + 1] = val[1];
    o.comps[i * o.comps_stride + 2] = val[2];
  }
  if (F != 3) {
    if (o.norms) o.norms[i * o.norms_stride] = val[F - 1];
    if (o.grads) {
#pragma unroll
      for (int a = 0; a < DIM; ++a) o.grads[i * o.grads_stride + a] = grad[a];
    }
  }
}

// Shared prologue: cell index, out-of-volume handling, sentinel semantics.
// Returns true when the row still needs evaluating.
// EXACT (float64 path): IEEE division, frac in double.  Otherwise the
// mixed-precision step (exact index, float frac, two float64 ops per axis).
template <int DIM, int F, bool EXACT>
__device__ __forceinline__ bool query_prologue(const arb_grid &g, const KParams &kp, double *q,
                                               int64_t i, int64_t qs, int wb,
                                               const arb_query_out &o, int32_t *status,
                                               typename std::conditional<EXACT, double, float>::type frac[DIM],
                                               int64_t &idx) {
  double *qr = q + i * qs;
  double qv[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) qv[a] = qr[a];
  CoordStep s;
  if constexpr (EXACT)
    s = coord_step<DIM, true>(qv, g, kp.inv_h, frac);
  else
    s = coord_step_fast<DIM>(qv, kp.ax, g, frac);
  append_oob(o, i, s.oob);
  if (s.oob && wb) {
    for (int64_t c = 0; c < qs; ++c) qr[c] = qnan();
  }
  if (o.inds) o.inds[i] = s.idx;
  idx = s.idx;
  if (s.oob || s.nan) {
    write_const<DIM, F>(o, i, qnan());
    return false;
  }
  if (s.idx > g.nc) {
    // the reference's alphamask lookup raises here (IndexError)
    set_status(status, ARB_ERR_CELL_INDEX);
    write_const<DIM, F>(o, i, qnan());
    return false;
  }
  if (s.idx == g.nc) {
    // in-volume query aliased onto the sentinel column (upper faces)
    write_const<DIM, F>(o, i, g.sentinel_nan ? qnan() : 0.0);
    return false;
  }
  return true;
}

// ---- row loaders ------------------------------------------------------------
// 4 consecutive grid points x F fields starting at flat point p.
template <int F>
__device__ __forceinline__ void load_row64(const double *grid, int64_t p, double v[4][F]) {
  const double *r = grid + p * F;
  if (F == 4) {
    const double2 *r2 = reinterpret_cast<const double2 *>(r);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const double2 a = __ldg(r2 + 2 * i), b = __ldg(r2 + 2 * i + 1);
      v[i][0] = a.x;
      v[i][1 % F] = a.y;
      v[i][2 % F] = b.x;
      v[i][3 % F] = b.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int f = 0; f < F; ++f) v[i][f] = __ldg(r + i * F + f);
  }
}

// Deltas against the reference point: (hi - rhi) + (lo - rlo) is accurate to
// float32 rounding of the DIFFERENCE, so gradients keep full relative
// precision even where |f| >> h |grad f|.
// (grid32 layout: see g32_load in arb_common.cuh.)
template <int F>
__device__ __forceinline__ void load_row32(const float *grid, int64_t npts, int64_t p, const float *rhi,
                                           const float *rlo, float v[4][F]) {
  if (F == 1) {
    const float2 *r = reinterpret_cast<const float2 *>(grid) + p;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 a = __ldg(r + i);
      v[i][0] = (a.x - rhi[0]) + (a.y - rlo[0]);
    }
  } else {
    const float4 *r4 = reinterpret_cast<const float4 *>(grid) + p;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 a = __ldg(r4 + i);
      v[i][0] = a.x - rhi[0];
      v[i][1 % F] = a.y - rhi[1 % F];
      v[i][2 % F] = a.z - rhi[2 % F];
      if (F == 4) v[i][3 % F] = (a.w - rhi[3 % F]) + (__ldg(grid + npts * 4 + p + i) - rlo[3 % F]);
    }
  }
}

template <int F, bool MIXED, typename T>
__device__ __forceinline__ void load_row(const arb_grid &g, int64_t npts, int64_t p, const float *rhi,
                                         const float *rlo, T v[4][F]) {
  if constexpr (MIXED)
    load_row32<F>(g.grid32, npts, p, rhi, rlo, v);
  else
    load_row64<F>(g.grid64, p, v);
}

// ---- 3D on-the-fly, float32 with gradient ----------------------------------
// Each gradient component is a difference along its own axis; formed from
// deltas to the cell corner it would inherit the float32 rounding of the
// OTHER axes' variation (error ~ eps * sum_b h_b |f_b| / (h_a |f_a|), over
// 1e-6 on coarse anisotropic grids).  So the gradient field is differenced
// along each axis first, from the (hi, lo) grid words:
//   d/dx: x-local deltas f[k][j][i] - f[k][j][1] per x-line,
//   d/dy: y-local deltas f[k][j][i] - f[k][1][i] (line j = 1 of the layer),
//   d/dz: z-local deltas f[k][j][i] - f[1][j][i] (layer k = 1),
// then smoothed over the other two axes (positive-dominated weights, no
// cancellation).  Values use corner deltas as before.  Layers and lines are
// visited in the order 1, 0, 2, 3 so the local references are loaded first.
// BLK says where the 4x4x4 block is read from: at(i, j, k) is the index of
// block point (i, j, k); with F = 1, hl(index) is its (hi, lo) pair; with
// F = 4, hi4(index) its float4 (hi_x, hi_y, hi_z, hi_n) and lo(index) lo_n.
struct Grid32Block3 {  // the mixed grid in global memory
  const float *g32;
  int64_t npts, sy, sz, base;  // strides of y, z; index of the block corner
  __device__ __forceinline__ int64_t at(int i, int j, int k) const { return base + k * sz + j * sy + i; }
  __device__ __forceinline__ float2 hl(int64_t p) const { return __ldg(reinterpret_cast<const float2 *>(g32) + p); }
  __device__ __forceinline__ float4 hi4(int64_t p) const { return __ldg(reinterpret_cast<const float4 *>(g32) + p); }
  __device__ __forceinline__ float lo(int64_t p) const { return __ldg(g32 + npts * 4 + p); }
  __device__ __forceinline__ void lo_row(int64_t p, float l[4]) const {
#pragma unroll
    for (int i = 0; i < 4; ++i) l[i] = __ldg(g32 + npts * 4 + p + i);
  }
  template <int F>
  __device__ __forceinline__ void load(int64_t p, int f, float &h, float &l) const {
    g32_load<F>(g32, npts, p, f, h, l);
  }
};

template <int F, class BLK>
__device__ __forceinline__ void eval_otf3_mixed_block(const BLK &blk, const KParams &kp, const float frac[3],
                                                      double val[F], double grad[3]) {
  constexpr int G = F - 1;  // the field whose gradient is returned (scalar or |B|)
  float wx[4], wy[4], wz[4], dx[4], dy[4], dz[4];
  cr_weights<float>(frac[0], wx);
  cr_weights<float>(frac[1], wy);
  cr_weights<float>(frac[2], wz);
  cr_dweights<float>(frac[0], dx);
  cr_dweights<float>(frac[1], dy);
  cr_dweights<float>(frac[2], dz);
  float rhi[F], rlo[F];
  const auto pr = blk.at(1, 1, 1);
#pragma unroll
  for (int f = 0; f < F; ++f) blk.template load<F>(pr, f, rhi[f], rlo[f]);
  float zh[4][4], zl[4][4], yh[4], yl[4];
  float acc[F], gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
  for (int f = 0; f < F; ++f) acc[f] = 0.f;
  constexpr int ORD[4] = {1, 0, 2, 3};
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const int k = ORD[kk];
    float ay[F], ayx = 0.f, ayy = 0.f;
#pragma unroll
    for (int f = 0; f < F; ++f) ay[f] = 0.f;
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int j = ORD[jj];
      const auto p = blk.at(0, j, k);
      float h[4], l[4], vv[4][3];
      if constexpr (F == 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float2 a = blk.hl(p + i);
          h[i] = a.x;
          l[i] = a.y;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 a = blk.hi4(p + i);
          vv[i][0] = a.x - rhi[0];
          vv[i][1] = a.y - rhi[1 % F];
          vv[i][2] = a.z - rhi[2 % F];
          h[i] = a.w;
          l[i] = blk.lo(p + i);
        }
      }
      if (k == 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          zh[j][i] = h[i];
          zl[j][i] = l[i];
        }
      }
      if (j == 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          yh[i] = h[i];
          yl[i] = l[i];
        }
      }
      // values: corner deltas
      float d[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) d[i] = (h[i] - rhi[G]) + (l[i] - rlo[G]);
      ay[G] += wy[j] * (wx[0] * d[0] + wx[1] * d[1] + wx[2] * d[2] + wx[3] * d[3]);
      if (F == 4) {
#pragma unroll
        for (int f = 0; f < 3; ++f)
          ay[f] += wy[j] * (wx[0] * vv[0][f] + wx[1] * vv[1][f] + wx[2] * vv[2][f] + wx[3] * vv[3][f]);
      }
      // d/dx from x-local deltas
      const float e0 = (h[0] - h[1]) + (l[0] - l[1]);
      const float e2 = (h[2] - h[1]) + (l[2] - l[1]);
      const float e3 = (h[3] - h[1]) + (l[3] - l[1]);
      ayx += wy[j] * (dx[0] * e0 + dx[2] * e2 + dx[3] * e3);
      // d/dy from y-local deltas
      if (j != 1) {
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) s += wx[i] * ((h[i] - yh[i]) + (l[i] - yl[i]));
        ayy += dy[j] * s;
      }
      // d/dz from z-local deltas
      if (k != 1) {
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) s += wx[i] * ((h[i] - zh[j][i]) + (l[i] - zl[j][i]));
        gz += (dz[k] * wy[j]) * s;
      }
    }
#pragma unroll
    for (int f = 0; f < F; ++f) acc[f] += wz[k] * ay[f];
    gx += wz[k] * ayx;
    gy += wz[k] * ayy;
  }
#pragma unroll
  for (int f = 0; f < F; ++f) val[f] = f2d_exact(rhi[f] + (rlo[f] + acc[f]));
  grad[0] = f2d_exact(gx * kp.inv_hf[0]);
  grad[1] = f2d_exact(gy * kp.inv_hf[1]);
  grad[2] = f2d_exact(gz * kp.inv_hf[2]);
}

// Packed float32 pairs (.f32x2): one instruction computes both components
// with the rounding of the scalar operation.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}

// 'both' fields (three components, values only, and |B| with its gradient),
// float32.  |B| is hi + lo per point.  The lo words (|lo| <= ulp(hi) / 2)
// are contracted as they are: their rounding errors are ~2^-24 of a quantity
// already ~2^-24 of |B|.  The hi words carry the variation, so each gradient
// component is formed from hi differences along its own axis (exact by
// Sterbenz's lemma where neighbouring values are within a factor of 2, and
// otherwise rounded relative to the difference itself):
//   d/dx from x-local differences hi[k][j][i] - hi[k][j][1],
//   d/dy from y-local differences hi[k][j][i] - hi[k][1][i],
//   d/dz from z-local differences hi[k][j][i] - hi[1][j][i],
// and the value from the x-local differences plus each row's own difference
// to the cell corner (1, 1, 1).  Components accumulate their float32 values
// directly.  Planes and rows are visited in the order 1, 0, 2, 3 so the
// references come first; pairs of products share one .f32x2 instruction.
// BLK as for eval_otf3_mixed_block (at, hi4, lo), plus lo_row(index, l):
// the lo words of the four points of an x-row from its first point.
template <class BLK>
__device__ __forceinline__ void eval_otf3_both_block(const BLK &blk, const KParams &kp, const float frac[3],
                                                     double val[4], double grad[3]) {
  float wx[4], wy[4], wz[4], dx[4], dy[4], dz[4];
  cr_weights<float>(frac[0], wx);
  cr_weights<float>(frac[1], wy);
  cr_weights<float>(frac[2], wz);
  cr_dweights<float>(frac[0], dx);
  cr_dweights<float>(frac[1], dy);
  cr_dweights<float>(frac[2], dz);
  const auto pc = blk.at(1, 1, 1);
  const float hc = blk.hi4(pc).w;
  float zr[4][4], yr[4];                     // hi of plane 1 (z references), of row 1 (y references)
  float2 Cxy = make_float2(0.f, 0.f);        // components
  float Cz = 0.f;
  float V = 0.f, GX = 0.f, GY = 0.f, GZ = 0.f;   // hi part: value (relative to the corner), gradients
  float LV = 0.f, LX = 0.f, LY = 0.f, LZ = 0.f;  // lo part
  constexpr int ORD[4] = {1, 0, 2, 3};
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const int k = ORD[kk];
    float2 cxy = make_float2(0.f, 0.f);
    float cz = 0.f, vp = 0.f, xp = 0.f, yp = 0.f, zp = 0.f, lp = 0.f, lxp = 0.f, lyp = 0.f;
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int j = ORD[jj];
      const auto p = blk.at(0, j, k);
      float4 a[4];
      float l[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = blk.hi4(p + i);
      blk.lo_row(p, l);
      float h[4] = {a[0].w, a[1].w, a[2].w, a[3].w};
      if (k == 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) zr[j][i] = h[i];
      }
      if (j == 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) yr[i] = h[i];
      }
      // components, and the lo words for the value (wx) and d/dx (dx)
      float2 rxy = make_float2(0.f, 0.f), rzl = make_float2(0.f, 0.f);
      float rlx = 0.f;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        rxy = ffma2(make_float2(wx[i], wx[i]), make_float2(a[i].x, a[i].y), rxy);
        rzl = ffma2(make_float2(wx[i], wx[i]), make_float2(a[i].z, l[i]), rzl);
        rlx = fmaf(dx[i], l[i], rlx);
      }
      // x-local differences: the value (plus the row's offset to the corner) and d/dx
      const float2 e02 = fsub2(make_float2(h[0], h[2]), make_float2(h[1], h[1]));
      const float e3 = h[3] - h[1];
      float2 vx = make_float2(h[1] - hc, 0.f);
      vx = ffma2(make_float2(wx[0], dx[0]), make_float2(e02.x, e02.x), vx);
      vx = ffma2(make_float2(wx[2], dx[2]), make_float2(e02.y, e02.y), vx);
      vx = ffma2(make_float2(wx[3], dx[3]), make_float2(e3, e3), vx);
      // y-local and z-local differences, contracted along x
      float ry = 0.f, rz = 0.f;
      if (j != 1 && k != 1) {
        float2 yz = make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < 4; ++i)
          yz = ffma2(make_float2(wx[i], wx[i]), fsub2(make_float2(h[i], h[i]), make_float2(yr[i], zr[j][i])), yz);
        ry = yz.x;
        rz = yz.y;
      } else if (j != 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) ry = fmaf(wx[i], h[i] - yr[i], ry);
      } else if (k != 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) rz = fmaf(wx[i], h[i] - zr[j][i], rz);
      }
      // along y
      cxy = ffma2(make_float2(wy[j], wy[j]), rxy, cxy);
      cz = fmaf(wy[j], rzl.x, cz);
      vp = fmaf(wy[j], vx.x, vp);
      xp = fmaf(wy[j], vx.y, xp);
      yp = fmaf(dy[j], ry, yp);
      zp = fmaf(wy[j], rz, zp);
      lp = fmaf(wy[j], rzl.y, lp);
      lxp = fmaf(wy[j], rlx, lxp);
      lyp = fmaf(dy[j], rzl.y, lyp);
    }
    // along z
    Cxy = ffma2(make_float2(wz[k], wz[k]), cxy, Cxy);
    Cz = fmaf(wz[k], cz, Cz);
    V = fmaf(wz[k], vp, V);
    GX = fmaf(wz[k], xp, GX);
    GY = fmaf(wz[k], yp, GY);
    GZ = fmaf(dz[k], zp, GZ);
    LV = fmaf(wz[k], lp, LV);
    LX = fmaf(wz[k], lxp, LX);
    LY = fmaf(wz[k], lyp, LY);
    LZ = fmaf(dz[k], lp, LZ);
  }
  val[0] = f2d_exact(Cxy.x);
  val[1] = f2d_exact(Cxy.y);
  val[2] = f2d_exact(Cz);
  val[3] = f2d_exact(hc + (V + LV));
  grad[0] = f2d_exact((GX + LX) * kp.inv_hf[0]);
  grad[1] = f2d_exact((GY + LY) * kp.inv_hf[1]);
  grad[2] = f2d_exact((GZ + LZ) * kp.inv_hf[2]);
}

template <int F>
__device__ __forceinline__ void eval_otf3_mixed_grad(const arb_grid &g, const KParams &kp, const int64_t c[3],
                                                     const float frac[3], double val[F], double grad[3]) {
  const int64_t nx = g.n[0], ny = g.n[1];
  Grid32Block3 blk;
  blk.g32 = g.grid32;
  blk.npts = grid_points(g);
  blk.sy = nx;
  blk.sz = nx * ny;
  blk.base = (c[2] * ny + c[1]) * nx + c[0];
  if constexpr (F == 4)
    eval_otf3_both_block(blk, kp, frac, val, grad);
  else
    eval_otf3_mixed_block<F>(blk, kp, frac, val, grad);
}

// Vector fields (values only) in float32: corner deltas of the three
// components; BLK as for eval_otf3_mixed_block (hi4 and at).
template <class BLK>
__device__ __forceinline__ void eval_otf3_vec_block(const BLK &blk, const float frac[3], double val[3]) {
  float wx[4], wy[4], wz[4];
  cr_weights<float>(frac[0], wx);
  cr_weights<float>(frac[1], wy);
  cr_weights<float>(frac[2], wz);
  const float4 r = blk.hi4(blk.at(1, 1, 1));  // reference point: the cell's own corner
  const float rhi[3] = {r.x, r.y, r.z};
  float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float ay[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const auto p = blk.at(0, j, k);
      float v[4][3];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float4 a = blk.hi4(p + i);
        v[i][0] = a.x - rhi[0];
        v[i][1] = a.y - rhi[1];
        v[i][2] = a.z - rhi[2];
      }
#pragma unroll
      for (int f = 0; f < 3; ++f)
        ay[f] += wy[j] * (wx[0] * v[0][f] + wx[1] * v[1][f] + wx[2] * v[2][f] + wx[3] * v[3][f]);
    }
#pragma unroll
    for (int f = 0; f < 3; ++f) acc[f] += wz[k] * ay[f];
  }
#pragma unroll
  for (int f = 0; f < 3; ++f) val[f] = f2d_exact(rhi[f] + (0.f + acc[f]));
}

// ---- 3D on-the-fly ---------------------------------------------------------
template <int F, bool MIXED>
__device__ __forceinline__ void eval_otf3(const arb_grid &g, const KParams &kp, const int64_t c[3],
                                          const typename std::conditional<MIXED, float, double>::type frac[3],
                                          double val[F], double grad[3]) {
  using T = typename std::conditional<MIXED, float, double>::type;
  constexpr bool GRAD = (F != 3);
  if constexpr (MIXED && GRAD) {
    eval_otf3_mixed_grad<F>(g, kp, c, frac, val, grad);
    return;
  }
  if constexpr (MIXED && F == 3) {
    Grid32Block3 blk;
    blk.g32 = g.grid32;
    blk.npts = grid_points(g);
    blk.sy = g.n[0];
    blk.sz = g.n[0] * g.n[1];
    blk.base = (c[2] * g.n[1] + c[1]) * g.n[0] + c[0];
    eval_otf3_vec_block(blk, frac, val);
    return;
  }
  const int64_t nx = g.n[0], ny = g.n[1];
  T wx[4], wy[4], wz[4], dx[4], dy[4], dz[4];
  cr_weights<T>((T)frac[0], wx);
  cr_weights<T>((T)frac[1], wy);
  cr_weights<T>((T)frac[2], wz);
  if (GRAD) {
    cr_dweights<T>((T)frac[0], dx);
    cr_dweights<T>((T)frac[1], dy);
    cr_dweights<T>((T)frac[2], dz);
  }
  float rhi[F], rlo[F];
  const int64_t npts = grid_points(g);
  if constexpr (MIXED) {
    // reference point: the cell's own corner, block offset (1, 1, 1)
    const int64_t pr = ((c[2] + 1) * ny + (c[1] + 1)) * nx + (c[0] + 1);
#pragma unroll
    for (int f = 0; f < F; ++f) g32_load<F>(g.grid32, npts, pr, f, rhi[f], rlo[f]);
  }
  T acc[F], gx = 0, gy = 0, gz = 0;
#pragma unroll
  for (int f = 0; f < F; ++f) acc[f] = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    T ay[F], ayx = 0, ayy = 0;
#pragma unroll
    for (int f = 0; f < F; ++f) ay[f] = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T v[4][F];
      load_row<F, MIXED, T>(g, npts, ((c[2] + k) * ny + (c[1] + j)) * nx + c[0], rhi, rlo, v);
      T ax[F];
#pragma unroll
      for (int f = 0; f < F; ++f)
        ax[f] = wx[0] * v[0][f] + wx[1] * v[1][f] + wx[2] * v[2][f] + wx[3] * v[3][f];
#pragma unroll
      for (int f = 0; f < F; ++f) ay[f] += wy[j] * ax[f];
      if (GRAD) {
        const T axd = dx[0] * v[0][F - 1] + dx[1] * v[1][F - 1] + dx[2] * v[2][F - 1] +
                      dx[3] * v[3][F - 1];
        ayx += wy[j] * axd;
        ayy += dy[j] * ax[F - 1];
      }
    }
#pragma unroll
    for (int f = 0; f < F; ++f) acc[f] += wz[k] * ay[f];
    if (GRAD) {
      gx += wz[k] * ayx;
      gy += wz[k] * ayy;
      gz += dz[k] * ay[F - 1];
    }
  }
#pragma unroll
  for (int f = 0; f < F; ++f) {
    if constexpr (MIXED)
      val[f] = f2d_exact(rhi[f] + (rlo[f] + acc[f]));
    else
      val[f] = (double)acc[f];
  }
  if (GRAD) {
    if constexpr (MIXED) {
      grad[0] = f2d_exact(gx * kp.inv_hf[0]);
      grad[1] = f2d_exact(gy * kp.inv_hf[1]);
      grad[2] = f2d_exact(gz * kp.inv_hf[2]);
    } else {
      grad[0] = (double)gx * kp.inv_h[0];
      grad[1] = (double)gy * kp.inv_h[1];
      grad[2] = (double)gz * kp.inv_h[2];
    }
  }
}

// ---- 4D on-the-fly, mixed precision ------------------------------------------
// The same contraction as eval_otf4 with float32 deltas taken hierarchically:
// each x-row against its own x-offset-1 point, each row's reference against
// the (1, 1, k, l) point (along y), those against (1, 1, 1, l) (along z) and
// those against the cell corner (along t).  Every delta is a difference along
// one axis, so the float32 rounding in a derivative along x, y or z no longer
// carries the field's variation along the later axes (the corner deltas did:
// a strongly t-dependent field cost its spatial gradient accuracy).  Rows,
// lines and slabs run in the order 1, 0, 2, 3 so that each reference is
// loaded before it is used; every grid point is loaded once.  BLK says where
// the 4x4x4x4 block is read from: at(i, j, k, l) is the index of block point
// (i, j, k, l) and load<F>(index, f, hi, lo) its (hi, lo) of field f.
struct Grid32Block {  // the mixed grid in global memory
  const float *g32;
  int64_t npts, sy, sz, st, base;  // strides of y, z, t; index of the block corner
  __device__ __forceinline__ int64_t at(int i, int j, int k, int l) const {
    return base + l * st + k * sz + j * sy + i;
  }
  template <int F>
  __device__ __forceinline__ void load(int64_t p, int f, float &hi, float &lo) const {
    g32_load<F>(g32, npts, p, f, hi, lo);
  }
};

template <int F, class BLK>
__device__ __forceinline__ void eval_otf4_mixed_block(const BLK &blk, const KParams &kp, const float frac[4],
                                                      double val[F], double grad[4]) {
  using T = float;
  T w[4][4], dw[4][4], hb[4][2], dhb[4][2];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    cr_weights<T>(frac[a], w[a]);
    cr_dweights<T>(frac[a], dw[a]);
    hermite_slope<T>(frac[a], hb[a], dhb[a]);
  }
  const auto pref = blk.at(1, 1, 1, 1);
#pragma unroll 1
  for (int f = 0; f < F; ++f) {
    const bool gradf = (F != 3) && (f == F - 1);
    float rhi = 0.f, rlo = 0.f;
    blk.template load<F>(pref, f, rhi, rlo);
    T V = 0, Vg[4] = {0, 0, 0, 0};
    T S[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) S[m] = 0;
    float hl = 0.f, ll = 0.f;  // point (1, 1, 1, l): reference of the z-deltas of slab l
    // the slab loop stays rolled: unrolled, the 256-point body overflowed the
    // instruction cache (instruction fetch was the bin kernel's first stall)
#pragma unroll 1
    for (int li = 0; li < 4; ++li) {
      const int l = li == 0 ? 1 : (li == 1 ? 0 : li);
      const T w3 = l == 0 ? w[3][0] : (l == 1 ? w[3][1] : (l == 2 ? w[3][2] : w[3][3]));
      const T dw3 = l == 0 ? dw[3][0] : (l == 1 ? dw[3][1] : (l == 2 ? dw[3][2] : dw[3][3]));
      T Az = 0, Azg[3] = {0, 0, 0};
      T E2[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) E2[m] = 0;
#pragma unroll
      for (int ki = 0; ki < 4; ++ki) {
        const int k = ki == 0 ? 1 : (ki == 1 ? 0 : ki);
        T Ay = 0, Ayx = 0, Ayy = 0;
        T E1[4] = {0, 0, 0, 0};
        float hj = 0.f, lj = 0.f;  // point (1, 1, k, l): reference of the y-deltas of line (k, l)
#pragma unroll
        for (int ji = 0; ji < 4; ++ji) {
          const int j = ji == 0 ? 1 : (ji == 1 ? 0 : ji);
          const auto p = blk.at(0, j, k, l);
          float h_[4], l_[4];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii) blk.template load<F>(p + ii, f, h_[ii], l_[ii]);
          if (j == 1) {
            hj = h_[1];
            lj = l_[1];
          }
          T d[4];  // along x, against the row's point at x offset 1
#pragma unroll
          for (int ii = 0; ii < 4; ++ii) d[ii] = (h_[ii] - h_[1]) + (l_[ii] - l_[1]);
          const T dy = (h_[1] - hj) + (l_[1] - lj);  // row reference against (1, 1, k, l)
          const T ax = (w[0][0] * d[0] + w[0][2] * d[2] + w[0][3] * d[3]) + dy;
          Ay += w[1][j] * ax;
          if (gradf) {
            const T axd = dw[0][0] * d[0] + dw[0][2] * d[2] + dw[0][3] * d[3];
            Ayx += w[1][j] * axd;
            Ayy += dw[1][j] * ax;
          }
          const T sj = (j >= 2) ? T(0.5) : T(-0.5);
          E1[0 + 2 * (j & 1)] += sj * (T(0.5) * (d[2] - d[0]));
          E1[1 + 2 * (j & 1)] += sj * (T(0.5) * d[3]);
        }
        if (k == 1) {
          hl = hj;
          ll = lj;
        }
        const T Ak = Ay + ((hj - hl) + (lj - ll));  // line reference against (1, 1, 1, l)
        Az += w[2][k] * Ak;
        if (gradf) {
          Azg[0] += w[2][k] * Ayx;
          Azg[1] += w[2][k] * Ayy;
          Azg[2] += dw[2][k] * Ak;
        }
        const T sk = (k >= 2) ? T(0.5) : T(-0.5);
#pragma unroll
        for (int m = 0; m < 4; ++m) E2[m + 4 * (k & 1)] += sk * E1[m];
      }
      const T Al = Az + ((hl - rhi) + (ll - rlo));  // slab reference against the corner
      V += w3 * Al;
      if (gradf) {
        Vg[0] += w3 * Azg[0];
        Vg[1] += w3 * Azg[1];
        Vg[2] += w3 * Azg[2];
        Vg[3] += dw3 * Al;
      }
      const T sl = (l >= 2) ? T(0.5) : T(-0.5);
      if (l & 1) {
#pragma unroll
        for (int m = 0; m < 8; ++m) S[m + 8] += sl * E2[m];
      } else {
#pragma unroll
        for (int m = 0; m < 8; ++m) S[m] += sl * E2[m];
      }
    }
    // T_c = S_{c-1} - S_c, contracted with the slope-Hermite tensor
    T Tc[16];
    Tc[0] = -S[0];
#pragma unroll
    for (int m = 1; m < 16; ++m) Tc[m] = S[m - 1] - S[m];
    T Cx[8], Cdx[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      Cx[m] = hb[0][0] * Tc[2 * m] + hb[0][1] * Tc[2 * m + 1];
      Cdx[m] = dhb[0][0] * Tc[2 * m] + dhb[0][1] * Tc[2 * m + 1];
    }
    T Cy[4], Cyx[4], Cyy[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      Cy[m] = hb[1][0] * Cx[2 * m] + hb[1][1] * Cx[2 * m + 1];
      Cyx[m] = hb[1][0] * Cdx[2 * m] + hb[1][1] * Cdx[2 * m + 1];
      Cyy[m] = dhb[1][0] * Cx[2 * m] + dhb[1][1] * Cx[2 * m + 1];
    }
    T Cz[2], Czx[2], Czy[2], Czz[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      Cz[m] = hb[2][0] * Cy[2 * m] + hb[2][1] * Cy[2 * m + 1];
      Czx[m] = hb[2][0] * Cyx[2 * m] + hb[2][1] * Cyx[2 * m + 1];
      Czy[m] = hb[2][0] * Cyy[2 * m] + hb[2][1] * Cyy[2 * m + 1];
      Czz[m] = dhb[2][0] * Cy[2 * m] + dhb[2][1] * Cy[2 * m + 1];
    }
    const T C = hb[3][0] * Cz[0] + hb[3][1] * Cz[1];
    val[f] = f2d_exact(rhi + (rlo + (V + C)));
    if (gradf) {
      const T G[4] = {Vg[0] + (hb[3][0] * Czx[0] + hb[3][1] * Czx[1]),
                      Vg[1] + (hb[3][0] * Czy[0] + hb[3][1] * Czy[1]),
                      Vg[2] + (hb[3][0] * Czz[0] + hb[3][1] * Czz[1]),
                      Vg[3] + (dhb[3][0] * Cz[0] + dhb[3][1] * Cz[1])};
#pragma unroll
      for (int a = 0; a < 4; ++a) grad[a] = f2d_exact(G[a] * kp.inv_hf[a]);
    }
  }
}

template <int F>
__device__ __forceinline__ void eval_otf4_mixed(const arb_grid &g, const KParams &kp, const int64_t c[4],
                                                const float frac[4], double val[F], double grad[4]) {
  const int64_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
  Grid32Block blk;
  blk.g32 = g.grid32;
  blk.npts = grid_points(g);
  blk.sy = nx;
  blk.sz = nx * ny;
  blk.st = nx * ny * nz;
  blk.base = ((c[3] * nz + c[2]) * ny + c[1]) * nx + c[0];
  eval_otf4_mixed_block<F>(blk, kp, frac, val, grad);
}

// ---- 4D on-the-fly ---------------------------------------------------------
// value = sum_o W_o(x) f_o  +  sum_c (H_{c+1}(x) - H_c(x)) S_c
// with W the 4-fold Catmull-Rom tensor, S_c the (1/16) mixed fourth
// difference centred on cell corner c, H_c(x) the tensor product of cubic
// slope-Hermite bases at corner c, H_16 = 0.  The second term is the
// reference's A minus kron(A1,A1,A1,A1) (D row 240 zero, rows 241..255
// shifted by one corner).
template <int F, bool MIXED>
__device__ __forceinline__ void eval_otf4(const arb_grid &g, const KParams &kp, const int64_t c[4],
                                          const typename std::conditional<MIXED, float, double>::type frac[4],
                                          double val[F], double grad[4]) {
  using T = typename std::conditional<MIXED, float, double>::type;
  if constexpr (MIXED) {
    eval_otf4_mixed<F>(g, kp, c, frac, val, grad);
    return;
  }
  const int64_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
  T w[4][4], dw[4][4], hb[4][2], dhb[4][2];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    cr_weights<T>((T)frac[a], w[a]);
    cr_dweights<T>((T)frac[a], dw[a]);
    hermite_slope<T>((T)frac[a], hb[a], dhb[a]);
  }
  const int64_t npts = grid_points(g);
  const int64_t pref = (((c[3] + 1) * nz + (c[2] + 1)) * ny + (c[1] + 1)) * nx + (c[0] + 1);
#pragma unroll 1
  for (int f = 0; f < F; ++f) {
    const bool gradf = (F != 3) && (f == F - 1);
    float rhi = 0.f, rlo = 0.f;
    if constexpr (MIXED) g32_load<F>(g.grid32, npts, pref, f, rhi, rlo);
    T V = 0, Vg[4] = {0, 0, 0, 0};
    T S[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) S[m] = 0;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      T Az = 0, Azg[4] = {0, 0, 0, 0};
      T E2[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) E2[m] = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        T Ay = 0, Ayx = 0, Ayy = 0;
        T E1[4] = {0, 0, 0, 0};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int64_t p = (((c[3] + l) * nz + (c[2] + k)) * ny + (c[1] + j)) * nx + c[0];
          T r[4];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii) {
            if constexpr (MIXED) {
              float h_, l_;
              g32_load<F>(g.grid32, npts, p + ii, f, h_, l_);
              r[ii] = (h_ - rhi) + (l_ - rlo);
            } else {
              r[ii] = __ldg(g.grid64 + (p + ii) * F + f);
            }
          }
          const T ax = w[0][0] * r[0] + w[0][1] * r[1] + w[0][2] * r[2] + w[0][3] * r[3];
          Ay += w[1][j] * ax;
          if (gradf) {
            const T axd = dw[0][0] * r[0] + dw[0][1] * r[1] + dw[0][2] * r[2] + dw[0][3] * r[3];
            Ayx += w[1][j] * axd;
            Ayy += dw[1][j] * ax;
          }
          const T sj = (j >= 2) ? T(0.5) : T(-0.5);
          E1[0 + 2 * (j & 1)] += sj * (T(0.5) * (r[2] - r[0]));
          E1[1 + 2 * (j & 1)] += sj * (T(0.5) * (r[3] - r[1]));
        }
        Az += w[2][k] * Ay;
        if (gradf) {
          Azg[0] += w[2][k] * Ayx;
          Azg[1] += w[2][k] * Ayy;
          Azg[2] += dw[2][k] * Ay;
        }
        const T sk = (k >= 2) ? T(0.5) : T(-0.5);
#pragma unroll
        for (int m = 0; m < 4; ++m) E2[m + 4 * (k & 1)] += sk * E1[m];
      }
      V += w[3][l] * Az;
      if (gradf) {
        Vg[0] += w[3][l] * Azg[0];
        Vg[1] += w[3][l] * Azg[1];
        Vg[2] += w[3][l] * Azg[2];
        Vg[3] += dw[3][l] * Az;
      }
      const T sl = (l >= 2) ? T(0.5) : T(-0.5);
#pragma unroll
      for (int m = 0; m < 8; ++m) S[m + 8 * (l & 1)] += sl * E2[m];
    }
    // T_c = S_{c-1} - S_c, then contract with the slope-Hermite tensor
    T Tc[16];
    Tc[0] = -S[0];
#pragma unroll
    for (int m = 1; m < 16; ++m) Tc[m] = S[m - 1] - S[m];
    T Cx[8], Cdx[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      Cx[m] = hb[0][0] * Tc[2 * m] + hb[0][1] * Tc[2 * m + 1];
      Cdx[m] = dhb[0][0] * Tc[2 * m] + dhb[0][1] * Tc[2 * m + 1];
    }
    T Cy[4], Cyx[4], Cyy[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      Cy[m] = hb[1][0] * Cx[2 * m] + hb[1][1] * Cx[2 * m + 1];
      Cyx[m] = hb[1][0] * Cdx[2 * m] + hb[1][1] * Cdx[2 * m + 1];
      Cyy[m] = dhb[1][0] * Cx[2 * m] + dhb[1][1] * Cx[2 * m + 1];
    }
    T Cz[2], Czx[2], Czy[2], Czz[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      Cz[m] = hb[2][0] * Cy[2 * m] + hb[2][1] * Cy[2 * m + 1];
      Czx[m] = hb[2][0] * Cyx[2 * m] + hb[2][1] * Cyx[2 * m + 1];
      Czy[m] = hb[2][0] * Cyy[2 * m] + hb[2][1] * Cyy[2 * m + 1];
      Czz[m] = dhb[2][0] * Cy[2 * m] + dhb[2][1] * Cy[2 * m + 1];
    }
    const T C = hb[3][0] * Cz[0] + hb[3][1] * Cz[1];
    const T total = V + C;
    if constexpr (MIXED)
      val[f] = f2d_exact(rhi + (rlo + total));
    else
      val[f] = (double)total;
    if (gradf) {
      const T G[4] = {Vg[0] + (hb[3][0] * Czx[0] + hb[3][1] * Czx[1]),
                      Vg[1] + (hb[3][0] * Czy[0] + hb[3][1] * Czy[1]),
                      Vg[2] + (hb[3][0] * Czz[0] + hb[3][1] * Czz[1]),
                      Vg[3] + (dhb[3][0] * Cz[0] + dhb[3][1] * Cz[1])};
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        if constexpr (MIXED)
          grad[a] = f2d_exact(G[a] * kp.inv_hf[a]);
        else
          grad[a] = (double)G[a] * kp.inv_h[a];
      }
    }
  }
}

// ---- table evaluation ------------------------------------------------------
// Horner along x for one 4-coefficient row: value and d/dx.
template <typename T>
__device__ __forceinline__ void horner_x(const T a[4], T x, T &v, T &d) {
  v = ((a[3] * x + a[2]) * x + a[1]) * x + a[0];
  d = (T(3) * a[3] * x + T(2) * a[2]) * x + a[1];
}

template <typename T>
__device__ __forceinline__ void load4(const T *p, T a[4]) {
  if constexpr (sizeof(T) == 8) {
    const double2 u = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 w = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    a[0] = u.x;
    a[1] = u.y;
    a[2] = w.x;
    a[3] = w.y;
  } else {
    const float4 u = __ldg(reinterpret_cast<const float4 *>(p));
    a[0] = u.x;
    a[1] = u.y;
    a[2] = u.z;
    a[3] = u.w;
  }
}

template <int DIM, int F, bool MIXED>
__device__ __forceinline__ void eval_tab(const arb_grid &g, const KParams &kp, const int64_t c[DIM],
                                         const typename std::conditional<MIXED, float, double>::type x[DIM],
                                         double val[F], double grad[DIM]) {
  using T = typename std::conditional<MIXED, float, double>::type;
  constexpr int M = DIM == 3 ? 64 : 256;
  const int64_t idx = flat_cell<DIM>(c, g);
  const T *tab = reinterpret_cast<const T *>(g.table) + idx * (int64_t)F * M;
#pragma unroll 1
  for (int f = 0; f < F; ++f) {
    const bool gradf = (F != 3) && (f == F - 1);
    const T *a = tab + f * M;
    // nested Horner: rows (ey, ez[, et]) of 4 x-coefficients
    T V = 0, G[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) G[d] = 0;
    const int NT = DIM == 4 ? 4 : 1;
#pragma unroll 1
    for (int et = NT - 1; et >= 0; --et) {
      T Vz = 0, Gz[3] = {0, 0, 0};
#pragma unroll
      for (int ez = 3; ez >= 0; --ez) {
        T Vy = 0, Gyx = 0, Gyy = 0;
#pragma unroll
        for (int ey = 3; ey >= 0; --ey) {
          T r[4];
          load4<T>(a + ((et * 4 + ez) * 4 + ey) * 4, r);
          T vx, dxv;
          horner_x<T>(r, x[0], vx, dxv);
          // Horner in y: derivative first (uses the old Vy)
          Gyy = Gyy * x[1] + Vy;
          Vy = Vy * x[1] + vx;
          Gyx = Gyx * x[1] + dxv;
        }
        Gz[2] = Gz[2] * x[2] + Vz;
        Vz = Vz * x[2] + Vy;
        Gz[0] = Gz[0] * x[2] + Gyx;
        Gz[1] = Gz[1] * x[2] + Gyy;
      }
      if (DIM == 4) {
        G[DIM - 1] = G[DIM - 1] * x[DIM - 1] + V;
        V = V * x[DIM - 1] + Vz;
        G[0] = G[0] * x[DIM - 1] + Gz[0];
        G[1] = G[1] * x[DIM - 1] + Gz[1];
        G[2] = G[2] * x[DIM - 1] + Gz[2];
      } else {
        V = Vz;
        G[0] = Gz[0];
        G[1] = Gz[1];
        G[2] = Gz[2];
      }
    }
    if constexpr (MIXED)
      val[f] = f2d_exact(V);
    else
      val[f] = V;
    if (gradf) {
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        if constexpr (MIXED)
          grad[d] = f2d_exact(G[d] * kp.inv_hf[d]);
        else
          grad[d] = (double)G[d] * kp.inv_h[d];
      }
    }
  }
}


static inline KParams make_kparams(const arb_grid *g) {
  KParams kp;
  for (int a = 0; a < 4; ++a) {
    const double h = a < g->dim ? g->h[a] : 1.0;
    kp.inv_h[a] = 1.0 / h;
    kp.inv_hf[a] = (float)(1.0 / h);
    unsigned long long lb, hb;
    const double lo = a < g->dim ? g->lo[a] : 0.0, hi = a < g->dim ? g->hi[a] : 0.0;
    memcpy(&lb, &lo, 8);
    memcpy(&hb, &hi, 8);
    kp.ax[a].lo_key = ord_key_bits(lb);
    kp.ax[a].hi_key = ord_key_bits(hb);
    kp.ax[a].lo = lo;
    kp.ax[a].h = h;
    kp.ax[a].inv_h = 1.0 / h;
    fast_axis_pairs(kp.ax[a], lo, hi, h);
  }
  return kp;
}

// Output descriptor with every row stride filled in (0 means packed).
static inline arb_query_out normalize_out(const arb_query_out &in, int dim) {
  arb_query_out o = in;
  if (o.comps_stride <= 0) o.comps_stride = 3;
  if (o.norms_stride <= 0) o.norms_stride = 1;
  if (o.grads_stride <= 0) o.grads_stride = dim;
  return o;
}

static inline int check_query_args(const arb_grid *g, const double *q, int64_t nq, int64_t qs,
                            const arb_query_out *out) {
  if (!g || !out || (nq > 0 && !q)) return ARB_ERR_INVALID;
  if (g->dim != 3 && g->dim != 4) return ARB_ERR_INVALID;
  if (qs < g->dim || nq < 0) return ARB_ERR_INVALID;
  if (g->nfield != 1 && g->nfield != 3 && g->nfield != 4) return ARB_ERR_INVALID;
  if (out->oob_rows && !out->oob_count) return ARB_ERR_INVALID;
  return ARB_OK;
}

}  // namespace arb
