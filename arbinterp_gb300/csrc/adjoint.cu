// Adjoint (backward) of the 3D scalar interpolant, and grid value updates.
//
// The reference has no backward pass.  For v(q) = sum_o W_o(x) f_o with
// W = w_x w_y w_z (Catmull-Rom weights of the fractional offset x), and the
// reference's gradient output grad_a(q) = (sum_o dW_o/dx_a f_o) / h_a:
//   dL/df_o  += dL/dv W_o + sum_a dL/dgrad_a (dW_o/dx_a) / h_a       (scatter)
//   dL/dq_a   = dL/dv grad_a + sum_b dL/dgrad_b H_ab                  (H = Hessian
//               of the interpolant, (sum_o d2W_o/dx_a dx_b f_o)/(h_a h_b))
// i.e. the transpose of the stencil-and-B^-1 map the forward applies.  The
// interpolant is C1 across cells, so dL/dq is the true derivative except
// on cell faces, where the Hessian term is one-sided.
#include "eval.cuh"

namespace arb {

template <bool MIXED>
__global__ void __launch_bounds__(256) adjoint3_kernel(arb_grid g, KParams kp, const double *q, int64_t nq,
                                                       int64_t qs, const double *dval, const double *dgrad,
                                                       void *grid_grad, double *q_grad, int32_t *status) {
  using T = typename std::conditional<MIXED, float, double>::type;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const double *qr = q + i * qs;
  double qv[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) qv[a] = qr[a];
  T fr[3];
  CoordStep s;
  if constexpr (MIXED)
    s = coord_step_fast<3>(qv, kp.ax, g, fr);
  else
    s = coord_step<3, true>(qv, g, kp.inv_h, fr);
  const bool dead = s.oob || s.nan || s.idx >= g.nc;
  if (!s.oob && !s.nan && s.idx > g.nc) set_status(status, ARB_ERR_CELL_INDEX);
  if (dead) {
    if (q_grad) q_grad[i * 3] = q_grad[i * 3 + 1] = q_grad[i * 3 + 2] = 0.0;
    return;
  }
  const T dv = dval ? (T)dval[i] : T(0);
  T dg[3] = {0, 0, 0};
  if (dgrad) {
    dg[0] = (T)dgrad[i * 3];
    dg[1] = (T)dgrad[i * 3 + 1];
    dg[2] = (T)dgrad[i * 3 + 2];
  }
  if (dv != dv) {  // a NaN upstream: no scatter, a NaN query gradient
    if (q_grad) q_grad[i * 3] = q_grad[i * 3 + 1] = q_grad[i * 3 + 2] = qnan();
    return;
  }
  int64_t c[3];
  cell_from_step<3>(s, g, c);
  T w[3][4], d1[3][4], d2[3][4];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    cr_weights<T>(fr[a], w[a]);
    cr_dweights<T>(fr[a], d1[a]);
    cr_d2weights<T>(fr[a], d2[a]);
  }
  T ih[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) ih[a] = MIXED ? (T)kp.inv_hf[a] : (T)kp.inv_h[a];
  // upstream folded into per-axis factors: c_ijk = dv wx wy wz + dgx dwx wy wz/hx + ...
  const T gx = dg[0] * ih[0], gy = dg[1] * ih[1], gz = dg[2] * ih[2];
  const int64_t nx = g.n[0], ny = g.n[1];
  const int64_t npts = grid_points(g);
  // forward values of the interpolant's derivatives (for dL/dq):
  // S[ox][oy][oz] = sum f * (d^ox w_x)(d^oy w_y)(d^oz w_z), total order <= 2
  T V = 0, G[3] = {0, 0, 0}, H[6] = {0, 0, 0, 0, 0, 0};  // H: xx yy zz xy xz yz
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t p = ((c[2] + k) * ny + (c[1] + j)) * nx + c[0];
      T f[4];
#pragma unroll
      for (int ii = 0; ii < 4; ++ii) {
        if constexpr (MIXED) {
          float hh, ll;
          g32_load<1>(g.grid32, npts, p + ii, 0, hh, ll);
          f[ii] = hh + ll;
        } else {
          f[ii] = __ldg(g.grid64 + p + ii);
        }
      }
      // scatter into the grid gradient
      const T yz = w[1][j] * w[2][k];
#pragma unroll
      for (int ii = 0; ii < 4; ++ii) {
        const T cval = dv * w[0][ii] * yz + gx * d1[0][ii] * yz + gy * w[0][ii] * d1[1][j] * w[2][k] +
                       gz * w[0][ii] * w[1][j] * d1[2][k];
        if (cval != T(0)) {
          if constexpr (MIXED)
            atomicAdd(reinterpret_cast<float *>(grid_grad) + p + ii, cval);
          else
            atomicAdd(reinterpret_cast<double *>(grid_grad) + p + ii, cval);
        }
      }
      if (q_grad) {
        const T a0 = w[0][0] * f[0] + w[0][1] * f[1] + w[0][2] * f[2] + w[0][3] * f[3];
        const T a1 = d1[0][0] * f[0] + d1[0][1] * f[1] + d1[0][2] * f[2] + d1[0][3] * f[3];
        const T a2 = d2[0][0] * f[0] + d2[0][1] * f[1] + d2[0][2] * f[2] + d2[0][3] * f[3];
        V += a0 * yz;
        G[0] += a1 * yz;
        G[1] += a0 * d1[1][j] * w[2][k];
        G[2] += a0 * w[1][j] * d1[2][k];
        H[0] += a2 * yz;
        H[1] += a0 * d2[1][j] * w[2][k];
        H[2] += a0 * w[1][j] * d2[2][k];
        H[3] += a1 * d1[1][j] * w[2][k];
        H[4] += a1 * w[1][j] * d1[2][k];
        H[5] += a0 * d1[1][j] * d1[2][k];
      }
    }
  }
  if (q_grad) {
    const T Hm[3][3] = {{H[0], H[3], H[4]}, {H[3], H[1], H[5]}, {H[4], H[5], H[2]}};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      T r = dv * G[a] * ih[a];
#pragma unroll
      for (int b = 0; b < 3; ++b) r += dg[b] * Hm[a][b] * ih[a] * ih[b];
      q_grad[i * 3 + a] = (double)r;
    }
  }
  (void)V;
}

// Replace the values of a scalar interpolant (grid order) and refresh its
// float32 split; the geometry stays.
template <typename TV>
__global__ void set_values_kernel(const TV *values, int64_t npts, double *grid64, float *grid32) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const double v = (double)values[p];
  grid64[p] = v;
  if (grid32) {
    float hi, lo;
    split_f32(v, hi, lo);
    reinterpret_cast<float2 *>(grid32)[p] = make_float2(hi, lo);
  }
}

}  // namespace arb

using namespace arb;

extern "C" int arb_adjoint(const arb_grid *g, int32_t precision, const double *q, int64_t nq,
                           int64_t q_stride, const double *dval, const double *dgrad, void *grid_grad,
                           double *q_grad, int32_t *status, arb_stream_t stream) {
  if (!g || (nq > 0 && !q) || q_stride < 3 || nq < 0) return ARB_ERR_INVALID;
  if (g->dim != 3 || g->nfield != 1) return ARB_ERR_UNSUPPORTED;
  if (!grid_grad) return ARB_ERR_INVALID;
  const bool mixed = precision == ARB_PREC_MIXED;
  if (mixed ? !g->grid32 : !g->grid64) return ARB_ERR_INVALID;
  if (nq == 0) return ARB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const KParams kp = make_kparams(g);
  const unsigned B = (unsigned)((nq + 255) / 256);
  if (mixed)
    adjoint3_kernel<true><<<B, 256, 0, s>>>(*g, kp, q, nq, q_stride, dval, dgrad, grid_grad, q_grad, status);
  else
    adjoint3_kernel<false><<<B, 256, 0, s>>>(*g, kp, q, nq, q_stride, dval, dgrad, grid_grad, q_grad, status);
  return launch_status();
}

extern "C" int arb_grid_set_values(const arb_grid *g, const void *values, int32_t values_f32,
                                   double *grid64, float *grid32, arb_stream_t stream) {
  if (!g || !values || !grid64 || g->nfield != 1) return ARB_ERR_INVALID;
  int64_t npts = g->n[0] * g->n[1] * g->n[2];
  if (g->dim == 4) npts *= g->n[3];
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned B = (unsigned)((npts + 255) / 256);
  if (values_f32)
    set_values_kernel<float><<<B, 256, 0, s>>>((const float *)values, npts, grid64, grid32);
  else
    set_values_kernel<double><<<B, 256, 0, s>>>((const double *)values, npts, grid64, grid32);
  return launch_status();
}
