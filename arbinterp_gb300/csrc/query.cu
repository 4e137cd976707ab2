// Query evaluation kernels: replace rQuery1/2/3 and sQuery1/2/3
// (src/ARBInterp/ARBInterp.py:213-521, 916-1258).
//
// Two strategies, both one thread per query row:
//   * on-the-fly (otf_*): gathers the 4^dim grid block of the query's cell
//     and contracts it with tensor-product Catmull-Rom weights.  This is the
//     reference's  p(x) . (A f)  regrouped as  (A^T p(x)) . f , exact in real
//     arithmetic because A = kron(A1, A1, A1) in 3D; in 4D the reference's A
//     carries an extra rank-16 term from its row-240 D-matrix off-by-one,
//     evaluated here from 16 mixed fourth-difference stencils.
//   * table (tab_*): gathers the cell's coefficient row(s) and evaluates the
//     monomial sum by Horner's rule.
//
// Precision: FP64 evaluates in float64 with IEEE division for the cell
// index.  MIXED reads the (hi, lo) float32 split of the grid (or a float32
// table) and evaluates in float32; the cell index and fractional offset are
// still formed in float64 so indices and NaN masks are bit-exact.
#include "eval.cuh"

namespace arb {

template <int F, bool MIXED>
__global__ void __launch_bounds__(256) otf3_kernel(arb_grid g, KParams kp, double *q, int64_t nq,
                                                   int64_t qs, int wb, arb_query_out o,
                                                   int32_t *status) {
  using T = typename std::conditional<MIXED, float, double>::type;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  T frac_[3];
  int64_t idx;
  if (!query_prologue<3, F, !MIXED>(g, kp, q, i, qs, wb, o, status, frac_, idx)) return;
  const T fr[3] = {frac_[0], frac_[1], frac_[2]};
  double val[F], grad[3];
  int64_t c[3];
  cell_coords<3>(idx, g, c);
  eval_otf3<F, MIXED>(g, kp, c, fr, val, grad);
  write_vals<3, F>(o, i, val, grad);
}

template <int F, bool MIXED>
__global__ void __launch_bounds__(128) otf4_kernel(arb_grid g, KParams kp, double *q, int64_t nq,
                                                   int64_t qs, int wb, arb_query_out o,
                                                   int32_t *status) {
  using T = typename std::conditional<MIXED, float, double>::type;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  T frac_[4];
  int64_t idx;
  if (!query_prologue<4, F, !MIXED>(g, kp, q, i, qs, wb, o, status, frac_, idx)) return;
  const T fr[4] = {frac_[0], frac_[1], frac_[2], frac_[3]};
  double val[F], grad[4] = {0, 0, 0, 0};
  int64_t c[4];
  cell_coords<4>(idx, g, c);
  eval_otf4<F, MIXED>(g, kp, c, fr, val, grad);
  write_vals<4, F>(o, i, val, grad);
}

template <int DIM, int F, bool MIXED>
__global__ void __launch_bounds__(256) tab_kernel(arb_grid g, KParams kp, double *q, int64_t nq,
                                                  int64_t qs, int wb, arb_query_out o,
                                                  int32_t *status) {
  using T = typename std::conditional<MIXED, float, double>::type;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  T x[DIM];
  int64_t idx;
  if (!query_prologue<DIM, F, !MIXED>(g, kp, q, i, qs, wb, o, status, x, idx)) return;
  double val[F], grad[DIM];
  int64_t c[DIM];
  cell_coords<DIM>(idx, g, c);
  eval_tab<DIM, F, MIXED>(g, kp, c, x, val, grad);
  write_vals<DIM, F>(o, i, val, grad);
}

}  // namespace arb

using namespace arb;

#define ARB_DISPATCH_F(KER, ...)                                \
  switch (g->nfield) {                                          \
    case 1: KER<1, __VA_ARGS__>; break;                         \
    case 3: KER<3, __VA_ARGS__>; break;                         \
    case 4: KER<4, __VA_ARGS__>; break;                         \
    default: return ARB_ERR_INVALID;                            \
  }

extern "C" int arb_query_eval_otf(const arb_grid *g, int32_t precision, double *q, int64_t nq,
                                  int64_t q_stride, int32_t q_writeback, const arb_query_out *out,
                                  int32_t *status, arb_stream_t stream) {
  int rc = check_query_args(g, q, nq, q_stride, out);
  if (rc) return rc;
  if (nq == 0) return ARB_OK;
  const bool mixed = precision == ARB_PREC_MIXED;
  if (mixed ? !g->grid32 : !g->grid64) return ARB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const arb_query_out out_norm = normalize_out(*out, g->dim);
  out = &out_norm;
  const KParams kp = make_kparams(g);
  if (g->dim == 3) {
    const int T = 256;
    const unsigned B = (unsigned)((nq + T - 1) / T);
#define L3(FF, MX) otf3_kernel<FF, MX><<<B, T, 0, s>>>(*g, kp, q, nq, q_stride, q_writeback, *out, status)
    if (mixed) {
      switch (g->nfield) { case 1: L3(1, true); break; case 3: L3(3, true); break; case 4: L3(4, true); break; }
    } else {
      switch (g->nfield) { case 1: L3(1, false); break; case 3: L3(3, false); break; case 4: L3(4, false); break; }
    }
#undef L3
  } else {
    const int T = 128;
    const unsigned B = (unsigned)((nq + T - 1) / T);
#define L4(FF, MX) otf4_kernel<FF, MX><<<B, T, 0, s>>>(*g, kp, q, nq, q_stride, q_writeback, *out, status)
    if (mixed) {
      switch (g->nfield) { case 1: L4(1, true); break; case 3: L4(3, true); break; case 4: L4(4, true); break; }
    } else {
      switch (g->nfield) { case 1: L4(1, false); break; case 3: L4(3, false); break; case 4: L4(4, false); break; }
    }
#undef L4
  }
  return launch_status();
}

extern "C" int arb_query_eval(const arb_grid *g, double *q, int64_t nq, int64_t q_stride,
                              int32_t q_writeback, const arb_query_out *out, int32_t *status,
                              arb_stream_t stream) {
  int rc = check_query_args(g, q, nq, q_stride, out);
  if (rc) return rc;
  if (!g->table) return ARB_ERR_INVALID;
  if (nq == 0) return ARB_OK;
  const bool mixed = g->table_prec == ARB_PREC_MIXED;
  cudaStream_t s = (cudaStream_t)stream;
  const arb_query_out out_norm = normalize_out(*out, g->dim);
  out = &out_norm;
  const KParams kp = make_kparams(g);
  const int T = 256;
  const unsigned B = (unsigned)((nq + T - 1) / T);
#define LT(D, FF, MX) tab_kernel<D, FF, MX><<<B, T, 0, s>>>(*g, kp, q, nq, q_stride, q_writeback, *out, status)
#define LTF(D, MX) switch (g->nfield) { case 1: LT(D, 1, MX); break; case 3: LT(D, 3, MX); break; case 4: LT(D, 4, MX); break; }
  if (g->dim == 3) {
    if (mixed) { LTF(3, true) } else { LTF(3, false) }
  } else {
    if (mixed) { LTF(4, true) } else { LTF(4, false) }
  }
#undef LTF
#undef LT
  return launch_status();
}
