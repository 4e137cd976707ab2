// Coefficient table (float64) and finite-difference planes.
//
// arb_coef_solve(FP64) replaces calcCoefficients1/2/3 + allCoeffs
// (src/ARBInterp/ARBInterp.py:523-525, 570-603; 4D 1260-1262, 1322-1355):
// alpha = A f[block] for every cell and field.  A is applied in factored
// form: 3D A == kron(A1, A1, A1) (Catmull-Rom A1) exactly, so alpha is three
// passes of the 4x4 A1 along x, y and z (480 flops instead of 8192); 4D A
// is kron(A1,A1,A1,A1) plus the rank-16 term of the reference's row-240 D
// off-by-one, added from 16 mixed fourth-difference stencils.
//
// Table layout [cell][F][M], M = 4^dim, monomial index ex + 4 ey + 16 ez
// (+ 64 et) — the transpose of the reference's (M, nc+1) arrays, so one
// query reads one contiguous row per field.
#include "arb_common.cuh"

namespace arb {

// In-place 1D Catmull-Rom coefficient transform of 4 samples g0..g3:
// a0 = g1, a1 = (g2-g0)/2, a2 = g0 - 5/2 g1 + 2 g2 - 1/2 g3,
// a3 = -1/2 g0 + 3/2 g1 - 3/2 g2 + 1/2 g3.
template <typename T>
__device__ __forceinline__ void a1_transform(T &g0, T &g1, T &g2, T &g3) {
  const T a0 = g1;
  const T a1 = T(0.5) * (g2 - g0);
  const T a2 = g0 - T(2.5) * g1 + T(2) * g2 - T(0.5) * g3;
  const T a3 = T(-0.5) * g0 + T(1.5) * g1 - T(1.5) * g2 + T(0.5) * g3;
  g0 = a0;
  g1 = a1;
  g2 = a2;
  g3 = a3;
}

// One thread per (cell, field) row.
template <int F, typename TO>
__global__ void __launch_bounds__(128) coef3_fp64_kernel(arb_grid g, int64_t cell0, int64_t ncells,
                                                         TO *table) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= ncells * F) return;
  const int64_t cell = cell0 + r / F;
  const int f = (int)(r % F);
  int64_t c[3];
  cell_coords<3>(cell, g, c);
  const int64_t nx = g.n[0], ny = g.n[1];
  double a[64];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t p = ((c[2] + k) * ny + (c[1] + j)) * nx + c[0];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[16 * k + 4 * j + i] = __ldg(g.grid64 + (p + i) * F + f);
    }
#pragma unroll
  for (int m = 0; m < 16; ++m) a1_transform(a[4 * m], a[4 * m + 1], a[4 * m + 2], a[4 * m + 3]);
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int i = 0; i < 4; ++i)
      a1_transform(a[16 * k + i], a[16 * k + 4 + i], a[16 * k + 8 + i], a[16 * k + 12 + i]);
#pragma unroll
  for (int m = 0; m < 16; ++m) a1_transform(a[m], a[16 + m], a[32 + m], a[48 + m]);
  TO *out = table + ((cell - cell0) * F + f) * 64;
  if constexpr (sizeof(TO) == 8) {
#pragma unroll
    for (int m = 0; m < 32; ++m)
      reinterpret_cast<double2 *>(out)[m] = make_double2(a[2 * m], a[2 * m + 1]);
  } else {
#pragma unroll
    for (int m = 0; m < 16; ++m)
      reinterpret_cast<float4 *>(out)[m] =
          make_float4((float)a[4 * m], (float)a[4 * m + 1], (float)a[4 * m + 2], (float)a[4 * m + 3]);
  }
}

// One warp per (cell, field) row; the 256-value block lives in shared memory.
template <int F, typename TO>
__global__ void __launch_bounds__(128) coef4_fp64_kernel(arb_grid g, int64_t cell0, int64_t ncells,
                                                         TO *table) {
  __shared__ double sm[4][256];
  __shared__ double sT[4][16];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r = blockIdx.x * (int64_t)4 + warp;
  if (r >= ncells * F) return;
  const int64_t cell = cell0 + r / F;
  const int f = (int)(r % F);
  int64_t c[4];
  cell_coords<4>(cell, g, c);
  const int64_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
  double *b = sm[warp];
  for (int e = lane; e < 256; e += 32) {
    const int i = e & 3, j = (e >> 2) & 3, k = (e >> 4) & 3, l = e >> 6;
    const int64_t p = (((c[3] + l) * nz + (c[2] + k)) * ny + (c[1] + j)) * nx + (c[0] + i);
    b[e] = __ldg(g.grid64 + p * F + f);
  }
  __syncwarp();
  // mixed fourth-difference stencils S_c, c = cx + 2cy + 4cz + 8ct:
  // (1/16) sum_b sign(b) f[c + 2b]; then T_c = S_{c-1} - S_c (S_{-1} = 0).
  double S = 0.0;
  if (lane < 16) {
    const int cx = lane & 1, cy = (lane >> 1) & 1, cz = (lane >> 2) & 1, ct = lane >> 3;
#pragma unroll
    for (int bb = 0; bb < 16; ++bb) {
      const int bx = bb & 1, by = (bb >> 1) & 1, bz = (bb >> 2) & 1, bt = bb >> 3;
      const int par = bx + by + bz + bt;
      const double v = b[(cx + 2 * bx) + 4 * (cy + 2 * by) + 16 * (cz + 2 * bz) + 64 * (ct + 2 * bt)];
      S += (par & 1) ? -v : v;  // sign = prod(2b-1) = (-1)^(4-par) = (-1)^par
    }
    S *= 0.0625;
  }
  const double Sprev = __shfl_up_sync(0xffffffffu, S, 1);
  if (lane < 16) sT[warp][lane] = (lane == 0 ? 0.0 : Sprev) - S;
  // separable Catmull-Rom transform along x, y, z, t (64 lines each)
#pragma unroll 1
  for (int ax = 0; ax < 4; ++ax) {
    const int st = 1 << (2 * ax);
    for (int line = lane; line < 64; line += 32) {
      // line enumerates the 64 index combinations of the other three axes
      const int lowmask = st - 1;
      const int base = (line & lowmask) + ((line & ~lowmask) << 2);
      a1_transform(b[base], b[base + st], b[base + 2 * st], b[base + 3 * st]);
    }
    __syncwarp();
  }
  // + sum_c T_c * coeffs of prod_a hb_{c_a}(x_a); hb_0 = t - 2t^2 + t^3,
  // hb_1 = -t^2 + t^3
  const double P0[4] = {0.0, 1.0, -2.0, 1.0};
  const double P1[4] = {0.0, 0.0, -1.0, 1.0};
  TO *out = table + ((cell - cell0) * F + f) * 256;
  for (int e = lane; e < 256; e += 32) {
    const int ex = e & 3, ey = (e >> 2) & 3, ez = (e >> 4) & 3, et = e >> 6;
    double acc = b[e];
#pragma unroll
    for (int cc = 0; cc < 16; ++cc) {
      const double px = (cc & 1) ? P1[ex] : P0[ex];
      const double py = (cc & 2) ? P1[ey] : P0[ey];
      const double pz = (cc & 4) ? P1[ez] : P0[ez];
      const double pt = (cc & 8) ? P1[et] : P0[et];
      acc += sT[warp][cc] * (px * py * pz * pt);
    }
    out[e] = (TO)acc;
  }
}

// Derivative kinds in the reference's D-matrix row order, as axis bitmasks
// (x = 1, y = 2, z = 4, t = 8).
__constant__ int kKinds3[8] = {0, 1, 2, 4, 3, 5, 6, 7};
__constant__ int kKinds4[16] = {0, 1, 2, 4, 8, 3, 5, 9, 6, 10, 12, 7, 11, 13, 14, 15};

template <int DIM, int F>
__global__ void fd_planes_kernel(arb_grid g, double *planes) {
  int64_t npts = 1;
  for (int a = 0; a < DIM; ++a) npts *= g.n[a];
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= npts) return;
  int64_t crd[DIM], stride[DIM];
  int64_t rem = p, st = 1;
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    crd[a] = rem % g.n[a];
    rem /= g.n[a];
    stride[a] = st;
    st *= g.n[a];
  }
  constexpr int NK = 1 << DIM;
  for (int r = 0; r < NK; ++r) {
    const int kind = DIM == 3 ? kKinds3[r] : kKinds4[r];
    bool inside = true;
    int nact = 0;
    for (int a = 0; a < DIM; ++a)
      if (kind >> a & 1) {
        inside &= crd[a] >= 1 && crd[a] <= g.n[a] - 2;
        ++nact;
      }
    for (int f = 0; f < F; ++f) {
      double acc = 0.0;
      if (inside) {
        for (int s = 0; s < (1 << nact); ++s) {
          int64_t off = 0;
          int bit = 0, neg = 0;
          for (int a = 0; a < DIM; ++a)
            if (kind >> a & 1) {
              const int sg = (s >> bit++) & 1;  // 1 -> +1 step, 0 -> -1 step
              off += sg ? stride[a] : -stride[a];
              neg += !sg;
            }
          const double v = g.grid64[(p + off) * F + f];
          acc += (neg & 1) ? -v : v;
        }
        acc = ldexp(acc, -nact);
      } else {
        acc = qnan();
      }
      planes[((int64_t)r * npts + p) * F + f] = acc;
    }
  }
}

}  // namespace arb

using namespace arb;

// float32 table from the float64 separable solve (rounded once).  Used for
// 4D and as the reference for the tensor-core 3D solve.
static int coef_solve_f32_simt(const arb_grid *g, int64_t cell0, int64_t ncells, float *table,
                               cudaStream_t s) {
  const int64_t rows = ncells * g->nfield;
  if (g->dim == 3) {
    const unsigned B = (unsigned)((rows + 127) / 128);
#define C3(FF) coef3_fp64_kernel<FF, float><<<B, 128, 0, s>>>(*g, cell0, ncells, table)
    switch (g->nfield) { case 1: C3(1); break; case 3: C3(3); break; case 4: C3(4); break; default: return ARB_ERR_INVALID; }
#undef C3
  } else {
    const unsigned B = (unsigned)((rows + 3) / 4);
#define C4(FF) coef4_fp64_kernel<FF, float><<<B, 128, 0, s>>>(*g, cell0, ncells, table)
    switch (g->nfield) { case 1: C4(1); break; case 3: C4(3); break; case 4: C4(4); break; default: return ARB_ERR_INVALID; }
#undef C4
  }
  return launch_status();
}

namespace arb {
int coef4_solve_tc(const arb_grid *g, int64_t cell0, int64_t ncells, float *table, int32_t *status,
                   cudaStream_t s);
int coef3_solve_tc(const arb_grid *g, int64_t cell0, int64_t ncells, float *table, int32_t *status,
                   cudaStream_t s);
}

// Mixed precision: 3D uses the split-BF16 tcgen05 GEMM; 4D (A not exact in
// BF16) the float64 separable solve rounded to float32.
static int coef_solve_mixed(const arb_grid *g, int64_t cell0, int64_t ncells, float *table,
                            int32_t *status, cudaStream_t s) {
  if (g->dim == 3 && g->grid32) return arb::coef3_solve_tc(g, cell0, ncells, table, status, s);
  if (g->dim == 4 && g->grid32) return arb::coef4_solve_tc(g, cell0, ncells, table, status, s);
  return coef_solve_f32_simt(g, cell0, ncells, table, s);
}

extern "C" int arb_coef_solve(const arb_grid *g, int32_t precision, int64_t cell0, int64_t ncells,
                              void *table, int32_t *status, arb_stream_t stream) {
  // the 3D mixed solve reads only the float32 split; every other solve the float64 grid
  const bool tc3 = precision == ARB_PREC_MIXED && g && g->grid32;   // 3D and 4D tensor-core solves
  if (!g || !table || (!tc3 && !g->grid64)) return ARB_ERR_INVALID;
  if (cell0 < 0 || ncells < 0 || cell0 + ncells > g->nc) return ARB_ERR_INVALID;
  if (ncells == 0) return ARB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == ARB_PREC_MIXED) return coef_solve_mixed(g, cell0, ncells, (float *)table, status, s);
  if (precision != ARB_PREC_FP64) return ARB_ERR_INVALID;
  const int64_t rows = ncells * g->nfield;
  if (g->dim == 3) {
    const int T = 128;
    const unsigned B = (unsigned)((rows + T - 1) / T);
#define C3(FF) coef3_fp64_kernel<FF, double><<<B, T, 0, s>>>(*g, cell0, ncells, (double *)table)
    switch (g->nfield) { case 1: C3(1); break; case 3: C3(3); break; case 4: C3(4); break; default: return ARB_ERR_INVALID; }
#undef C3
  } else if (g->dim == 4) {
    const unsigned B = (unsigned)((rows + 3) / 4);
#define C4(FF) coef4_fp64_kernel<FF, double><<<B, 128, 0, s>>>(*g, cell0, ncells, (double *)table)
    switch (g->nfield) { case 1: C4(1); break; case 3: C4(3); break; case 4: C4(4); break; default: return ARB_ERR_INVALID; }
#undef C4
  } else {
    return ARB_ERR_INVALID;
  }
  return launch_status();
}

extern "C" int arb_fd_planes(const arb_grid *g, double *planes, arb_stream_t stream) {
  if (!g || !planes || !g->grid64) return ARB_ERR_INVALID;
  int64_t npts = 1;
  for (int a = 0; a < g->dim; ++a) npts *= g->n[a];
  const int T = 256;
  const unsigned B = (unsigned)((npts + T - 1) / T);
  cudaStream_t s = (cudaStream_t)stream;
#define FP(D, FF) fd_planes_kernel<D, FF><<<B, T, 0, s>>>(*g, planes)
  if (g->dim == 3) {
    switch (g->nfield) { case 1: FP(3, 1); break; case 3: FP(3, 3); break; case 4: FP(3, 4); break; default: return ARB_ERR_INVALID; }
  } else if (g->dim == 4) {
    switch (g->nfield) { case 1: FP(4, 1); break; case 3: FP(4, 3); break; case 4: FP(4, 4); break; default: return ARB_ERR_INVALID; }
  } else {
    return ARB_ERR_INVALID;
  }
#undef FP
  return launch_status();
}
