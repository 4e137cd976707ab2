// Tensor-core coefficient solve (3D, mixed precision): the replacement of
// calcCoefficients1/2/3 + allCoeffs (src/ARBInterp/ARBInterp.py:523-525,
// 570-603) for float32 tables.
//
// For every (cell, field) row:  alpha = A . f[block],  A = inv(B) D (64x64,
// entries k/8 with |k| <= 125).  As a GEMM:
//   M = rows (cell, field), N = 64 monomials, K = 64 block points.
//
// Exact fixed-point split.  The block values enter as deltas against the
// cell's own corner value, d = f - f_ref, formed in float32 from the (hi, lo)
// grid split (alpha_000 is the only coefficient of magnitude |f|; the others
// scale with the field's variation).  Each row is scaled by a power of two
// S = 2^E >= max|d| and u = d / S is cut into three integers
//   u = h0 2^-10 + h1 2^-21 + h2 2^-32,   |h0| <= 2048, |h1|, |h2| <= 1024,
// each exact in FP16.  The B operand is 8 A, integers of at most 7 bits, also
// exact in FP16.  Every product h * 8A is an integer below 2^18 and a sum of
// 64 of them stays below 2^24, so each part's accumulation is EXACT in the
// float32 accumulator; the three parts go to three TMEM accumulators and are
// combined once in the epilogue,
//   alpha = 2^(E-13) (acc0 + 2^-11 (acc1 + 2^-11 acc2)).
// The only roundings are u's truncation at 2^-33 S and the final float32
// rounding of alpha, so the table matches alpha computed exactly from the
// float32 deltas and rounded to float32.  (A single accumulator over
// float32-split operands loses up to ~10x more to cancellation between
// partial sums on coarse, fast-varying grids.)
//
// CTA = 256 threads (8 warps), tile = 128 rows.  Thread t owns row t & 127
// (TMEM lane t & 127); its half (t >> 7) gathers block points 32h..32h+31
// and, in the epilogue, coefficients 32h..32h+31 of that row.  Twelve
// 128x64x16 MMAs per tile (3 parts x 4 K-chunks) are issued by one thread;
// accumulators use 3 x 64 of the 256 allocated TMEM columns.  Output rows are
// staged in padded shared memory and written with bulk async stores, which
// drain while the next tile is gathered.  Two CTAs per SM (shared memory
// above a third of the SM's keeps the 256-column TMEM allocations within the
// SM's 512 columns).
#include <cuda_fp16.h>

#include "arb_common.cuh"
#include "tc_ptx.cuh"

namespace arb {

namespace {

constexpr int TM = 128;                  // tile rows
constexpr int NT = 256;                  // threads per CTA
constexpr int KP = 64;                   // block points
constexpr int PARTS = 3;                 // FP16 fixed-point parts per value
constexpr int KT = KP * PARTS;           // 192
constexpr int A_SBO = (KT / 8) * 128;    // bytes between 8-row core-matrix groups
constexpr int A_BYTES = (TM / 8) * A_SBO;
constexpr int B_SBO = (KP / 8) * 128;
constexpr int B_BYTES = (64 / 8) * B_SBO;
constexpr int STAGE_STRIDE = 256 + 16;   // padded output row (conflict-free stores)
constexpr int TMEM_COLS = 256;
constexpr uint32_t WAIT_LIMIT = 1u << 22;
constexpr float kRound = 12582912.0f;    // 1.5 * 2^23: x + kRound - kRound = rint(x) for |x| < 2^22

struct TcSmem {
  unsigned char a[A_BYTES];
  unsigned char b[B_BYTES];
  unsigned char stage[TM * STAGE_STRIDE];
  float amax[2][TM];
  uint64_t mbar;
  uint32_t tmem_base;
};

__constant__ float kA1[4][4] = {{0.f, 1.f, 0.f, 0.f},
                                {-0.5f, 0.f, 0.5f, 0.f},
                                {1.f, -2.5f, 2.f, -0.5f},
                                {-0.5f, 1.5f, -1.5f, 0.5f}};

// byte offset of element (row, k) in the no-swizzle K-major layout
__device__ __forceinline__ uint32_t kmaj(int row, int k, int sbo) {
  return (uint32_t)((row >> 3) * sbo + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ float rint_f(float x) { return __fadd_rn(__fadd_rn(x, kRound), -kRound); }

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
  const __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// power-of-two scale exponent: S = 2^E > amax (E clamped to [-100, 126])
__device__ __forceinline__ int scale_exp(float amax) {
  const int eb = (int)((__float_as_uint(amax) >> 23) & 0xffu);
  return min(max(eb - 126, -100), 126);
}

}  // namespace

template <int F>
__global__ void __launch_bounds__(NT, 2) coef3_tc_kernel(arb_grid g, int64_t cell0, int64_t ncells,
                                                         float *table, int32_t *status) {
  extern __shared__ unsigned char smem_raw[];
  TcSmem &sm = *reinterpret_cast<TcSmem *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (TM - 1), half = tid >> 7;
  const int64_t rows = ncells * F;
  const int64_t npts = grid_points(g);
  const int64_t ntiles = (rows + TM - 1) / TM;
  const int64_t nx = g.n[0], ny = g.n[1];

  // B operand: B[n][k] = 8 A[n][k] = 8 A1[ex][ox] A1[ey][oy] A1[ez][oz]
  for (int e = tid; e < 64 * 64; e += NT) {
    const int n = e >> 6, k = e & 63;
    const float v = 8.f * kA1[n & 3][k & 3] * kA1[(n >> 2) & 3][(k >> 2) & 3] * kA1[n >> 4][k >> 4];
    *reinterpret_cast<__half *>(sm.b + kmaj(n, k, B_SBO)) = __float2half_rn(v);
  }
  if (warp == 0) {
    tc::tmem_alloc(&sm.tmem_base, TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&sm.mbar, 1);
    tc::fence_mbar_init();
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  const uint32_t idesc = tc::idesc_f16(0u, 128u, 64u);
  const uint32_t a_base = tc::smem_u32(sm.a), b_base = tc::smem_u32(sm.b);
  const uint32_t t_row = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(half * 32);
  uint32_t parity = 0;
  bool timed_out = false;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t r = tile * TM + row;
    float rhi = 0.f, rlo = 0.f, d[32], amax = 0.f;
    // ---- gather half of the 4x4x4 block as deltas to the corner -------------
    if (r < rows) {
      const int64_t cell = cell0 + r / F;
      const int f = (int)(r % F);
      int64_t c[3];
      cell_coords<3>(cell, g, c);
      const int64_t pref = ((c[2] + 1) * ny + (c[1] + 1)) * nx + (c[0] + 1);
      g32_load<F>(g.grid32, npts, pref, f, rhi, rlo);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int k = half * 32 + j;  // point index ox + 4 oy + 16 oz
        const int ox = k & 3, oy = (k >> 2) & 3, oz = k >> 4;
        const int64_t p = ((c[2] + oz) * ny + (c[1] + oy)) * nx + (c[0] + ox);
        float vh, vl;
        g32_load<F>(g.grid32, npts, p, f, vh, vl);
        d[j] = (vh - rhi) + (vl - rlo);
        amax = fmaxf(amax, fabsf(d[j]));
      }
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j) d[j] = 0.f;
    }
    sm.amax[half][row] = amax;
    __syncthreads();
    const int E = scale_exp(fmaxf(amax, sm.amax[half ^ 1][row]));
    const float inv_s = __uint_as_float((uint32_t)(127 - E) << 23);
    // ---- exact three-part FP16 fixed-point split into the A tile ----------
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      uint32_t w0[4], w1[4], w2[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        float h0[2], h1[2], h2[2];
#pragma unroll
        for (int w = 0; w < 2; ++w) {
          const float t0 = d[ch * 8 + v * 2 + w] * inv_s * 1024.f;
          h0[w] = rint_f(t0);
          const float t1 = (t0 - h0[w]) * 2048.f;
          h1[w] = rint_f(t1);
          h2[w] = rint_f((t1 - h1[w]) * 2048.f);
        }
        w0[v] = pack_h2(h0[0], h0[1]);
        w1[v] = pack_h2(h1[0], h1[1]);
        w2[v] = pack_h2(h2[0], h2[1]);
      }
      const int k = half * 32 + ch * 8;
      *reinterpret_cast<uint4 *>(sm.a + kmaj(row, k, A_SBO)) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
      *reinterpret_cast<uint4 *>(sm.a + kmaj(row, KP + k, A_SBO)) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
      *reinterpret_cast<uint4 *>(sm.a + kmaj(row, 2 * KP + k, A_SBO)) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    // ---- 12 MMAs of 128 x 64 x 16: part p accumulates into columns 64p -----
    if (tid == 0) {
      tc::tc_fence_after();
#pragma unroll
      for (int p = 0; p < PARTS; ++p)
#pragma unroll
        for (int kc = 0; kc < 4; ++kc) {
          const int s = p * 4 + kc;
          const uint64_t ad = tc::smem_desc(a_base + (uint32_t)(2 * s) * 128u, 128u, (uint32_t)A_SBO);
          const uint64_t bd = tc::smem_desc(b_base + (uint32_t)(2 * kc) * 128u, 128u, (uint32_t)B_SBO);
          tc::mma_f16(tmem + (uint32_t)(64 * p), ad, bd, idesc, kc > 0 ? 1u : 0u);
        }
      tc::mma_commit(&sm.mbar);
    }
    const bool ok = tc::mbar_wait_bounded(&sm.mbar, parity, WAIT_LIMIT);
    parity ^= 1u;
    if (!ok) set_status(status, ARB_ERR_TIMEOUT);
    tc::tc_fence_after();
    if (__syncthreads_or(!ok)) {
      timed_out = true;
      break;
    }
    // ---- epilogue: combine the exact part sums, stage, bulk-store ----------
    float a[32], t[32];
    tc::tmem_ld16(t_row + 128u, t);
    tc::tmem_ld16(t_row + 144u, t + 16);
    tc::tmem_ld16(t_row + 64u, a);
    tc::tmem_ld16(t_row + 80u, a + 16);
    tc::tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 32; ++j) t[j] = __fmaf_rn(t[j], 0x1p-11f, a[j]);
    tc::tmem_ld16(t_row, a);
    tc::tmem_ld16(t_row + 16u, a + 16);
    tc::tmem_wait_ld();
    const float so = __uint_as_float((uint32_t)(E - 13 + 127) << 23);
#pragma unroll
    for (int j = 0; j < 32; ++j) a[j] = __fmaf_rn(t[j], 0x1p-11f, a[j]) * so;
    if (half == 0) a[0] = rhi + (rlo + a[0]);
    tc::bulk_wait_read0();  // this slot's previous store has read its source
    unsigned char *st = sm.stage + row * STAGE_STRIDE + half * 128;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      *reinterpret_cast<float4 *>(st + 16 * q) = make_float4(a[4 * q], a[4 * q + 1], a[4 * q + 2], a[4 * q + 3]);
    tc::fence_proxy_async_smem();
    if (r < rows) {
      tc::bulk_store(table + r * 64 + half * 32, st, 128u);
      tc::bulk_commit();
    }
    tc::tc_fence_before();
  }
  tc::bulk_wait0();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  // after a timed-out wait, give the MMAs in flight one more bounded wait
  // before the accumulator columns are released
  if (timed_out) (void)tc::mbar_wait_bounded(&sm.mbar, parity ^ 1u, WAIT_LIMIT);
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

static int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

// Host launcher used by arb_coef_solve for 3D mixed precision.
int coef3_solve_tc(const arb_grid *g, int64_t cell0, int64_t ncells, float *table, int32_t *status,
                   cudaStream_t s) {
  if (!g->grid32) return ARB_ERR_INVALID;
  const size_t smem = sizeof(TcSmem) + 1024;
  static_assert(3 * (sizeof(TcSmem) + 1024) > 228 * 1024, "a third CTA per SM would oversubscribe TMEM");
  static bool attr = false;
  if (!attr) {
    const void *ks[3] = {(const void *)coef3_tc_kernel<1>, (const void *)coef3_tc_kernel<3>,
                         (const void *)coef3_tc_kernel<4>};
    for (const void *k : ks) {
      if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
          cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100) != cudaSuccess)
        return ARB_ERR_CUDA;
    }
    attr = true;
  }
  const int64_t rows = ncells * g->nfield;
  const int64_t tiles = (rows + TM - 1) / TM;
  static int per_sm = 0;
  if (!per_sm && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coef3_tc_kernel<4>, NT, smem) != cudaSuccess)
    return ARB_ERR_CUDA;
  per_sm = per_sm < 1 ? 1 : (per_sm > 2 ? 2 : per_sm);
  int64_t grid = (int64_t)num_sms() * per_sm;
  if (grid > tiles) grid = tiles;
  switch (g->nfield) {
    case 1: coef3_tc_kernel<1><<<(unsigned)grid, NT, smem, s>>>(*g, cell0, ncells, table, status); break;
    case 3: coef3_tc_kernel<3><<<(unsigned)grid, NT, smem, s>>>(*g, cell0, ncells, table, status); break;
    case 4: coef3_tc_kernel<4><<<(unsigned)grid, NT, smem, s>>>(*g, cell0, ncells, table, status); break;
    default: return ARB_ERR_INVALID;
  }
  return launch_status();
}

}  // namespace arb
