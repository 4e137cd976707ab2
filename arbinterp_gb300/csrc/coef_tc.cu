// Split-BF16 tensor-core coefficient solve (3D): the mixed-precision
// replacement of calcCoefficients1/2/3 + allCoeffs
// (src/ARBInterp/ARBInterp.py:523-525, 570-603).
//
// For every (cell, field) row:  alpha = A . f[block],  A = inv(B) D (64x64,
// entries k/8 with |k| <= 125, exact in BF16).  As a GEMM:
//   M = rows (cell, field), N = 64 monomials, K = 64 block points.
// A-operand rows hold the block values as deltas against the cell's own
// corner value, d = f - f_ref, formed in float32 from the (hi, lo) grid
// split, and d is split exactly into three BF16 terms d = d_hi + d_mid + d_lo,
// so the GEMM runs with K = 3 x 64 against A^T replicated three times.  The
// accumulators live in TMEM (128 lanes x 64 float32 columns); the epilogue
// adds f_ref back to alpha_000 and writes the float32 table row.
//
// Subtracting f_ref keeps every coefficient's relative error at float32
// level even where |f| >> h |grad f| (alpha_000 is the only coefficient of
// magnitude |f|; the rest scale with the field's variation), which is what
// keeps gradients within 1e-6 of the float64 path.
//
// One CTA = 128 threads = 4 warps; thread t owns tile row t (TMEM lane t).
// Persistent over tiles; up to 4 CTAs per SM (57 KB shared memory, 64 TMEM
// columns each).
#include <cuda_bf16.h>

#include "arb_common.cuh"
#include "tc_ptx.cuh"

namespace arb {

namespace {

constexpr int TM = 128;                  // tile rows
constexpr int KP = 64;                   // block points
constexpr int PARTS = 3;                 // BF16 terms per value
constexpr int KT = KP * PARTS;           // 192
constexpr int A_SBO = (KT / 8) * 128;    // bytes between 8-row core-matrix groups
constexpr int A_BYTES = (TM / 8) * A_SBO;
constexpr int B_SBO = (KP / 8) * 128;
constexpr int B_BYTES = (64 / 8) * B_SBO;
constexpr int STAGE_STRIDE = 256 + 16;   // padded output row (conflict-free stores)
constexpr uint32_t WAIT_LIMIT = 1u << 22;

static_assert(TM * STAGE_STRIDE <= A_BYTES, "staging must fit in the A tile");

struct TcSmem {
  unsigned char a[A_BYTES];
  unsigned char b[B_BYTES];
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

__device__ __forceinline__ uint32_t bf16_bits(float x) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x));
}

}  // namespace

template <int F>
__global__ void __launch_bounds__(128, 4) coef3_tc_kernel(arb_grid g, int64_t cell0, int64_t ncells,
                                                          float *table, int32_t *status) {
  extern __shared__ unsigned char smem_raw[];
  TcSmem &sm = *reinterpret_cast<TcSmem *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int64_t rows = ncells * F;
  const int64_t npts = grid_points(g);
  const int64_t ntiles = (rows + TM - 1) / TM;
  const int64_t nx = g.n[0], ny = g.n[1];

  // B operand: B[n][k] = A[n][k] = A1[ex][ox] A1[ey][oy] A1[ez][oz]
  for (int e = tid; e < 64 * 64; e += blockDim.x) {
    const int n = e >> 6, k = e & 63;
    const float v = kA1[n & 3][k & 3] * kA1[(n >> 2) & 3][(k >> 2) & 3] * kA1[n >> 4][k >> 4];
    *reinterpret_cast<__nv_bfloat16 *>(sm.b + kmaj(n, k, B_SBO)) = __float2bfloat16_rn(v);
  }
  if (warp == 0) {
    tc::tmem_alloc(&sm.tmem_base, 64);
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
  const uint32_t idesc = tc::idesc_f16(1u, 128u, 64u);
  const uint32_t a_base = tc::smem_u32(sm.a), b_base = tc::smem_u32(sm.b);
  uint32_t parity = 0;
  bool timed_out = false;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t r = tile * TM + tid;
    float rhi = 0.f, rlo = 0.f;
    // ---- gather the 4x4x4 block, delta, exact 3-term BF16 split ----------
    if (r < rows) {
      const int64_t cell = cell0 + r / F;
      const int f = (int)(r % F);
      int64_t c[3];
      cell_coords<3>(cell, g, c);
      const int64_t pref = ((c[2] + 1) * ny + (c[1] + 1)) * nx + (c[0] + 1);
      g32_load<F>(g.grid32, npts, pref, f, rhi, rlo);
#pragma unroll
      for (int ch = 0; ch < 8; ++ch) {  // 8 points = x-row pair (oy = 2ch&3 ..)
        uint32_t ph[4], pm[4], pl[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          uint32_t hb[2], mb[2], lb[2];
#pragma unroll
          for (int w = 0; w < 2; ++w) {
            const int k = ch * 8 + u * 2 + w;          // point index ox + 4 oy + 16 oz
            const int ox = k & 3, oy = (k >> 2) & 3, oz = k >> 4;
            const int64_t p = ((c[2] + oz) * ny + (c[1] + oy)) * nx + (c[0] + ox);
            float vh, vl;
            g32_load<F>(g.grid32, npts, p, f, vh, vl);
            const float d = (vh - rhi) + (vl - rlo);
            const __nv_bfloat16 h = __float2bfloat16_rn(d);
            const float r1 = d - __bfloat162float(h);
            const __nv_bfloat16 m = __float2bfloat16_rn(r1);
            const float r2 = r1 - __bfloat162float(m);
            hb[w] = (uint32_t)__bfloat16_as_ushort(h);
            mb[w] = (uint32_t)__bfloat16_as_ushort(m);
            lb[w] = bf16_bits(r2);
          }
          ph[u] = hb[0] | (hb[1] << 16);
          pm[u] = mb[0] | (mb[1] << 16);
          pl[u] = lb[0] | (lb[1] << 16);
        }
        *reinterpret_cast<uint4 *>(sm.a + kmaj(tid, ch * 8, A_SBO)) = make_uint4(ph[0], ph[1], ph[2], ph[3]);
        *reinterpret_cast<uint4 *>(sm.a + kmaj(tid, KP + ch * 8, A_SBO)) = make_uint4(pm[0], pm[1], pm[2], pm[3]);
        *reinterpret_cast<uint4 *>(sm.a + kmaj(tid, 2 * KP + ch * 8, A_SBO)) =
            make_uint4(pl[0], pl[1], pl[2], pl[3]);
      }
    } else {
#pragma unroll
      for (int ch = 0; ch < KT / 8; ++ch)
        *reinterpret_cast<uint4 *>(sm.a + kmaj(tid, ch * 8, A_SBO)) = make_uint4(0u, 0u, 0u, 0u);
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    // ---- 12 MMAs of 128 x 64 x 16 -----------------------------------------
    if (tid == 0) {
      tc::tc_fence_after();
#pragma unroll
      for (int s = 0; s < KT / 16; ++s) {
        const uint64_t ad = tc::smem_desc(a_base + (uint32_t)(2 * s) * 128u, 128u, (uint32_t)A_SBO);
        const uint64_t bd = tc::smem_desc(b_base + (uint32_t)(2 * (s & 3)) * 128u, 128u, (uint32_t)B_SBO);
        tc::mma_f16(tmem, ad, bd, idesc, s > 0 ? 1u : 0u);
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
    // ---- epilogue: TMEM -> registers -> padded staging -> bulk stores ------
    float acc[64];
#pragma unroll
    for (int q4 = 0; q4 < 4; ++q4) tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(q4 * 16), acc + 16 * q4);
    tc::tmem_wait_ld();
    acc[0] = rhi + (rlo + acc[0]);
    unsigned char *st = sm.a + tid * STAGE_STRIDE;
#pragma unroll
    for (int q = 0; q < 16; ++q)
      *reinterpret_cast<float4 *>(st + 16 * q) = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
    tc::fence_proxy_async_smem();
    if (r < rows) {
      tc::bulk_store(table + r * 64, st, 256u);
      tc::bulk_commit();
    }
    tc::bulk_wait_read0();
    tc::tc_fence_before();
    __syncthreads();
  }
  tc::bulk_wait0();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  // after a timed-out wait, give the MMAs in flight one more bounded wait
  // before the accumulator columns are released
  if (timed_out) (void)tc::mbar_wait_bounded(&sm.mbar, parity ^ 1u, WAIT_LIMIT);
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
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
  static bool attr = false;
  if (!attr) {
    // prefer the largest shared-memory carveout so several CTAs share an SM
    // (their gathers overlap each other's MMAs and epilogues)
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
  if (!per_sm && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coef3_tc_kernel<4>, 128, smem) != cudaSuccess)
    return ARB_ERR_CUDA;
  if (per_sm < 1) per_sm = 1;
  int64_t grid = (int64_t)num_sms() * per_sm;
  if (grid > tiles) grid = tiles;
  switch (g->nfield) {
    case 1: coef3_tc_kernel<1><<<(unsigned)grid, 128, smem, s>>>(*g, cell0, ncells, table, status); break;
    case 3: coef3_tc_kernel<3><<<(unsigned)grid, 128, smem, s>>>(*g, cell0, ncells, table, status); break;
    case 4: coef3_tc_kernel<4><<<(unsigned)grid, 128, smem, s>>>(*g, cell0, ncells, table, status); break;
    default: return ARB_ERR_INVALID;
  }
  return launch_status();
}

}  // namespace arb
