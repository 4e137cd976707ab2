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
// S = 2^E > max|d|, t = 2^10 d / S, and t is cut into three FP16 parts
//   t = h0 + h1 + 2^-22 h2,   h0 integer (|h0| <= 1024),
//   h1 a multiple of 2^-11 (|h1| <= 1/2),  |h2| <= 1024,
// h0 and h1 exact normal FP16 numbers.  The B operand is 8 A, integers of at
// most 7 bits, exact in FP16.  Every product h0 * 8A is an integer and every
// h1 * 8A a multiple of 2^-11, and their 64-term sums stay below 2^23 units,
// so those two accumulations are EXACT in the float32 accumulator; the third
// part carries only the last 2^-22 of t.  The parts accumulate into three
// TMEM accumulators and are combined once in the epilogue,
//   alpha = 2^(E-13) (acc0 + (acc1 + 2^-22 acc2)),
// so the table matches alpha computed exactly from the float32 deltas up to
// its own float32 rounding (plus ~2^-26 S).  A single accumulator over
// float32-split operands loses up to ~10x more to cancellation between
// partial sums on coarse, fast-varying grids.
//
// CTA = 256 threads (8 warps), tile = 128 rows.  Thread t owns row t & 127
// (TMEM lane t & 127); its half (t >> 7) gathers block points 32h..32h+31
// (block layers oz = 2h, 2h+1) and, in the epilogue, coefficients
// 32h..32h+31 of that row.  Twelve 128x64x16 MMAs per tile (3 parts x 4
// K-chunks) are issued by one thread; the accumulators use 3 x 64 of the 256
// allocated TMEM columns.  The tile's 128 output rows are one contiguous
// 32 KB range of the table: they are staged in shared memory in the 128-byte
// swizzled layout (conflict-free row-per-thread writes) and written by two
// TMA tensor stores, which drain while the next tile is gathered.  Two CTAs
// per SM (shared memory above a third of the SM's keeps the 256-column TMEM
// allocations within the SM's 512 columns).
#include <cuda.h>
#include <cuda_fp16.h>

#include <mutex>
#include <vector>

#include "arb_common.cuh"
#include "tc_ptx.cuh"

namespace arb {

namespace {

constexpr int TM = 128;                  // tile rows
constexpr int NT = 256;                  // threads per CTA
constexpr int KP = 64;                   // block points
constexpr int PARTS = 3;                 // FP16 parts per value
constexpr int KT = KP * PARTS;           // 192
constexpr int A_SBO = (KT / 8) * 128;    // bytes between 8-row core-matrix groups
constexpr int A_BYTES = (TM / 8) * A_SBO;
constexpr int B_SBO = (KP / 8) * 128;
constexpr int B_BYTES = (64 / 8) * B_SBO;
constexpr int BOX_BYTES = TM * 128;      // one half-row box: 128 rows x 32 floats
constexpr int TMEM_COLS = 256;
constexpr uint32_t WAIT_LIMIT = 1u << 22;
constexpr float kRound0 = 12582912.0f;   // 1.5 * 2^23: (x + c) - c rounds x to an integer (|x| < 2^22)
constexpr float kRound1 = 6144.0f;       // 1.5 * 2^12: (x + c) - c rounds x to a multiple of 2^-11

struct TcSmem {
  unsigned char a[A_BYTES];              // A tile, no-swizzle K-major (offset 0)
  unsigned char b[B_BYTES];              // B = 8 A (offset 48 KB)
  unsigned char stage[2][BOX_BYTES];     // output rows, 128-byte swizzled (offset 56 KB, 1 KB aligned)
  float amax[2][TM];
  uint64_t mbar;
  uint32_t tmem_base;
};

__constant__ float kA1[4][4] = {{0.f, 1.f, 0.f, 0.f},
                                {-0.5f, 0.f, 0.5f, 0.f},
                                {1.f, -2.5f, 2.f, -0.5f},
                                {-0.5f, 1.5f, -1.5f, 0.5f}};

// byte offset of element (row, k) in the no-swizzle K-major layout
__host__ __device__ __forceinline__ uint32_t kmaj(int row, int k, int sbo) {
  return (uint32_t)((row >> 3) * sbo + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// The 1 KB-aligned start of a kernel's dynamic shared memory, reached by an
// offset from the shared array itself: a pointer rounded through an integer
// loses the shared address space and every access through it becomes a
// generic load or store.
template <typename T>
__device__ __forceinline__ T &smem_aligned_1k(unsigned char *raw) {
  const uint32_t a = tc::smem_u32(raw);
  return *reinterpret_cast<T *>(raw + (((a + 1023u) & ~1023u) - a));
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
  const __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// power-of-two scale exponent: S = 2^E > amax (E clamped to [-100, 126])
__device__ __forceinline__ int scale_exp(float amax) {
  const int eb = (int)((__float_as_uint(amax) >> 23) & 0xffu);
  return min(max(eb - 126, -100), 126);
}

// Packed float32 pairs (Blackwell .f32x2): one instruction rounds both
// components exactly as the scalar operation does.
#define ARB_F32X2(name, op)                                                                            \
  __device__ __forceinline__ float2 name(float2 a, float2 b) {                                        \
    float2 d;                                                                                          \
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t" op      \
        " rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"                                                  \
        : "=f"(d.x), "=f"(d.y)                                                                         \
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                                     \
    return d;                                                                                          \
  }
ARB_F32X2(fadd2, "add.rn.f32x2")
ARB_F32X2(fsub2, "sub.rn.f32x2")
ARB_F32X2(fmul2, "mul.rn.f32x2")
#undef ARB_F32X2

// Two values at once: t -> (h0, h1, 2^-SH h2 parts) with t = h0 + h1 + 2^-SH h2;
// R1 rounds to the h1 grid (3D: 2^-11, SH = 22; 4D: 2^-10, SH = 20).
__device__ __forceinline__ void split3_pair(float2 t, float r1, float sh, float2 &h0, float2 &h1, float2 &h2) {
  const float2 R0 = make_float2(kRound0, kRound0), R1 = make_float2(r1, r1);
  h0 = fsub2(fadd2(t, R0), R0);
  const float2 r = fsub2(t, h0);
  h1 = fsub2(fadd2(r, R1), R1);
  h2 = fmul2(fsub2(r, h1), make_float2(sh, sh));
}


// four points along x of one block line: component f of grid32 (+ lo)
template <int F>
__device__ __forceinline__ void load_line(const float *hp, const float *lp, bool has_lo, float rhi, float rlo,
                                          float *d, float &amax) {
#pragma unroll
  for (int ox = 0; ox < 4; ox += 2) {
    float2 vh, vl = make_float2(0.f, 0.f);
    if (F == 1) {
      const float2 v0 = __ldg(reinterpret_cast<const float2 *>(hp) + ox);  // (hi, lo) points: 8-byte aligned
      const float2 v1 = __ldg(reinterpret_cast<const float2 *>(hp) + ox + 1);
      vh = make_float2(v0.x, v1.x);
      vl = make_float2(v0.y, v1.y);
    } else {
      vh = make_float2(__ldg(hp + 4 * ox), __ldg(hp + 4 * ox + 4));
      if (has_lo) vl = make_float2(__ldg(lp + ox), __ldg(lp + ox + 1));
    }
    const float2 dd = fadd2(fsub2(vh, make_float2(rhi, rhi)), fsub2(vl, make_float2(rlo, rlo)));
    d[ox] = dd.x;
    d[ox + 1] = dd.y;
    amax = fmaxf(amax, fmaxf(fabsf(dd.x), fabsf(dd.y)));
  }
}

}  // namespace

// Poll limit of the MMA-completion wait in coef3_tc's tile loop.  It is
// WAIT_LIMIT unless a test lowers it (arb_test_set_mma_wait_limit) to make
// that wait run out; the drain wait before the accumulator columns are
// released always keeps WAIT_LIMIT, so no MMA is in flight at kernel exit.
static __device__ uint32_t g_mma_wait_limit = WAIT_LIMIT;

template <int F>
__global__ void __launch_bounds__(NT, 2) coef3_tc_kernel(const __grid_constant__ CUtensorMap tmap, arb_grid g,
                                                         int64_t cell0, int64_t ncells, int32_t *status) {
  extern __shared__ unsigned char smem_raw[];
  TcSmem &sm = smem_aligned_1k<TcSmem>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (TM - 1), half = tid >> 7;
  const int64_t rows = ncells * F;
  const int64_t npts = grid_points(g);
  const int64_t ntiles = (rows + TM - 1) / TM;
  const int64_t nx = g.n[0], sy = g.n[0], sz = g.n[0] * g.n[1];   // point strides
  constexpr int PW = F == 1 ? 2 : 4;                                  // floats per point in grid32

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
  unsigned char *st_row = sm.stage[half] + row * 128;
  uint32_t parity = 0;
  bool timed_out = false;
  const uint32_t mma_wait_limit = g_mma_wait_limit;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t r = tile * TM + row;
    float rhi = 0.f, rlo = 0.f, d[32], amax = 0.f;
    // ---- gather block layers oz = 2h, 2h+1 as deltas to the corner ---------
    if (r < rows) {
      const int64_t cell = cell0 + r / F;
      const int f = F == 1 ? 0 : (int)(r % F);
      const bool has_lo = F == 1 || (F == 4 && f == 3);
      int64_t c[3];
      cell_coords<3>(cell, g, c);
      const int64_t p0 = (c[2] * g.n[1] + c[1]) * nx + c[0];          // block origin (ox = oy = oz = 0)
      const float *hb = g.grid32 + p0 * PW + f;
      const float *lb = g.grid32 + npts * 4 + p0;                     // lo of |B| (F = 4)
      const int64_t corner = sz + sy + 1;
      if (F == 1) {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(hb + corner * PW));
        rhi = v.x;
        rlo = v.y;
      } else {
        rhi = __ldg(hb + corner * PW);
        if (has_lo) rlo = __ldg(lb + corner);
      }
      const float *hp = hb + (2 * half) * sz * PW, *lp = lb + (2 * half) * sz;
#pragma unroll
      for (int oz = 0; oz < 2; ++oz) {
#pragma unroll
        for (int oy = 0; oy < 4; ++oy) {
          load_line<F>(hp, lp, has_lo, rhi, rlo, d + oz * 16 + oy * 4, amax);
          hp += sy * PW;
          lp += sy;
        }
        hp += (sz - 4 * sy) * PW;
        lp += sz - 4 * sy;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j) d[j] = 0.f;
    }
    sm.amax[half][row] = amax;
    __syncthreads();
    const int E = scale_exp(fmaxf(amax, sm.amax[half ^ 1][row]));
    const float c10 = __uint_as_float((uint32_t)(137 - E) << 23);    // 2^(10 - E)
    // ---- three-part FP16 split into the A tile ------------------------------
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      uint32_t w0[4], w1[4], w2[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        float2 h0, h1, h2;
        split3_pair(fmul2(make_float2(d[ch * 8 + v * 2], d[ch * 8 + v * 2 + 1]), make_float2(c10, c10)), kRound1,
                    4194304.0f, h0, h1, h2);
        w0[v] = pack_h2(h0.x, h0.y);
        w1[v] = pack_h2(h1.x, h1.y);
        w2[v] = pack_h2(h2.x, h2.y);
      }
      const int k = half * 32 + ch * 8;
      *reinterpret_cast<uint4 *>(sm.a + kmaj(row, k, A_SBO)) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
      *reinterpret_cast<uint4 *>(sm.a + kmaj(row, KP + k, A_SBO)) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
      *reinterpret_cast<uint4 *>(sm.a + kmaj(row, 2 * KP + k, A_SBO)) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    if (tid == 0) tc::bulk_wait_read0();  // the previous tile's stores have read the staging buffer
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
    const bool ok = tc::mbar_wait_bounded(&sm.mbar, parity, mma_wait_limit);
    parity ^= 1u;
    if (!ok) set_status(status, ARB_ERR_TIMEOUT);
    tc::tc_fence_after();
    if (__syncthreads_or(!ok)) {
      timed_out = true;
      break;
    }
    // ---- epilogue: combine the part sums, stage swizzled, TMA-store --------
    float a[32], t[32];
    tc::tmem_ld16(t_row + 128u, t);
    tc::tmem_ld16(t_row + 144u, t + 16);
    tc::tmem_ld16(t_row + 64u, a);
    tc::tmem_ld16(t_row + 80u, a + 16);
    tc::tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 32; ++j) t[j] = __fmaf_rn(t[j], 0x1p-22f, a[j]);
    tc::tmem_ld16(t_row, a);
    tc::tmem_ld16(t_row + 16u, a + 16);
    tc::tmem_wait_ld();
    const float so = __uint_as_float((uint32_t)(E - 13 + 127) << 23);   // 2^(E - 13)
#pragma unroll
    for (int j = 0; j < 32; ++j) a[j] = __fmul_rn(__fadd_rn(a[j], t[j]), so);
    if (half == 0) a[0] = rhi + (rlo + a[0]);
#pragma unroll
    for (int q = 0; q < 8; ++q)
      *reinterpret_cast<float4 *>(st_row + 16 * (q ^ (row & 7))) =
          make_float4(a[4 * q], a[4 * q + 1], a[4 * q + 2], a[4 * q + 3]);
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::tma_store_2d(&tmap, sm.stage[0], 0, (int32_t)(tile * TM));
      tc::tma_store_2d(&tmap, sm.stage[1], 32, (int32_t)(tile * TM));
      tc::bulk_commit();
    }
  }
  if (tid == 0) tc::bulk_wait0();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  // after a timed-out wait, give the MMAs in flight one more bounded wait
  // before the accumulator columns are released
  if (timed_out) (void)tc::mbar_wait_bounded(&sm.mbar, parity ^ 1u, WAIT_LIMIT);
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

// ---- full solves: warp-specialised, the block gather fed by TMA -------------
// allCoeffs over every cell.  A tile holds C = 128 / F consecutive cells of one
// x-row of cells (C x F rows of the table; the last tile of each row holds the
// row's remaining cells).  Its grid footprint -- C + 3 points along x, 4
// along y and z -- arrives in shared memory as 3D TMA boxes (zeros beyond the
// grid) and the gather reads the footprint from shared memory.
// Footprint boxes (the TMA rule: x * element size a multiple of 16 bytes):
//   F = 4: hi, 4 x 35 floats x 4 x 4 (x = 4 x0); lo of |B|, 40 x 4 x 4 floats
//          from x = x0 rounded down to a multiple of 4 (needs nx % 4 == 0);
//   F = 3: hi, 4 x 45 floats x 4 x 4;
//   F = 1: (hi, lo) pairs as 8-byte elements, 132 x 4 x 4, x0 even (needs nx
//          even: the row stride must be a multiple of 16 bytes).
// Grids that miss these rules, and partial solves, take coef3_tc_kernel.
//
// One CTA per SM, three roles working on consecutive tiles at once, each
// hand-off an mbarrier; footprints three-deep, A tiles and accumulators
// two-deep, one staging area (the epilogue waits for the previous tile's
// stores to have read it):
//   producers (8 warps): the gather of a footprint into row deltas, the
//       per-row scale, the three-part FP16 split into an A tile; thread t
//       owns half t >> 7 (block layers 2h, 2h+1) of row t & 127;
//   footprint loader (one thread of warp 12): the boxes three tiles ahead,
//       issued as soon as the producers have gathered from the buffer;
//   MMA issuer (one thread of warp 13): the 12 MMAs of each tile into one
//       of two TMEM accumulator stages (3 x 64 columns each, at columns 0
//       and 256).  Issuing a tile's MMAs takes about 1000 cycles; with the
//       box loads in the same thread the loads fell behind the producers;
//   epilogue (4 warps): warp 8 + w reads TMEM lanes 32w..32w+31 (a whole
//       row per thread), combines the three part sums, stages the rows
//       128-byte swizzled and one thread writes them with two TMA stores.
// So the split of one tile overlaps the MMAs of the previous one and the
// epilogue and stores of the one before, where coef3_tc runs that chain in
// order inside each CTA.  Every wait is bounded: a wait that runs out ORs
// ARB_ERR_TIMEOUT into the status word and raises a shared abort flag that
// ends every role's waits; the producer and epilogue warps leave their loops
// together (a barrier that ORs their failures), and before the accumulator
// columns are released and the CTA exits, the MMA issuer waits with the full
// limit for its last MMAs and the footprint loader for any box in flight.
namespace {
template <int F>
struct TmaShape;
template <>
struct TmaShape<4> {
  static constexpr int C = 32, HX = 35, LX = 40, HBYTES = 4 * HX * 16 * 4, LBYTES = LX * 16 * 4;
};
template <>
struct TmaShape<3> {
  static constexpr int C = 42, HX = 45, HBYTES = 4 * HX * 16 * 4, LBYTES = 0;
};
template <>
struct TmaShape<1> {
  static constexpr int C = 128, HX = 132, HBYTES = HX * 16 * 8, LBYTES = 0;
};
constexpr int FP_BYTES = 17408;  // >= every shape's HBYTES + LBYTES, a multiple of 1 KB

constexpr int WS_PROD = 256;                        // producer threads (warps 0-7)
constexpr int WS_EPI = 128;                         // epilogue threads (warps 8-11)
constexpr int WS_WARP_FP = (WS_PROD + WS_EPI) / 32;  // warp 12: footprint loads
constexpr int WS_WARP_MMA = WS_WARP_FP + 1;           // warp 13: MMA issue
constexpr int WS_THREADS = WS_PROD + WS_EPI + 64;
constexpr int WS_TMEM_COLS = 512;                   // two accumulator stages of 3 x 64 columns
constexpr uint32_t BAR_PROD = 1, BAR_EPI = 2;       // named barriers of the producer and epilogue warps
constexpr int WS_FP = 3;                            // footprint buffers: boxes three tiles ahead

struct WsSmem {
  unsigned char a[2][A_BYTES];             // A tiles, no-swizzle K-major (offset 0)
  unsigned char stage[2][BOX_BYTES];       // output rows of a tile: two 128-byte swizzled boxes (1 KB aligned)
  unsigned char b[B_BYTES];                // B = 8 A
  unsigned char fp[WS_FP][FP_BYTES];       // footprints
  float amax[2][2][TM];                    // [tile parity][half][row]
  float mrhi[4][TM], mrlo[4][TM];          // each row's corner value (hi, lo), by tile mod 4
  int mexp[4][TM];                         // each row's scale exponent
  uint64_t fp_full[WS_FP], fp_empty[WS_FP], a_full[2], a_empty[2], acc_full[2], acc_empty[2];
  uint32_t tmem_base;
  int abort;
};
static_assert(TmaShape<4>::HBYTES + TmaShape<4>::LBYTES <= FP_BYTES && TmaShape<3>::HBYTES <= FP_BYTES &&
                  TmaShape<1>::HBYTES <= FP_BYTES,
              "footprint buffer");
static_assert(offsetof(WsSmem, stage) % 1024 == 0 && offsetof(WsSmem, fp) % 1024 == 0 &&
                  offsetof(WsSmem, b) % 1024 == 0,
              "alignment");

// Bounded wait that also gives up once another role has raised the abort
// flag; a wait that runs out raises it.
__device__ __forceinline__ bool ws_wait(WsSmem &sm, uint64_t *bar, uint32_t parity, uint32_t limit,
                                        int32_t *status) {
  for (uint32_t it = 0; it < limit; ++it) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if (*(volatile int *)&sm.abort) return false;
  }
  set_status(status, ARB_ERR_TIMEOUT);
  *(volatile int *)&sm.abort = 1;
  return false;
}
}  // namespace

template <int F>
__global__ void __launch_bounds__(WS_THREADS, 1) coef3_tma_kernel(const __grid_constant__ CUtensorMap tmap_full,
                                                                  const __grid_constant__ CUtensorMap tmap_part,
                                                                  const __grid_constant__ CUtensorMap tmap_hi,
                                                                  const __grid_constant__ CUtensorMap tmap_lo,
                                                                  arb_grid g, int32_t *status) {
  using S = TmaShape<F>;
  extern __shared__ unsigned char smem_raw[];
  WsSmem &sm = smem_aligned_1k<WsSmem>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t ncx = g.n[0] - 3, ncy = g.n[1] - 3, ncz = g.n[2] - 3;
  const int64_t tpr = (ncx + S::C - 1) / S::C;          // tiles per x-row of cells
  const int rem = (int)(ncx - (tpr - 1) * S::C);         // cells in a row's last tile
  const int64_t ntiles = tpr * ncy * ncz;
  const int nloc = blockIdx.x < ntiles ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;

  for (int e = tid; e < 64 * 64; e += WS_THREADS) {
    const int n = e >> 6, k = e & 63;
    const float v = 8.f * kA1[n & 3][k & 3] * kA1[(n >> 2) & 3][(k >> 2) & 3] * kA1[n >> 4][k >> 4];
    *reinterpret_cast<__half *>(sm.b + kmaj(n, k, B_SBO)) = __float2half_rn(v);
  }
  if (warp == 0) {
    tc::tmem_alloc(&sm.tmem_base, WS_TMEM_COLS);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int s = 0; s < WS_FP; ++s) {
      tc::mbar_init(&sm.fp_full[s], 1);
      tc::mbar_init(&sm.fp_empty[s], WS_PROD / 32);
    }
    for (int s = 0; s < 2; ++s) {
      tc::mbar_init(&sm.a_full[s], WS_PROD / 32);
      tc::mbar_init(&sm.a_empty[s], 1);
      tc::mbar_init(&sm.acc_full[s], 1);
      tc::mbar_init(&sm.acc_empty[s], WS_EPI / 32);
    }
    sm.abort = 0;
    tc::fence_mbar_init();
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  auto tile_of = [&](int k) { return (int64_t)blockIdx.x + (int64_t)k * gridDim.x; };

  if (warp < WS_PROD / 32) {
    // ---- producers: gather, scale, split -----------------------------------
    const int row = tid & (TM - 1), half = tid >> 7;
    const int cl = row / F, f = row % F;                 // this row's cell in the tile, and field
    bool fail = false;
    for (int k = 0; k < nloc; ++k) {
      const int s = k & 1;
      const uint32_t ph = (uint32_t)(k >> 1) & 1u;
      const int64_t tile = tile_of(k);
      const int64_t xr = tile / tpr;
      const int x0 = (int)((tile - xr * tpr) * S::C);
      const int cnt = tile - xr * tpr == tpr - 1 ? rem : S::C;
      const int fs = k % WS_FP;
      bool ok = !fail && ws_wait(sm, &sm.fp_full[fs], (uint32_t)(k / WS_FP) & 1u, WAIT_LIMIT, status);
      float rhi = 0.f, rlo = 0.f, d[32], amax = 0.f;
#pragma unroll
      for (int j = 0; j < 32; ++j) d[j] = 0.f;
      if (ok && cl < cnt) {
        const unsigned char *fpb = sm.fp[fs];
        const float *fh = reinterpret_cast<const float *>(fpb);
        auto pt = [&](int ox, int oy, int oz, float &h, float &l) {
          const int P = (oz * 4 + oy) * S::HX + cl + ox;
          if constexpr (F == 1) {
            const float2 v = reinterpret_cast<const float2 *>(fpb)[P + (x0 & 1)];
            h = v.x;
            l = v.y;
          } else {
            h = fh[4 * P + f];
            l = 0.f;
            if constexpr (F == 4) {
              if (f == 3)
                l = reinterpret_cast<const float *>(fpb + S::HBYTES)[(oz * 4 + oy) * S::LX + cl + ox + (x0 & 3)];
            }
          }
        };
        pt(1, 1, 1, rhi, rlo);
#pragma unroll
        for (int oz = 0; oz < 2; ++oz)
#pragma unroll
          for (int oy = 0; oy < 4; ++oy)
#pragma unroll
            for (int ox = 0; ox < 4; ox += 2) {
              float h0, l0, h1, l1;
              pt(ox, oy, 2 * half + oz, h0, l0);
              pt(ox + 1, oy, 2 * half + oz, h1, l1);
              const float2 dd = fadd2(fsub2(make_float2(h0, h1), make_float2(rhi, rhi)),
                                      fsub2(make_float2(l0, l1), make_float2(rlo, rlo)));
              d[oz * 16 + oy * 4 + ox] = dd.x;
              d[oz * 16 + oy * 4 + ox + 1] = dd.y;
              amax = fmaxf(amax, fmaxf(fabsf(dd.x), fabsf(dd.y)));
            }
      }
      __syncwarp();
      if (ok && lane == 0) tc::mbar_arrive(&sm.fp_empty[fs]);  // this warp has read the footprint
      sm.amax[s][half][row] = amax;
      if (tc::named_bar_or(BAR_PROD, WS_PROD, !ok)) break;   // every producer leaves together
      const int E = scale_exp(fmaxf(amax, sm.amax[s][half ^ 1][row]));
      const float c10 = __uint_as_float((uint32_t)(137 - E) << 23);    // 2^(10 - E)
      ok = k < 2 || ws_wait(sm, &sm.a_empty[s], ph ^ 1u, WAIT_LIMIT, status);  // the MMAs of tile k - 2 are done
      if (ok) {
        unsigned char *at = sm.a[s];
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          uint32_t w0[4], w1[4], w2[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            float2 h0, h1, h2;
            split3_pair(fmul2(make_float2(d[ch * 8 + v * 2], d[ch * 8 + v * 2 + 1]), make_float2(c10, c10)),
                        kRound1, 4194304.0f, h0, h1, h2);
            w0[v] = pack_h2(h0.x, h0.y);
            w1[v] = pack_h2(h1.x, h1.y);
            w2[v] = pack_h2(h2.x, h2.y);
          }
          const int kk = half * 32 + ch * 8;
          *reinterpret_cast<uint4 *>(at + kmaj(row, kk, A_SBO)) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
          *reinterpret_cast<uint4 *>(at + kmaj(row, KP + kk, A_SBO)) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
          *reinterpret_cast<uint4 *>(at + kmaj(row, 2 * KP + kk, A_SBO)) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
        }
        if (half == 0) {
          sm.mrhi[k & 3][row] = rhi;
          sm.mrlo[k & 3][row] = rlo;
          sm.mexp[k & 3][row] = E;
        }
        tc::fence_proxy_async_smem();  // the A tile is visible to the tensor core
      }
      __syncwarp();
      if (ok && lane == 0) tc::mbar_arrive(&sm.a_full[s]);
      fail = !ok;
    }
  } else if (warp < (WS_PROD + WS_EPI) / 32) {
    // ---- epilogue: TMEM -> table rows ----------------------------------------
    const int ew = warp - WS_PROD / 32;                  // TMEM lanes 32 ew .. 32 ew + 31
    const int row = ew * 32 + lane;
    const uint32_t mma_wait_limit = g_mma_wait_limit;
    bool fail = false;
    for (int k = 0; k < nloc; ++k) {
      const int s = k & 1;
      const uint32_t ph = (uint32_t)(k >> 1) & 1u;
      const bool ok = !fail && ws_wait(sm, &sm.acc_full[s], ph, mma_wait_limit, status);
      tc::tc_fence_after();
      if (tid == WS_PROD) tc::bulk_wait_read0();          // the stores of tile k - 1 have read the staging
      if (tc::named_bar_or(BAR_EPI, WS_EPI, !ok)) break;
      const int64_t tile = tile_of(k);
      const int64_t xr = tile / tpr;
      const int64_t kx = tile - xr * tpr;
      const int cnt = kx == tpr - 1 ? rem : S::C;
      const int64_t row0 = (xr * ncx + kx * S::C) * F;   // first table row of the tile
      const int E = sm.mexp[k & 3][row];
      const float rhi = sm.mrhi[k & 3][row], rlo = sm.mrlo[k & 3][row];
      const float so = __uint_as_float((uint32_t)(E - 13 + 127) << 23);   // 2^(E - 13)
      const uint32_t t_row = tmem + ((uint32_t)(ew * 32) << 16) + (uint32_t)(256 * s);
#pragma unroll
      for (int q = 0; q < 4; ++q) {                      // coefficients 16q .. 16q + 15
        float p0[16], p1[16], p2[16];
        tc::tmem_ld16(t_row + (uint32_t)(16 * q), p0);
        tc::tmem_ld16(t_row + (uint32_t)(64 + 16 * q), p1);
        tc::tmem_ld16(t_row + (uint32_t)(128 + 16 * q), p2);
        tc::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; ++j) p0[j] = __fmul_rn(__fadd_rn(p0[j], __fmaf_rn(p2[j], 0x1p-22f, p1[j])), so);
        if (q == 0) p0[0] = rhi + (rlo + p0[0]);
        unsigned char *st_row = sm.stage[q >> 1] + row * 128;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int j = (q & 1) * 4 + c;                 // 16-byte chunk of the 128-byte row
          *reinterpret_cast<float4 *>(st_row + 16 * (j ^ (row & 7))) =
              make_float4(p0[4 * c], p0[4 * c + 1], p0[4 * c + 2], p0[4 * c + 3]);
        }
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&sm.acc_empty[s]);  // this warp has read the accumulator
      tc::fence_proxy_async_smem();
      tc::named_bar_sync(BAR_EPI, WS_EPI);
      if (tid == WS_PROD) {
        const CUtensorMap *tm = cnt == S::C ? &tmap_full : &tmap_part;
        tc::tma_store_2d(tm, sm.stage[0], 0, (int32_t)row0);
        tc::tma_store_2d(tm, sm.stage[1], 32, (int32_t)row0);
        tc::bulk_commit();
      }
    }
    if (tid == WS_PROD) tc::bulk_wait0();
  } else if (warp == WS_WARP_FP && lane == 0) {
    // ---- footprint loader: boxes WS_FP tiles ahead ---------------------------
    auto issue_fp = [&](int k) {
      const int s = k % WS_FP;
      const int64_t tile = tile_of(k);
      const int64_t xr = tile / tpr;
      const int x0 = (int)((tile - xr * tpr) * S::C);
      const int y = (int)(xr % ncy), z = (int)(xr / ncy);
      tc::mbar_arrive_expect_tx(&sm.fp_full[s], (uint32_t)(S::HBYTES + S::LBYTES));
      if constexpr (F == 1) {
        tc::tma_load_3d(sm.fp[s], &tmap_hi, x0 & ~1, y, z, &sm.fp_full[s]);
      } else {
        tc::tma_load_3d(sm.fp[s], &tmap_hi, 4 * x0, y, z, &sm.fp_full[s]);
        if constexpr (F == 4) tc::tma_load_3d(sm.fp[s] + S::HBYTES, &tmap_lo, x0 & ~3, y, z, &sm.fp_full[s]);
      }
    };
    int fp_issued = 0;
    for (; fp_issued < nloc && fp_issued < WS_FP; ++fp_issued) issue_fp(fp_issued);
    // the footprint WS_FP tiles ahead, as soon as the producers have read
    // tile k's buffer (after their gather, long before its A tile is ready)
    for (int k = 0; k + WS_FP < nloc; ++k) {
      if (!ws_wait(sm, &sm.fp_empty[k % WS_FP], (uint32_t)(k / WS_FP) & 1u, WAIT_LIMIT, status)) break;
      issue_fp(k + WS_FP);
      fp_issued = k + WS_FP + 1;
    }
    // no box load in flight when the CTA's shared memory is given back
    for (int kf = fp_issued - WS_FP > 0 ? fp_issued - WS_FP : 0; kf < fp_issued; ++kf)
      (void)tc::mbar_wait_bounded(&sm.fp_full[kf % WS_FP], (uint32_t)(kf / WS_FP) & 1u, WAIT_LIMIT);
  } else if (warp == WS_WARP_MMA && lane == 0) {
    // ---- MMA issue -----------------------------------------------------------
    int mma_done = 0;
    const uint32_t idesc = tc::idesc_f16(0u, 128u, 64u);
    const uint32_t b_base = tc::smem_u32(sm.b);
    for (int k = 0; k < nloc; ++k) {
      const int s = k & 1;
      const uint32_t ph = (uint32_t)(k >> 1) & 1u;
      if (!ws_wait(sm, &sm.a_full[s], ph, WAIT_LIMIT, status)) break;
      if (k >= 2 && !ws_wait(sm, &sm.acc_empty[s], ph ^ 1u, WAIT_LIMIT, status)) break;
      tc::tc_fence_after();
      const uint32_t a_base = tc::smem_u32(sm.a[s]);
#pragma unroll
      for (int p = 0; p < PARTS; ++p)
#pragma unroll
        for (int kc = 0; kc < 4; ++kc) {
          const int c = p * 4 + kc;
          const uint64_t ad = tc::smem_desc(a_base + (uint32_t)(2 * c) * 128u, 128u, (uint32_t)A_SBO);
          const uint64_t bd = tc::smem_desc(b_base + (uint32_t)(2 * kc) * 128u, 128u, (uint32_t)B_SBO);
          tc::mma_f16(tmem + (uint32_t)(256 * s + 64 * p), ad, bd, idesc, kc > 0 ? 1u : 0u);
        }
      tc::mma_commit(&sm.a_empty[s]);    // A[s] may be rewritten
      tc::mma_commit(&sm.acc_full[s]);   // the accumulator is ready
      mma_done = k + 1;
    }
    // no MMA in flight when the accumulator columns are released (they
    // complete in order: the last one suffices)
    if (mma_done > 0) {
      const int kl = mma_done - 1;
      (void)tc::mbar_wait_bounded(&sm.acc_full[kl & 1], (uint32_t)(kl >> 1) & 1u, WAIT_LIMIT);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tmem, WS_TMEM_COLS);
}

static int num_sms() {
  return device_sms();
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  });
  return fn;
}

// Test hook: sets the poll limit of coef3_tc's MMA-completion wait on the
// current device (limit < 0 restores the default).
extern "C" int arb_test_set_mma_wait_limit(int64_t limit) {
  const uint32_t v = limit < 0 ? WAIT_LIMIT : (limit > (int64_t)WAIT_LIMIT ? WAIT_LIMIT : (uint32_t)limit);
  return cudaMemcpyToSymbol(g_mma_wait_limit, &v, sizeof(v)) == cudaSuccess ? ARB_OK : ARB_ERR_CUDA;
}

// Host launcher used by arb_coef_solve for 3D mixed precision.  The table is
// written as a 2D tensor [rows][64] float32 (rows = ncells x nfield) through
// 128-row x 32-float boxes in the 128-byte swizzled layout.
// Full solves through coef3_tma_kernel; returns ARB_ERR_UNSUPPORTED (nothing
// launched) where the grid misses the TMA rules, so the caller falls back.
template <int F>
static int coef3_solve_tma(const arb_grid *g, float *table, int32_t *status, cudaStream_t s, EncodeTiled encode) {
  using S = TmaShape<F>;
  const int64_t nx = g->n[0], ny = g->n[1], nz = g->n[2];
  if ((F == 4 && nx % 4 != 0) || (F == 1 && nx % 2 != 0)) return ARB_ERR_UNSUPPORTED;
  const int64_t rows = g->nc * F;
  if (rows >= ((int64_t)1 << 31) || nx > ((int64_t)1 << 30) || ny > ((int64_t)1 << 30) || nz > ((int64_t)1 << 30))
    return ARB_ERR_UNSUPPORTED;
  const int64_t ncx = nx - 3;
  const int64_t tpr = (ncx + S::C - 1) / S::C;
  const int rem = (int)(ncx - (tpr - 1) * S::C);
  const size_t smem = sizeof(WsSmem) + 1024;
  static std::once_flag once[MAX_DEVICES];
  static int per_sm_dev[MAX_DEVICES];
  static cudaError_t attr_err[MAX_DEVICES];
  const int dev = current_device();
  if (dev < 0) return ARB_ERR_CUDA;
  std::call_once(once[dev], [&] {
    attr_err[dev] = cudaFuncSetAttribute(coef3_tma_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr_err[dev] == cudaSuccess)
      attr_err[dev] = cudaFuncSetAttribute(coef3_tma_kernel<F>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    // one CTA per SM (its 512 TMEM columns are the whole SM's)
    per_sm_dev[dev] = 1;
  });
  if (attr_err[dev] != cudaSuccess) return ARB_ERR_CUDA;
  const cuuint32_t estr[3] = {1, 1, 1};
  CUtensorMap tm_full, tm_part, tm_hi, tm_lo;
  {  // table rows: full tiles and the last tile of each row
    const cuuint64_t dims[2] = {64, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {64 * sizeof(float)};
    const cuuint32_t box_f[2] = {32, (cuuint32_t)(S::C * F)}, box_p[2] = {32, (cuuint32_t)(rem * F)};
    if (encode(&tm_full, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, table, dims, strides, box_f, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS ||
        encode(&tm_part, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, table, dims, strides, box_p, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return ARB_ERR_CUDA;
  }
  {  // grid footprints
    float *g32 = const_cast<float *>(g->grid32);
    if (F == 1) {
      const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
      const cuuint64_t strides[2] = {(cuuint64_t)(8 * nx), (cuuint64_t)(8 * nx * ny)};
      const cuuint32_t box[3] = {(cuuint32_t)S::HX, 4, 4};
      if (encode(&tm_hi, CU_TENSOR_MAP_DATA_TYPE_INT64, 3, g32, dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return ARB_ERR_CUDA;
    } else {
      const cuuint64_t dims[3] = {(cuuint64_t)(4 * nx), (cuuint64_t)ny, (cuuint64_t)nz};
      const cuuint64_t strides[2] = {(cuuint64_t)(16 * nx), (cuuint64_t)(16 * nx * ny)};
      const cuuint32_t box[3] = {(cuuint32_t)(4 * S::HX), 4, 4};
      if (encode(&tm_hi, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, g32, dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return ARB_ERR_CUDA;
    }
    tm_lo = tm_hi;
    if (F == 4) {
      const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
      const cuuint64_t strides[2] = {(cuuint64_t)(4 * nx), (cuuint64_t)(4 * nx * ny)};
      const cuuint32_t box[3] = {(cuuint32_t)TmaShape<4>::LX, 4, 4};
      if (encode(&tm_lo, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, g32 + 4 * nx * ny * nz, dims, strides, box, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return ARB_ERR_CUDA;
    }
  }
  const int64_t tiles = tpr * (ny - 3) * (nz - 3);
  int64_t grid = (int64_t)num_sms() * per_sm_dev[dev];
  if (grid > tiles) grid = tiles;
  if (grid < 1) return ARB_OK;
  coef3_tma_kernel<F><<<(unsigned)grid, WS_THREADS, smem, s>>>(tm_full, tm_part, tm_hi, tm_lo, *g, status);
  return launch_status();
}

int coef3_solve_tc(const arb_grid *g, int64_t cell0, int64_t ncells, float *table, int32_t *status,
                   cudaStream_t s) {
  if (!g->grid32 || ((uintptr_t)table & 15u)) return ARB_ERR_INVALID;
  const EncodeTiled encode = encode_fn();
  if (!encode) return ARB_ERR_CUDA;
  if (cell0 == 0 && ncells == g->nc) {
    int rc = ARB_ERR_UNSUPPORTED;
    switch (g->nfield) {
      case 1: rc = coef3_solve_tma<1>(g, table, status, s, encode); break;
      case 3: rc = coef3_solve_tma<3>(g, table, status, s, encode); break;
      case 4: rc = coef3_solve_tma<4>(g, table, status, s, encode); break;
      default: break;
    }
    if (rc != ARB_ERR_UNSUPPORTED) return rc;
  }
  const size_t smem = sizeof(TcSmem) + 1024;
  static_assert(3 * (sizeof(TcSmem) + 1024 + 1024) > 228 * 1024, "a third CTA per SM would oversubscribe TMEM");
  static_assert(offsetof(TcSmem, stage) % 1024 == 0, "swizzled boxes need 1 KB alignment");
  // one-time setup per device (function attributes are per device)
  static std::once_flag once[MAX_DEVICES];
  static int per_sm_dev[MAX_DEVICES];
  static cudaError_t attr_err[MAX_DEVICES];
  const int dev = current_device();
  if (dev < 0) return ARB_ERR_CUDA;
  std::call_once(once[dev], [&] {
    attr_err[dev] = cudaSuccess;
    const void *ks[3] = {(const void *)coef3_tc_kernel<1>, (const void *)coef3_tc_kernel<3>,
                         (const void *)coef3_tc_kernel<4>};
    for (const void *k : ks) {
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      if (e != cudaSuccess) attr_err[dev] = e;
    }
    int smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    int n = (int)(smem_sm / (int64_t)(smem + 1024));
    per_sm_dev[dev] = n < 1 ? 1 : (n > 2 ? 2 : n);
  });
  if (attr_err[dev] != cudaSuccess) return ARB_ERR_CUDA;
  const int per_sm = per_sm_dev[dev];
  const int F = g->nfield;
  if (F != 1 && F != 3 && F != 4) return ARB_ERR_INVALID;
  // one tensor map covers at most 2^31 rows; larger solves go in chunks
  const int64_t max_cells = ((int64_t)1 << 31) / F;
  for (int64_t done = 0; done < ncells; done += max_cells) {
    const int64_t nc = ncells - done < max_cells ? ncells - done : max_cells;
    const int64_t rows = nc * F;
    CUtensorMap tmap;
    const cuuint64_t dims[2] = {64, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {64 * sizeof(float)};
    const cuuint32_t box[2] = {32, TM};
    const cuuint32_t estr[2] = {1, 1};
    if (encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, table + done * F * 64, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return ARB_ERR_CUDA;
    const int64_t tiles = (rows + TM - 1) / TM;
    int64_t grid = (int64_t)num_sms() * per_sm;
    if (grid > tiles) grid = tiles;
    switch (F) {
      case 1: coef3_tc_kernel<1><<<(unsigned)grid, NT, smem, s>>>(tmap, *g, cell0 + done, nc, status); break;
      case 3: coef3_tc_kernel<3><<<(unsigned)grid, NT, smem, s>>>(tmap, *g, cell0 + done, nc, status); break;
      default: coef3_tc_kernel<4><<<(unsigned)grid, NT, smem, s>>>(tmap, *g, cell0 + done, nc, status); break;
    }
    const int rc = launch_status();
    if (rc != ARB_OK) return rc;
  }
  return ARB_OK;
}


// ============================================================================
// 4D: the 256x256 product (calcCoefficients1/2/3 and allCoeffs of quadcubic,
// src/ARBInterp/ARBInterp.py:1260-1262, 1322-1355), rows = (cell, field),
// K = the 256 block samples, B = 16 A4 (integers, |.| <= 624, exact in FP16;
// row absolute sums <= 20740).  The same exact split with bounds for that
// matrix: t = 2^9 d / S = h0 + h1 + 2^-20 h2, h0 and h2 integers with
// |h| <= 512, h1 a multiple of 2^-10 with |h1| <= 1/2; then every part's
// 256-term sum stays below 2^24 of its own unit and accumulates exactly.
// Three parts x 256 monomials would need 768 TMEM columns (an SM has 512),
// so each 128-row tile runs the monomials in two halves of 128 (3 x 128
// columns) from an A tile kept whole in shared memory (128 rows x 768 FP16 =
// 192 KB); B arrives in 16 KB chunks (128 monomials x 64 samples, already in
// the core-matrix layout) by single bulk copies, double-buffered, and the two
// chunk buffers double as the 128-byte-swizzled staging of the output boxes
// (128 rows x 32 coefficients) drained by TMA tensor stores.  One CTA of 256
// threads per SM (shared memory and TMEM both allow one).
namespace {
constexpr int T4_M = 128, T4_NT = 256, T4_KP = 256, T4_KT = 768, T4_NH = 128, T4_KC = 64;
constexpr int T4_A_SBO = (T4_KT / 8) * 128;       // 12288
constexpr int T4_A_BYTES = (T4_M / 8) * T4_A_SBO;  // 196608
constexpr int T4_B_SBO = (T4_KC / 8) * 128;        // 1024
constexpr int T4_B_BYTES = (T4_NH / 8) * T4_B_SBO; // 16384
constexpr int T4_TMEM = 512;
constexpr float kRound10 = 12288.0f;                // 1.5 * 2^13: rounds to a multiple of 2^-10

struct Tc4Smem {
  unsigned char a[T4_A_BYTES];
  unsigned char b[2][T4_B_BYTES];
  float amax[2][T4_M];
  uint64_t mbar_b[2];
  uint64_t mbar_mma[2];
  uint32_t tmem_base;
  int32_t bad;
};

// Two values at once: t -> (h0, h1, h2) with t = h0 + h1 + 2^-20 h2, h2 an integer
__device__ __forceinline__ void split3_4d_pair(float2 t, float2 &h0, float2 &h1, float2 &h2) {
  const float2 R0 = make_float2(kRound0, kRound0), R10 = make_float2(kRound10, kRound10);
  h0 = fsub2(fadd2(t, R0), R0);
  const float2 r = fsub2(t, h0);
  h1 = fsub2(fadd2(r, R10), R10);
  h2 = fsub2(fadd2(fmul2(fsub2(r, h1), make_float2(1048576.0f, 1048576.0f)), R0), R0);
}

}  // namespace

// B = 16 A4 as FP16 in 8 chunks [half][K-chunk] of the no-swizzle K-major
// core-matrix layout (filled once per device from the host).
static __device__ __align__(256) unsigned short g_b4[8 * T4_B_BYTES / 2];

template <int F>
__global__ void __launch_bounds__(T4_NT, 1) coef4_tc_kernel(const __grid_constant__ CUtensorMap tmap, arb_grid g,
                                                            int64_t cell0, int64_t ncells, int32_t *status) {
  extern __shared__ unsigned char smem_raw[];
  Tc4Smem &sm = smem_aligned_1k<Tc4Smem>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & (T4_M - 1), half = tid >> 7;
  const int64_t rows = ncells * F;
  const int64_t npts = grid_points(g);
  const int64_t ntiles = (rows + T4_M - 1) / T4_M;
  const int64_t sy = g.n[0], sz = g.n[0] * g.n[1], st = g.n[0] * g.n[1] * g.n[2];
  constexpr int PW = F == 1 ? 2 : 4;
  const unsigned char *b4 = reinterpret_cast<const unsigned char *>(g_b4);

  if (warp == 0) {
    tc::tmem_alloc(&sm.tmem_base, T4_TMEM);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&sm.mbar_b[i], 1);
      tc::mbar_init(&sm.mbar_mma[i], 1);
    }
    sm.bad = 0;
    tc::fence_mbar_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  const uint32_t idesc = tc::idesc_f16(0u, 128u, 128u);
  const uint32_t a_base = tc::smem_u32(sm.a);
  const uint32_t t_lane = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  uint32_t pb[2] = {0u, 0u}, pm[2] = {0u, 0u};  // phases (meaningful in thread 0)

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t r = tile * T4_M + row;
    float rhi = 0.f, rlo = 0.f, amax = 0.f;
    const float *hb = nullptr, *lb = nullptr;
    bool has_lo = false;
    if (r < rows) {
      const int64_t cell = cell0 + r / F;
      const int f = F == 1 ? 0 : (int)(r % F);
      has_lo = F == 1 || (F == 4 && f == 3);
      int64_t c[4];
      cell_coords<4>(cell, g, c);
      const int64_t p0 = ((c[3] * g.n[2] + c[2]) * g.n[1] + c[1]) * g.n[0] + c[0];
      hb = g.grid32 + p0 * PW + f;
      lb = g.grid32 + npts * 4 + p0;
      const int64_t corner = st + sz + sy + 1;
      float vl = 0.f;
      g32_load<F>(g.grid32, npts, p0 + corner, f, rhi, vl);
      rlo = vl;
      // pass 1: the row's largest |delta| over this thread's 128 samples
#pragma unroll 1
      for (int ot = 0; ot < 2; ++ot)
#pragma unroll
        for (int oz = 0; oz < 4; ++oz)
#pragma unroll
          for (int oy = 0; oy < 4; ++oy) {
            const int64_t line = (2 * half + ot) * st + oz * sz + oy * sy;
#pragma unroll
            for (int ox = 0; ox < 4; ox += 2) {
              float2 vh, vl2 = make_float2(0.f, 0.f);
              if (F == 1) {
                const float2 v0 = __ldg(reinterpret_cast<const float2 *>(hb) + line + ox);
                const float2 v1 = __ldg(reinterpret_cast<const float2 *>(hb) + line + ox + 1);
                vh = make_float2(v0.x, v1.x);
                vl2 = make_float2(v0.y, v1.y);
              } else {
                vh = make_float2(__ldg(hb + (line + ox) * 4), __ldg(hb + (line + ox + 1) * 4));
                if (has_lo) vl2 = make_float2(__ldg(lb + line + ox), __ldg(lb + line + ox + 1));
              }
              const float2 dd = fadd2(fsub2(vh, make_float2(rhi, rhi)), fsub2(vl2, make_float2(rlo, rlo)));
              amax = fmaxf(amax, fmaxf(fabsf(dd.x), fabsf(dd.y)));
            }
          }
    }
    sm.amax[half][row] = amax;
    __syncthreads();
    const int E = scale_exp(fmaxf(amax, sm.amax[half ^ 1][row]));
    const float c9 = __uint_as_float((uint32_t)(127 + 9 - E) << 23);  // 2^(9 - E)
    // pass 2: split into the A tile (8 consecutive samples = two x-lines per store)
#pragma unroll 1
    for (int ot = 0; ot < 2; ++ot)
#pragma unroll
      for (int oz = 0; oz < 4; ++oz)
#pragma unroll
        for (int oy = 0; oy < 4; oy += 2) {
          float d[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) d[u] = 0.f;
          if (r < rows) {
#pragma unroll
            for (int l2 = 0; l2 < 2; ++l2) {
              const int64_t line = (2 * half + ot) * st + oz * sz + (oy + l2) * sy;
#pragma unroll
              for (int ox = 0; ox < 4; ox += 2) {
                float2 vh, vl2 = make_float2(0.f, 0.f);
                if (F == 1) {
                  const float2 v0 = __ldg(reinterpret_cast<const float2 *>(hb) + line + ox);
                  const float2 v1 = __ldg(reinterpret_cast<const float2 *>(hb) + line + ox + 1);
                  vh = make_float2(v0.x, v1.x);
                  vl2 = make_float2(v0.y, v1.y);
                } else {
                  vh = make_float2(__ldg(hb + (line + ox) * 4), __ldg(hb + (line + ox + 1) * 4));
                  if (has_lo) vl2 = make_float2(__ldg(lb + line + ox), __ldg(lb + line + ox + 1));
                }
                const float2 dd = fadd2(fsub2(vh, make_float2(rhi, rhi)), fsub2(vl2, make_float2(rlo, rlo)));
                d[l2 * 4 + ox] = dd.x;
                d[l2 * 4 + ox + 1] = dd.y;
              }
            }
          }
          uint32_t w0[4], w1[4], w2[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            float2 h0, h1, h2;
            split3_4d_pair(fmul2(make_float2(d[2 * v], d[2 * v + 1]), make_float2(c9, c9)), h0, h1, h2);
            w0[v] = pack_h2(h0.x, h0.y);
            w1[v] = pack_h2(h1.x, h1.y);
            w2[v] = pack_h2(h2.x, h2.y);
          }
          const int k = half * 128 + ot * 64 + oz * 16 + oy * 4;  // sample index ox + 4oy + 16oz + 64ot
          *reinterpret_cast<uint4 *>(sm.a + kmaj(row, k, T4_A_SBO)) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
          *reinterpret_cast<uint4 *>(sm.a + kmaj(row, T4_KP + k, T4_A_SBO)) =
              make_uint4(w1[0], w1[1], w1[2], w1[3]);
          *reinterpret_cast<uint4 *>(sm.a + kmaj(row, 2 * T4_KP + k, T4_A_SBO)) =
              make_uint4(w2[0], w2[1], w2[2], w2[3]);
        }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    if (tid == 0) tc::bulk_wait_read0();  // staging boxes of the previous tile have been read
    __syncthreads();
    const float so = __uint_as_float((uint32_t)(E - 13 + 127) << 23);  // 2^(E - 13)

    for (int nh = 0; nh < 2; ++nh) {
      // ---- MMAs for monomials [128 nh, 128 nh + 128): 4 K-chunks x 3 parts x 4 ----
      if (tid == 0) {
        tc::tc_fence_after();
        bool ok = true;
        for (int i = 0; i < 2; ++i) {
          tc::mbar_arrive_expect_tx(&sm.mbar_b[i], T4_B_BYTES);
          tc::bulk_load(sm.b[i], b4 + (size_t)(nh * 4 + i) * T4_B_BYTES, T4_B_BYTES, &sm.mbar_b[i]);
        }
        for (int kc = 0; kc < 4 && ok; ++kc) {
          const int buf = kc & 1;
          ok = tc::mbar_wait_bounded(&sm.mbar_b[buf], pb[buf], WAIT_LIMIT);
          pb[buf] ^= 1u;
          if (!ok) break;
          const uint32_t b_base = tc::smem_u32(sm.b[buf]);
#pragma unroll
          for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const uint32_t ka = (uint32_t)(p * T4_KP + kc * T4_KC + ks * 16);
              const uint64_t ad = tc::smem_desc(a_base + (ka / 8) * 128u, 128u, (uint32_t)T4_A_SBO);
              const uint64_t bd = tc::smem_desc(b_base + (uint32_t)ks * 256u, 128u, (uint32_t)T4_B_SBO);
              tc::mma_f16(tmem + (uint32_t)(p * T4_NH), ad, bd, idesc, (kc | ks) ? 1u : 0u);
            }
          tc::mma_commit(&sm.mbar_mma[buf]);
          if (kc >= 1 && kc + 1 < 4) {
            // the previous chunk's MMAs release its buffer for chunk kc + 1
            const int pbuf = buf ^ 1;
            ok = tc::mbar_wait_bounded(&sm.mbar_mma[pbuf], pm[pbuf], WAIT_LIMIT);
            pm[pbuf] ^= 1u;
            if (ok) {
              tc::mbar_arrive_expect_tx(&sm.mbar_b[pbuf], T4_B_BYTES);
              tc::bulk_load(sm.b[pbuf], b4 + (size_t)(nh * 4 + kc + 1) * T4_B_BYTES, T4_B_BYTES, &sm.mbar_b[pbuf]);
            }
          }
        }
        // chunks 2 and 3 (buffers 0 and 1) are the last commits outstanding
        for (int i = 0; i < 2 && ok; ++i) {
          ok = tc::mbar_wait_bounded(&sm.mbar_mma[i], pm[i], WAIT_LIMIT);
          pm[i] ^= 1u;
        }
        if (!ok) {
          set_status(status, ARB_ERR_TIMEOUT);
          sm.bad = 1;
        }
      }
      tc::tc_fence_before();
      __syncthreads();
      tc::tc_fence_after();
      if (sm.bad) break;
      // ---- epilogue: thread (row, q) combines monomials 64 q .. 64 q + 63 of this half ----
      const int q = half;
#pragma unroll 1
      for (int sub = 0; sub < 2; ++sub) {
        const uint32_t col = (uint32_t)(q * 64 + sub * 32);
        float a[32], t[32];
        tc::tmem_ld16(t_lane + 2u * T4_NH + col, t);
        tc::tmem_ld16(t_lane + 2u * T4_NH + col + 16u, t + 16);
        tc::tmem_ld16(t_lane + T4_NH + col, a);
        tc::tmem_ld16(t_lane + T4_NH + col + 16u, a + 16);
        tc::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 32; ++j) t[j] = __fmaf_rn(t[j], 0x1p-20f, a[j]);
        tc::tmem_ld16(t_lane + col, a);
        tc::tmem_ld16(t_lane + col + 16u, a + 16);
        tc::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 32; ++j) a[j] = __fmul_rn(__fadd_rn(a[j], t[j]), so);
        if (nh == 0 && q == 0 && sub == 0) a[0] = rhi + (rlo + a[0]);
        if (tid == 0) tc::bulk_wait_read0();  // the staging box is free again
        __syncthreads();
        unsigned char *st_row = sm.b[q] + row * 128;
#pragma unroll
        for (int c = 0; c < 8; ++c)
          *reinterpret_cast<float4 *>(st_row + 16 * (c ^ (row & 7))) =
              make_float4(a[4 * c], a[4 * c + 1], a[4 * c + 2], a[4 * c + 3]);
        tc::fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
          tc::tma_store_2d(&tmap, sm.b[0], nh * 128 + 0 * 64 + sub * 32, (int32_t)(tile * T4_M));
          tc::tma_store_2d(&tmap, sm.b[1], nh * 128 + 1 * 64 + sub * 32, (int32_t)(tile * T4_M));
          tc::bulk_commit();
        }
      }
      // the next half's chunk copies land in the staging buffers: wait for the reads
      tc::tc_fence_before();
      if (tid == 0) tc::bulk_wait_read0();
      __syncthreads();
    }
    if (sm.bad) break;
  }
  if (tid == 0) {
    tc::bulk_wait0();
    if (sm.bad) {
      // after a timed-out wait: one more bounded wait for work still in flight
      for (int i = 0; i < 2; ++i) {
        (void)tc::mbar_wait_bounded(&sm.mbar_mma[i], pm[i], WAIT_LIMIT);
        (void)tc::mbar_wait_bounded(&sm.mbar_b[i], pb[i], WAIT_LIMIT);
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tmem, T4_TMEM);
}

// 16 A4 (the reference's 4D A scaled by 16: integers) in the chunked FP16 layout.
static void build_b4_host(std::vector<__half> &out) {
  static const double A1h[4][4] = {{0, 1, 0, 0}, {-0.5, 0, 0.5, 0}, {1, -2.5, 2, -0.5}, {-0.5, 1.5, -1.5, 0.5}};
  static const double HB[2][4] = {{0, 1, -2, 1}, {0, 0, -1, 1}};  // t - 2t^2 + t^3, -t^2 + t^3
  auto h_c = [&](int c, int n) {  // slope-Hermite tensor coefficient of monomial n for corner c (h_16 = 0)
    if (c >= 16) return 0.0;
    double v = 1.0;
    for (int a = 0; a < 4; ++a) v *= HB[(c >> a) & 1][(n >> (2 * a)) & 3];
    return v;
  };
  auto s_c = [&](int c, int k) {  // mixed fourth-difference stencil of corner c at block sample k
    double v = 1.0;
    for (int a = 0; a < 4; ++a) {
      const int b = (c >> a) & 1, o = (k >> (2 * a)) & 3;
      v *= o == b ? -0.5 : (o == b + 2 ? 0.5 : 0.0);
    }
    return v;
  };
  out.assign(8 * T4_B_BYTES / 2, __float2half(0.f));
  for (int n = 0; n < 256; ++n)
    for (int k = 0; k < 256; ++k) {
      double v = 1.0;
      for (int a = 0; a < 4; ++a) v *= A1h[(n >> (2 * a)) & 3][(k >> (2 * a)) & 3];
      for (int c = 0; c < 16; ++c) v += (h_c(c + 1, n) - h_c(c, n)) * s_c(c, k);
      const int nh = n >> 7, nl = n & 127, kc = k >> 6, kl = k & 63;
      const size_t off = (size_t)(nh * 4 + kc) * T4_B_BYTES + kmaj(nl, kl, T4_B_SBO);
      out[off / 2] = __float2half((float)(16.0 * v));
    }
}

int coef4_solve_tc(const arb_grid *g, int64_t cell0, int64_t ncells, float *table, int32_t *status,
                   cudaStream_t s) {
  if (!g->grid32 || ((uintptr_t)table & 15u)) return ARB_ERR_INVALID;
  const EncodeTiled encode = encode_fn();
  if (!encode) return ARB_ERR_CUDA;
  const size_t smem = sizeof(Tc4Smem) + 1024;
  static_assert(sizeof(Tc4Smem) + 1024 <= 232448, "shared memory above the per-CTA limit");
  static std::mutex mu;
  static bool filled[MAX_DEVICES] = {};
  static bool attr[MAX_DEVICES] = {};
  const int dev = current_device();
  if (dev < 0) return ARB_ERR_CUDA;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!filled[dev]) {
      std::vector<__half> host;
      build_b4_host(host);
      if (cudaMemcpyToSymbol(g_b4, host.data(), host.size() * sizeof(__half)) != cudaSuccess) return ARB_ERR_CUDA;
      filled[dev] = true;
    }
    if (!attr[dev]) {
      const void *ks[3] = {(const void *)coef4_tc_kernel<1>, (const void *)coef4_tc_kernel<3>,
                           (const void *)coef4_tc_kernel<4>};
      for (const void *k : ks)
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
          return ARB_ERR_CUDA;
      attr[dev] = true;
    }
  }
  const int F = g->nfield;
  if (F != 1 && F != 3 && F != 4) return ARB_ERR_INVALID;
  const int64_t max_cells = ((int64_t)1 << 31) / F;
  for (int64_t done = 0; done < ncells; done += max_cells) {
    const int64_t nc = ncells - done < max_cells ? ncells - done : max_cells;
    const int64_t rows = nc * F;
    CUtensorMap tmap;
    const cuuint64_t dims[2] = {256, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {256 * sizeof(float)};
    const cuuint32_t box[2] = {32, T4_M};
    const cuuint32_t estr[2] = {1, 1};
    if (encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, table + done * F * 256, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return ARB_ERR_CUDA;
    const int64_t tiles = (rows + T4_M - 1) / T4_M;
    int64_t grid = num_sms();
    if (grid > tiles) grid = tiles;
    switch (F) {
      case 1: coef4_tc_kernel<1><<<(unsigned)grid, T4_NT, smem, s>>>(tmap, *g, cell0 + done, nc, status); break;
      case 3: coef4_tc_kernel<3><<<(unsigned)grid, T4_NT, smem, s>>>(tmap, *g, cell0 + done, nc, status); break;
      default: coef4_tc_kernel<4><<<(unsigned)grid, T4_NT, smem, s>>>(tmap, *g, cell0 + done, nc, status); break;
    }
    const int rc = launch_status();
    if (rc != ARB_OK) return rc;
  }
  return ARB_OK;
}

}  // namespace arb
