// Cell-grouped query evaluation.
//
// Random query order makes every query's 4^dim grid block (or coefficient
// row) a cold gather from a field far larger than L2.  Here the queries are
// first grouped by spatial bin (8^3 cells in 3D, 4^4 in 4D) with a counting
// sort, then evaluated bin by bin, so neighbouring threads share grid data in
// L1/L2 and each grid point is fetched from HBM about once.
//
//   count    : cell index + fractional offset (exactly the reference's
//              iu = (q - IntMin)/h, floor, flat index), the out-of-volume
//              bookkeeping of rQuery (NaN rows, queryInds) and the bin
//              histogram (fire-and-forget atomics)
//   scan     : exclusive prefix sum of the bin histogram
//   place    : the same coordinate step again, a slot in the query's bin
//              (atomic on the running offset) and one 32-byte record
//              (packed cell, row, fraction) written there; afterwards
//              hist[b] is the end of bin b
//   evaluate : on-the-fly or table evaluation in bin order, outputs written
//              to the query's original row
// Recomputing the coordinate step (float32 pipe in mixed precision) is
// cheaper than storing it: the unsorted intermediates and a separate scatter
// pass cost three partial-sector writes per query, the record one full one.
// The evaluation pass does no float64 arithmetic and no integer division in
// mixed precision.
#include <cuda.h>

#include <mutex>

#include "eval.cuh"

namespace arb {

// Bin-ordered query record: packed cell (or CELL_SPECIAL | code), the
// query's row and its fractional offsets (float32 in mixed precision: 32
// bytes, one sector; float64: 48 bytes).
template <typename T>
struct QRec;
template <>
struct __align__(32) QRec<float> {
  unsigned long long cell;
  uint32_t row;
  float f[4];
  uint32_t pad;
};
template <>
struct __align__(16) QRec<double> {
  unsigned long long cell;
  uint32_t row;
  uint32_t pad;
  double f[4];
};
static_assert(sizeof(QRec<float>) == 32 && sizeof(QRec<double>) == 48, "record sizes");

struct SortedWork {
  uint32_t *hist;  // nbins + 1: counts, exclusive offsets after the scan, bin ends after placement
  void *rec;       // nq records (QRec<float> or QRec<double>), bin order
};

struct BinGeom {
  int64_t nb[4];     // bins per axis
  int64_t nbins;     // product (the special bin is index nbins)
  int shift;         // log2 cells per bin edge
};

static inline BinGeom bin_geom(const arb_grid *g) {
  BinGeom b;
  b.shift = (g->bin_shift > 0 && g->bin_shift <= 8) ? g->bin_shift : (g->dim == 3 ? 3 : 2);
  b.nbins = 1;
  for (int a = 0; a < 4; ++a) {
    if (a < g->dim) {
      const int64_t cells = g->n[a] - 3;
      b.nb[a] = (cells + (1 << b.shift) - 1) >> b.shift;
    } else {
      b.nb[a] = 1;
    }
    b.nbins *= b.nb[a];
  }
  return b;
}

static inline size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

static size_t carve(SortedWork *w, void *base, const arb_grid *g, int precision, int64_t nq) {
  const BinGeom bg = bin_geom(g);
  const size_t tsz = precision == ARB_PREC_MIXED ? 4 : 8;
  size_t off = 0;
  char *p = (char *)base;
  auto take = [&](size_t bytes) {
    void *r = p ? (void *)(p + off) : nullptr;
    off += align_up(bytes);
    return r;
  };
  SortedWork t;
  t.hist = (uint32_t *)take(sizeof(uint32_t) * (bg.nbins + 1));
  t.rec = take((tsz == 4 ? sizeof(QRec<float>) : sizeof(QRec<double>)) * nq);
  if (w) *w = t;
  return off;
}

// Coordinate step of query row i: cell index, fraction, packed cell word
// and bin (the special bin nbins for rows that need no evaluation).
template <int DIM, bool EXACT, typename T>
__device__ __forceinline__ CoordStep bin_step(const arb_grid &g, const KParams &kp, const BinGeom &bg,
                                              const double *qr, T frac[DIM], unsigned long long &cw, int64_t &bin,
                                              bool &bad_index) {
  double qv[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) qv[a] = qr[a];
  CoordStep s;
  if constexpr (EXACT)
    s = coord_step<DIM, true>(qv, g, kp.inv_h, frac);
  else
    s = coord_step_fast<DIM>(qv, kp.ax, g, frac);
  bin = bg.nbins;
  bad_index = false;
  if (s.oob || s.nan) {
    cw = CELL_SPECIAL;
  } else if (s.idx > g.nc) {
    bad_index = true;
    cw = CELL_SPECIAL;
  } else if (s.idx == g.nc) {
    cw = CELL_SPECIAL | 1ULL;
  } else {
    int64_t c[DIM];
    cell_from_step<DIM>(s, g, c);
    cw = pack_cell<DIM>(c);
    bin = c[DIM - 1] >> bg.shift;
#pragma unroll
    for (int a = DIM - 2; a >= 0; --a) bin = bin * bg.nb[a] + (c[a] >> bg.shift);
  }
  return s;
}

template <int DIM, bool EXACT, typename T>
__global__ void __launch_bounds__(256) bin_count_kernel(arb_grid g, KParams kp, BinGeom bg, double *q, int64_t nq,
                                                        int64_t qs, int wb, arb_query_out o, int32_t *status,
                                                        SortedWork w) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  double *qr = q + i * qs;
  T frac[DIM];
  unsigned long long cw;
  int64_t bin;
  bool bad;
  const CoordStep s = bin_step<DIM, EXACT, T>(g, kp, bg, qr, frac, cw, bin, bad);
  append_oob(o, i, s.oob);
  if (o.inds) o.inds[i] = s.idx;
  if (bad) set_status(status, ARB_ERR_CELL_INDEX);
  atomicAdd(&w.hist[bin], 1u);
  // the caller's out-of-volume rows become NaN (the place pass reads them
  // back as NaN rows: the same special bin)
  if (s.oob && wb)
    for (int64_t c = 0; c < qs; ++c) qr[c] = qnan();
}

template <int DIM, bool EXACT, typename T>
__global__ void __launch_bounds__(256) bin_place_kernel(arb_grid g, KParams kp, BinGeom bg, const double *q,
                                                        int64_t nq, int64_t qs, SortedWork w) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  T frac[DIM];
  unsigned long long cw;
  int64_t bin;
  bool bad;
  (void)bin_step<DIM, EXACT, T>(g, kp, bg, q + i * qs, frac, cw, bin, bad);
  const uint32_t pos = atomicAdd(&w.hist[bin], 1u);
  QRec<T> r;
  r.cell = cw;
  r.row = (uint32_t)i;
#pragma unroll
  for (int a = 0; a < 4; ++a) r.f[a] = a < DIM ? frac[a] : T(0);
  r.pad = 0;
  if constexpr (sizeof(T) == 4) {
    // one 32-byte store: a whole sector, no partial-sector merge in L2
    const uint32_t *u = reinterpret_cast<const uint32_t *>(&r);
    asm volatile("st.global.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(reinterpret_cast<QRec<T> *>(w.rec) + pos),
                 "r"(u[0]), "r"(u[1]), "r"(u[2]), "r"(u[3]), "r"(u[4]), "r"(u[5]), "r"(u[6]), "r"(u[7])
                 : "memory");
  } else {
    reinterpret_cast<QRec<T> *>(w.rec)[pos] = r;
  }
}

// Exclusive scan of n counters in one block (n up to a few million).
__global__ void __launch_bounds__(1024) scan_kernel(uint32_t *hist, int64_t n) {
  __shared__ uint32_t part[1024];
  const int64_t per = (n + blockDim.x - 1) / blockDim.x;
  const int64_t b = threadIdx.x * per, e = min(b + per, n);
  uint32_t sum = 0;
  for (int64_t k = b; k < e; ++k) sum += hist[k];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const uint32_t v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = part[threadIdx.x] - sum;
  for (int64_t k = b; k < e; ++k) {
    const uint32_t c = hist[k];
    hist[k] = run;
    run += c;
  }
}

template <int DIM, int F, bool MIXED, bool TABLE>
__global__ void __launch_bounds__(DIM == 3 ? 256 : 128) eval_sorted_kernel(arb_grid g, KParams kp,
                                                                           int64_t nq, arb_query_out o,
                                                                           SortedWork w) {
  using T = typename std::conditional<MIXED, float, double>::type;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nq) return;
  const QRec<T> r = reinterpret_cast<const QRec<T> *>(w.rec)[t];
  const unsigned long long cw = r.cell;
  const int64_t i = r.row;
  if (cw & CELL_SPECIAL) {
    write_const<DIM, F>(o, i, (cw & 1ULL) && !g.sentinel_nan ? 0.0 : qnan());
    return;
  }
  int64_t c[DIM];
  unpack_cell<DIM>(cw, c);
  T fr[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) fr[a] = r.f[a];
  double val[F], grad[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) grad[a] = 0.0;
  if constexpr (TABLE) {
    eval_tab<DIM, F, MIXED>(g, kp, c, fr, val, grad);
  } else if constexpr (DIM == 3) {
    eval_otf3<F, MIXED>(g, kp, c, fr, val, grad);
  } else {
    eval_otf4<F, MIXED>(g, kp, c, fr, val, grad);
  }
  write_vals<DIM, F>(o, i, val, grad);
}

// 3D, four fields ('both' mode), mixed precision: 4 lanes per query, lane
// s owning grid point s of every x-row.  A row is 4 points x float4
// (hi_x, hi_y, hi_z, hi_n) = 64 bytes plus 4 x float lo_n, so the 4 lanes of
// a query read it with one 16-byte and one 4-byte load each.  Each lane
// contracts its 16 rows over y and z (components from their float32 values
// as deltas to the cell corner; |B| from (hi, lo) deltas so its gradient keeps
// full precision), then the 4 lanes reduce over x with two butterfly
// shuffles.  Each block walks COOP_CHUNK consecutive sorted queries (about
// one spatial bin) so the bin's grid footprint stays in that SM's L1.
constexpr int COOP_CHUNK = 256;

__global__ void __launch_bounds__(256) eval_sorted_coop4_kernel(arb_grid g, KParams kp, int64_t nq,
                                                                arb_query_out o, SortedWork w) {
  const int lane = threadIdx.x & 31;
  const int p = lane & 3;
  const int64_t t0 = (int64_t)blockIdx.x * COOP_CHUNK;
  const int64_t t1 = min(t0 + COOP_CHUNK, nq);
  const int64_t nx = g.n[0], ny = g.n[1];
  const int64_t npts = grid_points(g);
  const float4 *g4 = reinterpret_cast<const float4 *>(g.grid32);
  const float *glo = g.grid32 + npts * 4;
  const unsigned mask = 0xfu << (lane & 28);
  for (int64_t t = t0 + (threadIdx.x >> 2); t < t1; t += blockDim.x >> 2) {  // groups stay converged
    const QRec<float> r = reinterpret_cast<const QRec<float> *>(w.rec)[t];
    const unsigned long long cw = r.cell;
    const int64_t i = r.row;
    if (cw & CELL_SPECIAL) {
      if (p == 0) write_const<3, 4>(o, i, (cw & 1ULL) && !g.sentinel_nan ? 0.0 : qnan());
      continue;
    }
    int64_t c[3];
    unpack_cell<3>(cw, c);
    const float fx = r.f[0], fy = r.f[1], fz = r.f[2];
    float wx[4], dx[4], wy[4], dy[4], wz[4], dz[4];
    cr_weights<float>(fx, wx);
    cr_dweights<float>(fx, dx);
    cr_weights<float>(fy, wy);
    cr_dweights<float>(fy, dy);
    cr_weights<float>(fz, wz);
    cr_dweights<float>(fz, dz);
    const int64_t pref = ((c[2] + 1) * ny + (c[1] + 1)) * nx + (c[0] + 1);
    const float4 ref = __ldg(g4 + pref);
    const float rlo = __ldg(glo + pref);
    float Sx = 0.f, Sy_ = 0.f, Sz_ = 0.f, Sn = 0.f, Gy = 0.f, Gz = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t pt = ((c[2] + k) * ny + (c[1] + j)) * nx + c[0] + p;
        const float4 v = __ldg(g4 + pt);
        const float lo = __ldg(glo + pt);
        const float dn = (v.w - ref.w) + (lo - rlo);
        const float wyz = wy[j] * wz[k];
        Sx += wyz * (v.x - ref.x);
        Sy_ += wyz * (v.y - ref.y);
        Sz_ += wyz * (v.z - ref.z);
        Sn += wyz * dn;
        Gy += (dy[j] * wz[k]) * dn;
        Gz += (wy[j] * dz[k]) * dn;
      }
    }
    float Vx = wx[p] * Sx, Vy = wx[p] * Sy_, Vz = wx[p] * Sz_, Vn = wx[p] * Sn;
    float Gx = dx[p] * Sn;
    Gy *= wx[p];
    Gz *= wx[p];
#pragma unroll
    for (int off = 1; off <= 2; off <<= 1) {
      Vx += __shfl_xor_sync(mask, Vx, off);
      Vy += __shfl_xor_sync(mask, Vy, off);
      Vz += __shfl_xor_sync(mask, Vz, off);
      Vn += __shfl_xor_sync(mask, Vn, off);
      Gx += __shfl_xor_sync(mask, Gx, off);
      Gy += __shfl_xor_sync(mask, Gy, off);
      Gz += __shfl_xor_sync(mask, Gz, off);
    }
    const double nv = f2d_exact(ref.w + (rlo + Vn));
    if (interleaved_rows<3, 4>(o)) {
      if (p == 0)
        st_v4(o.comps + i * 8, f2d_exact(ref.x + Vx), f2d_exact(ref.y + Vy), f2d_exact(ref.z + Vz), nv);
      else if (p == 2)
        st_v4(o.comps + i * 8 + 4, f2d_exact(Gx * kp.inv_hf[0]), f2d_exact(Gy * kp.inv_hf[1]),
              f2d_exact(Gz * kp.inv_hf[2]), 0.0);
    } else if (p == 0) {
      if (o.comps) {
        o.comps[i * o.comps_stride + 0] = f2d_exact(ref.x + Vx);
        o.comps[i * o.comps_stride + 1] = f2d_exact(ref.y + Vy);
        o.comps[i * o.comps_stride + 2] = f2d_exact(ref.z + Vz);
      }
    } else if (p == 1) {
      if (o.norms) o.norms[i * o.norms_stride] = nv;
    } else if (p == 2) {
      if (o.grads) {
        o.grads[i * o.grads_stride + 0] = f2d_exact(Gx * kp.inv_hf[0]);
        o.grads[i * o.grads_stride + 1] = f2d_exact(Gy * kp.inv_hf[1]);
        o.grads[i * o.grads_stride + 2] = f2d_exact(Gz * kp.inv_hf[2]);
      }
    }
  }
}

// ---- bin-staged evaluation (3D, mixed, 8^3-cell bins) -------------------------
// One CTA per bin (round-robin over bins): the bin's footprint of 11^3 grid
// points (8 cells + 3 per axis) is copied into shared memory with cp.async,
// double-buffered so the next bin's copy overlaps this bin's queries, and
// every query of the bin gathers its 4x4x4 block from shared memory.  Reading
// the block from L1 instead costs ~3 L1 wavefronts per (query, x-row) because
// the 8 queries of a warp touch 16 scattered 64-byte and 16-byte segments;
// from shared memory it is about one.
constexpr int BIN_EDGE = 8;
constexpr int TILE_EDGE = BIN_EDGE + 3;
constexpr int TILE_PTS = TILE_EDGE * TILE_EDGE * TILE_EDGE;

template <int F>
struct BinTile;
// hi planes are 124 points apart (121 used): 124 * 16 B = 1984 B is 64 B
// modulo the 128-byte bank cycle, so a query's x-rows in planes k and k+1
// (read by one 8-thread phase of a 128-bit load) fall on complementary banks.
constexpr int HI_PLANE = 124;
constexpr int HI_PTS = TILE_EDGE * HI_PLANE;
template <>
struct BinTile<4> {          // (hi_x, hi_y, hi_z, hi_n) and lo_n per point
  float4 hi[HI_PTS];         // [z][HI_PLANE] with rows of TILE_EDGE points
  float lo[TILE_PTS];        // [z][y][x], unpadded
};
template <>
struct BinTile<1> {          // (hi, lo) per point
  float2 v[TILE_PTS];
};
template <>
struct BinTile<3> {          // (hi_x, hi_y, hi_z, 0) per point
  float4 v[TILE_PTS];
};

__device__ __forceinline__ void cp_async16(void *sdst, const void *gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void *sdst, const void *gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void *sdst, const void *gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// grid-point origin of bin b (x fastest)
__device__ __forceinline__ void bin_origin(int64_t b, const BinGeom &bg, int64_t o[3]) {
  o[0] = (b % bg.nb[0]) * BIN_EDGE;
  const int64_t r = b / bg.nb[0];
  o[1] = (r % bg.nb[1]) * BIN_EDGE;
  o[2] = (r / bg.nb[1]) * BIN_EDGE;
}

// Copy bin b's footprint into `t` (points outside the grid are skipped: no
// cell of the bin reads them).
template <int F>
__device__ __forceinline__ void load_bin_tile(const arb_grid &g, const BinGeom &bg, int64_t b, BinTile<F> &t) {
  int64_t o[3];
  bin_origin(b, bg, o);
  const int64_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const int64_t npts = nx * ny * nz;
  for (int e = threadIdx.x; e < TILE_PTS; e += blockDim.x) {
    const int lx = e % TILE_EDGE, r = e / TILE_EDGE;
    const int ly = r % TILE_EDGE, lz = r / TILE_EDGE;
    const int64_t x = o[0] + lx, y = o[1] + ly, z = o[2] + lz;
    if (x >= nx || y >= ny || z >= nz) continue;
    const int64_t p = (z * ny + y) * nx + x;
    if (F == 4) {
      cp_async16(&reinterpret_cast<BinTile<4> &>(t).hi[lz * HI_PLANE + ly * TILE_EDGE + lx],
                 reinterpret_cast<const float4 *>(g.grid32) + p);
      cp_async4(&reinterpret_cast<BinTile<4> &>(t).lo[e], g.grid32 + npts * 4 + p);
    } else if (F == 3) {
      cp_async16(&reinterpret_cast<BinTile<3> &>(t).v[e], reinterpret_cast<const float4 *>(g.grid32) + p);
    } else {
      cp_async8(&reinterpret_cast<BinTile<1> &>(t).v[e], reinterpret_cast<const float2 *>(g.grid32) + p);
    }
  }
}

// Packed float32 FMA on (x, y) pairs: d = a * b + c per component.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

template <int F>
__global__ void __launch_bounds__(256, 4) eval_bin_kernel(arb_grid g, KParams kp, BinGeom bg, int64_t nq,
                                                       arb_query_out o, SortedWork w) {
  extern __shared__ __align__(16) unsigned char bin_smem[];
  BinTile<F> *tiles = reinterpret_cast<BinTile<F> *>(bin_smem);
  const int lane = threadIdx.x & 31;
  const int g8 = lane & 7;        // lane within the query's group; also the output column it writes
  const int p = lane & 3;         // x offset in the 4x4x4 block
  const int h = g8 >> 2;          // z parity: this lane reads planes h and h + 2
  const unsigned mask = 0xffu << (lane & 24);
  const int64_t nbins = bg.nbins;
  int stage = 0;
  int64_t b = blockIdx.x;
  // after placement hist[b] is the end of bin b; bins with no query need no copy
  auto bin_begin = [&](int64_t bb) { return bb > 0 ? (int64_t)w.hist[bb - 1] : (int64_t)0; };
  auto count = [&](int64_t bb) { return bb < nbins ? (int64_t)w.hist[bb] - bin_begin(bb) : 0; };
  if (count(b) > 0) load_bin_tile<F>(g, bg, b, tiles[0]);
  cp_async_commit();
  for (; b < nbins; b += gridDim.x) {
    const int64_t bn = b + gridDim.x;
    if (count(bn) > 0) load_bin_tile<F>(g, bg, bn, tiles[stage ^ 1]);
    cp_async_commit();
    const int64_t t0 = bin_begin(b), t1 = w.hist[b];
    cp_async_wait1();
    __syncthreads();
    if (t1 > t0) {
      const BinTile<F> &T = tiles[stage];
      int64_t og[3];
      bin_origin(b, bg, og);
      if (F == 4) {
        // 8 lanes per query: lane (p, h) owns x offset p of the rows in
        // planes h and h + 2, so each 8-thread phase of a 128-bit shared load
        // reads one query's two x-rows on complementary banks.  The next
        // record is loaded while this one is evaluated.
        const QRec<float> *recs = reinterpret_cast<const QRec<float> *>(w.rec);
        const int64_t tstep = blockDim.x >> 3;
        int64_t t = t0 + (threadIdx.x >> 3);
        QRec<float> rnext;
        if (t < t1) rnext = recs[t];
        for (; t < t1; t += tstep) {
          const QRec<float> r = rnext;
          if (t + tstep < t1) rnext = recs[t + tstep];
          const int64_t i = r.row;
          int64_t c[3];
          unpack_cell<3>(r.cell, c);
          const int cx = (int)(c[0] - og[0]), cy = (int)(c[1] - og[1]), cz = (int)(c[2] - og[2]);
          const int lph = cz * HI_PLANE + cy * TILE_EDGE + cx;     // block corner in hi
          const int lpl = (cz * TILE_EDGE + cy) * TILE_EDGE + cx;  // block corner in lo
          const float fx = r.f[0], fy = r.f[1], fz = r.f[2];
          float wx[4], dx[4], wy[4], dy[4], wz[4], dz[4];
          cr_weights<float>(fx, wx);
          cr_dweights<float>(fx, dx);
          cr_weights<float>(fy, wy);
          cr_dweights<float>(fy, dy);
          cr_weights<float>(fz, wz);
          cr_dweights<float>(fz, dz);
          const float nref = reinterpret_cast<const BinTile<4> &>(T).hi[lph + HI_PLANE + TILE_EDGE + 1].w;
          const float rlo = reinterpret_cast<const BinTile<4> &>(T).lo[lpl + TILE_EDGE * TILE_EDGE + TILE_EDGE + 1];
          // this lane's weights, selected in registers
          const float wzk[2] = {h ? wz[1] : wz[0], h ? wz[3] : wz[2]};
          const float dzk[2] = {h ? dz[1] : dz[0], h ? dz[3] : dz[2]};
          const float wxp = (p & 2) ? ((p & 1) ? wx[3] : wx[2]) : ((p & 1) ? wx[1] : wx[0]);
          const float dxp = (p & 2) ? ((p & 1) ? dx[3] : dx[2]) : ((p & 1) ? dx[1] : dx[0]);
          // Components (values only) accumulate raw float32 values; |B|
          // accumulates deltas to the corner so its derivatives keep full
          // relative precision.  y first, then z: d/dz reuses the layer sums.
          float2 Sxy = make_float2(0.f, 0.f), Szn = make_float2(0.f, 0.f);
          float Gy = 0.f, Gz = 0.f;
#pragma unroll
          for (int kk = 0; kk < 2; ++kk) {
            const int k = 2 * kk + h;
            float2 axy = make_float2(0.f, 0.f), azn = make_float2(0.f, 0.f);
            float gy = 0.f;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const float4 v = reinterpret_cast<const BinTile<4> &>(T).hi[lph + k * HI_PLANE + j * TILE_EDGE + p];
              const float lo = reinterpret_cast<const BinTile<4> &>(T).lo[lpl + (k * TILE_EDGE + j) * TILE_EDGE + p];
              const float dn = (v.w - nref) + (lo - rlo);
              const float2 wj = make_float2(wy[j], wy[j]);
              axy = ffma2(wj, make_float2(v.x, v.y), axy);
              azn = ffma2(wj, make_float2(v.z, dn), azn);
              gy += dy[j] * dn;
            }
            const float2 wk = make_float2(wzk[kk], wzk[kk]);
            Sxy = ffma2(wk, axy, Sxy);
            Szn = ffma2(wk, azn, Szn);
            Gy += wzk[kk] * gy;
            Gz += dzk[kk] * azn.y;
          }
          // Reduce-scatter over the 8 lanes of the group (butterfly on lane
          // bits 2, 1, 0): lane g8 ends with the sum of output column g8 of
          // (Vx, Vy, Vz, Vn, Gx, Gy, Gz, 0).
          float u[4];
          {
            const float v8[8] = {wxp * Sxy.x, wxp * Sxy.y, wxp * Szn.x, wxp * Szn.y,
                                 dxp * Szn.y, wxp * Gy, wxp * Gz, 0.f};
#pragma unroll
            for (int m = 0; m < 4; ++m) {
              const float send = h ? v8[m] : v8[m + 4];
              u[m] = (h ? v8[m + 4] : v8[m]) + __shfl_xor_sync(mask, send, 4);
            }
          }
          const bool b1 = (p & 2) != 0, b0 = (p & 1) != 0;
          float u2[2];
#pragma unroll
          for (int m = 0; m < 2; ++m) {
            const float send = b1 ? u[m] : u[m + 2];
            u2[m] = (b1 ? u[m + 2] : u[m]) + __shfl_xor_sync(mask, send, 2);
          }
          const float val = (b0 ? u2[1] : u2[0]) + __shfl_xor_sync(mask, b0 ? u2[0] : u2[1], 1);
          // column g8 as the caller's float64
          const float ih = g8 == 4 ? kp.inv_hf[0] : (g8 == 5 ? kp.inv_hf[1] : kp.inv_hf[2]);
          const float x = g8 == 3 ? nref + (rlo + val) : (g8 >= 4 ? val * ih : val);
          const double out = g8 == 7 ? 0.0 : f2d_exact(x);
          if (interleaved_rows<3, 4>(o)) {
            o.comps[i * 8 + g8] = out;      // a group writes its 64-byte row
          } else if (g8 < 3) {
            if (o.comps) o.comps[i * o.comps_stride + g8] = out;
          } else if (g8 == 3) {
            if (o.norms) o.norms[i * o.norms_stride] = out;
          } else if (g8 < 7) {
            if (o.grads) o.grads[i * o.grads_stride + (g8 - 4)] = out;
          }
        }
      }
    }
    __syncthreads();  // this stage is refilled two bins later
    stage ^= 1;
  }
  // records that need no evaluation (out of volume, NaN, sentinel column)
  for (int64_t t = bin_begin(nbins) + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nq;
       t += (int64_t)gridDim.x * blockDim.x) {
    const QRec<float> r = reinterpret_cast<const QRec<float> *>(w.rec)[t];
    write_const<3, F>(o, r.row, (r.cell & 1ULL) && !g.sentinel_nan ? 0.0 : qnan());
  }
}

static int sm_count_sorted() { return device_sms(); }

// Launches the bin-staged kernel when it applies (3D, mixed, 'both' fields,
// 8^3-cell bins); returns false otherwise.
static bool launch_eval_bin(const arb_grid *g, const KParams &kp, const BinGeom &bg, int64_t nq,
                            const arb_query_out *out, const SortedWork &w, cudaStream_t s) {
  if (g->dim != 3 || g->nfield != 4 || bg.shift != 3) return false;
  const size_t smem = 2 * sizeof(BinTile<4>);
  static bool attr[MAX_DEVICES] = {};
  const int dev = current_device();
  if (dev < 0) return false;
  if (!attr[dev]) {
    if (cudaFuncSetAttribute(eval_bin_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return false;
    attr[dev] = true;
  }
  int64_t grid = (int64_t)sm_count_sorted() * 4;  // 4 resident per SM (64 registers)
  if (grid > bg.nbins) grid = bg.nbins;
  if (grid < 1) grid = 1;
  eval_bin_kernel<4><<<(unsigned)grid, 256, smem, s>>>(*g, kp, bg, nq, *out, w);
  return true;
}

// ---- bin-staged evaluation (3D, mixed, scalar / norm or vector fields) -------
// rQuery2 (ARBInterp.py:399-455, scalar and norm fields: one (hi, lo) field)
// and rQuery1 (ARBInterp.py:344-397, vector fields: three components, values
// only) on the fly: the bin's 11^3 points staged in shared memory as in
// eval_bin, one query per thread evaluating eval_otf3_mixed_block /
// eval_otf3_vec_block on the staged block (the code the global-memory kernel
// runs, so the same bits).
constexpr int BINF_THREADS = 128;

template <int F>
struct TileBlock3 {  // a 4x4x4 block inside a staged tile
  // F = 1: (hi, lo) pairs, read by hl and load; F = 3: float4 components,
  // read by hi4 (the accessors of the other layout are never instantiated)
  const typename std::conditional<F == 1, float2, float4>::type *v;
  int base;  // tile index of the block corner
  __device__ __forceinline__ int at(int i, int j, int k) const {
    return base + (k * TILE_EDGE + j) * TILE_EDGE + i;
  }
  __device__ __forceinline__ float2 hl(int p) const { return v[p]; }
  __device__ __forceinline__ float4 hi4(int p) const { return v[p]; }
  template <int FF>
  __device__ __forceinline__ void load(int p, int, float &hi, float &lo) const {
    const float2 x = v[p];
    hi = x.x;
    lo = x.y;
  }
};

template <int F>
__global__ void __launch_bounds__(BINF_THREADS) eval_binf_kernel(arb_grid g, KParams kp, BinGeom bg, int64_t nq,
                                                                 arb_query_out o, SortedWork w) {
  extern __shared__ __align__(16) unsigned char binf_smem[];
  BinTile<F> *tiles = reinterpret_cast<BinTile<F> *>(binf_smem);
  const int64_t nbins = bg.nbins;
  const QRec<float> *recs = reinterpret_cast<const QRec<float> *>(w.rec);
  int stage = 0;
  int64_t b = blockIdx.x;
  // after placement hist[b] is the end of bin b; bins with no query need no copy
  auto bin_begin = [&](int64_t bb) { return bb > 0 ? (int64_t)w.hist[bb - 1] : (int64_t)0; };
  auto count = [&](int64_t bb) { return bb < nbins ? (int64_t)w.hist[bb] - bin_begin(bb) : 0; };
  if (count(b) > 0) load_bin_tile<F>(g, bg, b, tiles[0]);
  cp_async_commit();
  for (; b < nbins; b += gridDim.x) {
    const int64_t bn = b + gridDim.x;
    if (count(bn) > 0) load_bin_tile<F>(g, bg, bn, tiles[stage ^ 1]);
    cp_async_commit();
    const int64_t t0 = bin_begin(b), t1 = w.hist[b];
    cp_async_wait1();
    __syncthreads();
    if (t1 > t0) {
      int64_t og[3];
      bin_origin(b, bg, og);
      for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
        const QRec<float> r = recs[t];
        int64_t c[3];
        unpack_cell<3>(r.cell, c);
        TileBlock3<F> blk;
        blk.v = tiles[stage].v;
        blk.base = (int)(((c[2] - og[2]) * TILE_EDGE + (c[1] - og[1])) * TILE_EDGE + (c[0] - og[0]));
        const float fr[3] = {r.f[0], r.f[1], r.f[2]};
        double val[F], grad[3] = {0.0, 0.0, 0.0};
        if constexpr (F == 1)
          eval_otf3_mixed_block<1>(blk, kp, fr, val, grad);
        else
          eval_otf3_vec_block(blk, fr, val);
        write_vals<3, F>(o, r.row, val, grad);
      }
    }
    __syncthreads();  // this stage is refilled two bins later
    stage ^= 1;
  }
  // records that need no evaluation (out of volume, NaN, sentinel column)
  for (int64_t t = bin_begin(nbins) + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nq;
       t += (int64_t)gridDim.x * blockDim.x) {
    const QRec<float> r = recs[t];
    write_const<3, F>(o, r.row, (r.cell & 1ULL) && !g.sentinel_nan ? 0.0 : qnan());
  }
}

// Launches the 3D one-field / vector bin-staged kernel when it applies (3D,
// mixed, F = 1 or 3, 8^3-cell bins); returns false otherwise.
template <int F>
static bool launch_eval_binf(const arb_grid *g, const KParams &kp, const BinGeom &bg, int64_t nq,
                             const arb_query_out *out, const SortedWork &w, cudaStream_t s) {
  const size_t smem = 2 * sizeof(BinTile<F>);
  static int per_sm[MAX_DEVICES] = {};
  const int dev = current_device();
  if (dev < 0) return false;
  if (!per_sm[dev]) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, eval_binf_kernel<F>, BINF_THREADS, smem) !=
            cudaSuccess ||
        n < 1)
      return false;
    per_sm[dev] = n;
  }
  int64_t grid = (int64_t)sm_count_sorted() * per_sm[dev];
  if (grid > bg.nbins) grid = bg.nbins;
  if (grid < 1) grid = 1;
  eval_binf_kernel<F><<<(unsigned)grid, BINF_THREADS, smem, s>>>(*g, kp, bg, nq, *out, w);
  return true;
}

static bool launch_eval_bin1(const arb_grid *g, const KParams &kp, const BinGeom &bg, int64_t nq,
                             const arb_query_out *out, const SortedWork &w, cudaStream_t s) {
  if (g->dim != 3 || bg.shift != 3) return false;
  if (g->nfield == 1) return launch_eval_binf<1>(g, kp, bg, nq, out, w, s);
  if (g->nfield == 3) return launch_eval_binf<3>(g, kp, bg, nq, out, w, s);
  return false;
}

// ---- bin-staged evaluation (4D, mixed, one scalar field, 4^4-cell bins) -------
// rQuery2 of the 4D class (ARBInterp.py:1129-1189) on the fly.
// As eval_bin in 3D: one CTA per bin (round-robin), the bin's 7^4-point
// footprint of (hi, lo) pairs copied into shared memory with cp.async and
// double-buffered, one thread per query evaluating eval_otf4_mixed_block on
// the staged block.  From global memory each thread's 8-byte loads touch a
// different 128-byte line per instruction and the kernel was L1-bound; shared
// memory serves a warp's 32 scattered 8-byte loads in a few wavefronts.
constexpr int BIN4_EDGE = 4;
constexpr int TILE4_EDGE = BIN4_EDGE + 3;
constexpr int TILE4_PTS = TILE4_EDGE * TILE4_EDGE * TILE4_EDGE * TILE4_EDGE;
constexpr int BIN4_THREADS = 128;

struct BinTile4 {
  float2 v[TILE4_PTS];  // [t][z][y][x] (hi, lo)
};

struct TileBlock4 {  // a 4x4x4x4 block inside a staged tile
  const float2 *v;
  int base;  // tile index of the block corner
  __device__ __forceinline__ int at(int i, int j, int k, int l) const {
    return base + ((l * TILE4_EDGE + k) * TILE4_EDGE + j) * TILE4_EDGE + i;
  }
  template <int F>
  __device__ __forceinline__ void load(int p, int, float &hi, float &lo) const {
    const float2 x = v[p];
    hi = x.x;
    lo = x.y;
  }
};

__device__ __forceinline__ void bin_origin4(int64_t b, const BinGeom &bg, int64_t o[4]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = (b % bg.nb[a]) * BIN4_EDGE;
    b /= bg.nb[a];
  }
  o[3] = b * BIN4_EDGE;
}

__device__ __forceinline__ void load_bin_tile4(const arb_grid &g, const BinGeom &bg, int64_t b, BinTile4 &t) {
  int64_t o[4];
  bin_origin4(b, bg, o);
  const int64_t nx = g.n[0], ny = g.n[1], nz = g.n[2], nt = g.n[3];
  const float2 *g2 = reinterpret_cast<const float2 *>(g.grid32);
  for (int e = threadIdx.x; e < TILE4_PTS; e += blockDim.x) {
    int r = e;
    const int lx = r % TILE4_EDGE;
    r /= TILE4_EDGE;
    const int ly = r % TILE4_EDGE;
    r /= TILE4_EDGE;
    const int lz = r % TILE4_EDGE, lt = r / TILE4_EDGE;
    const int64_t x = o[0] + lx, y = o[1] + ly, z = o[2] + lz, tt = o[3] + lt;
    if (x >= nx || y >= ny || z >= nz || tt >= nt) continue;
    cp_async8(&t.v[e], g2 + ((tt * nz + z) * ny + y) * nx + x);
  }
}

__global__ void __launch_bounds__(BIN4_THREADS) eval_bin4_kernel(arb_grid g, KParams kp, BinGeom bg, int64_t nq,
                                                                 arb_query_out o, SortedWork w) {
  extern __shared__ __align__(16) unsigned char bin4_smem[];
  BinTile4 *tiles = reinterpret_cast<BinTile4 *>(bin4_smem);
  const int64_t nbins = bg.nbins;
  const QRec<float> *recs = reinterpret_cast<const QRec<float> *>(w.rec);
  int stage = 0;
  int64_t b = blockIdx.x;
  // after placement hist[b] is the end of bin b; bins with no query need no copy
  auto bin_begin = [&](int64_t bb) { return bb > 0 ? (int64_t)w.hist[bb - 1] : (int64_t)0; };
  auto count = [&](int64_t bb) { return bb < nbins ? (int64_t)w.hist[bb] - bin_begin(bb) : 0; };
  if (count(b) > 0) load_bin_tile4(g, bg, b, tiles[0]);
  cp_async_commit();
  for (; b < nbins; b += gridDim.x) {
    const int64_t bn = b + gridDim.x;
    if (count(bn) > 0) load_bin_tile4(g, bg, bn, tiles[stage ^ 1]);
    cp_async_commit();
    const int64_t t0 = bin_begin(b), t1 = w.hist[b];
    cp_async_wait1();
    __syncthreads();
    if (t1 > t0) {
      int64_t og[4];
      bin_origin4(b, bg, og);
      for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
        const QRec<float> r = recs[t];
        int64_t c[4];
        unpack_cell<4>(r.cell, c);
        TileBlock4 blk;
        blk.v = tiles[stage].v;
        blk.base = (int)((((c[3] - og[3]) * TILE4_EDGE + (c[2] - og[2])) * TILE4_EDGE + (c[1] - og[1])) *
                             TILE4_EDGE +
                         (c[0] - og[0]));
        const float fr[4] = {r.f[0], r.f[1], r.f[2], r.f[3]};
        double val[1], grad[4];
        eval_otf4_mixed_block<1>(blk, kp, fr, val, grad);
        write_vals<4, 1>(o, r.row, val, grad);
      }
    }
    __syncthreads();  // this stage is refilled two bins later
    stage ^= 1;
  }
  // records that need no evaluation (out of volume, NaN, sentinel column)
  for (int64_t t = bin_begin(nbins) + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nq;
       t += (int64_t)gridDim.x * blockDim.x) {
    const QRec<float> r = recs[t];
    write_const<4, 1>(o, r.row, (r.cell & 1ULL) && !g.sentinel_nan ? 0.0 : qnan());
  }
}

// Launches the 4D bin-staged kernel when it applies (4D, mixed, one scalar
// field, 4^4-cell bins); returns false otherwise.
static bool launch_eval_bin4(const arb_grid *g, const KParams &kp, const BinGeom &bg, int64_t nq,
                             const arb_query_out *out, const SortedWork &w, cudaStream_t s) {
  if (g->dim != 4 || g->nfield != 1 || bg.shift != 2) return false;
  const size_t smem = 2 * sizeof(BinTile4);
  static int per_sm[MAX_DEVICES] = {};
  const int dev = current_device();
  if (dev < 0) return false;
  if (!per_sm[dev]) {
    if (cudaFuncSetAttribute(eval_bin4_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return false;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, eval_bin4_kernel, BIN4_THREADS, smem) != cudaSuccess ||
        n < 1)
      return false;
    per_sm[dev] = n;
  }
  int64_t grid = (int64_t)sm_count_sorted() * per_sm[dev];
  if (grid > bg.nbins) grid = bg.nbins;
  if (grid < 1) grid = 1;
  eval_bin4_kernel<<<(unsigned)grid, BIN4_THREADS, smem, s>>>(*g, kp, bg, nq, *out, w);
  return true;
}

template <int DIM, bool MIXED>
static void launch_bin(const arb_grid *g, const KParams &kp, const BinGeom &bg, double *q, int64_t nq,
                       int64_t qs, int wb, const arb_query_out *out, int32_t *status, const SortedWork &w,
                       cudaStream_t s) {
  using T = typename std::conditional<MIXED, float, double>::type;
  const int TB = 256;
  const unsigned B = (unsigned)((nq + TB - 1) / TB);
  bin_count_kernel<DIM, !MIXED, T><<<B, TB, 0, s>>>(*g, kp, bg, q, nq, qs, wb, *out, status, w);
  scan_kernel<<<1, 1024, 0, s>>>(w.hist, bg.nbins + 1);
  bin_place_kernel<DIM, !MIXED, T><<<B, TB, 0, s>>>(*g, kp, bg, q, nq, qs, w);
}

// Table evaluation, 8 lanes per query.  A cell's block is F fields x R rows
// (ey + 4 ez [+ 16 et]; R = 16 in 3D, 64 in 4D) of 4 x-coefficients; lane j
// loads rows j + 8 i of every field (ey = j & 3, ez alternating between
// j >> 2 and j >> 2 + 2, et = i >> 1), so each load instruction of a group
// reads one contiguous 128-byte line (float table; two with a double table)
// and a warp's four queries four lines.  Each lane evaluates its rows along x
// (Horner) and weights them by y^ey z^ez t^et (and the derivative weights for
// the gradient field); three butterfly shuffles reduce and the group's first
// lane writes the row.  Each block walks TAB_CHUNK consecutive sorted queries.
constexpr int TAB_CHUNK = 256;

template <int DIM, int F, bool MIXED>
__global__ void __launch_bounds__(256) eval_tab_coop_kernel(arb_grid g, KParams kp, int64_t nq, arb_query_out o,
                                                            SortedWork w) {
  using T = typename std::conditional<MIXED, float, double>::type;
  constexpr int M = DIM == 3 ? 64 : 256, NR = M / 32;  // rows per lane and field
  constexpr bool GRAD = F != 3;
  const int lane = threadIdx.x & 31, j = lane & 7;
  const unsigned gmask = 0xffu << (lane & 24);
  const int64_t t0 = (int64_t)blockIdx.x * TAB_CHUNK;
  const int64_t t1 = min(t0 + TAB_CHUNK, nq);
  const T *tab = reinterpret_cast<const T *>(g.table);
  const int ey = j & 3, jz = j >> 2;
  for (int64_t t = t0 + (threadIdx.x >> 3); t < t1; t += blockDim.x >> 3) {
    const QRec<T> r = reinterpret_cast<const QRec<T> *>(w.rec)[t];
    const unsigned long long cw = r.cell;
    const int64_t i = r.row;
    if (cw & CELL_SPECIAL) {
      if (j == 0) write_const<DIM, F>(o, i, (cw & 1ULL) && !g.sentinel_nan ? 0.0 : qnan());
      continue;
    }
    int64_t c[DIM];
    unpack_cell<DIM>(cw, c);
    const T x = r.f[0], y = r.f[1], z = r.f[2];
    // y^ey, z^jz, z^(jz+2) and their derivatives: selects, not indexing
    const T y2 = y * y, z2 = z * z;
    const T wy = ey == 0 ? T(1) : ey == 1 ? y : ey == 2 ? y2 : y2 * y;
    const T dwy = ey == 0 ? T(0) : ey == 1 ? T(1) : ey == 2 ? T(2) * y : T(3) * y2;
    const T wza = jz ? z : T(1), wzb = jz ? z2 * z : z2;
    const T dwza = jz ? T(1) : T(0), dwzb = jz ? T(3) * z2 : T(2) * z;
    T wt[4] = {T(1), T(1), T(1), T(1)}, dwt[4] = {T(0), T(0), T(0), T(0)};
    if constexpr (DIM == 4) {
      const T u = r.f[3], u2 = u * u;
      wt[1] = u;
      wt[2] = u2;
      wt[3] = u2 * u;
      dwt[1] = T(1);
      dwt[2] = T(2) * u;
      dwt[3] = T(3) * u2;
    }
    const T *blk = tab + flat_cell<DIM>(c, g) * (int64_t)(F * M);
    T V[F], G[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) G[d] = T(0);
#pragma unroll
    for (int f = 0; f < F; ++f) {
      V[f] = T(0);
#pragma unroll
      for (int k = 0; k < NR; ++k) {
        T a[4], v, dx;
        load4<T>(blk + f * M + (j + 8 * k) * 4, a);
        horner_x<T>(a, x, v, dx);
        const T wz = (k & 1) ? wzb : wza, dwz = (k & 1) ? dwzb : dwza;
        const T wyz = wy * wz * wt[k >> 1];
        V[f] += v * wyz;
        if (GRAD && f == F - 1) {
          G[0] += dx * wyz;
          G[1] += v * (dwy * wz * wt[k >> 1]);
          G[2] += v * (wy * dwz * wt[k >> 1]);
          if constexpr (DIM == 4) G[3] += v * (wy * wz * dwt[k >> 1]);
        }
      }
    }
#pragma unroll
    for (int m = 1; m < 8; m <<= 1) {
#pragma unroll
      for (int f = 0; f < F; ++f) V[f] += __shfl_xor_sync(gmask, V[f], m);
      if (GRAD) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) G[d] += __shfl_xor_sync(gmask, G[d], m);
      }
    }
    if (j == 0) {
      double val[F], grad[DIM];
#pragma unroll
      for (int f = 0; f < F; ++f) {
        if constexpr (MIXED)
          val[f] = f2d_exact(V[f]);
        else
          val[f] = V[f];
      }
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        if (!GRAD)
          grad[d] = 0.0;
        else if constexpr (MIXED)
          grad[d] = f2d_exact(G[d] * kp.inv_hf[d]);
        else
          grad[d] = (double)G[d] * kp.inv_h[d];
      }
      write_vals<DIM, F>(o, i, val, grad);
    }
  }
}

template <int DIM, bool MIXED>
static void launch_eval(const arb_grid *g, const KParams &kp, int64_t nq, const arb_query_out *out,
                        const SortedWork &w, bool table, cudaStream_t s) {
  if (DIM == 3 && MIXED && !table && launch_eval_bin(g, kp, bin_geom(g), nq, out, w, s)) return;
  if (DIM == 3 && MIXED && !table && launch_eval_bin1(g, kp, bin_geom(g), nq, out, w, s)) return;
  if (DIM == 4 && MIXED && !table && launch_eval_bin4(g, kp, bin_geom(g), nq, out, w, s)) return;
  const int TE = DIM == 3 ? 256 : 128;
  const unsigned BE = (unsigned)((nq + TE - 1) / TE);
#define ES(FF, TAB) eval_sorted_kernel<DIM, FF, MIXED, TAB><<<BE, TE, 0, s>>>(*g, kp, nq, *out, w)
  if (table) {
    const unsigned BT = (unsigned)((nq + TAB_CHUNK - 1) / TAB_CHUNK);
#define ET(FF) eval_tab_coop_kernel<DIM, FF, MIXED><<<BT, 256, 0, s>>>(*g, kp, nq, *out, w)
    switch (g->nfield) { case 1: ET(1); break; case 3: ET(3); break; default: ET(4); break; }
#undef ET
  } else if (DIM == 3 && MIXED && g->nfield == 4) {
    const unsigned BC = (unsigned)((nq + COOP_CHUNK - 1) / COOP_CHUNK);
    eval_sorted_coop4_kernel<<<BC, 256, 0, s>>>(*g, kp, nq, *out, w);
  } else {
    switch (g->nfield) { case 1: ES(1, false); break; case 3: ES(3, false); break; default: ES(4, false); break; }
  }
#undef ES
}

}  // namespace arb

using namespace arb;

// ---- allocation-free variant --------------------------------------------------
// Scratch of arb_query_eval_sorted_noalloc: a file-scope device array that
// every GPU which loads this library holds until the process exits.  Host code
// must not pass the symbol itself to a kernel (on the host it is only a
// stand-in); its device address is looked up with cudaGetSymbolAddress, with
// the device current, the first time that device's context calls, and again
// only if the device's context has changed since (a cudaDeviceReset loads the
// module anew, at a possibly different address).
static __device__ __align__(256) unsigned char g_noalloc_scratch[ARB_NOALLOC_SCRATCH_BYTES];

// Unique id of the calling thread's current context (0 if none or unknown).
static unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult r;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &r) == cudaSuccess &&
        r == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(p);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &r) == cudaSuccess &&
        r == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(p);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) != CUDA_SUCCESS)
    id = 0;
  return id;
}

static void *noalloc_scratch(int *rc) {
  static std::mutex mu;
  static void *ptrs[MAX_DEVICES] = {};
  static unsigned long long ctx_ids[MAX_DEVICES] = {};
  const int dev = current_device();
  if (dev < 0) {
    *rc = ARB_ERR_CUDA;
    return nullptr;
  }
  const unsigned long long id = current_context_id();
  std::lock_guard<std::mutex> lock(mu);
  if (!ptrs[dev] || ctx_ids[dev] != id) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
      *rc = ARB_ERR_CUDA;
      return nullptr;
    }
    ptrs[dev] = p;
    ctx_ids[dev] = current_context_id();  // the lookup may have made the primary context current
  }
  return ptrs[dev];
}

extern "C" size_t arb_query_sorted_work_bytes(const arb_grid *g, int32_t precision, int64_t nq) {
  if (!g || nq < 0 || (g->dim != 3 && g->dim != 4)) return 0;
  return carve(nullptr, nullptr, g, precision, nq);
}

extern "C" int arb_query_eval_sorted(const arb_grid *g, int32_t precision, int32_t use_table,
                                     double *q, int64_t nq, int64_t q_stride, int32_t q_writeback,
                                     const arb_query_out *out, void *work, size_t work_bytes,
                                     int32_t *status, arb_stream_t stream) {
  int rc = check_query_args(g, q, nq, q_stride, out);
  if (rc) return rc;
  if (nq == 0) return ARB_OK;
  if (!work || !status) return ARB_ERR_INVALID;
  if (nq >= (int64_t)1 << 32) return ARB_ERR_UNSUPPORTED;
  const int bits = g->dim == 3 ? cell_bits<3>() : cell_bits<4>();
  for (int a = 0; a < g->dim; ++a)
    if (g->n[a] - 3 >= ((int64_t)1 << bits)) return ARB_ERR_UNSUPPORTED;  // cells per axis
  const bool mixed = precision == ARB_PREC_MIXED;
  if (use_table) {
    if (!g->table || g->table_prec != precision) return ARB_ERR_INVALID;
  } else if (mixed ? !g->grid32 : !g->grid64) {
    return ARB_ERR_INVALID;
  }
  SortedWork w;
  if (carve(&w, work, g, precision, nq) > work_bytes) return ARB_ERR_INVALID;
  const BinGeom bg = bin_geom(g);
  cudaStream_t s = (cudaStream_t)stream;
  const arb_query_out out_norm = normalize_out(*out, g->dim);
  out = &out_norm;
  if (cudaMemsetAsync(w.hist, 0, sizeof(uint32_t) * (bg.nbins + 1), s) != cudaSuccess) return ARB_ERR_CUDA;
  const KParams kp = make_kparams(g);
  if (g->dim == 3) {
    if (mixed) {
      launch_bin<3, true>(g, kp, bg, q, nq, q_stride, q_writeback, out, status, w, s);
      launch_eval<3, true>(g, kp, nq, out, w, use_table, s);
    } else {
      launch_bin<3, false>(g, kp, bg, q, nq, q_stride, q_writeback, out, status, w, s);
      launch_eval<3, false>(g, kp, nq, out, w, use_table, s);
    }
  } else {
    if (mixed) {
      launch_bin<4, true>(g, kp, bg, q, nq, q_stride, q_writeback, out, status, w, s);
      launch_eval<4, true>(g, kp, nq, out, w, use_table, s);
    } else {
      launch_bin<4, false>(g, kp, bg, q, nq, q_stride, q_writeback, out, status, w, s);
      launch_eval<4, false>(g, kp, nq, out, w, use_table, s);
    }
  }
  return launch_status();
}

// Binning only: the first half of arb_query_eval_sorted.  The workspace then
// holds the bin-ordered records, which depend on the query points and the
// grid geometry but not on the field values.
extern "C" int arb_query_bin(const arb_grid *g, int32_t precision, double *q, int64_t nq, int64_t q_stride,
                             int32_t q_writeback, const arb_query_out *out, void *work, size_t work_bytes,
                             int32_t *status, arb_stream_t stream) {
  int rc = check_query_args(g, q, nq, q_stride, out);
  if (rc) return rc;
  if (nq == 0) return ARB_OK;
  if (!work || !status) return ARB_ERR_INVALID;
  if (nq >= (int64_t)1 << 32) return ARB_ERR_UNSUPPORTED;
  const int bits = g->dim == 3 ? cell_bits<3>() : cell_bits<4>();
  for (int a = 0; a < g->dim; ++a)
    if (g->n[a] - 3 >= ((int64_t)1 << bits)) return ARB_ERR_UNSUPPORTED;
  SortedWork w;
  if (carve(&w, work, g, precision, nq) > work_bytes) return ARB_ERR_INVALID;
  const BinGeom bg = bin_geom(g);
  cudaStream_t s = (cudaStream_t)stream;
  const arb_query_out out_norm = normalize_out(*out, g->dim);
  out = &out_norm;
  if (cudaMemsetAsync(w.hist, 0, sizeof(uint32_t) * (bg.nbins + 1), s) != cudaSuccess) return ARB_ERR_CUDA;
  const KParams kp = make_kparams(g);
  const bool mixed = precision == ARB_PREC_MIXED;
  if (g->dim == 3) {
    if (mixed) launch_bin<3, true>(g, kp, bg, q, nq, q_stride, q_writeback, out, status, w, s);
    else launch_bin<3, false>(g, kp, bg, q, nq, q_stride, q_writeback, out, status, w, s);
  } else {
    if (mixed) launch_bin<4, true>(g, kp, bg, q, nq, q_stride, q_writeback, out, status, w, s);
    else launch_bin<4, false>(g, kp, bg, q, nq, q_stride, q_writeback, out, status, w, s);
  }
  return launch_status();
}

// Evaluation only, from a workspace filled by arb_query_bin for the same
// query rows and a grid of the same geometry (values may differ).
extern "C" int arb_query_eval_binned(const arb_grid *g, int32_t precision, int32_t use_table, int64_t nq,
                                     const arb_query_out *out, void *work, size_t work_bytes,
                                     arb_stream_t stream) {
  if (!g || !out || nq < 0 || (g->dim != 3 && g->dim != 4)) return ARB_ERR_INVALID;
  if (nq == 0) return ARB_OK;
  if (!work) return ARB_ERR_INVALID;
  const bool mixed = precision == ARB_PREC_MIXED;
  if (use_table) {
    if (!g->table || g->table_prec != precision) return ARB_ERR_INVALID;
  } else if (mixed ? !g->grid32 : !g->grid64) {
    return ARB_ERR_INVALID;
  }
  SortedWork w;
  if (carve(&w, work, g, precision, nq) > work_bytes) return ARB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const arb_query_out out_norm = normalize_out(*out, g->dim);
  out = &out_norm;
  const KParams kp = make_kparams(g);
  if (g->dim == 3) {
    if (mixed) launch_eval<3, true>(g, kp, nq, out, w, use_table, s);
    else launch_eval<3, false>(g, kp, nq, out, w, use_table, s);
  } else {
    if (mixed) launch_eval<4, true>(g, kp, nq, out, w, use_table, s);
    else launch_eval<4, false>(g, kp, nq, out, w, use_table, s);
  }
  return launch_status();
}

extern "C" int arb_query_eval_sorted_noalloc(const arb_grid *g, int32_t precision, int32_t use_table,
                                             double *q, int64_t nq, int64_t q_stride, int32_t q_writeback,
                                             const arb_query_out *out, int32_t *status,
                                             arb_stream_t stream) {
  int rc = check_query_args(g, q, nq, q_stride, out);
  if (rc) return rc;
  if (nq == 0) return ARB_OK;
  if (!status) return ARB_ERR_INVALID;
  const size_t need = arb_query_sorted_work_bytes(g, precision, nq);
  if (need == 0) return ARB_ERR_INVALID;
  if (need > (size_t)ARB_NOALLOC_SCRATCH_BYTES) return ARB_ERR_CAPACITY;
  void *ws = noalloc_scratch(&rc);
  if (!ws) return rc;
  return arb_query_eval_sorted(g, precision, use_table, q, nq, q_stride, q_writeback, out, ws, need,
                               status, stream);
}
