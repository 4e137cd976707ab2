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
//              bookkeeping of rQuery (NaN rows, queryInds) and the sub-bin
//              histogram (fire-and-forget atomics)
//   scan     : exclusive prefix sum of the histogram into a second array
//              (the counts stay), and with bank classes one 32-byte header
//              per bin (its start and its 16 class counts)
//   place    : the same coordinate step again, a rank inside the query's
//              sub-bin (an atomic that counts the histogram back down to
//              zero), the bin's header (one load) and one 32-byte record
//              (packed cell, row, fraction) written at its final position
//   evaluate : on-the-fly or table evaluation in record order, outputs
//              written to the query's original row
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

// Placement header of a bin with 16 bank classes: where its records start
// and how many each class holds, so the placement pass reads one sector
// per query instead of the bin's 17 offsets.
struct __align__(32) BinHdr {
  uint32_t cnt[4];  // class k's count in byte k & 3 of cnt[k >> 2] (when ovf == 0)
  uint32_t start;   // offs of the bin's class 0 sub-bin
  uint32_t ovf;     // a class holds more than 255 queries: read the offsets instead
  uint32_t pad[2];
};
static_assert(sizeof(BinHdr) == 32, "header size");

struct SortedWork {
  uint32_t *hist;   // nsub + 1 sub-bin counts; placement counts them back down to zero
  uint32_t *offs;   // nsub + 1 exclusive offsets: sub-bin sb holds records [offs[sb], offs[sb + 1]),
                    // the special sub-bin nsub [offs[nsub], nq)
  uint32_t *part;   // per-block totals of the scan
  BinHdr *hdr;      // nbins placement headers (bins with bank classes; null otherwise)
  void *rec;        // nq records (QRec<float> or QRec<double>) in bin order; with bank classes each
                    // bin's records are in its bank schedule (see bank_slot)
};

struct BinGeom {
  int64_t nb[4];     // bins per axis
  int64_t nbins;     // product
  int shift;         // log2 cells per bin edge
  int cls;           // log2 bank classes per bin (4: 3D mixed 8^3-cell bins and 4D mixed scalar
                     // 4^4-cell bins; 0 otherwise)
  int64_t nsub;      // nbins << cls sub-bins (bin-major); the special sub-bin is index nsub
};

// Bank class of a cell inside its 8^3-cell bin: the index, mod 16, of the
// cell's corner point in an unpadded 11 x 11 x 11 tile (x + 11 y + 121 z,
// with 121 = 9 mod 16).  Mod 8 it is the corner's 16-byte bank group in the
// tile of float4 points, mod 16 its 8-byte slot in the tile of float2 pairs.
// Bin origins are multiples of 8 on every axis, so the class from the global
// cell coordinates is the local one plus 0 or 8 for the whole bin: 8
// consecutive classes stay distinct mod 8, and 16 distinct mod 16.
__host__ __device__ __forceinline__ int bank_class(int64_t cx, int64_t cy, int64_t cz) {
  return (int)((cx + 11 * cy + 9 * cz) & 15);
}

// 4D: the 8-byte bank slot (mod 16) of the cell's corner point in an unpadded
// 7^4 tile of (hi, lo) pairs (x + 7 y + 49 z + 343 t, with 49 = 1 and
// 343 = 7 mod 16).  Bin origins are multiples of 4, so the class from the
// global cell coordinates is the local one plus a constant per bin: the
// classes of one bin still map to 16 distinct slots.
__host__ __device__ __forceinline__ int bank_class4(int64_t cx, int64_t cy, int64_t cz, int64_t ct) {
  return (int)((cx + 7 * cy + cz + 7 * ct) & 15);
}

static inline BinGeom bin_geom(const arb_grid *g, int precision) {
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
  b.cls = 0;
  if (precision == ARB_PREC_MIXED) {
    if (g->dim == 3 && b.shift == 3) b.cls = 4;
    if (g->dim == 4 && b.shift == 2 && g->nfield == 1) b.cls = 4;
  }
  b.nsub = b.nbins << b.cls;
  return b;
}

static inline size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

// Exclusive scan of the sub-bin histogram: SCAN_THREADS x SCAN_PER counters
// per block, two launches (block totals, then the scan with carry-in).
constexpr int SCAN_THREADS = 1024, SCAN_PER = 8;
constexpr int64_t SCAN_CHUNK = (int64_t)SCAN_THREADS * SCAN_PER;

static inline int64_t scan_blocks(int64_t n) { return (n + SCAN_CHUNK - 1) / SCAN_CHUNK; }

static size_t carve(SortedWork *w, void *base, const arb_grid *g, int precision, int64_t nq) {
  const BinGeom bg = bin_geom(g, precision);
  const size_t tsz = precision == ARB_PREC_MIXED ? 4 : 8;
  size_t off = 0;
  char *p = (char *)base;
  auto take = [&](size_t bytes) {
    void *r = p ? (void *)(p + off) : nullptr;
    off += align_up(bytes);
    return r;
  };
  SortedWork t;
  t.hist = (uint32_t *)take(sizeof(uint32_t) * (bg.nsub + 1));
  t.offs = (uint32_t *)take(sizeof(uint32_t) * (bg.nsub + 1));
  t.part = (uint32_t *)take(sizeof(uint32_t) * scan_blocks(bg.nsub + 1));
  t.hdr = bg.cls ? (BinHdr *)take(sizeof(BinHdr) * bg.nbins) : nullptr;
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
  bin = bg.nsub;
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
    if constexpr (DIM == 3) {
      if (bg.cls) bin = (bin << 4) | bank_class(c[0], c[1], c[2]);
    } else {
      if (bg.cls) bin = (bin << 4) | bank_class4(c[0], c[1], c[2], c[3]);
    }
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

// Position of the query of rank r in class c of a bin whose NC class
// sub-bins start at o[0..NC-1] (o[NC]: the bin's end), in the bin's bank
// schedule: round robin over the classes, level l holding the l-th query of
// every class with more than l, classes in increasing order within a level.
// So every NC consecutive records of a level with all classes present have
// NC distinct bank classes, wherever the NC start.
template <int NC>
__device__ __forceinline__ uint32_t bank_slot(const uint32_t o[NC + 1], int c, uint32_t r) {
  uint32_t pos = o[0];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    const uint32_t n = o[k + 1] - o[k];
    pos += min(n, r) + ((k < c && n > r) ? 1u : 0u);
  }
  return pos;
}

// bank_slot from a bin header: start, and the 16 class counts as bytes.
__device__ __forceinline__ uint32_t bank_slot_hdr(const uint32_t cnt[4], uint32_t start, int c, uint32_t r) {
  uint32_t pos = start;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const uint32_t n = (cnt[k >> 2] >> (8 * (k & 3))) & 255u;
    pos += min(n, r) + ((k < c && n > r) ? 1u : 0u);
  }
  return pos;
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
  // rank inside the sub-bin (any order: the count runs back down to zero)
  const uint32_t r = atomicSub(&w.hist[bin], 1u) - 1u;
  uint32_t pos;
  if (bg.cls && bin < bg.nsub) {
    constexpr int NC = 16;  // the class sub-bins of one bin
    uint32_t h[8];
    asm volatile("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(h[0]), "=r"(h[1]), "=r"(h[2]), "=r"(h[3]), "=r"(h[4]), "=r"(h[5]), "=r"(h[6]), "=r"(h[7])
                 : "l"(w.hdr + (bin >> 4)));
    if (!h[5]) {
      pos = bank_slot_hdr(h, h[4], (int)(bin & (NC - 1)), r);
    } else {
      const int64_t b0 = bin & ~(int64_t)(NC - 1);
      uint32_t o[NC + 1];
#pragma unroll
      for (int k = 0; k <= NC; ++k) o[k] = w.offs[b0 + k];
      pos = bank_slot<NC>(o, (int)(bin & (NC - 1)), r);
    }
  } else {
    pos = w.offs[bin] + r;
  }
  QRec<T> rec;
  rec.cell = cw;
  rec.row = (uint32_t)i;
#pragma unroll
  for (int a = 0; a < 4; ++a) rec.f[a] = a < DIM ? frac[a] : T(0);
  rec.pad = 0;
  if constexpr (sizeof(T) == 4) {
    // one 32-byte store: a whole sector, no partial-sector merge in L2
    const uint32_t *u = reinterpret_cast<const uint32_t *>(&rec);
    asm volatile("st.global.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(reinterpret_cast<QRec<T> *>(w.rec) + pos),
                 "r"(u[0]), "r"(u[1]), "r"(u[2]), "r"(u[3]), "r"(u[4]), "r"(u[5]), "r"(u[6]), "r"(u[7])
                 : "memory");
  } else {
    reinterpret_cast<QRec<T> *>(w.rec)[pos] = rec;
  }
}

// Block totals of the histogram chunks (SCAN_CHUNK counters per block).
__global__ void __launch_bounds__(SCAN_THREADS) scan_part_kernel(const uint32_t *hist, int64_t n, uint32_t *part) {
  __shared__ uint32_t wsum[SCAN_THREADS / 32];
  const int64_t b = blockIdx.x * SCAN_CHUNK + (int64_t)threadIdx.x * SCAN_PER;
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_PER; ++k)
    if (b + k < n) sum += hist[b + k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t v = wsum[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

// Exclusive scan of each chunk into offs, offset by the totals of the chunks
// before it (the counts in hist stay for the placement pass).
__global__ void __launch_bounds__(SCAN_THREADS) scan_apply_kernel(const uint32_t *hist, int64_t n,
                                                                  const uint32_t *part, uint32_t *offs,
                                                                  BinHdr *hdr, int64_t nbins) {
  __shared__ uint32_t wsum[SCAN_THREADS / 32];
  __shared__ uint32_t carry_s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // carry-in: the totals of the chunks before this one
  uint32_t c = 0;
  for (int64_t k = threadIdx.x; k < blockIdx.x; k += SCAN_THREADS) c += part[k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0) wsum[warp] = c;
  __syncthreads();
  if (warp == 0) {
    uint32_t v = wsum[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) carry_s = v;
  }
  __syncthreads();
  const uint32_t carry = carry_s;
  __syncthreads();  // wsum is reused below
  const int64_t b = blockIdx.x * SCAN_CHUNK + (int64_t)threadIdx.x * SCAN_PER;
  uint32_t v[SCAN_PER], sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_PER; ++k) {
    v[k] = b + k < n ? hist[b + k] : 0u;
    sum += v[k];
  }
  // inclusive warp scan of the thread totals, then of the warp totals
  uint32_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t x = wsum[lane], xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += y;
    }
    wsum[lane] = xi - x;  // exclusive prefix of the warp totals
  }
  __syncthreads();
  uint32_t run = carry + wsum[warp] + (incl - sum);
#pragma unroll
  for (int k = 0; k < SCAN_PER; ++k) {
    if (b + k < n) offs[b + k] = run;
    run += v[k];
  }
  if (hdr) {
    // bins of 16 class counters: this thread holds classes 0-7 (even lane)
    // or 8-15 (odd lane) of bin b / 16; the even lane writes the header
    uint32_t c0 = 0, c1 = 0, ovf = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      c0 |= min(v[k], 255u) << (8 * k);
      c1 |= min(v[k + 4], 255u) << (8 * k);
      ovf |= (v[k] > 255u) | (v[k + 4] > 255u);
    }
    const uint32_t d0 = __shfl_down_sync(0xffffffffu, c0, 1), d1 = __shfl_down_sync(0xffffffffu, c1, 1);
    const uint32_t dovf = __shfl_down_sync(0xffffffffu, ovf, 1);
    const int64_t bin = b >> 4;
    if (!(lane & 1) && bin < nbins) {
      const uint32_t start = carry + wsum[warp] + (incl - sum);
      asm volatile("st.global.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(hdr + bin), "r"(c0), "r"(c1),
                   "r"(d0), "r"(d1), "r"(start), "r"(ovf | dovf), "r"(0u), "r"(0u)
                   : "memory");
    }
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

// ---- bin-staged evaluation (3D, mixed, 8^3-cell bins) -------------------------
// rQuery1/2/3 (ARBInterp.py:344-521) on the fly for the three field layouts
// of mixed precision: F = 1 (scalar and norm fields: one (hi, lo) field),
// F = 3 (vector fields: three components, values only) and F = 4 ('both':
// three components plus |B| as (hi, lo)).
//
// One CTA per bin (round-robin over bins): the bin's footprint of 11^3 grid
// points (8 cells + 3 per axis) is copied into shared memory with cp.async,
// double-buffered so the next bin's copy overlaps this bin's queries, and one
// thread per query evaluates eval_otf3_mixed_block / eval_otf3_vec_block on
// the staged block -- the code the global-memory kernels run, so binned and
// unbinned queries return the same bits, and every gradient component is
// differenced along its own axis first.
//
// Bank order.  The tiles are unpadded, x fastest: point (x, y, z) at
// e = x + 11 y + 121 z, so point (i, j, k) of the block of local cell
// (cx, cy, cz) has e = bank_class(cx, cy, cz) + i + 11 j + 9 k + const
// (mod 16): in the float4 tile its 16-byte bank group is e mod 8, in the
// float2 tile of lo pairs its 8-byte slot e mod 16.  The placement pass
// orders each bin's queries into 16 sub-bins by class and writes them round
// robin over the classes 0..15, so in a level with all 16 classes each
// quarter-warp (the 8 threads of one phase of a 16-byte load) holds 8
// consecutive classes, distinct mod 8, and each half-warp (one phase of an
// 8-byte load) 16 distinct classes: one wavefront each, where random queries
// need about three for the 16-byte loads and two for the 8-byte ones.  Where
// fewer classes are left in a bin, its last queries conflict as random
// queries would.
constexpr int BIN_EDGE = 8;
constexpr int TILE_EDGE = BIN_EDGE + 3;
constexpr int TILE_PTS = TILE_EDGE * TILE_EDGE * TILE_EDGE;
constexpr int BINC_THREADS = 128;

template <int F>
struct BinTile;
template <>
struct BinTile<4> {          // (hi_x, hi_y, hi_z, hi_n) per point; lo_n of each point and of its x successor
  float4 hi[TILE_PTS];
  float2 lo2[TILE_PTS];      // lo2[e] = (lo_n[e], lo_n[e + 1]): an x-row's four lo words in two 8-byte loads
};
template <>
struct BinTile<1> {          // (hi, lo) per point
  float2 v[TILE_PTS];
};
template <>
struct BinTile<3> {          // (hi_x, hi_y, hi_z, 0) per point
  float4 v[TILE_PTS];
};

// Copy the footprint of the bin whose tile origin is o into `t` (points
// outside the grid are skipped: no cell of the bin reads them).
template <int F>
__device__ __forceinline__ void load_bin_tile(const arb_grid &g, const int o[3], BinTile<F> &t) {
  const int64_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const int64_t npts = nx * ny * nz;
  for (int e = threadIdx.x; e < TILE_PTS; e += blockDim.x) {
    const int lx = e % TILE_EDGE, r = e / TILE_EDGE;
    const int ly = r % TILE_EDGE, lz = r / TILE_EDGE;
    const int64_t x = o[0] + lx, y = o[1] + ly, z = o[2] + lz;
    if (x >= nx || y >= ny || z >= nz) continue;
    const int64_t p = (z * ny + y) * nx + x;
    if constexpr (F == 4) {
      cp_async16(&t.hi[e], reinterpret_cast<const float4 *>(g.grid32) + p);
      cp_async4(&t.lo2[e].x, g.grid32 + npts * 4 + p);
      if (lx + 1 < TILE_EDGE && x + 1 < nx) cp_async4(&t.lo2[e].y, g.grid32 + npts * 4 + p + 1);
    } else if constexpr (F == 3) {
      cp_async16(&t.v[e], reinterpret_cast<const float4 *>(g.grid32) + p);
    } else {
      cp_async8(&t.v[e], reinterpret_cast<const float2 *>(g.grid32) + p);
    }
  }
}

template <int F>
struct TileBlock3;  // a 4x4x4 block inside a staged tile
template <>
struct TileBlock3<4> {
  const float4 *h4;
  const float2 *l2;
  int base;  // tile index of the block corner
  __device__ __forceinline__ int at(int i, int j, int k) const {
    return base + (k * TILE_EDGE + j) * TILE_EDGE + i;
  }
  __device__ __forceinline__ float4 hi4(int p) const { return h4[p]; }
  __device__ __forceinline__ float lo(int p) const { return l2[p].x; }
  __device__ __forceinline__ void lo_row(int p, float l[4]) const {
    const float2 a = l2[p], b = l2[p + 2];
    l[0] = a.x;
    l[1] = a.y;
    l[2] = b.x;
    l[3] = b.y;
  }
};
template <>
struct TileBlock3<1> {
  const float2 *v;
  int base;
  __device__ __forceinline__ int at(int i, int j, int k) const {
    return base + (k * TILE_EDGE + j) * TILE_EDGE + i;
  }
  __device__ __forceinline__ float2 hl(int p) const { return v[p]; }
  template <int FF>
  __device__ __forceinline__ void load(int p, int, float &hi, float &lo) const {
    const float2 x = v[p];
    hi = x.x;
    lo = x.y;
  }
};
template <>
struct TileBlock3<3> {
  const float4 *v;
  int base;
  __device__ __forceinline__ int at(int i, int j, int k) const {
    return base + (k * TILE_EDGE + j) * TILE_EDGE + i;
  }
  __device__ __forceinline__ float4 hi4(int p) const { return v[p]; }
};

// One CTA per bin (round-robin over bins, so the CTAs work on neighbouring
// bins at the same time and their tiles' shared halo points are read from
// HBM about once): the bin's tile is copied into shared memory with
// cp.async, double-buffered so the next bin's copy overlaps this bin's
// queries, and thread t of the CTA evaluates records t, t + BINC_THREADS, ...
// of the bin, which placement wrote in the bin's bank schedule.
template <int F>
__global__ void __launch_bounds__(BINC_THREADS, F == 4 ? 3 : (F == 3 ? 5 : 4)) eval_binc_kernel(arb_grid g, KParams kp, BinGeom bg,
                                                                   int64_t nq, arb_query_out o, SortedWork w) {
  extern __shared__ __align__(16) unsigned char binc_smem[];
  BinTile<F> *tiles = reinterpret_cast<BinTile<F> *>(binc_smem);
  const int64_t nbins = bg.nbins;
  const QRec<float> *recs = reinterpret_cast<const QRec<float> *>(w.rec);
  // bin b holds records [offs[16 b], offs[16 b + 16]) (its 16 class sub-bins)
  const int cls = bg.cls;
  auto begin = [&](int64_t bb) { return w.offs[bb << cls]; };
  auto count = [&](int64_t bb) { return bb < nbins ? w.offs[(bb + 1) << cls] - begin(bb) : 0u; };
  auto origin = [&](int64_t bb, int og[3]) {
    og[0] = (int)((bb % bg.nb[0]) * BIN_EDGE);
    const int64_t r = bb / bg.nb[0];
    og[1] = (int)((r % bg.nb[1]) * BIN_EDGE);
    og[2] = (int)((r / bg.nb[1]) * BIN_EDGE);
  };
  int stage = 0;
  int64_t b = blockIdx.x;
  int og[3];
  if (count(b) > 0) {
    origin(b, og);
    load_bin_tile<F>(g, og, tiles[0]);
  }
  cp_async_commit();
  for (; b < nbins; b += gridDim.x) {
    const int64_t bn = b + gridDim.x;
    if (count(bn) > 0) {
      origin(bn, og);
      load_bin_tile<F>(g, og, tiles[stage ^ 1]);
    }
    cp_async_commit();
    const uint32_t t0 = begin(b), t1 = t0 + count(b);
    cp_async_wait1();
    __syncthreads();
    if (t1 > t0) {
      origin(b, og);
      // the next record is loaded while this one is evaluated
      QRec<float> rnext;
      if (t0 + threadIdx.x < t1) rnext = recs[t0 + threadIdx.x];
      for (uint32_t t = t0 + threadIdx.x; t < t1; t += BINC_THREADS) {
        const QRec<float> r = rnext;
        if (t + BINC_THREADS < t1) rnext = recs[t + BINC_THREADS];
        int64_t c[3];
        unpack_cell<3>(r.cell, c);
        const int bi = (((int)c[2] - og[2]) * TILE_EDGE + ((int)c[1] - og[1])) * TILE_EDGE + ((int)c[0] - og[0]);
        const float fr[3] = {r.f[0], r.f[1], r.f[2]};
        double val[F], grad[3] = {0.0, 0.0, 0.0};
        TileBlock3<F> blk;
        if constexpr (F == 4) {
          blk.h4 = tiles[stage].hi;
          blk.l2 = tiles[stage].lo2;
        } else {
          blk.v = tiles[stage].v;
        }
        blk.base = bi;
        if constexpr (F == 3)
          eval_otf3_vec_block(blk, fr, val);
        else if constexpr (F == 4)
          eval_otf3_both_block(blk, kp, fr, val, grad);
        else
          eval_otf3_mixed_block<F>(blk, kp, fr, val, grad);
        write_vals<3, F>(o, r.row, val, grad);
      }
    }
    __syncthreads();  // this stage is refilled two bins later
    stage ^= 1;
  }
  // records that need no evaluation (out of volume, NaN, sentinel column)
  for (int64_t t = (int64_t)w.offs[bg.nsub] + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nq;
       t += (int64_t)gridDim.x * blockDim.x) {
    const QRec<float> r = recs[t];
    write_const<3, F>(o, r.row, (r.cell & 1ULL) && !g.sentinel_nan ? 0.0 : qnan());
  }
}

static int sm_count_sorted() { return device_sms(); }

// Launches the bank-ordered bin kernel when it applies (3D, mixed, 8^3-cell
// bins with bank classes); returns false otherwise.
template <int F>
static bool launch_eval_binc_f(const arb_grid *g, const KParams &kp, const BinGeom &bg, int64_t nq,
                               const arb_query_out *out, const SortedWork &w, cudaStream_t s) {
  const size_t smem = 2 * sizeof(BinTile<F>);
  static int per_sm[MAX_DEVICES] = {};
  const int dev = current_device();
  if (dev < 0) return false;
  if (!per_sm[dev]) {
    if (cudaFuncSetAttribute(eval_binc_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return false;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, eval_binc_kernel<F>, BINC_THREADS, smem) !=
            cudaSuccess ||
        n < 1)
      return false;
    per_sm[dev] = n;
  }
  int64_t grid = (int64_t)sm_count_sorted() * per_sm[dev];
  if (grid > bg.nbins) grid = bg.nbins;
  if (grid < 1) grid = 1;
  eval_binc_kernel<F><<<(unsigned)grid, BINC_THREADS, smem, s>>>(*g, kp, bg, nq, *out, w);
  return true;
}

static bool launch_eval_binc(const arb_grid *g, const KParams &kp, const BinGeom &bg, int64_t nq,
                             const arb_query_out *out, const SortedWork &w, cudaStream_t s) {
  if (g->dim != 3 || bg.shift != 3 || bg.cls != 4) return false;
  if (g->nfield == 1) return launch_eval_binc_f<1>(g, kp, bg, nq, out, w, s);
  if (g->nfield == 3) return launch_eval_binc_f<3>(g, kp, bg, nq, out, w, s);
  if (g->nfield == 4) return launch_eval_binc_f<4>(g, kp, bg, nq, out, w, s);
  return false;
}

// ---- bin-staged evaluation (4D, mixed, one scalar field, 4^4-cell bins) -------
// rQuery2 of the 4D class (ARBInterp.py:1129-1189) on the fly.
// As eval_bin in 3D: one CTA per bin (round-robin), the bin's 7^4-point
// footprint of (hi, lo) pairs copied into shared memory with cp.async and
// double-buffered, one thread per query evaluating eval_otf4_mixed_block on
// the staged block.  From global memory each thread's 8-byte loads touch a
// different 128-byte line per instruction and the kernel was L1-bound.
// Bank order: an 8-byte shared load is served half-warp by half-warp, 16
// slots of 8 bytes per wavefront, and point (i, j, k, l) of the block of a
// cell of class c (bank_class4) lies in slot (c + i + 7 j + k + 7 l + const)
// mod 16; placement writes each bin's queries round robin over its 16
// classes, so in every level with all 16 classes a half-warp's 16 loads hit
// 16 distinct slots: one wavefront, where 16 random queries need about three.
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
  // bin b holds records [offs[b << cls], offs[(b + 1) << cls]) (its class
  // sub-bins, in the bin's bank schedule); bins with no query need no copy
  const int cls = bg.cls;
  auto bin_begin = [&](int64_t bb) { return (int64_t)w.offs[bb << cls]; };
  auto count = [&](int64_t bb) { return bb < nbins ? (int64_t)w.offs[(bb + 1) << cls] - bin_begin(bb) : 0; };
  if (count(b) > 0) load_bin_tile4(g, bg, b, tiles[0]);
  cp_async_commit();
  for (; b < nbins; b += gridDim.x) {
    const int64_t bn = b + gridDim.x;
    if (count(bn) > 0) load_bin_tile4(g, bg, bn, tiles[stage ^ 1]);
    cp_async_commit();
    const int64_t t0 = bin_begin(b), t1 = w.offs[(b + 1) << cls];
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
  for (int64_t t = (int64_t)w.offs[bg.nsub] + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nq;
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
  const int64_t nh = bg.nsub + 1, nb = scan_blocks(nh);
  scan_part_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(w.hist, nh, w.part);
  scan_apply_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(w.hist, nh, w.part, w.offs, w.hdr, bg.nbins);
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
  const BinGeom bg = bin_geom(g, MIXED ? ARB_PREC_MIXED : ARB_PREC_FP64);
  if (DIM == 3 && MIXED && !table && launch_eval_binc(g, kp, bg, nq, out, w, s)) return;
  if (DIM == 4 && MIXED && !table && launch_eval_bin4(g, kp, bg, nq, out, w, s)) return;
  const int TE = DIM == 3 ? 256 : 128;
  const unsigned BE = (unsigned)((nq + TE - 1) / TE);
#define ES(FF, TAB) eval_sorted_kernel<DIM, FF, MIXED, TAB><<<BE, TE, 0, s>>>(*g, kp, nq, *out, w)
  if (table) {
    const unsigned BT = (unsigned)((nq + TAB_CHUNK - 1) / TAB_CHUNK);
#define ET(FF) eval_tab_coop_kernel<DIM, FF, MIXED><<<BT, 256, 0, s>>>(*g, kp, nq, *out, w)
    switch (g->nfield) { case 1: ET(1); break; case 3: ET(3); break; default: ET(4); break; }
#undef ET
  } else {
    switch (g->nfield) { case 1: ES(1, false); break; case 3: ES(3, false); break; default: ES(4, false); break; }
  }
#undef ES
}

// ---- bin-grouped adjoint (3D scalar, mixed) ----------------------------------
// The backward of rQuery2 (ARBInterp.py:399-454), as arb_adjoint computes it
// per query, but grouped by the 8^3-cell bins of the query pass: the bin's
// (hi, lo) tile is staged as for the forward (the dL/dq terms read the
// interpolant's gradient and Hessian from it), and dL/df is accumulated in a
// shared-memory tile of the bin's 11^3 points with shared atomics, then
// added to the grid gradient once per point and bin.  A query scatters 64
// values, so with ~250 queries per bin (1e6 queries on 128^3) the global
// atomics fall from 64 per query to 1331 per bin.
constexpr int ADJ_THREADS = 128;

__global__ void __launch_bounds__(ADJ_THREADS) adjoint_bin_kernel(arb_grid g, KParams kp, BinGeom bg, int64_t nq,
                                                                  const double *dval, const double *dgrad,
                                                                  float *grid_grad, double *q_grad, SortedWork w) {
  extern __shared__ __align__(16) unsigned char adj_smem[];
  BinTile<1> *tiles = reinterpret_cast<BinTile<1> *>(adj_smem);
  float *gt = reinterpret_cast<float *>(adj_smem + 2 * sizeof(BinTile<1>));  // dL/df of the bin's points
  const int64_t nbins = bg.nbins;
  const QRec<float> *recs = reinterpret_cast<const QRec<float> *>(w.rec);
  const int cls = bg.cls;
  auto begin = [&](int64_t bb) { return w.offs[bb << cls]; };
  auto count = [&](int64_t bb) { return bb < nbins ? w.offs[(bb + 1) << cls] - begin(bb) : 0u; };
  auto origin = [&](int64_t bb, int og[3]) {
    og[0] = (int)((bb % bg.nb[0]) * BIN_EDGE);
    const int64_t r = bb / bg.nb[0];
    og[1] = (int)((r % bg.nb[1]) * BIN_EDGE);
    og[2] = (int)((r / bg.nb[1]) * BIN_EDGE);
  };
  const int64_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const float ih[3] = {kp.inv_hf[0], kp.inv_hf[1], kp.inv_hf[2]};
  for (int e = threadIdx.x; e < TILE_PTS; e += blockDim.x) gt[e] = 0.f;
  int stage = 0;
  int64_t b = blockIdx.x;
  int og[3];
  if (count(b) > 0) {
    origin(b, og);
    load_bin_tile<1>(g, og, tiles[0]);
  }
  cp_async_commit();
  for (; b < nbins; b += gridDim.x) {
    const int64_t bn = b + gridDim.x;
    if (count(bn) > 0) {
      origin(bn, og);
      load_bin_tile<1>(g, og, tiles[stage ^ 1]);
    }
    cp_async_commit();
    const uint32_t t0 = begin(b), t1 = t0 + count(b);
    cp_async_wait1();
    __syncthreads();
    if (t1 > t0) {
      origin(b, og);
      const float2 *tv = tiles[stage].v;
      for (uint32_t t = t0 + threadIdx.x; t < t1; t += ADJ_THREADS) {
        const QRec<float> r = recs[t];
        const int64_t row = r.row;
        const float dv = dval ? (float)dval[row] : 0.f;
        float dg[3] = {0.f, 0.f, 0.f};
        if (dgrad) {
          dg[0] = (float)dgrad[row * 3];
          dg[1] = (float)dgrad[row * 3 + 1];
          dg[2] = (float)dgrad[row * 3 + 2];
        }
        if (dv != dv) {  // a NaN upstream: no scatter, a NaN query gradient
          if (q_grad) q_grad[row * 3] = q_grad[row * 3 + 1] = q_grad[row * 3 + 2] = qnan();
          continue;
        }
        int64_t c[3];
        unpack_cell<3>(r.cell, c);
        const int base = (((int)c[2] - og[2]) * TILE_EDGE + ((int)c[1] - og[1])) * TILE_EDGE + ((int)c[0] - og[0]);
        float wgt[3][4], d1[3][4], d2[3][4];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          cr_weights<float>(r.f[a], wgt[a]);
          cr_dweights<float>(r.f[a], d1[a]);
          cr_d2weights<float>(r.f[a], d2[a]);
        }
        const float gx = dg[0] * ih[0], gy = dg[1] * ih[1], gz = dg[2] * ih[2];
        float G[3] = {0.f, 0.f, 0.f}, H[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // H: xx yy zz xy xz yz
#pragma unroll
        for (int k = 0; k < 4; ++k) {
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int p = base + (k * TILE_EDGE + j) * TILE_EDGE;
            const float yz = wgt[1][j] * wgt[2][k];
            float f[4];
#pragma unroll
            for (int ii = 0; ii < 4; ++ii) {
              const float2 hl = tv[p + ii];
              f[ii] = hl.x + hl.y;
              const float cval = dv * wgt[0][ii] * yz + gx * d1[0][ii] * yz + gy * wgt[0][ii] * d1[1][j] * wgt[2][k] +
                                 gz * wgt[0][ii] * wgt[1][j] * d1[2][k];
              if (cval != 0.f) atomicAdd(gt + p + ii, cval);
            }
            if (q_grad) {
              const float a0 = wgt[0][0] * f[0] + wgt[0][1] * f[1] + wgt[0][2] * f[2] + wgt[0][3] * f[3];
              const float a1 = d1[0][0] * f[0] + d1[0][1] * f[1] + d1[0][2] * f[2] + d1[0][3] * f[3];
              const float a2 = d2[0][0] * f[0] + d2[0][1] * f[1] + d2[0][2] * f[2] + d2[0][3] * f[3];
              G[0] += a1 * yz;
              G[1] += a0 * d1[1][j] * wgt[2][k];
              G[2] += a0 * wgt[1][j] * d1[2][k];
              H[0] += a2 * yz;
              H[1] += a0 * d2[1][j] * wgt[2][k];
              H[2] += a0 * wgt[1][j] * d2[2][k];
              H[3] += a1 * d1[1][j] * wgt[2][k];
              H[4] += a1 * wgt[1][j] * d1[2][k];
              H[5] += a0 * d1[1][j] * d1[2][k];
            }
          }
        }
        if (q_grad) {
          const float Hm[3][3] = {{H[0], H[3], H[4]}, {H[3], H[1], H[5]}, {H[4], H[5], H[2]}};
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            float v = dv * G[a] * ih[a];
#pragma unroll
            for (int bb = 0; bb < 3; ++bb) v += dg[bb] * Hm[a][bb] * ih[a] * ih[bb];
            q_grad[row * 3 + a] = (double)v;
          }
        }
      }
    }
    __syncthreads();  // the bin's scatter is complete; this stage is refilled two bins later
    if (t1 > t0) {
      // one global atomic per touched point of the bin (each thread clears what it flushes)
      for (int e = threadIdx.x; e < TILE_PTS; e += blockDim.x) {
        const float v = gt[e];
        if (v == 0.f) continue;
        gt[e] = 0.f;
        const int lx = e % TILE_EDGE, rr = e / TILE_EDGE;
        const int64_t x = og[0] + lx, y = og[1] + rr % TILE_EDGE, z = og[2] + rr / TILE_EDGE;
        if (x < nx && y < ny && z < nz) atomicAdd(grid_grad + (z * ny + y) * nx + x, v);
      }
    }
    stage ^= 1;
  }
  // rows outside the volume, NaN rows and the sentinel column: no gradient
  if (q_grad)
    for (int64_t t = (int64_t)w.offs[bg.nsub] + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nq;
         t += (int64_t)gridDim.x * blockDim.x) {
      const int64_t row = recs[t].row;
      q_grad[row * 3] = q_grad[row * 3 + 1] = q_grad[row * 3 + 2] = 0.0;
    }
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
  const BinGeom bg = bin_geom(g, precision);
  cudaStream_t s = (cudaStream_t)stream;
  const arb_query_out out_norm = normalize_out(*out, g->dim);
  out = &out_norm;
  if (cudaMemsetAsync(w.hist, 0, sizeof(uint32_t) * (bg.nsub + 1), s) != cudaSuccess) return ARB_ERR_CUDA;
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
  const BinGeom bg = bin_geom(g, precision);
  cudaStream_t s = (cudaStream_t)stream;
  const arb_query_out out_norm = normalize_out(*out, g->dim);
  out = &out_norm;
  if (cudaMemsetAsync(w.hist, 0, sizeof(uint32_t) * (bg.nsub + 1), s) != cudaSuccess) return ARB_ERR_CUDA;
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

// Bin-grouped adjoint of a 3D scalar interpolant in mixed precision: the
// contract of arb_adjoint (float32 grid_grad, which it accumulates into),
// with caller-owned scratch of arb_adjoint_work_bytes() bytes.
extern "C" size_t arb_adjoint_work_bytes(const arb_grid *g, int64_t nq) {
  if (!g || nq < 0 || g->dim != 3) return 0;
  arb_grid gb = *g;
  gb.bin_shift = 3;
  return carve(nullptr, nullptr, &gb, ARB_PREC_MIXED, nq);
}

extern "C" int arb_adjoint_binned(const arb_grid *g, int32_t precision, const double *q, int64_t nq,
                                  int64_t q_stride, const double *dval, const double *dgrad, void *grid_grad,
                                  double *q_grad, void *work, size_t work_bytes, int32_t *status,
                                  arb_stream_t stream) {
  if (!g || (nq > 0 && !q) || q_stride < 3 || nq < 0 || !grid_grad || !status) return ARB_ERR_INVALID;
  if (g->dim != 3 || g->nfield != 1 || precision != ARB_PREC_MIXED) return ARB_ERR_UNSUPPORTED;
  if (!g->grid32) return ARB_ERR_INVALID;
  if (nq == 0) return ARB_OK;
  if (!work) return ARB_ERR_INVALID;
  if (nq >= (int64_t)1 << 32) return ARB_ERR_UNSUPPORTED;
  for (int a = 0; a < 3; ++a)
    if (g->n[a] - 3 >= ((int64_t)1 << cell_bits<3>())) return ARB_ERR_UNSUPPORTED;
  arb_grid gb = *g;
  gb.bin_shift = 3;  // 8^3-cell bins: the staged tiles' shape
  SortedWork w;
  if (carve(&w, work, &gb, precision, nq) > work_bytes) return ARB_ERR_INVALID;
  const BinGeom bg = bin_geom(&gb, precision);
  cudaStream_t s = (cudaStream_t)stream;
  arb_query_out none{};
  const arb_query_out out = normalize_out(none, 3);
  if (cudaMemsetAsync(w.hist, 0, sizeof(uint32_t) * (bg.nsub + 1), s) != cudaSuccess) return ARB_ERR_CUDA;
  const KParams kp = make_kparams(&gb);
  launch_bin<3, true>(&gb, kp, bg, const_cast<double *>(q), nq, q_stride, 0, &out, status, w, s);
  const size_t smem = 2 * sizeof(BinTile<1>) + sizeof(float) * TILE_PTS;
  static int per_sm[MAX_DEVICES] = {};
  const int dev = current_device();
  if (dev < 0) return ARB_ERR_CUDA;
  if (!per_sm[dev]) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, adjoint_bin_kernel, ADJ_THREADS, smem) != cudaSuccess ||
        n < 1)
      return ARB_ERR_CUDA;
    per_sm[dev] = n;
  }
  int64_t grid = (int64_t)sm_count_sorted() * per_sm[dev];
  if (grid > bg.nbins) grid = bg.nbins;
  if (grid < 1) grid = 1;
  adjoint_bin_kernel<<<(unsigned)grid, ADJ_THREADS, smem, s>>>(gb, kp, bg, nq, dval, dgrad, (float *)grid_grad,
                                                               q_grad, w);
  return launch_status();
}
