// Batched persistent evaluation: many 3D interpolants (fields) and their
// query sets in one launch.  No counterpart in the reference (one object per
// field, ARB:8-621); per field it computes exactly what rQuery1/2/3 do
// (ARB:344-521).
//
// The query sets are concatenated; each is cut into tiles of `tile_rows`
// rows, and tiles are numbered field by field (tile_off is the prefix sum of
// tiles per field).  One CTA per SM slot loops: it takes the next tile from a
// global atomic counter, loads that field's descriptor into shared memory
// and evaluates the tile's rows, on the fly from the grid or from the
// field's coefficient table when the descriptor carries one.  Dynamic
// scheduling keeps uneven fields (1e3 .. 1e6 rows, 16^3 .. 128^3 grids)
// balanced, and fields are processed roughly in order so each field's grid
// stays L2-resident while its tiles run.
#include "eval.cuh"

namespace arb {

// Axis a of the kernel parameters of grid g (make_kparams, on the device).
__device__ void make_kparams_axis(const arb_grid &g, int a, KParams &kp) {
  const double h = a < g.dim ? g.h[a] : 1.0;
  const double lo = a < g.dim ? g.lo[a] : 0.0, hi = a < g.dim ? g.hi[a] : 0.0;
  kp.inv_h[a] = 1.0 / h;
  kp.inv_hf[a] = (float)(1.0 / h);
  kp.ax[a].lo_key = ord_key_bits((unsigned long long)__double_as_longlong(lo));
  kp.ax[a].hi_key = ord_key_bits((unsigned long long)__double_as_longlong(hi));
  kp.ax[a].lo = lo;
  kp.ax[a].h = h;
  kp.ax[a].inv_h = 1.0 / h;
  fast_axis_pairs(kp.ax[a], lo, hi, h);
}

// One warp takes the next tile from the counter and fills descriptor slot
// `slot` (tile, field, grid, kernel parameters): a 32-ary search of the
// fields' first tiles (one load per lane and step), the grid copied by the
// lanes, the parameters of axis a by lane a.
static_assert(sizeof(arb_grid) % 8 == 0, "grid descriptor copied in 8-byte words");
struct TileSlot {
  arb_grid g;
  KParams kp;
  int64_t tile;
  int32_t field;
};

__device__ __forceinline__ void acquire_tile(const arb_grid *grids, int32_t nfields, const int64_t *tile_off,
                                             int64_t ntiles, unsigned long long *counter, TileSlot &ts) {
  const int lane = threadIdx.x & 31;
  unsigned long long t = 0;
  if (lane == 0) t = atomicAdd(counter, 1ULL);
  const int64_t tile = (int64_t)__shfl_sync(0xffffffffu, t, 0);
  if (tile < ntiles) {
    // last field f with tile_off[f] <= tile (tile_off[0] = 0)
    int32_t lo = 0, hi = nfields - 1;
    while (lo < hi) {
      const int32_t step = (hi - lo + 32) / 32;  // ceil((hi - lo + 1) / 32)
      const int32_t piv = lo + lane * step;
      const bool ok = piv <= hi && tile_off[piv] <= tile;
      const unsigned m = __ballot_sync(0xffffffffu, ok);  // lane 0 always holds
      const int last = 31 - __clz(m);
      const int32_t nlo = lo + last * step;
      hi = min(hi, nlo + step - 1);
      lo = nlo;
    }
    const arb_grid &src = grids[lo];
    const uint64_t *w = reinterpret_cast<const uint64_t *>(&src);
    uint64_t *d = reinterpret_cast<uint64_t *>(&ts.g);
    for (int k = lane; k < (int)(sizeof(arb_grid) / 8); k += 32) d[k] = w[k];
    if (lane < 4) make_kparams_axis(src, lane, ts.kp);
    if (lane == 0) ts.field = lo;
  }
  if (lane == 0) ts.tile = tile;
}

template <int F, bool MIXED>
__device__ __forceinline__ void batched_rows(const arb_grid &g, const KParams &kp, double *q, int64_t q0,
                                             int64_t q1, int64_t qs, int wb, const arb_query_out &o,
                                             int32_t *status) {
  using T = typename std::conditional<MIXED, float, double>::type;
  for (int64_t i = q0 + threadIdx.x; i < q1; i += blockDim.x) {
    T fr[3];
    int64_t idx;
    if (!query_prologue<3, F, !MIXED>(g, kp, q, i, qs, wb, o, status, fr, idx)) continue;
    int64_t c[3];
    cell_coords<3>(idx, g, c);
    double val[F], grad[3] = {0, 0, 0};
    if (g.table)
      eval_tab<3, F, MIXED>(g, kp, c, fr, val, grad);
    else
      eval_otf3<F, MIXED>(g, kp, c, fr, val, grad);
    write_vals<3, F>(o, i, val, grad);
  }
}

// FF: the fields' common count (1, 3, 4), compiled alone (no registers or
// spills for the other counts' paths); 0 dispatches on each descriptor's
// count.  Mixed precision: two CTAs per SM (the register file caps the
// on-the-fly evaluator at 16 warps per SM).  Tiles come from an atomic
// counter; warp 0 takes the next tile and fills its descriptor slot while
// the CTA evaluates the current one (two slots), so the dependent loads of
// the take (counter, field search, descriptor) do not hold the CTA at the
// barrier between tiles.
template <bool MIXED, int FF>
__global__ void __launch_bounds__(256, MIXED ? 2 : 1) batched_kernel(const arb_grid *grids, int32_t nfields,
                                                      const int64_t *q_off, const int64_t *tile_off,
                                                      int64_t ntiles, int32_t tile_rows, double *q,
                                                      int64_t qs, int wb, arb_query_out o,
                                                      unsigned long long *counter, int32_t *status) {
  __shared__ TileSlot slots[2];
  if (threadIdx.x < 32) acquire_tile(grids, nfields, tile_off, ntiles, counter, slots[0]);
  __syncthreads();
  for (int cur = 0;; cur ^= 1) {
    const TileSlot &ts = slots[cur];
    const int64_t tile = ts.tile;
    if (tile >= ntiles) break;
    if (threadIdx.x < 32) acquire_tile(grids, nfields, tile_off, ntiles, counter, slots[cur ^ 1]);
    const int32_t f = ts.field;
    const int64_t q0 = q_off[f] + (tile - tile_off[f]) * tile_rows;
    const int64_t q1 = min(q0 + (int64_t)tile_rows, q_off[f + 1]);
    if constexpr (FF != 0) {
      batched_rows<FF, MIXED>(ts.g, ts.kp, q, q0, q1, qs, wb, o, status);
    } else {
      switch (ts.g.nfield) {
        case 1: batched_rows<1, MIXED>(ts.g, ts.kp, q, q0, q1, qs, wb, o, status); break;
        case 3: batched_rows<3, MIXED>(ts.g, ts.kp, q, q0, q1, qs, wb, o, status); break;
        default: batched_rows<4, MIXED>(ts.g, ts.kp, q, q0, q1, qs, wb, o, status); break;
      }
    }
    __syncthreads();  // this slot is refilled two tiles later; the other one is complete
  }
}

static int sm_count() { return device_sms(); }

}  // namespace arb

using namespace arb;

extern "C" int arb_batched_launch(const arb_grid *grids, int32_t nfields, int32_t nfield, const int64_t *q_off,
                                  const int64_t *tile_off, int64_t ntiles, int32_t tile_rows,
                                  int32_t precision, double *q, int64_t q_stride, int32_t q_writeback,
                                  const arb_query_out *out, unsigned long long *counter, int32_t *status,
                                  arb_stream_t stream) {
  if (!grids || nfields <= 0 || !q_off || !tile_off || !out || !counter || tile_rows <= 0 || q_stride < 3)
    return ARB_ERR_INVALID;
  if (nfield != 0 && nfield != 1 && nfield != 3 && nfield != 4) return ARB_ERR_INVALID;
  if (out->oob_rows && !out->oob_count) return ARB_ERR_INVALID;
  if (ntiles == 0) return ARB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const arb_query_out out_norm = normalize_out(*out, 3);
  out = &out_norm;
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s) != cudaSuccess) return ARB_ERR_CUDA;
  const int per_sm = 8;
  int64_t grid = (int64_t)sm_count() * per_sm;
  if (grid > ntiles) grid = ntiles;
#define BK(MX, FF)                                                                                          \
  batched_kernel<MX, FF><<<(unsigned)grid, 256, 0, s>>>(grids, nfields, q_off, tile_off, ntiles, tile_rows, q, \
                                                        q_stride, q_writeback, *out, counter, status)
  const bool mixed = precision == ARB_PREC_MIXED;
  switch (nfield) {
    case 1: if (mixed) BK(true, 1); else BK(false, 1); break;
    case 3: if (mixed) BK(true, 3); else BK(false, 3); break;
    case 4: if (mixed) BK(true, 4); else BK(false, 4); break;
    default: if (mixed) BK(true, 0); else BK(false, 0); break;
  }
#undef BK
  return launch_status();
}
