// Field ingest: axis discovery and scatter of field rows into the z-major
// (x fastest, t slowest) grid.  Replaces the reference's three/four argsorts
// and exact-equality axis scans (src/ARBInterp/ARBInterp.py:528-568,
// 1264-1320).
//
// For a full tensor grid the position of a row in the reference's
// lexicographic sort is ix + nx*(iy + ny*(iz + nz*it)) with i_a the rank of
// the row's a-coordinate among that axis' samples, so the sort becomes an
// index pass (binary search per axis, inverse permutation) plus a gather
// pass with coalesced writes, with no global sort.  Rows that are not a full tensor
// grid (missing or duplicate points, a coordinate not on its axis) set
// ARB_ERR_IRREGULAR_GRID instead of silently producing garbage.
#include <climits>

#include "arb_common.cuh"

namespace arb {

// Order-preserving map of a double onto uint64 (for atomicMin).
__device__ __forceinline__ unsigned long long ord_key(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}

template <typename TF>
__device__ __forceinline__ double ld(const TF *p) { return (double)p[0]; }

struct AxesWork {
  unsigned long long minkey[4];
  unsigned long long count[4];
};

__global__ void axes_init_kernel(AxesWork *w) {
  if (threadIdx.x < 4) {
    w->minkey[threadIdx.x] = ~0ULL;
    w->count[threadIdx.x] = 0ULL;
  }
}

// Appends every row that lies on an axis line through row 0 (all other
// coordinates equal to row 0's).  For a full tensor grid each such line
// carries exactly that axis' samples, the same set the reference reads off
// the lines through the first sorted row; the index pass then checks that
// every row lies on the grid.  NaN coordinates mark the grid irregular.
template <typename TF>
__global__ void axes_collect_kernel(const TF *field, int64_t npts, int ncol, int dim, AxesWork *w,
                                    double *raw_axes, int64_t cap, int32_t *status) {
  double r0[4];
  for (int a = 0; a < dim; ++a) r0[a] = ld(field + a);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v[4];
    int neq = 0, which = -1;
    bool bad = false;
    for (int a = 0; a < dim; ++a) {
      v[a] = ld(field + i * ncol + a);
      bad |= (v[a] != v[a]);
      if (v[a] != r0[a]) {
        ++neq;
        which = a;
      }
    }
    if (bad) set_status(status, ARB_ERR_IRREGULAR_GRID);
    if (neq > 1 || bad) continue;
    // neq == 0: row 0 itself belongs to every axis line
    for (int a = 0; a < dim; ++a) {
      if (neq == 1 && a != which) continue;
      const unsigned long long slot = atomicAdd(&w->count[a], 1ULL);
      if ((int64_t)slot < cap)
        raw_axes[a * cap + slot] = v[a];
      else
        set_status(status, ARB_ERR_CAPACITY);
    }
  }
}

// Rank sort of each (short) axis list; equal samples mean duplicate points.
__global__ void axes_sort_kernel(const double *raw_axes, const AxesWork *w, int dim, int64_t cap,
                                 double *axis_out, int64_t *axis_count, int32_t *status) {
  const int a = blockIdx.y;
  const int64_t n = (int64_t)min(w->count[a], (unsigned long long)cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) axis_count[a] = (int64_t)w->count[a];
  const double *src = raw_axes + a * cap;
  extern __shared__ double tile[];
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const double v = i < n ? src[i] : 0.0;
    int64_t rank = 0;
    bool dup = false;
    for (int64_t t0 = 0; t0 < n; t0 += blockDim.x) {
      __syncthreads();
      if (t0 + threadIdx.x < n) tile[threadIdx.x] = src[t0 + threadIdx.x];
      __syncthreads();
      const int64_t lim = min((int64_t)blockDim.x, n - t0);
      if (i < n) {
        for (int64_t j = 0; j < lim; ++j) {
          const double u = tile[j];
          rank += (u < v);
          dup |= (u == v) && (t0 + j != i);
        }
      }
    }
    if (i < n) {
      if (dup) set_status(status, ARB_ERR_IRREGULAR_GRID);
      axis_out[a * cap + rank] = v;
    }
  }
}

// Binary search of an ordered key among n sorted axis keys; -1 if absent.
__device__ __forceinline__ int64_t find_key(const unsigned long long *keys, int64_t n,
                                            unsigned long long k) {
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < k)
      lo = mid + 1;
    else
      hi = mid;
  }
  return keys[lo] == k ? lo : -1;
}

// Pass 1 (row order): grid slot of every row from exact axis-key lookups
// (integer compares on order-preserving keys; no float64 pipe work), and the
// inverse permutation inv[slot] = row.  inv is 4 bytes per point and stays
// L2-resident while rows land in scattered slots; a second claim of a slot
// is a duplicate point.
template <typename TF>
__global__ void __launch_bounds__(256) ingest_index_kernel(const TF *field, int64_t npts, int ncol,
                                                           int dim, const double *axes, int64_t cap,
                                                           int64_t n0, int64_t n1, int64_t n2,
                                                           int64_t n3, uint32_t *inv,
                                                           int32_t *status) {
  extern __shared__ unsigned long long skeys[];
  const int64_t nn[4] = {n0, n1, n2, n3};
  int64_t off[4];
  int64_t tot = 0;
  for (int a = 0; a < dim; ++a) {
    off[a] = tot;
    tot += nn[a];
  }
  for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) {
    int a = 0;
    while (a + 1 < dim && e >= off[a + 1]) ++a;
    skeys[e] = ord_key(axes[a * cap + (e - off[a])]);
  }
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts;
       i += (int64_t)gridDim.x * blockDim.x) {
    const TF *row = field + i * ncol;
    int64_t dest = 0;
    bool ok = true;
    // Rows of a warp usually share all but their fastest-varying coordinate:
    // when a coordinate is equal across the warp, one lane searches for it.
    const unsigned act = __activemask();
    const int leader = __ffs(act) - 1;
    const int lane = threadIdx.x & 31;
    for (int a = dim - 1; a >= 0; --a) {
      const unsigned long long key = ord_key((double)row[a]);
      const unsigned long long k0 = __shfl_sync(act, key, leader);
      int64_t r;
      if (__all_sync(act, key == k0)) {
        r = lane == leader ? find_key(skeys + off[a], nn[a], key) : 0;
        r = __shfl_sync(act, r, leader);
      } else {
        r = find_key(skeys + off[a], nn[a], key);
      }
      ok &= (r >= 0);
      dest = dest * nn[a] + (r < 0 ? 0 : r);
    }
    if (!ok) {
      set_status(status, ARB_ERR_IRREGULAR_GRID);
      continue;
    }
    if (atomicExch(&inv[dest], (uint32_t)i) != 0xffffffffu) set_status(status, ARB_ERR_IRREGULAR_GRID);
  }
}

// field value as float64 without the float64 pipe
template <typename TF>
__device__ __forceinline__ double to_f64(TF v) {
  if constexpr (sizeof(TF) == 8)
    return (double)v;
  else
    return f2d_exact(v);
}

// ||(bx, by, bz)|| for float64 components as a float32 pair hi + lo, in
// float32 arithmetic only, and each component rounded to float32 (ch, the
// grid's hi of that component).  The components are rescaled by the power of
// two of the largest (exact, on the exponent bits) and split on their bits
// (split_f32_trunc_bits: h + l is the scaled component to 2^-47 relative).  Then
// double-float: error-free squares via FMA, two-sum accumulation, one Newton
// correction of the float32 square root.  Accurate to ~2^-45 relative, below
// the pair's own resolution.  ch is h rounded to nearest-even on the dropped
// bits, rescaled (exact where the component and its scaled value are normal
// float32 numbers; other components take split_f32).  Scaled components
// below 2^-74 add nothing to the norm.  Returns false (caller takes the
// float64 norm) for a largest component outside [2^-90, 2^90], zeros,
// infinities and NaN.
__device__ __forceinline__ bool norm_f32pair(double bx, double by, double bz, float &hi, float &lo,
                                             float ch[3]) {
  const long long bb[3] = {__double_as_longlong(bx), __double_as_longlong(by), __double_as_longlong(bz)};
  int ex[3], em = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    ex[a] = (int)((bb[a] >> 52) & 0x7ff);
    em = max(em, ex[a]);
  }
  if (em < 1023 - 90 || em > 1023 + 90) return false;
  const int sc = em - 1023;
  const float f = __int_as_float((sc + 127) << 23);        // 2^sc, exact rescale
  float h[3], l[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int es = ex[a] - sc;                              // biased exponent of the scaled component
    if (es >= 949) {
      split_f32_trunc_bits((unsigned long long)(bb[a] - ((long long)sc << 52)), h[a], l[a]);
    } else {
      h[a] = 0.f;
      l[a] = 0.f;
    }
    if (es >= 949 && ex[a] >= 897) {
      // round h to nearest even on the dropped bits (the same bits scaled or not)
      const unsigned rem = (unsigned)bb[a] & 0x1fffffffu;
      const unsigned hb = __float_as_uint(h[a]);
      const bool up = rem > 0x10000000u || (rem == 0x10000000u && (hb & 1u));
      ch[a] = __uint_as_float(hb + (up ? 1u : 0u)) * f;
    } else {
      float t;
      split_f32(__longlong_as_double(bb[a]), ch[a], t);
    }
  }
  float s = 0.f, e = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float p = __fmul_rn(h[a], h[a]);
    const float pe = __fmaf_rn(h[a], h[a], -p);           // exact error of the square
    const float t = __fadd_rn(s, p);                       // two-sum s + p
    const float bp = __fsub_rn(t, s);
    const float te = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    e = __fadd_rn(e, __fadd_rn(te, __fmaf_rn(2.f * h[a], l[a], pe)));
    s = t;
  }
  const float S = __fadd_rn(s, e), Slo = __fsub_rn(e, __fsub_rn(S, s));   // renormalise
  const float r = __fsqrt_rn(S);                           // S in [1, 12)
  const float res = __fadd_rn(__fmaf_rn(-r, r, S), Slo);   // S + Slo - r^2
  const float rc = __fmul_rn(res, __fdividef(0.5f, r));
  const float h0 = __fadd_rn(r, rc);
  hi = h0 * f;
  lo = __fsub_rn(rc, __fsub_rn(h0, r)) * f;
  return true;
}

// Per-mode interpolated fields of one row written to grid slot `dest`:
// grid64, grid32 (hi/lo split, layout of g32_load in arb_common.cuh) and the
// raw value columns.  With grid32 (mixed precision) and float64 components
// the norm comes from norm_f32pair (float32 pipe); otherwise it is the
// float64 norm NumPy computes.
template <typename TF, int KIND>
__device__ __forceinline__ void write_slot(const TF *row, int64_t dest, int64_t npts, int dim, double *grid64,
                                           float *grid32, double *raw_out) {
  constexpr int F = (KIND == ARB_KIND_VECTOR) ? 3 : (KIND == ARB_KIND_BOTH ? 4 : 1);
  double out[4];
  float nhi = 0.f, nlo = 0.f, chi[3];
  bool nsplit = false;   // norm pair and component hi from norm_f32pair
  if (KIND == ARB_KIND_SCALAR) {
    out[0] = to_f64(row[dim]);
  } else {
    const TF bx = row[dim], by = row[dim + 1], bz = row[dim + 2];
    out[0] = to_f64(bx);
    out[1] = to_f64(by);
    out[2] = to_f64(bz);
    if (KIND == ARB_KIND_NORM || KIND == ARB_KIND_BOTH) {
      // ||B|| at the grid point in the field's own precision, as NumPy's
      // norm evaluates it: sqrt((bx*bx + by*by) + bz*bz).
      double nrm;
      if (sizeof(TF) == 8 && grid32 && norm_f32pair(out[0], out[1], out[2], nhi, nlo, chi)) {
        // the float64 value is needed only for grid64 (grid32 takes the pair)
        nrm = grid64 ? f2d_exact(nhi) + f2d_exact(nlo) : 0.0;
        nsplit = true;
      } else if (sizeof(TF) == 8) {
        nrm = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn((double)bx, (double)bx), __dmul_rn((double)by, (double)by)),
                                   __dmul_rn((double)bz, (double)bz)));
      } else {
        nrm = f2d_exact(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn((float)bx, (float)bx), __fmul_rn((float)by, (float)by)),
                                             __fmul_rn((float)bz, (float)bz))));
      }
      if (KIND == ARB_KIND_NORM)
        out[0] = nrm;
      else
        out[3] = nrm;
    }
    if (raw_out) {
      raw_out[dest * 3 + 0] = (double)bx;
      raw_out[dest * 3 + 1] = (double)by;
      raw_out[dest * 3 + 2] = (double)bz;
    }
  }
  if (grid64) {
    if (F == 4) {
      reinterpret_cast<double2 *>(grid64)[dest * 2] = make_double2(out[0], out[1 % F]);
      reinterpret_cast<double2 *>(grid64)[dest * 2 + 1] = make_double2(out[2 % F], out[3 % F]);
    } else {
#pragma unroll
      for (int f = 0; f < F; ++f) grid64[dest * F + f] = out[f];
    }
  }
  if (grid32) {
    float hi[4], lo[4];
#pragma unroll
    for (int f = 0; f < F; ++f) {
      if (nsplit && f == F - 1) {
        hi[f] = nhi;
        lo[f] = nlo;
      } else if (nsplit && F == 4) {
        hi[f] = chi[f];   // components: hi only
        lo[f] = 0.f;
      } else {
        split_f32(out[f], hi[f], lo[f]);
      }
    }
    if (F == 4) {
      reinterpret_cast<float4 *>(grid32)[dest] = make_float4(hi[0], hi[1 % F], hi[2 % F], hi[3 % F]);
      grid32[npts * 4 + dest] = lo[3 % F];
    } else if (F == 3) {
      reinterpret_cast<float4 *>(grid32)[dest] = make_float4(hi[0], hi[1 % F], hi[2 % F], 0.f);
    } else {
      reinterpret_cast<float2 *>(grid32)[dest] = make_float2(hi[0], lo[0]);
    }
  }
  if (KIND == ARB_KIND_SCALAR && raw_out) raw_out[dest] = out[0];
}

// Pass 2 (grid order): each slot reads its row and writes the per-mode
// interpolated fields with coalesced stores.
template <typename TF, int KIND>
__global__ void __launch_bounds__(256) ingest_gather_kernel(const TF *field, int64_t npts, int ncol,
                                                            int dim, const uint32_t *inv,
                                                            double *grid64, float *grid32,
                                                            double *raw_out, int32_t *status) {
  for (int64_t dest = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; dest < npts;
       dest += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t src = inv[dest];
    if (src == 0xffffffffu) {
      set_status(status, ARB_ERR_IRREGULAR_GRID);
      continue;
    }
    write_slot<TF, KIND>(field + (int64_t)src * ncol, dest, npts, dim, grid64, grid32, raw_out);
  }
}

// ---- single-pass ingest of rows in meshgrid order ---------------------------
// Rows in meshgrid order are lexicographic over the axes in some axis order,
// each axis ascending or descending: row = sum_a stride_a * j_a with j_a the
// sample's position along the row order (i_a or n_a - 1 - i_a) and the
// strides the running products of the axis lengths.  NumPy's meshgrid +
// reshape and the reference's own sort (ARB:530) produce such orders.  The
// probe reads the axes straight off the lines through row 0 (the lines the
// axis pass collects); the gather then maps every grid slot to its row
// arithmetically and checks the row's coordinates against the slot's axis
// samples, so a field in any other order is detected, never misplaced.
struct OrderWork {
  int64_t stride[4];  // signed: negative for an axis descending along the rows
  int64_t n[4];
  int32_t ok;
};

template <typename TF>
__global__ void __launch_bounds__(256) ordered_probe_kernel(const TF *field, int64_t npts, int ncol, int dim,
                                                            int64_t cap, double *axis_out, int64_t *axis_count,
                                                            OrderWork *w, int32_t *status) {
  __shared__ long long first_stop;
  const int tid = threadIdx.x;
  if (tid == 0)  // axes the probe does not find keep a count of 0 (the caller need not clear them)
    for (int a = 0; a < dim; ++a) axis_count[a] = 0;
  double r0[4];
  for (int a = 0; a < dim; ++a) r0[a] = (double)field[a];
  int64_t stride = 1;
  unsigned used = 0;
  bool ok = true;
  for (int step = 0; step < dim && ok; ++step) {
    if (stride >= npts) {
      ok = false;
      break;
    }
    // the one axis that changes between row 0 and row `stride`
    int which = -1, nd = 0;
    for (int a = 0; a < dim; ++a) {
      const double v = (double)field[stride * ncol + a];
      if (!(v == r0[a])) {
        ++nd;
        which = a;
      }
    }
    if (nd != 1 || ((used >> which) & 1u)) {
      ok = false;
      break;
    }
    const bool asc = (double)field[stride * ncol + which] > r0[which];
    // line length: first k >= 1 whose row leaves the line through row 0 or
    // breaks the strict monotonicity of the axis samples
    int64_t n = -1;
    for (int64_t base = 1; base <= cap + 1; base += blockDim.x) {
      if (tid == 0) first_stop = LLONG_MAX;
      __syncthreads();
      const int64_t k = base + tid;
      bool stop = k * stride >= npts;
      if (!stop) {
        const TF *row = field + k * stride * ncol;
        for (int a = 0; a < dim; ++a)
          if (a != which && !((double)row[a] == r0[a])) stop = true;
        const double cur = (double)row[which], prev = (double)field[(k - 1) * stride * ncol + which];
        if (!(asc ? cur > prev : cur < prev)) stop = true;
      }
      if (stop) atomicMin(&first_stop, (long long)k);
      __syncthreads();
      const long long fs = first_stop;
      __syncthreads();
      if (fs != LLONG_MAX) {
        n = fs;
        break;
      }
    }
    if (n < 4 || n > cap) {
      ok = false;
      break;
    }
    for (int64_t k = tid; k < n; k += blockDim.x)
      axis_out[which * cap + (asc ? k : n - 1 - k)] = (double)field[k * stride * ncol + which];
    if (tid == 0) {
      w->stride[which] = asc ? stride : -stride;
      w->n[which] = n;
      axis_count[which] = n;
    }
    used |= 1u << which;
    stride *= n;
  }
  if (ok && stride != npts) ok = false;
  if (tid == 0) {
    w->ok = ok ? 1 : 0;
    if (!ok) set_status(status, ARB_ERR_IRREGULAR_GRID);
  }
}

// One field row into registers: 16-byte loads when the row is 16-byte
// aligned (float64 rows of an even column count), scalar loads otherwise.
template <typename TF, int NC>
__device__ __forceinline__ void load_field_row(const TF *row, TF v[NC]) {
  if constexpr (sizeof(TF) == 8 && NC % 2 == 0) {
    const double2 *r2 = reinterpret_cast<const double2 *>(row);
#pragma unroll
    for (int k = 0; k < NC / 2; ++k) {
      const double2 t = __ldg(r2 + k);
      v[2 * k] = t.x;
      v[2 * k + 1] = t.y;
    }
  } else if constexpr (sizeof(TF) == 4 && NC == 4) {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(row));
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
  } else {
#pragma unroll
    for (int k = 0; k < NC; ++k) v[k] = __ldg(row + k);
  }
}

template <typename TF, int KIND, int DIM>
__global__ void __launch_bounds__(256) ordered_gather_kernel(const TF *field, int64_t npts, int ncol,
                                                             const double *axes, int64_t cap, const OrderWork *w,
                                                             double *grid64, float *grid32, double *raw_out,
                                                             int32_t *status) {
  // rows whose fastest axis is x: slot order is row order (up to direction),
  // both sides coalesced; other orders go through ordered_tile_kernel
  if (!w->ok || (w->stride[0] != 1 && w->stride[0] != -1)) return;
  uint32_t nn[DIM];
  int64_t st[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    nn[a] = (uint32_t)w->n[a];
    st[a] = w->stride[a];
  }
  for (int64_t dest = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; dest < npts;
       dest += (int64_t)gridDim.x * blockDim.x) {
    uint32_t u = (uint32_t)dest;  // npts < 2^32
    int64_t src = 0;
    uint32_t idx[DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      const uint32_t q = a + 1 < DIM ? u / nn[a] : 0u;
      idx[a] = u - q * nn[a];
      u = q;
      src += st[a] > 0 ? (int64_t)idx[a] * st[a] : (int64_t)(nn[a] - 1u - idx[a]) * (-st[a]);
    }
    constexpr int NC = DIM + (KIND == ARB_KIND_SCALAR ? 1 : 3);
    TF row[NC];
    load_field_row<TF, NC>(field + src * NC, row);
    bool ok = true;
#pragma unroll
    for (int a = 0; a < DIM; ++a)  // bitwise, as the general path's key lookup
      ok &= __double_as_longlong(to_f64(row[a])) == __double_as_longlong(__ldg(axes + a * cap + idx[a]));
    if (!ok) set_status(status, ARB_ERR_IRREGULAR_GRID);
    write_slot<TF, KIND>(row, dest, npts, DIM, grid64, grid32, raw_out);
  }
}

// Rows whose fastest axis S is not x (e.g. meshgrid(..., indexing='ij') with
// x slowest): consecutive grid slots come from rows |stride_x| apart, so a
// direct gather reads one scattered row per slot.  Instead a CTA takes a
// 32 (x) x 16 (S) tile at fixed other coordinates, reads its 512 rows with
// consecutive threads on consecutive rows (S runs along the rows: 16 rows
// per half-warp), keeps them in shared memory, and writes the slots with
// consecutive threads on consecutive x.  Persistent over tiles.  The kernel
// is bound by instruction issue and latency, so the indices are 32-bit
// (npts < 2^32), a tile's digits (x tile, S tile, the other axes) advance by
// the grid stride with carries instead of being divided out of the tile
// number, and the tile is 16 rows deep along S so that five CTAs fit an SM
// (26 KB each for six float64 columns; 32 x 32 tiles: four, 250 against
// 223 us at 256^3).
constexpr int OT = 32, OS = 16;

template <typename TF, int KIND, int DIM>
__global__ void __launch_bounds__(256) ordered_tile_kernel(const TF *field, int64_t npts, const double *axes,
                                                           int64_t cap, const OrderWork *w, double *grid64,
                                                           float *grid32, double *raw_out, int32_t *status) {
  constexpr int NC = DIM + (KIND == ARB_KIND_SCALAR ? 1 : 3);
  if (!w->ok || w->stride[0] == 1 || w->stride[0] == -1) return;
  extern __shared__ __align__(16) unsigned char ot_smem[];
  // one plane per column (structure of arrays): the load phase writes
  // consecutive words, the write phase reads words OS + 1 apart (odd), both
  // without bank conflicts beyond the two wavefronts 8-byte values need
  TF(*tile)[OT][OS + 1] = reinterpret_cast<TF(*)[OT][OS + 1]>(ot_smem);
  uint32_t nn[DIM], sa[DIM], ps[DIM];
  bool neg[DIM];
  int S = 1;
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    const int64_t st = w->stride[a];
    nn[a] = (uint32_t)w->n[a];
    neg[a] = st < 0;
    sa[a] = (uint32_t)(st < 0 ? -st : st);
    if (st == 1 || st == -1) S = a;
  }
  ps[0] = 1;  // slot strides (x fastest)
#pragma unroll
  for (int a = 1; a < DIM; ++a) ps[a] = ps[a - 1] * nn[a - 1];
  // digits of a tile number: x tile, S tile, then the other axes (slowest last)
  uint32_t rad[DIM];
  int ax[DIM];  // axis of digit k >= 2
  rad[0] = (nn[0] + OT - 1) / OT;
  rad[1] = (nn[S] + OS - 1) / OS;
  uint32_t ntiles = rad[0] * rad[1];
  {
    int k = 2;
#pragma unroll
    for (int a = 1; a < DIM; ++a)
      if (a != S) {
        ax[k] = a;
        rad[k] = nn[a];
        ntiles *= nn[a];
        ++k;
      }
  }
  uint32_t dig[DIM], step[DIM];
  {
    uint32_t t = blockIdx.x, g = gridDim.x;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      dig[k] = k + 1 < DIM ? t % rad[k] : t;
      step[k] = k + 1 < DIM ? g % rad[k] : g;
      t /= rad[k];
      g /= rad[k];
    }
  }
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    uint32_t i[DIM];
#pragma unroll
    for (int k = 2; k < DIM; ++k) i[ax[k]] = dig[k];
    // load: consecutive threads read consecutive rows (along S)
#pragma unroll
    for (int e = threadIdx.x; e < OT * OS; e += 256) {
      const int k = e / OS, j = e % OS;
      i[0] = dig[0] * OT + k;
      i[S] = dig[1] * OS + j;
      if (i[0] < nn[0] && i[S] < nn[S]) {
        uint32_t src = 0;
#pragma unroll
        for (int a = 0; a < DIM; ++a) src += (neg[a] ? nn[a] - 1u - i[a] : i[a]) * sa[a];
        TF v[NC];
        load_field_row<TF, NC>(field + (size_t)src * NC, v);
#pragma unroll
        for (int c = 0; c < NC; ++c) tile[c][k][j] = v[c];
      }
    }
    __syncthreads();
    // write: consecutive threads write consecutive slots (along x)
#pragma unroll
    for (int e = threadIdx.x; e < OT * OS; e += 256) {
      const int k = e / OT, tx = e % OT;
      i[0] = dig[0] * OT + tx;
      i[S] = dig[1] * OS + k;
      if (i[0] < nn[0] && i[S] < nn[S]) {
        TF row[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) row[c] = tile[c][tx][k];
        uint32_t dest = 0;
        bool ok = true;
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
          dest += i[a] * ps[a];
          ok &= __double_as_longlong(to_f64(row[a])) == __double_as_longlong(__ldg(axes + a * cap + i[a]));
        }
        if (!ok) set_status(status, ARB_ERR_IRREGULAR_GRID);
        write_slot<TF, KIND>(row, dest, npts, DIM, grid64, grid32, raw_out);
      }
    }
    __syncthreads();
    // next tile: add the grid stride digit by digit (each digit stays below
    // twice its radix, so one conditional subtraction carries it)
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      dig[k] += step[k] + c;
      if (k + 1 < DIM) {
        c = dig[k] >= rad[k] ? 1u : 0u;
        dig[k] -= c ? rad[k] : 0u;
      }
    }
  }
}

template <typename TF, int KIND, int DIM>
static void launch_ordered_tile(const void *field, int64_t npts, const double *axes, int64_t cap,
                                const OrderWork *w, double *grid64, float *grid32, double *raw_out, int32_t *status,
                                cudaStream_t s) {
  constexpr int NC = DIM + (KIND == ARB_KIND_SCALAR ? 1 : 3);
  const size_t smem = sizeof(TF) * OT * (OS + 1) * NC;
  static int per_sm[MAX_DEVICES] = {};  // resident CTAs per SM (registers and shared memory)
  const int dev = current_device();
  if (dev >= 0 && !per_sm[dev]) {
    cudaFuncSetAttribute(ordered_tile_kernel<TF, KIND, DIM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ordered_tile_kernel<TF, KIND, DIM>, 256, smem) !=
            cudaSuccess ||
        n < 1)
      n = 4;
    per_sm[dev] = n;
  }
  const int sms = device_sms();
  int64_t grid = (int64_t)sms * (dev >= 0 ? per_sm[dev] : 4);
  const int64_t tiles_max = npts / (OT * 4) + 1;  // no more CTAs than that (each loops over the tiles)
  if (grid > tiles_max) grid = tiles_max;
  ordered_tile_kernel<TF, KIND, DIM><<<(unsigned)grid, 256, smem, s>>>((const TF *)field, npts, axes, cap, w,
                                                                       grid64, grid32, raw_out, status);
}

static int grid_blocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 64) b = 152 * 64;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace arb

using namespace arb;

extern "C" size_t arb_ingest_axes_work_bytes(int32_t dim) {
  (void)dim;
  return (sizeof(AxesWork) > sizeof(OrderWork) ? sizeof(AxesWork) : sizeof(OrderWork)) + 256;
}

extern "C" int arb_ingest_axes(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                               int32_t dim, int64_t axis_cap, double *axis_out, int64_t *axis_count,
                               void *work, size_t work_bytes, int32_t *status, arb_stream_t stream) {
  if (!field || !axis_out || !axis_count || !work || !status) return ARB_ERR_INVALID;
  if ((dim != 3 && dim != 4) || npts <= 0 || ncol < dim + 1 || axis_cap <= 0 ||
      axis_cap > ARB_MAX_AXIS_CAP || work_bytes < arb_ingest_axes_work_bytes(dim))
    return ARB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  AxesWork *w = (AxesWork *)work;
  // The unsorted axis lists are staged in the second half of axis_out
  // (callers allocate 2 * dim * axis_cap doubles).
  double *raw = axis_out + (int64_t)dim * axis_cap;
  axes_init_kernel<<<1, 32, 0, s>>>(w);
  const int T = 256;
  const int B = grid_blocks(npts, T);
  if (field_is_f32) {
    axes_collect_kernel<float>
        <<<B, T, 0, s>>>((const float *)field, npts, ncol, dim, w, raw, axis_cap, status);
  } else {
    axes_collect_kernel<double>
        <<<B, T, 0, s>>>((const double *)field, npts, ncol, dim, w, raw, axis_cap, status);
  }
  int sb = (int)((axis_cap + T - 1) / T);
  if (sb > 1024) sb = 1024;
  axes_sort_kernel<<<dim3(sb, dim), T, T * sizeof(double), s>>>(raw, w, dim, axis_cap, axis_out,
                                                                axis_count, status);
  return launch_status();
}

extern "C" int arb_ingest_scatter(const void *field, int32_t field_is_f32, int64_t npts,
                                  int32_t ncol, int32_t dim, const double *axes, int64_t axis_cap,
                                  const int64_t *n, int32_t kind, double *grid64, float *grid32,
                                  double *raw_out, uint32_t *claim, int32_t *status,
                                  arb_stream_t stream) {
  if (!field || !axes || !n || (!grid64 && !grid32) || !claim || !status) return ARB_ERR_INVALID;
  if (dim != 3 && dim != 4) return ARB_ERR_INVALID;
  int64_t prod = 1;
  for (int a = 0; a < dim; ++a) {
    if (n[a] < 4 || n[a] > axis_cap) return ARB_ERR_INVALID;
    prod *= n[a];
  }
  if (prod != npts) return ARB_ERR_IRREGULAR_GRID;
  const int nval = ncol - dim;
  if (kind == ARB_KIND_SCALAR ? nval != 1 : nval != 3) return ARB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  if (npts >= (int64_t)0xffffffffLL) return ARB_ERR_UNSUPPORTED;
  if (cudaMemsetAsync(claim, 0xff, sizeof(uint32_t) * npts, s) != cudaSuccess) return ARB_ERR_CUDA;
  const int T = 256;
  const int B = grid_blocks(npts, T);
  const int64_t n3 = dim == 4 ? n[3] : 1;
  int64_t tot = 0;
  for (int a = 0; a < dim; ++a) tot += n[a];
  const size_t ksm = sizeof(unsigned long long) * (size_t)tot;
  if (ksm > 200 * 1024) return ARB_ERR_UNSUPPORTED;
  if (ksm > 48 * 1024) {
    cudaFuncSetAttribute(ingest_index_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ksm);
    cudaFuncSetAttribute(ingest_index_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ksm);
  }
  if (field_is_f32)
    ingest_index_kernel<float><<<B, T, ksm, s>>>((const float *)field, npts, ncol, dim, axes, axis_cap, n[0],
                                                 n[1], n[2], n3, claim, status);
  else
    ingest_index_kernel<double><<<B, T, ksm, s>>>((const double *)field, npts, ncol, dim, axes, axis_cap,
                                                  n[0], n[1], n[2], n3, claim, status);
#define ARB_GATHER(TF, K)                                                                             \
  ingest_gather_kernel<TF, K><<<B, T, 0, s>>>((const TF *)field, npts, ncol, dim, claim, grid64, grid32, \
                                              raw_out, status)
#define ARB_GATHER_KIND(TF)                                         \
  switch (kind) {                                                   \
    case ARB_KIND_SCALAR: ARB_GATHER(TF, ARB_KIND_SCALAR); break;   \
    case ARB_KIND_VECTOR: ARB_GATHER(TF, ARB_KIND_VECTOR); break;   \
    case ARB_KIND_NORM: ARB_GATHER(TF, ARB_KIND_NORM); break;       \
    case ARB_KIND_BOTH: ARB_GATHER(TF, ARB_KIND_BOTH); break;       \
    default: return ARB_ERR_INVALID;                                \
  }
  if (field_is_f32) {
    ARB_GATHER_KIND(float)
  } else {
    ARB_GATHER_KIND(double)
  }
#undef ARB_GATHER_KIND
#undef ARB_GATHER
  return launch_status();
}

static int ordered_args_ok(const void *field, int64_t npts, int32_t ncol, int32_t dim, int32_t kind,
                           int64_t axis_cap, size_t work_bytes) {
  if (!field) return ARB_ERR_INVALID;
  if ((dim != 3 && dim != 4) || npts <= 0 || axis_cap <= 0 || axis_cap > ARB_MAX_AXIS_CAP ||
      work_bytes < arb_ingest_axes_work_bytes(dim))
    return ARB_ERR_INVALID;
  const int nval = ncol - dim;
  if (kind == ARB_KIND_SCALAR ? nval != 1 : nval != 3) return ARB_ERR_INVALID;
  if (npts >= (int64_t)0xffffffffLL) return ARB_ERR_UNSUPPORTED;
  return ARB_OK;
}

static void launch_ordered_probe(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol, int32_t dim,
                                 int64_t axis_cap, double *axis_out, int64_t *axis_count, OrderWork *w,
                                 int32_t *status, cudaStream_t s) {
  if (field_is_f32)
    ordered_probe_kernel<float><<<1, 256, 0, s>>>((const float *)field, npts, ncol, dim, axis_cap, axis_out,
                                                  axis_count, w, status);
  else
    ordered_probe_kernel<double><<<1, 256, 0, s>>>((const double *)field, npts, ncol, dim, axis_cap, axis_out,
                                                   axis_count, w, status);
}

static int launch_ordered_fill(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol, int32_t dim,
                               int32_t kind, int64_t axis_cap, const double *axis_out, const OrderWork *w,
                               double *grid64, float *grid32, double *raw_out, int32_t *status, cudaStream_t s) {
  const int T = 256;
  const int B = grid_blocks(npts, T);
#define ARB_OGATHER(TF, K)                                                                                 \
  if (dim == 3) {                                                                                          \
    ordered_gather_kernel<TF, K, 3><<<B, T, 0, s>>>((const TF *)field, npts, ncol, axis_out, axis_cap, w,    \
                                                    grid64, grid32, raw_out, status);                        \
    launch_ordered_tile<TF, K, 3>(field, npts, axis_out, axis_cap, w, grid64, grid32, raw_out, status, s); \
  } else {                                                                                                 \
    ordered_gather_kernel<TF, K, 4><<<B, T, 0, s>>>((const TF *)field, npts, ncol, axis_out, axis_cap, w,    \
                                                    grid64, grid32, raw_out, status);                        \
    launch_ordered_tile<TF, K, 4>(field, npts, axis_out, axis_cap, w, grid64, grid32, raw_out, status, s); \
  }
#define ARB_OGATHER_KIND(TF)                                         \
  switch (kind) {                                                    \
    case ARB_KIND_SCALAR: ARB_OGATHER(TF, ARB_KIND_SCALAR); break;   \
    case ARB_KIND_VECTOR: ARB_OGATHER(TF, ARB_KIND_VECTOR); break;   \
    case ARB_KIND_NORM: ARB_OGATHER(TF, ARB_KIND_NORM); break;       \
    case ARB_KIND_BOTH: ARB_OGATHER(TF, ARB_KIND_BOTH); break;       \
    default: return ARB_ERR_INVALID;                                 \
  }
  if (field_is_f32) {
    ARB_OGATHER_KIND(float)
  } else {
    ARB_OGATHER_KIND(double)
  }
#undef ARB_OGATHER_KIND
#undef ARB_OGATHER
  return ARB_OK;
}

extern "C" int arb_ingest_ordered(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                                  int32_t dim, int32_t kind, int64_t axis_cap, double *axis_out,
                                  int64_t *axis_count, double *grid64, float *grid32, double *raw_out,
                                  void *work, size_t work_bytes, int32_t *status, arb_stream_t stream) {
  if (!axis_out || !axis_count || (!grid64 && !grid32) || !work || !status) return ARB_ERR_INVALID;
  int rc = ordered_args_ok(field, npts, ncol, dim, kind, axis_cap, work_bytes);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  OrderWork *w = (OrderWork *)work;
  launch_ordered_probe(field, field_is_f32, npts, ncol, dim, axis_cap, axis_out, axis_count, w, status, s);
  rc = launch_ordered_fill(field, field_is_f32, npts, ncol, dim, kind, axis_cap, axis_out, w, grid64, grid32,
                           raw_out, status, s);
  return rc ? rc : launch_status();
}

extern "C" int arb_ingest_ordered_probe(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                                        int32_t dim, int32_t kind, int64_t axis_cap, double *axis_out,
                                        int64_t *axis_count, void *work, size_t work_bytes, int32_t *status,
                                        arb_stream_t stream) {
  if (!axis_out || !axis_count || !work || !status) return ARB_ERR_INVALID;
  const int rc = ordered_args_ok(field, npts, ncol, dim, kind, axis_cap, work_bytes);
  if (rc) return rc;
  launch_ordered_probe(field, field_is_f32, npts, ncol, dim, axis_cap, axis_out, axis_count, (OrderWork *)work,
                       status, (cudaStream_t)stream);
  return launch_status();
}

extern "C" int arb_ingest_ordered_fill(const void *field, int32_t field_is_f32, int64_t npts, int32_t ncol,
                                       int32_t dim, int32_t kind, int64_t axis_cap, const double *axis_out,
                                       const void *work, size_t work_bytes, double *grid64, float *grid32,
                                       double *raw_out, int32_t *status, arb_stream_t stream) {
  if (!axis_out || (!grid64 && !grid32) || !work || !status) return ARB_ERR_INVALID;
  const int rc = ordered_args_ok(field, npts, ncol, dim, kind, axis_cap, work_bytes);
  if (rc) return rc;
  const int r2 = launch_ordered_fill(field, field_is_f32, npts, ncol, dim, kind, axis_cap, axis_out,
                                     (const OrderWork *)work, grid64, grid32, raw_out, status, (cudaStream_t)stream);
  return r2 ? r2 : launch_status();
}

__global__ void ingest_summary_kernel(const double *axes, int64_t cap, const int64_t *count, int dim,
                                      int32_t *status, double *out) {
  if (threadIdx.x != 0) return;
  out[0] = (double)*status;
  *status = 0;
  for (int a = 0; a < 4; ++a) {
    const int64_t n = a < dim ? count[a] : 0;
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    out[1 + a] = (double)n;
    out[5 + 3 * a] = n >= 1 ? axes[a * cap] : nan;
    out[6 + 3 * a] = n >= 2 ? axes[a * cap + 1] : nan;
    out[7 + 3 * a] = n >= 2 ? axes[a * cap + n - 2] : nan;
  }
}

extern "C" int arb_ingest_summary(const double *axes, int64_t axis_cap, const int64_t *axis_count, int32_t dim,
                                  int32_t *status, double *out, arb_stream_t stream) {
  if (!axes || !axis_count || !status || !out || (dim != 3 && dim != 4) || axis_cap <= 0) return ARB_ERR_INVALID;
  ingest_summary_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(axes, axis_cap, axis_count, dim, status, out);
  return launch_status();
}

extern "C" int arb_status_fetch(int32_t *status, arb_stream_t stream) {
  if (!status) return ARB_ERR_INVALID;
  int32_t h = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&h, status, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return ARB_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return ARB_ERR_CUDA;
  if (h != 0 && cudaMemsetAsync(status, 0, sizeof(int32_t), s) != cudaSuccess) return ARB_ERR_CUDA;
  return h;
}

extern "C" int arb_status_clear(int32_t *status, arb_stream_t stream) {
  if (!status) return ARB_ERR_INVALID;
  return cudaMemsetAsync(status, 0, sizeof(int32_t), (cudaStream_t)stream) == cudaSuccess ? ARB_OK : ARB_ERR_CUDA;
}

extern "C" const char *arb_version(void) { return "arbinterp-gb300 0.1.0 sm_103a"; }
