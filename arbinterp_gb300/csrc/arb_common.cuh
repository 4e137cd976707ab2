// Shared device helpers for the sm_103a interpolation kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/arbinterp.h"

#define ARB_MAX_AXIS_CAP (1 << 20)

namespace arb {

// -- status helpers ----------------------------------------------------------
__device__ __forceinline__ void set_status(int32_t *status, int32_t bits) {
  if (status) atomicOr(status, bits);
}

static inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ARB_OK : ARB_ERR_CUDA;
}

// -- per-device host caches -----------------------------------------------------
// Function attributes (shared-memory limits) and __device__ constants are
// per device, so launchers keep their one-time setup per device index.
constexpr int MAX_DEVICES = 64;

// The current device's index, or -1 when there is none (or it is out of range).
static inline int current_device() {
  int d = -1;
  return (cudaGetDevice(&d) == cudaSuccess && d >= 0 && d < MAX_DEVICES) ? d : -1;
}

// Streaming multiprocessors of the current device (cached per device).
static inline int device_sms() {
  static int n[MAX_DEVICES] = {};
  const int d = current_device();
  if (d < 0) return 148;
  if (!n[d]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d);
    n[d] = v > 0 ? v : 148;
  }
  return n[d];
}

// -- Catmull-Rom weights ------------------------------------------------------
// The reference's 3D A = inv(B) D is exactly kron(A1, A1, A1) with A1 the
// 4x4 Catmull-Rom matrix (cubic Hermite with central-difference slopes), so
// p(x) . (A f) == sum_o w(x)_o f_o with w(t) = A1^T [1, t, t^2, t^3].
template <typename T>
__device__ __forceinline__ void cr_weights(T t, T w[4]) {
  const T h = T(0.5);
  w[0] = t * (-h + t * (T(1) - h * t));
  w[1] = T(1) + t * t * (T(-2.5) + T(1.5) * t);
  w[2] = t * (h + t * (T(2) - T(1.5) * t));
  w[3] = t * t * (-h + h * t);
}

template <typename T>
__device__ __forceinline__ void cr_dweights(T t, T d[4]) {
  d[0] = T(-0.5) + t * (T(2) - T(1.5) * t);
  d[1] = t * (T(-5) + T(4.5) * t);
  d[2] = T(0.5) + t * (T(4) - T(4.5) * t);
  d[3] = t * (T(-1) + T(1.5) * t);
}

template <typename T>
__device__ __forceinline__ void cr_d2weights(T t, T d[4]) {
  d[0] = T(2) - T(3) * t;
  d[1] = T(-5) + T(9) * t;
  d[2] = T(4) - T(9) * t;
  d[3] = T(-1) + T(3) * t;
}

// Cubic Hermite basis for the slope at t=0 (c=0) and at t=1 (c=1), and their
// derivatives: the 1D factors of the inv(B) columns of the d4f/dxdydzdt rows.
template <typename T>
__device__ __forceinline__ void hermite_slope(T t, T hb[2], T dhb[2]) {
  const T u = T(1) - t;
  hb[0] = t * u * u;
  hb[1] = t * t * (t - T(1));
  dhb[0] = T(1) + t * (T(-4) + T(3) * t);
  dhb[1] = t * (T(3) * t - T(2));
}

// -- coordinate step ---------------------------------------------------------
// The reference computes iu = (q - IntMin) / h in float64, floors it, and
// builds the flat cell index from the floors (ARB:471-483).  Division must
// be the IEEE one so floors (hence cell indices) are bit-exact.
struct CoordStep {
  int64_t idx;       // flat cell index, as the reference computes it
  int64_t fl[4];     // per-axis floors (valid when !oob && !nan)
  bool oob;          // some coordinate outside [lo, hi]  -> row written NaN
  bool nan;          // some coordinate NaN (row not rewritten, outputs NaN)
};

// exact == true: IEEE division (used by the float64 path).
// exact == false: multiply by 1/h and fall back to the division only when the
// product lies within a few ulps of an integer, so floor() still matches.
template <int DIM, bool EXACT>
__device__ __forceinline__ CoordStep coord_step(const double *qrow, const arb_grid &g,
                                                const double *inv_h, double frac[DIM]) {
  CoordStep s;
  s.oob = false;
  s.nan = false;
  int64_t fl[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    const double q = qrow[a];
    if (q < g.lo[a] || q > g.hi[a]) s.oob = true;
    if (q != q) s.nan = true;
    const double d = q - g.lo[a];
    double iu, k;
    if (EXACT) {
      iu = d / g.h[a];
      k = floor(iu);
    } else {
      iu = d * inv_h[a];
      k = floor(iu);
      const double guard = fmax(fabs(iu), 1.0) * 1.7763568394002505e-15;  // 8 ulp(1)
      if (iu - k < guard || (k + 1.0) - iu < guard) {
        iu = d / g.h[a];
        k = floor(iu);
      }
    }
    frac[a] = iu - k;
    fl[a] = (int64_t)k;
  }
#pragma unroll
  for (int a = 0; a < DIM; ++a) s.fl[a] = fl[a];
  if (s.oob || s.nan) {
    s.idx = g.nc;
    return s;
  }
  int64_t idx = fl[DIM - 1];
#pragma unroll
  for (int a = DIM - 2; a >= 0; --a) idx = idx * (g.n[a] - 3) + fl[a];
  s.idx = idx;
  return s;
}

// Order-preserving map of a double onto uint64: a < b <=> key(a) < key(b)
// for non-NaN values, so bounds tests run on the integer pipe.
__host__ __device__ __forceinline__ unsigned long long ord_key_bits(unsigned long long b) {
  return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}

__device__ __forceinline__ void split_f32(double v, float &hi, float &lo);
__device__ __forceinline__ void split_f32_trunc(unsigned long long b, float &hi, float &lo);

// x unchanged, its origin hidden from the optimiser (no instruction): bit
// tests on a reinterpreted double are then not turned into float64 compares.
__device__ __forceinline__ unsigned long long opaque_u64(unsigned long long x) {
  asm("" : "+l"(x));
  return x;
}

struct FastAxis {
  unsigned long long lo_key, hi_key;  // ord keys of IntMin / IntMax
  double lo, h, inv_h;
  float loh, lol, ih, il;             // float32 pairs of IntMin and 1/h
  int df;                             // the float32 double-float step applies on this axis
};

// Float32 pairs of IntMin and 1/h, and whether the double-float step of
// coord_step_fast applies: the interpolation range spans at most 2^20 cells
// from the origin ((|IntMin| + |IntMax|) / h <= 2^20) and the values lie where
// float32 pairs hold them (0 or [2^-80, 2^100] in magnitude).
__host__ __device__ inline void fast_axis_pairs(FastAxis &f, double lo, double hi, double h) {
  const double ih = 1.0 / h;
#ifdef __CUDA_ARCH__
  split_f32(lo, f.loh, f.lol);
  split_f32(ih, f.ih, f.il);
#else
  f.loh = (float)lo;
  f.lol = (float)(lo - (double)f.loh);
  f.ih = (float)ih;
  f.il = (float)(ih - (double)f.ih);
#endif
  auto in_range = [](double v) {
    const double m = v < 0 ? -v : v;
    return m == 0.0 || (m >= 0x1p-80 && m <= 0x1p100);
  };
  const double alo = lo < 0 ? -lo : lo, ahi = hi < 0 ? -hi : hi;
  f.df = (h > 0.0 && in_range(lo) && in_range(hi) && in_range(ih) && ih > 0.0 && (alo + ahi) * ih <= 0x1p20) ? 1
                                                                                                         : 0;
}

// Mixed-precision coordinate step: the cell index is bit-exact (it equals
// floor((q - IntMin) / h) with IEEE division, as the reference computes it)
// and the fractional offset is returned to 2^-24.  Float64-pipe work per
// axis: one subtraction and one multiplication; the floor and the fraction
// come from the product's bit pattern with integer operations.  Only when
// the product lies within 8 ulps of an integer (where multiplying by 1/h
// and dividing by h could floor differently) is the IEEE division redone.
// The float64 step of one axis: (q - IntMin) * (1/h), floored, with the
// reference's own division where the product lands within 8 ulps of an
// integer.  Out of line, so the float32 fast path never issues these
// float64-pipe instructions speculatively; it is the main path only for an
// axis spanning more than 2^20 cells.
struct AxisStep {
  int64_t k;
  float fr;
};

static __device__ __noinline__ AxisStep axis_step_f64(double q, const FastAxis &ax) {
  const double d = q - ax.lo;
  double iu = d * ax.inv_h;
  const unsigned long long b = (unsigned long long)__double_as_longlong(iu);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  int64_t kk = 0;
  float fr = 0.f;
  bool redo = (e > 30);
  if (e >= -1 && e <= 30) {
    const int nf = 52 - e;  // 22 .. 53 fraction bits
    const unsigned long long m = (b & 0xfffffffffffffULL) | (1ULL << 52);
    const unsigned long long one = 1ULL << nf;
    const unsigned long long fb = m & (one - 1);
    kk = (int64_t)(m >> nf);
    redo = (fb < 8ULL) || (fb > one - 8ULL);
    // top 24 bits of the fraction, converted exactly, times 2^-24
    const unsigned f24 = (unsigned)(nf >= 24 ? (fb >> (nf - 24)) : (fb << (24 - nf)));
    // f24 * 2^-24 exactly, without an int->float conversion instruction
    const float f23 = __fsub_rn(__uint_as_float(0x4b000000u | (f24 >> 1)), 8388608.f);
    fr = __fmaf_rn(f23, 2.f, (f24 & 1u) ? 1.f : 0.f) * 5.9604644775390625e-08f;
  } else if (e < -1) {
    fr = __double2float_rn(iu);  // iu < 0.5: floor is 0
  }
  if (redo) {
    iu = d / ax.h;
    const double kf = floor(iu);
    kk = (int64_t)kf;
    fr = (float)(iu - kf);
  }
  AxisStep r;
  r.k = kk;
  r.fr = fr;
  return r;
}

template <int DIM>
__device__ __forceinline__ CoordStep coord_step_fast(const double *qrow, const FastAxis *ax,
                                                     const arb_grid &g, float frac[DIM]) {
  CoordStep s;
  s.oob = false;
  s.nan = false;
  int64_t fl[DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    const double q = qrow[a];
    // the bits are opaque to the optimiser, so the NaN and range tests below
    // stay integer operations instead of being folded into float64 compares
    // (the float64 pipe issues about one warp instruction per 15 cycles per SM)
    const unsigned long long qb = opaque_u64((unsigned long long)__double_as_longlong(q));
    const bool isnan = (qb & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL;
    const unsigned long long k = ord_key_bits(qb);
    const bool out = !isnan && (k < ax[a].lo_key || k > ax[a].hi_key);
    s.nan |= isnan;
    s.oob |= out;
    if (isnan || out) {
      fl[a] = 0;
      frac[a] = 0.f;
      continue;
    }
    if (ax[a].df) {
      // (q - IntMin) / h in float32 double-float arithmetic: q and IntMin
      // as float pairs (residuals 2^-47 and 2^-48 relative), an exact
      // two-sum of the high parts, times the pair of 1/h.  Error < 2^-24 in
      // cell units (span <= 2^20 cells); the reference's own float64
      // roundings move iu by <= 2^-31.  So the floor is the reference's
      // whenever the fraction is 2^-20 or more away from a cell face;
      // otherwise the float64 steps below decide.
      float qh, ql;
      split_f32_trunc(qb, qh, ql);
      const float sh = __fsub_rn(qh, ax[a].loh);
      const float bv = __fsub_rn(sh, qh);
      const float se = __fadd_rn(__fsub_rn(qh, __fsub_rn(sh, bv)), __fsub_rn(-ax[a].loh, bv));
      const float st = __fadd_rn(se, __fsub_rn(ql, ax[a].lol));
      const float ph = __fmul_rn(sh, ax[a].ih);
      const float pe = __fmaf_rn(sh, ax[a].ih, -ph);
      const float pl = __fmaf_rn(sh, ax[a].il, __fmaf_rn(st, ax[a].ih, pe));
      float kf = __fsub_rn(__fadd_rn(ph, 8388608.f), 8388608.f);  // nearest integer (0 <= ph < 2^21)
      if (kf > ph) kf = __fsub_rn(kf, 1.f);
      float fr = __fadd_rn(__fsub_rn(ph, kf), pl);
      if (fr < 0.f) {
        kf = __fsub_rn(kf, 1.f);
        fr = __fadd_rn(fr, 1.f);
      } else if (fr >= 1.f) {
        kf = __fadd_rn(kf, 1.f);
        fr = __fsub_rn(fr, 1.f);
      }
      if (kf >= 0.f && fr >= 0x1p-20f && fr <= 1.f - 0x1p-20f) {
        fl[a] = (int64_t)(__float_as_int(__fadd_rn(kf, 8388608.f)) - 0x4b000000);
        frac[a] = fr;
        continue;
      }
    }
    const AxisStep r = axis_step_f64(q, ax[a]);
    fl[a] = r.k;
    frac[a] = r.fr;
  }
#pragma unroll
  for (int a = 0; a < DIM; ++a) s.fl[a] = fl[a];
  if (s.oob || s.nan) {
    s.idx = g.nc;
    return s;
  }
  int64_t idx = fl[DIM - 1];
#pragma unroll
  for (int a = DIM - 2; a >= 0; --a) idx = idx * (g.n[a] - 3) + fl[a];
  s.idx = idx;
  return s;
}

// Cell coordinates of a flat index (the reference's upper-face aliasing
// falls out of this: (nPos, iy, iz) decodes as (0, iy+1, iz)).
// 64-bit integer division runs on the float64 pipe on this GPU, so indices
// below 2^32 (every practical grid) take the 32-bit unsigned path.
template <int DIM>
__device__ __forceinline__ void cell_coords(int64_t idx, const arb_grid &g, int64_t c[DIM]) {
  if (idx < 0x100000000LL) {
    uint32_t u = (uint32_t)idx;
#pragma unroll
    for (int a = 0; a < DIM - 1; ++a) {
      const uint32_t m = (uint32_t)(g.n[a] - 3);
      const uint32_t qd = u / m;
      c[a] = (int64_t)(u - qd * m);
      u = qd;
    }
    c[DIM - 1] = (int64_t)u;
    return;
  }
#pragma unroll
  for (int a = 0; a < DIM - 1; ++a) {
    const int64_t m = g.n[a] - 3;
    c[a] = idx % m;
    idx /= m;
  }
  c[DIM - 1] = idx;
}

// ---- packed cell coordinates (bin-ordered query records) -------------------
// 21 bits per axis in 3D, 15 in 4D; bit 63 marks a row that needs no
// evaluation (low bits 0: NaN row; 1: in-volume row whose flat index equals
// nc, the reference's sentinel column).
constexpr unsigned long long CELL_SPECIAL = 1ULL << 63;
template <int DIM>
__host__ __device__ constexpr int cell_bits() { return DIM == 3 ? 21 : 15; }

template <int DIM>
__device__ __forceinline__ unsigned long long pack_cell(const int64_t c[DIM]) {
  unsigned long long w = 0;
#pragma unroll
  for (int a = DIM - 1; a >= 0; --a) w = (w << cell_bits<DIM>()) | (unsigned long long)c[a];
  return w;
}
template <int DIM>
__device__ __forceinline__ void unpack_cell(unsigned long long w, int64_t c[DIM]) {
  const unsigned long long m = (1ULL << cell_bits<DIM>()) - 1;
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    c[a] = (int64_t)(w & m);
    w >>= cell_bits<DIM>();
  }
}
// Flat cell index from coordinates (no division).
template <int DIM>
__device__ __forceinline__ int64_t flat_cell(const int64_t c[DIM], const arb_grid &g) {
  int64_t idx = c[DIM - 1];
#pragma unroll
  for (int a = DIM - 2; a >= 0; --a) idx = idx * (g.n[a] - 3) + c[a];
  return idx;
}
// Cell coordinates of an in-volume step: the floors themselves, unless one
// sits on an upper face (floor == cells on that axis), where the reference's
// flat index aliases onto another cell and is decoded.
template <int DIM>
__device__ __forceinline__ void cell_from_step(const CoordStep &s, const arb_grid &g, int64_t c[DIM]) {
  bool face = false;
#pragma unroll
  for (int a = 0; a < DIM; ++a) face |= s.fl[a] >= g.n[a] - 3;
  if (face) {
    cell_coords<DIM>(s.idx, g, c);
  } else {
#pragma unroll
    for (int a = 0; a < DIM; ++a) c[a] = s.fl[a];
  }
}

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000LL); }

// ---- mixed-precision grid (grid32) layout -----------------------------------
//   F = 1: [npts] float2 (hi, lo)               value + gradient field
//   F = 3: [npts] float4 (hi_x, hi_y, hi_z, 0)   components: values only
//   F = 4: [npts] float4 (hi_x, hi_y, hi_z, hi_n), then [npts] float lo_n
// hi = RN(v), lo = RN(v - hi).  Only the field whose gradient is returned
// keeps lo; a value interpolated from float32-rounded samples is within
// ~2 eps32 max|f| of the float64 one (Catmull-Rom weights sum to 1 with
// absolute sum <= 1.25 per axis), whereas a gradient needs the residual.
template <int F>
__host__ __device__ constexpr int g32_floats_per_point() { return F == 1 ? 2 : (F == 3 ? 4 : 5); }

__device__ __forceinline__ int64_t grid_points(const arb_grid &g) {
  int64_t n = g.n[0] * g.n[1] * g.n[2];
  if (g.dim == 4) n *= g.n[3];
  return n;
}

// hi / lo of field f at point p (lo = 0 for fields stored without residual).
template <int F>
__device__ __forceinline__ void g32_load(const float *g32, int64_t npts, int64_t p, int f, float &hi,
                                         float &lo) {
  if (F == 1) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(g32) + p);
    hi = v.x;
    lo = v.y;
  } else {
    hi = __ldg(g32 + p * 4 + f);
    lo = (F == 4 && f == 3) ? __ldg(g32 + npts * 4 + p) : 0.f;
  }
}

// float -> double on the integer pipe (exact for normal numbers and zeros;
// subnormals, infinities and NaN take the conversion instruction).
// Rare conversions kept out of line: a call cannot be hoisted, so the common
// path never issues the float64-pipe instruction speculatively.
static __device__ __noinline__ double f2d_slow(float f) { return (double)f; }

__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((unsigned long long)u << 32));
  if (e == 0u || e == 0xffu) return f2d_slow(f);
  const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(e + 896u) << 52) |
                               ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)b);
}

// Split a double into float32 hi = RN(v) and lo = RN(v - hi) with integer
// operations (bit-identical to the float64-pipe conversions) for
// 2^-45 <= |v| < 2^127; other magnitudes fall back to the conversions.
static __device__ __noinline__ float2 split_f32_slow(double v) {
  const float hi = __double2float_rn(v);
  return make_float2(hi, __double2float_rn(v - (double)hi));
}

__device__ __forceinline__ void split_f32(double v, float &hi, float &lo) {
  const unsigned long long b = opaque_u64((unsigned long long)__double_as_longlong(v));  // integer tests only
  const int E = (int)((b >> 52) & 0x7ff);
  if (E < 978 || E > 1023 + 126) {
    const float2 r = split_f32_slow(v);  // out of line: never speculated
    hi = r.x;
    lo = r.y;
    return;
  }
  const unsigned long long m = b & 0xfffffffffffffULL;
  const unsigned top = (unsigned)(m >> 29);          // 23 kept mantissa bits
  const unsigned r = (unsigned)(m & 0x1fffffffULL);   // 29 dropped bits
  const bool up = (r > 0x10000000u) || (r == 0x10000000u && (top & 1u));
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  hi = __uint_as_float(sign | ((((unsigned)(E - 1023 + 127)) << 23) + top + (up ? 1u : 0u)));
  const int rs = up ? (int)r - 0x20000000 : (int)r;   // v - hi in units of 2^(E-1075), |rs| <= 2^28
  // RN(rs) without the int->float conversion instruction: rs = a 2^12 + b
  // with both halves exact as magic-number floats, one rounded add
  const int a = rs >> 12, bq = rs & 0xfff;
  const float fa = __fsub_rn(__int_as_float(0x4b400000 + a), 12582912.f);
  const float fb = __fsub_rn(__int_as_float(0x4b400000 + bq), 12582912.f);
  const float l = __fadd_rn(__fmul_rn(fa, 4096.f), fb) * __uint_as_float(((unsigned)(E - 948)) << 23);
  lo = sign ? -l : l;
}

// Asynchronous global -> shared copies (cp.async): 16 bytes bypassing L1,
// 8 and 4 bytes through it; groups committed and waited on per thread.
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

// Split a double into float32 hi + lo with hi = v truncated to 24
// significand bits and lo = RN(v - hi) (the 29 dropped bits, rounded once),
// so |v - (hi + lo)| <= 2^-47 |v|: cheaper than split_f32 (no rounding of
// hi) where only the sum matters.  Both forms take the bits of v; the _bits
// form requires the biased exponent E of v in [949, 1149]
// (2^-74 <= |v| < 2^127).
__device__ __forceinline__ void split_f32_trunc_bits(unsigned long long b, float &hi, float &lo) {
  const unsigned h32 = (unsigned)(b >> 32), l32 = (unsigned)b;
  const int E = (int)((h32 >> 20) & 0x7ff);
  const unsigned sign = h32 & 0x80000000u;
  hi = __uint_as_float(sign | ((unsigned)(E - 896) << 23) | ((h32 & 0xfffffu) << 3) | (l32 >> 29));
  // the dropped bits as a float without the conversion instruction:
  // r = x 2^12 + y, both halves exact as magic-number floats, one rounded add
  const unsigned r = l32 & 0x1fffffffu;
  const float fx = __fsub_rn(__int_as_float(0x4b400000 + (int)(r >> 12)), 12582912.f);
  const float fy = __fsub_rn(__int_as_float(0x4b400000 + (int)(r & 0xfffu)), 12582912.f);
  const float l = __fadd_rn(__fmul_rn(fx, 4096.f), fy) * __uint_as_float((unsigned)(E - 948) << 23);
  lo = sign ? -l : l;
}

// Other magnitudes: split_f32, out of line (never speculated on the fast path).
static __device__ __noinline__ float2 split_f32_trunc_slow(double v) {
  float hi, lo;
  split_f32(v, hi, lo);
  return make_float2(hi, lo);
}

__device__ __forceinline__ void split_f32_trunc(unsigned long long b, float &hi, float &lo) {
  const int E = (int)((b >> 52) & 0x7ff);
  if (E < 949 || E > 1023 + 126) {
    const float2 r = split_f32_trunc_slow(__longlong_as_double((long long)b));
    hi = r.x;
    lo = r.y;
    return;
  }
  split_f32_trunc_bits(b, hi, lo);
}

// Warp-aggregated append of an out-of-volume row index.
__device__ __forceinline__ void append_oob(const arb_query_out &o, int64_t row, bool pred) {
  if (!o.oob_rows) return;
  const unsigned mask = __ballot_sync(__activemask(), pred);
  if (!pred) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(o.oob_count, (unsigned long long)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  const int rank = __popc(mask & ((1u << lane) - 1));
  o.oob_rows[base + rank] = row;
}

}  // namespace arb
