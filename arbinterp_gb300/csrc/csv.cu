// GPU reader for the field files the reference loads with
//     np.genfromtxt(path, delimiter=',')
// (examples/3D_ARBInterpExample.py:14,37, examples/4D_ARBInterpExample.py:14,38;
// the files are N x 4..7 tables, README.md:64-72).
//
// Semantics follow genfromtxt with a delimiter, a comment character and
// skip_header, on ASCII text opened in text mode:
//   * lines end at "\n", "\r\n" or a lone "\r" (universal newlines);
//   * everything from the comment character on is dropped, then spaces are
//     stripped from both ends; a line left empty is skipped;
//   * the first remaining line fixes the column count; a later line with a
//     different count is an error (reported with numpy's line numbering);
//   * every token goes through Python's float(): surrounding ASCII
//     whitespace (TAB..CR, space), an optional sign, inf/infinity/nan in any
//     case, digits with single underscores between digits, an optional
//     point and exponent; anything else (and an empty token) reads as NaN.
// Decimal-to-binary conversion is correctly rounded (round half to even,
// subnormals, overflow to infinity), bit-identical to float():
//   1. w <= 2^53 and |q| <= 22: one IEEE multiply or divide of exact operands;
//   2. otherwise the first 19 significant digits w times a 128-bit
//      truncation T of 10^q (csv_pow10.cuh) bound the value from below and
//      above; when both bounds round to the same double, that is the answer
//      (rounding is monotone);
//   3. else the line is queued and csv_exact_kernel compares the value with
//      the midpoint of the two candidates in exact big-integer arithmetic
//      (all significant digits up to 800, beyond which only "nonzero"
//      matters: a midpoint has at most 768 significant decimal digits).
// Method 2 is the bound-and-check scheme of D. Lemire, "Number parsing at a
// gigabyte per second", Software: Practice and Experience 51(8), 2021;
// method 3 is the classic exact comparison (W. D. Clinger, "How to read
// floating point numbers accurately", PLDI 1990).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/arbinterp.h"
#include "arb_common.cuh"
#include "csv_pow10.cuh"

namespace arb {
namespace csv {

constexpr int CHUNK_THREADS = 256;
constexpr int64_t CHUNK = CHUNK_THREADS * 64;  // bytes per count/starts CTA
constexpr int LINES_PER_CTA = 256;
constexpr int STAGE_BYTES = 40 * 1024;
constexpr int MAX_DIGITS = 800;
constexpr int LIMBS = 168;  // 5376 bits: the largest operand of the exact comparison is < 4800 bits
constexpr int EXACT_THREADS = 64;
constexpr int64_t NONE = INT64_MAX;
constexpr uint64_t NAN_BITS = 0x7ff8000000000000ull, INF_BITS = 0x7ff0000000000000ull;
constexpr uint64_t SIGN = 0x8000000000000000ull;

__device__ const double kExact10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                        1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

__device__ __forceinline__ bool is_ws(unsigned c) { return c == 32u || (c - 9u) < 5u; }
__device__ __forceinline__ bool is_digit(unsigned c) { return (c - 48u) < 10u; }
__device__ __forceinline__ bool is_eol(unsigned c) { return c == 10u || c == 13u; }

// ---- eight bytes at a time (SWAR on 64-bit words, byte 0 = lowest address) ------
constexpr uint64_t ONES = 0x0101010101010101ull, HIGHS = 0x8080808080808080ull;

// 0x80 in every byte of x equal to c, 0 elsewhere (exact: no carries between bytes)
__device__ __forceinline__ uint64_t eq8(uint64_t x, unsigned c) {
  const uint64_t y = x ^ (ONES * (uint64_t)c);
  return ~(((y & 0x7f7f7f7f7f7f7f7full) + 0x7f7f7f7f7f7f7f7full) | y) & HIGHS;
}
__device__ __forceinline__ bool all_digits8(uint64_t x) {
  return ((x & 0xf0f0f0f0f0f0f0f0ull) == 0x3030303030303030ull) &&
         (((x + 0x0606060606060606ull) & 0xf0f0f0f0f0f0f0f0ull) == 0x3030303030303030ull);
}
// Value of 8 ASCII digits (first byte most significant): pairs, then quads,
// then the octet, each step a multiply-add of adjacent lanes.
__device__ __forceinline__ uint32_t digits8(uint64_t x) {
  x -= 0x3030303030303030ull;
  x = (x * 10u + (x >> 8)) & 0x00ff00ff00ff00ffull;
  x = (x * 100u + (x >> 16)) & 0x0000ffff0000ffffull;
  return (uint32_t)((x * 10000u + (x >> 32)) & 0xffffffffull);
}
// bytes 0..k-1 of a word (k in 0..8)
__device__ __forceinline__ uint64_t below(int k) { return k >= 8 ? ~0ull : ((1ull << (8 * k)) - 1); }

// Text byte x at p[x - off]: staged in shared memory (STAGED; the stage is
// padded so an 8-byte read never leaves it) or read from global memory.
template <bool STAGED>
struct Src {
  const uint8_t *p;
  int64_t off;
  __device__ __forceinline__ unsigned at(int64_t x) const { return p[x - off]; }
  // bytes x .. x+7; callers keep x + 8 within the text
  __device__ __forceinline__ uint64_t load8(int64_t x) const {
    if constexpr (STAGED) {
      const int64_t r = x - off;
      const uint64_t *w = reinterpret_cast<const uint64_t *>(p + (r & ~(int64_t)7));
      const int sh = (int)(r & 7) * 8;
      const uint64_t lo = w[0];
      return sh ? (lo >> sh) | (w[1] << (64 - sh)) : lo;
    } else {
      uint64_t v = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) v |= (uint64_t)p[x - off + k] << (8 * k);
      return v;
    }
  }
};

// ---- token grammar (Python float) --------------------------------------------
struct Dec {
  uint64_t w;    // first 19 significant digits
  int64_t q;     // value = w * 10^q (digits past the 19th dropped)
  int32_t nd;    // digits in w
  uint8_t neg, trunc, kind;  // kind: 0 number, 1 inf, 2 nan, 3 invalid or empty
};

template <bool ST>
__device__ __forceinline__ bool word_is(const Src<ST> &s, int64_t i, int64_t len, const char *w, int n) {
  if (len != n) return false;
  for (int k = 0; k < n; ++k)
    if ((s.at(i + k) | 0x20u) != (unsigned)w[k]) return false;
  return true;
}

// Exponent part at s[i] (just past 'e'/'E'); returns the position after it,
// or -1 if malformed.  e saturates at 1e9.
template <bool ST>
__device__ __forceinline__ int64_t parse_exp(const Src<ST> &s, int64_t i, int64_t j, int64_t &e) {
  bool eneg = false;
  if (i < j && (s.at(i) == '+' || s.at(i) == '-')) {
    eneg = s.at(i) == '-';
    ++i;
  }
  int64_t v = 0;
  int nd = 0;
  for (; i < j; ++i) {
    const unsigned c = s.at(i);
    if (is_digit(c)) {
      v = v * 10 + (c - 48u);
      if (v > 1000000000) v = 1000000000;
      ++nd;
    } else if (c == '_') {
      if (!(is_digit(s.at(i - 1)) && i + 1 < j && is_digit(s.at(i + 1)))) return -1;
    } else {
      break;
    }
  }
  if (nd == 0) return -1;
  e = eneg ? -v : v;
  return i;
}

template <bool ST>
__device__ Dec parse_token(const Src<ST> &s, int64_t i, int64_t j) {
  Dec r{0, 0, 0, 0, 0, 3};
  while (i < j && is_ws(s.at(i))) ++i;
  while (j > i && is_ws(s.at(j - 1))) --j;
  if (i == j) return r;
  const int64_t i0 = i;
  if (s.at(i) == '+' || s.at(i) == '-') {
    r.neg = s.at(i) == '-';
    ++i;
  }
  if (i < j && ((s.at(i) | 0x20u) == 'i' || (s.at(i) | 0x20u) == 'n')) {
    if (word_is(s, i, j - i, "inf", 3) || word_is(s, i, j - i, "infinity", 8)) r.kind = 1;
    else if (word_is(s, i, j - i, "nan", 3)) r.kind = 2;
    return r;
  }
  uint64_t w = 0;
  int nd = 0;
  int64_t q = 0, ndig = 0;
  bool seen = false, point = false, trunc = false;
  while (i < j) {
    if (nd <= 11 && i + 8 <= j) {  // eight digits at once while w * 10^8 + v stays below 10^19
      const uint64_t x = s.load8(i);
      if (all_digits8(x)) {
        const uint32_t v = digits8(x);
        if (seen || v) {
          int sig = 8;
          if (!seen) {
            const uint64_t nz = ~eq8(x, '0') & HIGHS;  // nonzero digits
            sig = 8 - ((__ffsll((long long)nz) - 1) >> 3);
            seen = true;
          }
          w = w * 100000000ull + v;
          nd += sig;
        }
        q -= point ? 8 : 0;
        ndig += 8;
        i += 8;
        continue;
      }
    }
    const unsigned c = s.at(i);
    if (is_digit(c)) {
      const unsigned d = c - 48u;
      ++ndig;
      if (seen || d) {
        seen = true;
        if (nd < 19) {
          w = w * 10 + d;
          ++nd;
          q -= point;
        } else {
          trunc |= d != 0;
          q += !point;
        }
      } else {
        q -= point;
      }
    } else if (c == '_') {
      if (!(i > i0 && is_digit(s.at(i - 1)) && i + 1 < j && is_digit(s.at(i + 1)))) return r;
    } else if (c == '.') {
      if (point) return r;
      point = true;
    } else {
      break;
    }
    ++i;
  }
  if (ndig == 0) return r;
  if (i < j && (s.at(i) | 0x20u) == 'e') {
    int64_t e = 0;
    i = parse_exp(s, i + 1, j, e);
    if (i < 0) return r;
    q += e;
  }
  if (i != j) return r;
  r.w = w;
  r.q = q;
  r.nd = nd;
  r.trunc = trunc;
  r.kind = 0;
  return r;
}

// ---- 128-bit bound and round -------------------------------------------------
// Bits of RN(X * 2^(b - lz)) with X = (W << lz) * T (+ (W << lz) when addW):
// the rounding of an exact integer, magnitude only.  carry: X overflowed
// 192 bits (never for the table's T, reported as undecided).
__device__ __forceinline__ uint64_t round_prod(uint64_t W, bool addW, uint64_t thi, uint64_t tlo, int b,
                                               bool &carry, bool *same_plus_w = nullptr) {
  const int lz = __clzll((long long)W);
  const uint64_t Wn = W << lz;
  uint64_t x0 = Wn * tlo;
  const uint64_t c0 = __umul64hi(Wn, tlo);
  uint64_t x1 = Wn * thi;
  uint64_t x2 = __umul64hi(Wn, thi);
  x1 += c0;
  x2 += x1 < c0;
  carry = false;
  if (addW) {
    x0 += Wn;
    const uint64_t k0 = x0 < Wn;
    x1 += k0;
    const uint64_t k1 = k0 & (x1 == 0);
    x2 += k1;
    carry = k1 && x2 == 0;
  }
  const int p = (x2 >> 63) ? 191 : 190;  // X >= 2^190: W << lz >= 2^63, T >= 2^127
  const int ebias = b - lz;
  if (p + ebias > 1023) return INF_BITS;
  int c = p - 52;
  if (c + ebias < -1074) c = -1074 - ebias;  // subnormal: the grid is 2^-1074
  if (c > 192) return 0;                     // below half the smallest subnormal
  const int sh = c - 128, rs = c - 129;      // sh in [10, 64], rs in [9, 63]
  uint64_t m = sh >= 64 ? 0 : (x2 >> sh);
  const uint64_t r = (x2 >> rs) & 1u;
  const uint64_t s = ((x2 & ((1ull << rs) - 1)) | x1 | x0) != 0;
  // X + (W << lz) rounds the same way when the addition cannot carry into
  // the top word (the round bit and mantissa live there) and X is already
  // inexact below the round bit
  if (same_plus_w) *same_plus_w = x1 != ~0ull && s;
  m += r & (s | (m & 1u));
  const uint64_t bits = ((uint64_t)(c + ebias + 1074) << 52) + m;
  return bits > INF_BITS ? INF_BITS : bits;
}

// Magnitude bits of the correctly rounded value when decided; otherwise the
// rounding of the lower bound (a candidate for the exact pass).
__device__ __forceinline__ uint64_t fast_convert(const Dec &d, bool &decided) {
  decided = true;
  if (d.w == 0) return 0;
  if (!d.trunc && d.w <= (1ull << 53) && d.q >= -22 && d.q <= 22) {
    const double x = __ull2double_rn(d.w);
    const double v = d.q >= 0 ? __dmul_rn(x, kExact10[d.q]) : __ddiv_rn(x, kExact10[-d.q]);
    return (uint64_t)__double_as_longlong(v);
  }
  if (d.q > 308) return INF_BITS;
  if (d.q + d.nd <= -324) return 0;
  const int k = (int)d.q - kPow10Min;
  const uint64_t thi = kPow10T[k][0], tlo = kPow10T[k][1];
  const int b = kPow10B[k];
  const bool exact = d.q >= 0 && d.q <= 55;
  bool cy, same = false;
  const uint64_t lo = round_prod(d.w, false, thi, tlo, b, cy, &same);
  if (exact && !d.trunc) return lo;
  if (!d.trunc && same) return lo;  // the upper bound (W << lz) * (T + 1) rounds alike
  const uint64_t hi = round_prod(d.trunc ? d.w + 1 : d.w, !exact, thi, tlo, b, cy);
  if (cy || hi != lo) decided = false;
  return lo;
}

__device__ __forceinline__ uint64_t token_bits(const Dec &d, bool &decided) {
  decided = true;
  switch (d.kind) {
    case 0: {
      const uint64_t m = fast_convert(d, decided);
      return d.neg ? (m | SIGN) : m;
    }
    case 1: return d.neg ? (INF_BITS | SIGN) : INF_BITS;
    case 2: return d.neg ? (NAN_BITS | SIGN) : NAN_BITS;
    default: return NAN_BITS;
  }
}

// ---- exact comparison (big integers, little-endian 32-bit limbs) -------------
struct Big {
  uint32_t *l;
  int n;
};

__device__ bool big_mul_add(Big &a, uint32_t m, uint32_t add) {
  uint64_t carry = add;
  for (int k = 0; k < a.n; ++k) {
    const uint64_t t = (uint64_t)a.l[k] * m + carry;
    a.l[k] = (uint32_t)t;
    carry = t >> 32;
  }
  if (carry) {
    if (a.n >= LIMBS) return false;
    a.l[a.n++] = (uint32_t)carry;
  }
  return true;
}

__device__ bool big_mul_pow5(Big &a, int64_t e) {
  const uint32_t p5[14] = {1u, 5u, 25u, 125u, 625u, 3125u, 15625u, 78125u, 390625u, 1953125u, 9765625u,
                           48828125u, 244140625u, 1220703125u};
  bool ok = true;
  for (; e >= 13 && ok; e -= 13) ok = big_mul_add(a, p5[13], 0);
  if (ok && e > 0) ok = big_mul_add(a, p5[e], 0);
  return ok;
}

__device__ bool big_shl(Big &a, int64_t bits) {
  if (a.n == 0 || bits == 0) return true;
  const int64_t words = bits >> 5;
  const int rem = (int)(bits & 31);
  const int top = a.n + (int)words + (rem ? 1 : 0);
  if (words >= LIMBS || top > LIMBS) return false;
  if (rem) {
    a.l[a.n + words] = 0;
    for (int k = a.n - 1; k >= 0; --k) {
      a.l[k + words + 1] |= a.l[k] >> (32 - rem);
      a.l[k + words] = a.l[k] << rem;
    }
  } else {
    for (int k = a.n - 1; k >= 0; --k) a.l[k + words] = a.l[k];
  }
  for (int64_t k = 0; k < words; ++k) a.l[k] = 0;
  a.n = top;
  while (a.n > 0 && a.l[a.n - 1] == 0) --a.n;
  return true;
}

__device__ int big_cmp(const Big &a, const Big &b) {
  if (a.n != b.n) return a.n < b.n ? -1 : 1;
  for (int k = a.n - 1; k >= 0; --k)
    if (a.l[k] != b.l[k]) return a.l[k] < b.l[k] ? -1 : 1;
  return 0;
}

// Correctly rounded magnitude of the (valid, finite-number) token s[i, j),
// starting from cand, a double no larger than the answer.
__device__ uint64_t exact_convert(const Src<false> &s, int64_t i, int64_t j, uint64_t cand, uint32_t *scratch,
                                  int32_t *err) {
  while (i < j && is_ws(s.at(i))) ++i;
  while (j > i && is_ws(s.at(j - 1))) --j;
  if (i < j && (s.at(i) == '+' || s.at(i) == '-')) ++i;
  Big D{scratch, 0};
  int nd = 0, chunk_n = 0;
  uint32_t chunk = 0;
  int64_t qd = 0;
  bool sticky = false, seen = false, point = false, ok = true;
  const uint32_t p10[10] = {1u, 10u, 100u, 1000u, 10000u, 100000u, 1000000u, 10000000u, 100000000u, 1000000000u};
  for (; i < j; ++i) {
    const unsigned c = s.at(i);
    if ((c | 0x20) == 'e') break;
    if (is_digit(c)) {
      const unsigned d = c - 48u;
      if (seen || d) {
        seen = true;
        if (nd < MAX_DIGITS) {
          chunk = chunk * 10 + d;
          ++nd;
          qd -= point;
          if (++chunk_n == 9) {
            ok &= big_mul_add(D, p10[9], chunk);
            chunk = 0;
            chunk_n = 0;
          }
        } else {
          sticky |= d != 0;
          qd += !point;
        }
      } else {
        qd -= point;
      }
    } else if (c == '.') {
      point = true;
    }
  }
  if (chunk_n) ok &= big_mul_add(D, p10[chunk_n], chunk);
  if (i < j) {
    int64_t e = 0;
    parse_exp(s, i + 1, j, e);
    qd += e;
  }
  Big X{scratch + LIMBS, 0}, Y{scratch + 2 * LIMBS, 0};
  for (int it = 0; it < 4 && ok; ++it) {
    if (cand >= INF_BITS) return INF_BITS;
    const uint64_t ex = cand >> 52;
    const uint64_t m1 = (cand & ((1ull << 52) - 1)) | (ex ? (1ull << 52) : 0);
    const int64_t K = (ex ? (int64_t)ex - 1075 : -1074) - 1;  // midpoint (2 m1 + 1) 2^K
    const uint64_t M = 2 * m1 + 1;
    for (int k = 0; k < D.n; ++k) X.l[k] = D.l[k];
    X.n = D.n;
    Y.l[0] = (uint32_t)M;
    Y.l[1] = (uint32_t)(M >> 32);
    Y.n = Y.l[1] ? 2 : 1;
    const int64_t a2 = qd;
    ok &= qd >= 0 ? big_mul_pow5(X, qd) : big_mul_pow5(Y, -qd);
    ok &= a2 >= K ? big_shl(X, a2 - K) : big_shl(Y, K - a2);
    if (!ok) break;
    const int cmp = big_cmp(X, Y);
    if (cmp < 0) return cand;
    if (cmp == 0 && !sticky) return (m1 & 1u) ? cand + 1 : cand;
    ++cand;  // above the midpoint: the next double up is the new candidate
  }
  if (err) atomicOr(err, ARB_ERR_CAPACITY);
  return cand;
}

// ---- line walking --------------------------------------------------------------
// Content of the line starting at p, limited to lim: [a, b) after the
// comment cut and the strip of spaces; nvals values (0: nothing left).
struct LineSpan {
  int64_t a, b;
  int32_t nvals;
};

template <bool ST>
__device__ __forceinline__ LineSpan line_span(const Src<ST> &s, int64_t p, int64_t lim, int delim, int comment) {
  int64_t first = -1, last = -1;
  int32_t nd_all = 0, nd_first = 0, nd_last = 0;
  while (p < lim) {
    if (p + 8 <= lim) {
      const uint64_t x = s.load8(p);
      uint64_t end = eq8(x, 10u) | eq8(x, 13u);
      if (comment >= 0) end |= eq8(x, (unsigned)comment);
      const uint64_t valid = end ? below((__ffsll((long long)end) - 1) >> 3) : ~0ull;
      const uint64_t del = eq8(x, (unsigned)delim) & valid;
      const uint64_t ns = ~eq8(x, 32u) & HIGHS & valid;
      if (ns) {
        const int fb = (__ffsll((long long)ns) - 1) >> 3, lb = (63 - __clzll((long long)ns)) >> 3;
        if (first < 0) {
          first = p + fb;
          nd_first = nd_all + __popcll(del & below(fb));
        }
        last = p + lb;
        nd_last = nd_all + __popcll(del & below(lb + 1));
      }
      nd_all += __popcll(del);
      if (end) break;
      p += 8;
    } else {
      const unsigned c = s.at(p);
      if (is_eol(c) || (int)c == comment) break;
      const bool isd = (int)c == delim;
      nd_all += isd;
      if (c != 32u) {
        if (first < 0) {
          first = p;
          nd_first = nd_all - isd;
        }
        last = p;
        nd_last = nd_all;
      }
      ++p;
    }
  }
  LineSpan r;
  r.a = first;
  r.b = last + 1;
  r.nvals = first < 0 ? 0 : nd_last - nd_first + 1;
  return r;
}

// Next delimiter at or after ts before b (b if none).
template <bool ST>
__device__ __forceinline__ int64_t next_delim(const Src<ST> &s, int64_t ts, int64_t b, int delim) {
  while (ts < b) {
    if (ts + 8 <= b) {
      const uint64_t m = eq8(s.load8(ts), (unsigned)delim);
      if (m) return ts + ((__ffsll((long long)m) - 1) >> 3);
      ts += 8;
    } else {
      if ((int)s.at(ts) == delim) return ts;
      ++ts;
    }
  }
  return b;
}

// Bytes [a, b) of the text for the CTA's lines, staged into shared memory
// (16 bytes of padding past the stage) when they fit; returns whether they did
// and sets off so that text byte x is at sm[x - off].
__device__ __forceinline__ bool stage_bytes(const uint8_t *t, int64_t n, int64_t a, int64_t b, uint8_t *sm,
                                            int64_t &off) {
  const int64_t a16 = a & ~(int64_t)15;
  off = a16;
  if (b - a16 > STAGE_BYTES) return false;
  const int64_t nvec = (b - a16 + 15) >> 4;
  for (int64_t k = threadIdx.x; k < nvec; k += blockDim.x) {
    const int64_t p = a16 + 16 * k;
    if (p + 16 <= n) {
      *reinterpret_cast<uint4 *>(sm + 16 * k) = __ldg(reinterpret_cast<const uint4 *>(t + p));
    } else {
      for (int e = 0; e < 16; ++e) sm[16 * k + e] = p + e < n ? t[p + e] : (uint8_t)0;
    }
  }
  return true;
}

// ---- kernels -------------------------------------------------------------------
__global__ void init_kernel(arb_csv_info *info) {
  info->nlines = 0;
  info->first_nonascii = NONE;
  info->first_data_line = NONE;
  info->ncols = 0;
  info->nrows = 0;
  info->ninvalid = 0;
  info->nexact = 0;
  info->nqueued = 0;
  info->error = 0;
  info->reserved = 0;
}

// Terminators ('\n', or '\r' not followed by '\n') in t[p0, p1) in order;
// records the first byte >= 0x80.  p0 is a multiple of 16.
// One 8-byte word at text position p of a chunk: its terminators in order.
// next_lf: the byte after the word is '\n'.
template <class F>
__device__ __forceinline__ void word_terms(uint64_t x, int64_t p, bool next_lf, int64_t &nonascii, F &f) {
  if ((x & HIGHS) && nonascii == NONE) nonascii = p + ((__ffsll((long long)(x & HIGHS)) - 1) >> 3);
  const uint64_t lf = eq8(x, 10u);
  uint64_t term = lf;
  const uint64_t cr = eq8(x, 13u);
  if (cr) term |= cr & ~((lf >> 8) | (next_lf ? (0x80ull << 56) : 0ull));  // CR not followed by LF
  while (term) {
    f(p + ((__ffsll((long long)term) - 1) >> 3));
    term &= term - 1;
  }
}

// Terminators ('\n', or '\r' not followed by '\n') in t[p0, p1) in order;
// records the first byte >= 0x80.  p0 is a multiple of 16.
template <class F>
__device__ __forceinline__ void for_each_term(const uint8_t *t, int64_t n, int64_t p0, int64_t p1, int64_t &nonascii,
                                              F &&f) {
  for (int64_t p = p0; p < p1; p += 16) {
    if (p + 16 <= n) {
      const uint4 v = __ldg(reinterpret_cast<const uint4 *>(t + p));
      const uint64_t x0 = (uint64_t)v.x | ((uint64_t)v.y << 32), x1 = (uint64_t)v.z | ((uint64_t)v.w << 32);
      word_terms(x0, p, (x1 & 0xffu) == 10u, nonascii, f);
      const bool lf16 = (x1 >> 56) == 13u && p + 16 < n && t[p + 16] == 10u;
      word_terms(x1, p + 8, lf16, nonascii, f);
    } else {
      for (int64_t q = p; q < n && q < p + 16; ++q) {
        const unsigned c = t[q];
        if ((c & 0x80u) && nonascii == NONE) nonascii = q;
        if (c == 10u || (c == 13u && (q + 1 >= n || t[q + 1] != 10u))) f(q);
      }
    }
  }
}

__device__ __forceinline__ int64_t block_sum_i64(int64_t v, int64_t *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  int64_t s = 0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
  return s;  // valid in thread 0
}

// Exclusive prefix of v over the block (blockDim.x <= 1024); total in *tot.
__device__ __forceinline__ int64_t block_excl_i64(int64_t v, int64_t *red, int64_t *tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
  int64_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) red[warp] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int k = 0; k < nw; ++k) {
      const int64_t c = red[k];
      red[k] = run;
      run += c;
    }
    *tot = run;
  }
  __syncthreads();
  return red[warp] + x - v;
}

__global__ void __launch_bounds__(CHUNK_THREADS) count_kernel(const uint8_t *t, int64_t n, int64_t *counts,
                                                              arb_csv_info *info) {
  __shared__ int64_t red[CHUNK_THREADS / 32];
  const int64_t p0 = blockIdx.x * CHUNK + (int64_t)threadIdx.x * 64;
  const int64_t p1 = p0 + 64 < n ? p0 + 64 : n;
  int64_t cnt = 0, nonascii = NONE;
  if (p0 < n) for_each_term(t, n, p0, p1, nonascii, [&](int64_t) { ++cnt; });
  if (nonascii != NONE) atomicMin(reinterpret_cast<unsigned long long *>(&info->first_nonascii),
                                  (unsigned long long)nonascii);
  const int64_t s = block_sum_i64(cnt, red);
  if (threadIdx.x == 0) counts[blockIdx.x] = s;
}

// Single-block exclusive scan of v[0, m) in place; returns the total.
__device__ int64_t scan_block(int64_t *v, int64_t m, int64_t *red, int64_t *tot) {
  const int64_t per = (m + blockDim.x - 1) / blockDim.x;
  const int64_t b = threadIdx.x * per, e = b + per < m ? b + per : m;
  int64_t sum = 0;
  for (int64_t k = b; k < e; ++k) sum += v[k];
  int64_t run = block_excl_i64(sum, red, tot);
  for (int64_t k = b; k < e; ++k) {
    const int64_t c = v[k];
    v[k] = run;
    run += c;
  }
  __syncthreads();
  return *tot;
}

__global__ void __launch_bounds__(1024) line_scan_kernel(const uint8_t *t, int64_t n, int64_t *counts,
                                                         int64_t nchunks, arb_csv_info *info) {
  __shared__ int64_t red[32];
  __shared__ int64_t tot;
  const int64_t terms = scan_block(counts, nchunks, red, &tot);
  if (threadIdx.x == 0) {
    const bool open_last = n > 0 && t[n - 1] != 10u && t[n - 1] != 13u;
    info->nlines = terms + (open_last ? 1 : 0);
    if (info->first_nonascii == NONE) info->first_nonascii = -1;
  }
}

__global__ void __launch_bounds__(CHUNK_THREADS) starts_kernel(const uint8_t *t, int64_t n, const int64_t *base,
                                                               int64_t *starts, int64_t nlines) {
  __shared__ int64_t red[CHUNK_THREADS / 32];
  __shared__ int64_t tot;
  const int64_t p0 = blockIdx.x * CHUNK + (int64_t)threadIdx.x * 64;
  const int64_t p1 = p0 + 64 < n ? p0 + 64 : n;
  int64_t cnt = 0, na = NONE;
  if (p0 < n) for_each_term(t, n, p0, p1, na, [&](int64_t) { ++cnt; });
  int64_t k = base[blockIdx.x] + block_excl_i64(cnt, red, &tot);
  if (blockIdx.x == 0 && threadIdx.x == 0 && nlines > 0) starts[0] = 0;
  if (cnt)
    for_each_term(t, n, p0, p1, na, [&](int64_t p) {
      if (k + 1 < nlines) starts[k + 1] = p + 1;
      ++k;
    });
}

template <bool ST>
__device__ __forceinline__ void classify_line(const Src<ST> &s, int64_t l, int64_t start, int64_t lim, int delim,
                                              int comment, int64_t skip_header, int32_t *nvals, uint2 *spans,
                                              int64_t &first) {
  const LineSpan sp = line_span(s, start, lim, delim, comment);
  const int32_t nv = l < skip_header ? 0 : sp.nvals;
  nvals[l] = nv;
  if (nv > 0) {
    const int64_t ra = sp.a - start, rb = sp.b - start;
    spans[l] = rb < 0xffffffffll ? make_uint2((unsigned)ra, (unsigned)rb) : make_uint2(0xffffffffu, 0xffffffffu);
    first = first < l ? first : l;
  }
}

__global__ void __launch_bounds__(LINES_PER_CTA) classify_kernel(const uint8_t *t, int64_t n, const int64_t *starts,
                                                                 int64_t nlines, int delim, int comment,
                                                                 int64_t skip_header, int32_t *nvals, uint2 *spans,
                                                                 arb_csv_info *info) {
  __shared__ __align__(16) uint8_t sm[STAGE_BYTES + 16];
  __shared__ unsigned long long first_sm;
  const int64_t L0 = (int64_t)blockIdx.x * LINES_PER_CTA;
  const int64_t L1 = L0 + LINES_PER_CTA < nlines ? L0 + LINES_PER_CTA : nlines;
  const int64_t a = starts[L0], b = L1 < nlines ? starts[L1] : n;
  int64_t off;
  const bool staged = stage_bytes(t, n, a, b, sm, off);
  if (threadIdx.x == 0) first_sm = (unsigned long long)NONE;
  __syncthreads();
  const int64_t l = L0 + threadIdx.x;
  int64_t first = NONE;
  if (l < L1) {
    if (staged) classify_line(Src<true>{sm, off}, l, starts[l], b, delim, comment, skip_header, nvals, spans, first);
    else classify_line(Src<false>{t, 0}, l, starts[l], b, delim, comment, skip_header, nvals, spans, first);
  }
  // one atomic per CTA: the first line with values
  for (int o = 16; o > 0; o >>= 1) {
    const int64_t y = __shfl_down_sync(0xffffffffu, first, o);
    first = y < first ? y : first;
  }
  if ((threadIdx.x & 31) == 0 && first != NONE) atomicMin(&first_sm, (unsigned long long)first);
  __syncthreads();
  if (threadIdx.x == 0 && first_sm != (unsigned long long)NONE)
    atomicMin(reinterpret_cast<unsigned long long *>(&info->first_data_line), first_sm);
}

__global__ void __launch_bounds__(LINES_PER_CTA) rows_kernel(const int32_t *nvals, int64_t nlines, int64_t *cta_count,
                                                             arb_csv_info *info) {
  __shared__ int64_t red[LINES_PER_CTA / 32];
  const int64_t first = info->first_data_line;
  const int32_t ncols = first == NONE ? 0 : nvals[first];
  const int64_t l = (int64_t)blockIdx.x * LINES_PER_CTA + threadIdx.x;
  const int32_t nv = l < nlines ? nvals[l] : 0;
  const int64_t valid = nv > 0 && nv == ncols;
  if (nv > 0 && nv != ncols) atomicAdd(reinterpret_cast<unsigned long long *>(&info->ninvalid), 1ull);
  const int64_t s = block_sum_i64(valid, red);
  if (threadIdx.x == 0) cta_count[blockIdx.x] = s;
}

__global__ void __launch_bounds__(1024) row_scan_kernel(int64_t *cta, int64_t nctas, const int32_t *nvals,
                                                        arb_csv_info *info) {
  __shared__ int64_t red[32];
  __shared__ int64_t tot;
  const int64_t rows = scan_block(cta, nctas, red, &tot);
  if (threadIdx.x == 0) {
    const int64_t first = info->first_data_line;
    info->nrows = rows;
    info->ncols = first == NONE ? 0 : nvals[first];
    if (first == NONE) info->first_data_line = -1;
  }
}

// Tokens of the content [a, b): each parsed and written to out_row[c];
// returns true when every token was decided by the fast paths.
template <bool ST>
__device__ __forceinline__ bool parse_line(const Src<ST> &s, int64_t a, int64_t b, int delim, int64_t ncols,
                                           double *out_row) {
  bool all = true;
  int64_t ts = a;
  for (int64_t c = 0; c < ncols; ++c) {
    const int64_t te = next_delim(s, ts, b, delim);
    const Dec d = parse_token(s, ts, te);
    bool ok;
    out_row[c] = __longlong_as_double((long long)token_bits(d, ok));
    all &= ok;
    ts = te + 1;
  }
  return all;
}

template <bool ST>
__device__ __forceinline__ bool parse_one(const Src<ST> &s, int64_t start, int64_t lim, uint2 sp, int delim,
                                          int comment, int64_t ncols, double *out_row) {
  int64_t a = start + sp.x, b = start + sp.y;
  if (sp.x == 0xffffffffu) {  // a line longer than 4 GB: walk it again
    const LineSpan r = line_span(s, start, lim, delim, comment);
    a = r.a;
    b = r.b;
  }
  return parse_line(s, a, b, delim, ncols, out_row);
}

__global__ void __launch_bounds__(LINES_PER_CTA) parse_kernel(const uint8_t *t, int64_t n, const int64_t *starts,
                                                              int64_t nlines, const int32_t *nvals, const uint2 *spans,
                                                              const int64_t *cta_base, int delim, int comment,
                                                              int64_t ncols, double *out, int64_t *queue,
                                                              arb_csv_info *info) {
  __shared__ __align__(16) uint8_t sm[STAGE_BYTES + 16];
  __shared__ int64_t red[LINES_PER_CTA / 32];
  __shared__ int64_t tot;
  const int64_t L0 = (int64_t)blockIdx.x * LINES_PER_CTA;
  const int64_t L1 = L0 + LINES_PER_CTA < nlines ? L0 + LINES_PER_CTA : nlines;
  const int64_t a = starts[L0], b = L1 < nlines ? starts[L1] : n;
  int64_t off;
  const bool staged = stage_bytes(t, n, a, b, sm, off);
  const int64_t l = L0 + threadIdx.x;
  const int32_t nv = l < L1 ? nvals[l] : 0;
  const bool valid = nv > 0 && nv == ncols;
  const int64_t row = cta_base[blockIdx.x] + block_excl_i64(valid ? 1 : 0, red, &tot);  // also syncs the stage
  if (!valid) return;
  const uint2 sp = spans[l];
  double *dst = out + row * ncols;
  const bool ok = staged ? parse_one(Src<true>{sm, off}, starts[l], b, sp, delim, comment, ncols, dst)
                         : parse_one(Src<false>{t, 0}, starts[l], b, sp, delim, comment, ncols, dst);
  if (!ok) {
    const unsigned long long k = atomicAdd(reinterpret_cast<unsigned long long *>(&info->nqueued), 1ull);
    queue[2 * k] = l;
    queue[2 * k + 1] = row;
  }
}

__global__ void __launch_bounds__(EXACT_THREADS) exact_kernel(const uint8_t *t, int64_t n, const int64_t *starts,
                                                              int64_t nlines, int delim, int comment, int64_t ncols,
                                                              double *out, const int64_t *queue, uint32_t *scratch,
                                                              arb_csv_info *info) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  uint32_t *mine = scratch + tid * (3 * LIMBS);
  const int64_t nq = info->nqueued;
  const Src<false> s{t, 0};
  for (int64_t k = tid; k < nq; k += nthreads) {
    const int64_t l = queue[2 * k], row = queue[2 * k + 1];
    const int64_t lim = l + 1 < nlines ? starts[l + 1] : n;
    const LineSpan sp = line_span(s, starts[l], lim, delim, comment);
    int64_t ts = sp.a;
    for (int64_t c = 0; c < ncols; ++c) {
      const int64_t te = next_delim(s, ts, sp.b, delim);
      const Dec d = parse_token(s, ts, te);
      bool ok;
      const uint64_t bits = token_bits(d, ok);
      if (!ok) {
        const uint64_t m = exact_convert(s, ts, te, bits & ~SIGN, mine, &info->error);
        out[row * ncols + c] = __longlong_as_double((long long)(d.neg ? (m | SIGN) : m));
        atomicAdd(reinterpret_cast<unsigned long long *>(&info->nexact), 1ull);
      }
      ts = te + 1;
    }
  }
}

static int exact_grid() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                 cudaSuccess || sms <= 0)
    sms = 152;
  return sms;
}

static inline int64_t nchunks_of(int64_t nbytes) { return nbytes > 0 ? (nbytes + CHUNK - 1) / CHUNK : 1; }
static inline int64_t nctas_of(int64_t nlines) { return nlines > 0 ? (nlines + LINES_PER_CTA - 1) / LINES_PER_CTA : 1; }

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct LinesWork {
  int64_t *starts, *cta, *queue;
  uint2 *spans;
  uint32_t *scratch;
};

static size_t lines_layout(int64_t nlines, int grid, void *base, LinesWork *w) {
  const size_t s0 = align256((size_t)(nlines > 0 ? nlines : 1) * 8);
  const size_t s1 = align256((size_t)(nctas_of(nlines) + 1) * 8);
  const size_t s2 = align256((size_t)(nlines > 0 ? nlines : 1) * 16);
  const size_t s3 = align256((size_t)(nlines > 0 ? nlines : 1) * 8);
  const size_t s4 = (size_t)grid * EXACT_THREADS * 3 * LIMBS * 4;
  if (w) {
    char *p = static_cast<char *>(base);
    w->starts = reinterpret_cast<int64_t *>(p);
    w->cta = reinterpret_cast<int64_t *>(p + s0);
    w->queue = reinterpret_cast<int64_t *>(p + s0 + s1);
    w->spans = reinterpret_cast<uint2 *>(p + s0 + s1 + s2);
    w->scratch = reinterpret_cast<uint32_t *>(p + s0 + s1 + s2 + s3);
  }
  return s0 + s1 + s2 + s3 + s4;
}

static bool args_ok(const uint8_t *text, int64_t nbytes, int delim, int comment) {
  if (nbytes < 0 || (nbytes > 0 && !text) || ((uintptr_t)text & 15u)) return false;
  if (delim < 1 || delim > 127 || delim == 10 || delim == 13) return false;
  if (comment != -1 && (comment < 1 || comment > 127 || comment == 10 || comment == 13 || comment == delim))
    return false;
  return true;
}

}  // namespace csv
}  // namespace arb

using namespace arb::csv;

extern "C" size_t arb_csv_count_work_bytes(int64_t nbytes) {
  return nbytes < 0 ? 0 : (size_t)(nchunks_of(nbytes) + 1) * 8;
}

extern "C" int arb_csv_count(const uint8_t *text, int64_t nbytes, void *work, size_t work_bytes, arb_csv_info *info,
                             arb_stream_t stream) {
  if (!info || !work || !args_ok(text, nbytes, ',', -1) || work_bytes < arb_csv_count_work_bytes(nbytes) ||
      ((uintptr_t)work & 7u))
    return ARB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nch = nchunks_of(nbytes);
  int64_t *counts = static_cast<int64_t *>(work);
  init_kernel<<<1, 1, 0, s>>>(info);
  if (nbytes > 0) {
    count_kernel<<<(unsigned)nch, CHUNK_THREADS, 0, s>>>(text, nbytes, counts, info);
  } else if (cudaMemsetAsync(counts, 0, 8, s) != cudaSuccess) {
    return ARB_ERR_CUDA;
  }
  line_scan_kernel<<<1, 1024, 0, s>>>(text, nbytes, counts, nbytes > 0 ? nch : 1, info);
  return arb::launch_status();
}

extern "C" size_t arb_csv_lines_work_bytes(int64_t nlines) {
  return nlines < 0 ? 0 : lines_layout(nlines, exact_grid(), nullptr, nullptr);
}

extern "C" int arb_csv_split(const uint8_t *text, int64_t nbytes, int64_t nlines, int32_t delimiter, int32_t comment,
                             int64_t skip_header, const void *count_work, void *lines_work, size_t lines_work_bytes,
                             int32_t *nvals, arb_csv_info *info, arb_stream_t stream) {
  if (!info || !count_work || !lines_work || !nvals || nlines <= 0 || skip_header < 0 ||
      !args_ok(text, nbytes, delimiter, comment) || lines_work_bytes < arb_csv_lines_work_bytes(nlines) ||
      ((uintptr_t)lines_work & 255u))
    return ARB_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  LinesWork w;
  lines_layout(nlines, exact_grid(), lines_work, &w);
  const int64_t nch = nchunks_of(nbytes);
  const int64_t nctas = nctas_of(nlines);
  starts_kernel<<<(unsigned)nch, CHUNK_THREADS, 0, s>>>(text, nbytes, static_cast<const int64_t *>(count_work),
                                                        w.starts, nlines);
  classify_kernel<<<(unsigned)nctas, LINES_PER_CTA, 0, s>>>(text, nbytes, w.starts, nlines, delimiter, comment,
                                                            skip_header, nvals, w.spans, info);
  rows_kernel<<<(unsigned)nctas, LINES_PER_CTA, 0, s>>>(nvals, nlines, w.cta, info);
  row_scan_kernel<<<1, 1024, 0, s>>>(w.cta, nctas, nvals, info);
  return arb::launch_status();
}

extern "C" int arb_csv_parse(const uint8_t *text, int64_t nbytes, int64_t nlines, int32_t delimiter, int32_t comment,
                             void *lines_work, size_t lines_work_bytes, const int32_t *nvals, double *out,
                             int64_t nrows, int64_t ncols, arb_csv_info *info, arb_stream_t stream) {
  if (!info || !lines_work || !nvals || nlines <= 0 || nrows < 0 || ncols < 0 || (nrows > 0 && (!out || ncols == 0)) ||
      !args_ok(text, nbytes, delimiter, comment) || lines_work_bytes < arb_csv_lines_work_bytes(nlines) ||
      ((uintptr_t)lines_work & 255u) || ((uintptr_t)out & 7u))
    return ARB_ERR_INVALID;
  if (nrows == 0) return ARB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const int grid = exact_grid();
  LinesWork w;
  lines_layout(nlines, grid, lines_work, &w);
  const int64_t nctas = nctas_of(nlines);
  parse_kernel<<<(unsigned)nctas, LINES_PER_CTA, 0, s>>>(text, nbytes, w.starts, nlines, nvals, w.spans, w.cta,
                                                         delimiter, comment, ncols, out, w.queue, info);
  exact_kernel<<<(unsigned)grid, EXACT_THREADS, 0, s>>>(text, nbytes, w.starts, nlines, delimiter, comment, ncols,
                                                        out, w.queue, w.scratch, info);
  return arb::launch_status();
}
