// Float results of the two double-precision expressions the reference's
// filters evaluate once per event, computed exactly with integer arithmetic:
//
//   f32_int_minus_f64(r, A) = (float)((double)r - A)   DenseFilter::Apply,
//                             dark subtraction (dense_filter.cpp:163)
//   f32_mul_f64(v, g)       = (float)((double)v * g)   flatfield scaling
//                             (dense_filter.cpp:171, sparse_filter.cpp:152)
//
// Both are double-rounded in the reference: the exact value is rounded to the
// nearest double, and that double to the nearest float (ties to even each
// time).  Here the exact value is formed as a two-word (2 x 64-bit) integer
// times a power of two, rounded to 53 significant bits and then to 24, and the
// float is assembled from its bits, with 64-bit integer operations only.
// GB300 executes FP64 at a small fraction of its integer and FP32 rate, and
// these run once per event.  Operands outside the handled range (|A| outside
// [2^-12, 2^30) but not 0, subnormal, infinite or NaN operands, results outside
// the normal float range) return false, and the caller evaluates the
// expression in double precision instead.
//
// The header is plain C++ as well, so that a host checker can compare it with
// double arithmetic.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define XG_EMU_HD __host__ __device__ __forceinline__
#else
#define XG_EMU_HD inline
#endif

namespace xg {

XG_EMU_HD int emu_clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// Rounds m (> 0) to at most `bits` significant bits, ties to even; the shift
// is added to e, so m * 2^e keeps its (rounded) value.
XG_EMU_HD uint64_t emu_round64(uint64_t m, int bits, int &e) {
  const int nb = 64 - emu_clz64(m);
  if (nb <= bits) return m;
  int sh = nb - bits;
  uint64_t q = m >> sh;
  const uint64_t rem = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (q & 1))) q += 1;
  if (q >> bits) {  // rounding carried into a new leading bit
    q >>= 1;
    sh += 1;
  }
  e += sh;
  return q;
}

// The same for hi * 2^64 + lo (> 0) with at most bits + 63 significant bits.
XG_EMU_HD uint64_t emu_round128(uint64_t hi, uint64_t lo, int bits, int &e) {
  if (hi == 0) return emu_round64(lo, bits, e);
  int sh = 128 - emu_clz64(hi) - bits;  // in [1, 63]
  uint64_t q = (hi << (64 - sh)) | (lo >> sh);
  const uint64_t rem = lo & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (q & 1))) q += 1;
  if (q >> bits) {
    q >>= 1;
    sh += 1;
  }
  e += sh;
  return q;
}

XG_EMU_HD float emu_f32_from_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, 4);
  return f;
#endif
}

XG_EMU_HD uint64_t emu_f64_bits(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  memcpy(&b, &d, 8);
  return b;
#endif
}

XG_EMU_HD uint32_t emu_f32_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
#endif
}

// (-1)^neg * m * 2^e, with 0 < m < 2^24, as a normal float; false when the
// value is outside the normal float range.
XG_EMU_HD bool emu_pack_f32(bool neg, uint64_t m, int e, float &out) {
  const int nb = 64 - emu_clz64(m);
  const uint32_t mm = (uint32_t)m << (24 - nb);  // 24 significant bits
  const int E = e + nb - 1;                      // value = 1.f * 2^E
  if (E < -126 || E > 127) return false;
  out = emu_f32_from_bits((neg ? 0x80000000u : 0u) | ((uint32_t)(E + 127) << 23) |
                          (mm & 0x7fffffu));
  return true;
}

// (float)((double)r - A) for an integer r with |r| < 2^16.  |A| is split
// into its integer part Ai and its fraction F * 2^-64 (exact while
// 2^-12 <= |A| < 2^30), so that r - A = n + G * 2^-64 with an integer n and
// 0 <= G < 2^64, a value of at most 95 significant bits.
XG_EMU_HD bool f32_int_minus_f64(int32_t r, double A, float &out) {
  const uint64_t b = emu_f64_bits(A);
  const int eb = (int)((b >> 52) & 0x7ff);
  const uint64_t fr = b & ((1ull << 52) - 1);
  const bool na = (b >> 63) != 0;
  if (eb == 0 && fr == 0) {  // r - (+-0) = r, and 0 - 0 = +0
    out = (float)r;
    return true;
  }
  const int E = eb - 1023;  // |A| = 1.f * 2^E
  if (E < -12 || E > 29) return false;
  const uint64_t mA = fr | (1ull << 52);
  const int64_t Ai = E >= 0 ? (int64_t)(mA >> (52 - E)) : 0;
  const uint64_t F = mA << (E + 12);  // the fraction bits, scaled by 2^64
  int64_t n;
  uint64_t G;
  if (!na) {  // r - Ai - F 2^-64 = (r - Ai - 1) + (2^64 - F) 2^-64
    n = (int64_t)r - Ai - (F ? 1 : 0);
    G = F ? (uint64_t)0 - F : 0;
  } else {  // r + Ai + F 2^-64
    n = (int64_t)r + Ai;
    G = F;
  }
  bool neg = false;
  uint64_t hi, lo;
  if (n >= 0) {
    hi = (uint64_t)n;
    lo = G;
  } else {  // |x| = -n - G 2^-64
    neg = true;
    hi = (uint64_t)(-n) - (G ? 1 : 0);
    lo = G ? (uint64_t)0 - G : 0;
  }
  if (hi == 0 && lo == 0) {
    out = 0.f;
    return true;
  }
  int e = -64;
  uint64_t M = emu_round128(hi, lo, 53, e);  // the double difference (>= 2^-64: normal)
  M = emu_round64(M, 24, e);                  // then the float
  return emu_pack_f32(neg, M, e, out);
}

// (float)((double)v * g): the 77-bit product of the significands from two
// 32-bit halves of g's.
XG_EMU_HD bool f32_mul_f64(float v, double g, float &out) {
  const uint32_t vb = emu_f32_bits(v);
  const uint64_t gb = emu_f64_bits(g);
  const int ev = (int)((vb >> 23) & 0xff), eg = (int)((gb >> 52) & 0x7ff);
  const uint32_t fv = vb & 0x7fffffu;
  const uint64_t fg = gb & ((1ull << 52) - 1);
  const bool neg = ((vb >> 31) != 0) != ((gb >> 63) != 0);
  if (ev == 0xff || eg == 0x7ff) return false;
  if ((ev == 0 && fv == 0) || (eg == 0 && fg == 0)) {
    out = emu_f32_from_bits(neg ? 0x80000000u : 0u);
    return true;
  }
  if (ev == 0 || eg == 0) return false;
  const uint64_t mv = fv | 0x800000u, mg = fg | (1ull << 52);
  const uint64_t plo = mv * (mg & 0xffffffffu);  // < 2^56
  const uint64_t phi = mv * (mg >> 32);          // < 2^45
  const uint64_t lo = plo + (phi << 32);
  const uint64_t hi = (phi >> 32) + (lo < plo ? 1 : 0);
  int e = (ev - 150) + (eg - 1075);
  uint64_t M = emu_round128(hi, lo, 53, e);
  const int Ed = e + (64 - emu_clz64(M)) - 1;  // the double must be normal
  if (Ed < -1022 || Ed > 1023) return false;
  M = emu_round64(M, 24, e);
  return emu_pack_f32(neg, M, e, out);
}

}  // namespace xg
