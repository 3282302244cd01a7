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

// ---- per-pixel forms for the dense filter's inner loop
//
// The dark level A and the flatfield g are fixed per pixel, so their
// decomposition is done once.  For A in [2^-12, 2^30): c0 = ceil(A) and
// G = (c0 - A) * 2^64 (exact), so that r - A = (r - c0) + G * 2^-64.  For g
// normal and positive: its 53-bit significand and exponent.

struct EmuSubPrep {
  int32_t c0;   // INT32_MIN: use f32_int_minus_f64
  uint64_t G;
};

XG_EMU_HD EmuSubPrep emu_sub_prep(double A) {
  EmuSubPrep q{INT32_MIN, 0};
  const uint64_t b = emu_f64_bits(A);
  const int eb = (int)((b >> 52) & 0x7ff);
  const int E = eb - 1023;
  if ((b >> 63) || eb == 0 || E < -12 || E > 29) return q;
  const uint64_t mA = (b & ((1ull << 52) - 1)) | (1ull << 52);
  const int64_t Ai = E >= 0 ? (int64_t)(mA >> (52 - E)) : 0;
  const uint64_t F = mA << (E + 12);
  q.c0 = (int32_t)(Ai + (F ? 1 : 0));
  q.G = F ? (uint64_t)0 - F : 0;
  return q;
}

// (float)((double)r - A) given the prep, for 1 <= r - c0 < 2^24: the value
// n + G 2^-64 with n = r - c0 >= 1 has b = bitlen(n) integer bits, so the
// double keeps 53 - b fraction bits of G and the float 24 - b of those.
XG_EMU_HD float f32_sub_fast(int32_t n, uint64_t G) {
  if (G == 0) return (float)n;
  const int b = 64 - emu_clz64((uint64_t)(uint32_t)n);  // bitlen(n), 1 .. 24
  const int sh1 = 11 + b;                                            // 12 .. 35
  uint64_t f = G >> sh1;
  const uint64_t rem = G & ((1ull << sh1) - 1), half = 1ull << (sh1 - 1);
  if (rem > half || (rem == half && (f & 1))) f += 1;
  if (f >> (53 - b)) {  // the double rounded up to the integer n + 1
    return (float)(n + 1);
  }
  uint64_t m = ((uint64_t)n << (24 - b)) | (f >> 29);
  const uint64_t rem2 = f & ((1ull << 29) - 1), half2 = 1ull << 28;
  if (rem2 > half2 || (rem2 == half2 && (m & 1))) m += 1;
  // m <= 2^24 and the scale 2^-(24-b) are exact in float
  return (float)(uint32_t)m * emu_f32_from_bits((uint32_t)(127 - (24 - b)) << 23);
}

struct EmuMulPrep {
  int32_t eg;   // INT32_MIN: use f32_mul_f64
  uint64_t mg;  // 53-bit significand of g
};

XG_EMU_HD EmuMulPrep emu_mul_prep(double g) {
  EmuMulPrep q{INT32_MIN, 0};
  const uint64_t b = emu_f64_bits(g);
  const int eb = (int)((b >> 52) & 0x7ff);
  if ((b >> 63) || eb == 0 || eb == 0x7ff) return q;
  q.eg = eb - 1075;
  q.mg = (b & ((1ull << 52) - 1)) | (1ull << 52);
  return q;
}

// (float)((double)v * g) given the prep, for a normal v > 0; false when the
// result leaves the normal float range.  The significand product has 76 or
// 77 bits.
XG_EMU_HD bool f32_mul_fast(float v, const EmuMulPrep &g, float &out) {
  const uint32_t vb = emu_f32_bits(v);
  const int ev = (int)(vb >> 23);  // v > 0: no sign bit
  if (ev == 0 || ev == 0xff) return false;
  const uint64_t mv = (vb & 0x7fffffu) | 0x800000u;
  const uint64_t plo = mv * (g.mg & 0xffffffffu), phi = mv * (g.mg >> 32);
  const uint64_t lo = plo + (phi << 32);
  const uint64_t hi = (phi >> 32) + (lo < plo ? 1 : 0);  // 2^11 <= hi < 2^13
  int sh = (hi >> 12) ? 24 : 23;                          // bits beyond 53
  uint64_t q = (hi << (64 - sh)) | (lo >> sh);
  const uint64_t rem = lo & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (q & 1))) q += 1;
  if (q >> 53) {
    q >>= 1;
    sh += 1;
  }
  uint64_t m = q >> 29;
  const uint64_t rem2 = q & ((1ull << 29) - 1), half2 = 1ull << 28;
  if (rem2 > half2 || (rem2 == half2 && (m & 1))) m += 1;
  int e = (ev - 150) + g.eg + sh + 29;
  if (m >> 24) {
    m >>= 1;
    e += 1;
  }
  const int E = e + 23;  // value = 1.m * 2^E
  if (E < -126 || E > 127) return false;
  out = emu_f32_from_bits(((uint32_t)(E + 127) << 23) | ((uint32_t)m & 0x7fffffu));
  return true;
}

}  // namespace xg
