// Host check of csrc/f64emu.cuh against double arithmetic (built and run by
// test_f64emu.py).  Prints "<mismatches> <fallbacks> <double_rounding_cases> <checked>";
// fallbacks counts in-range operands that were refused.
//
//  * (float)((double)r - A): every r in [-32768, 32767] for dark levels A
//    drawn around typical CCD offsets, over a wide range of exponents, just
//    beside integers, negative, and constructed so that r - A lies within a
//    fraction of a double ulp of a float midpoint (where rounding to double
//    first and then to float differs from rounding once);
//  * (float)((double)v * g): v from the dark-subtracted values and random
//    floats, g around 1 (gains) and over a wide exponent range, and g = m / v
//    rounded to double for float midpoints m (products within a few double
//    ulps of a midpoint).
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "f64emu.cuh"

using namespace xg;

static uint64_t rng_state = 0x243F6A8885A308D3ull;
static uint64_t next_u64() {
  uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double uniform() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

static uint32_t fbits(float f) {
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
}

static long long mismatches = 0, fallbacks = 0, dr_cases = 0, checked = 0;

// the float nearest to the exact value, rounded once (for counting the cases
// where double rounding decides the result); long double arithmetic is not
// portable, so the exact difference is formed here as r * 2^k - m_A in
// unsigned __int128
static bool single_round_differs_sub(int32_t r, double A, float got) {
  uint64_t b;
  memcpy(&b, &A, 8);
  const int eb = (int)((b >> 52) & 0x7ff);
  if (eb == 0) return false;
  const int k = 1075 - eb;
  if (k <= 0 || k > 100) return false;
  typedef __int128 i128;
  typedef unsigned __int128 u128;
  const i128 mA = (i128)((b & ((1ull << 52) - 1)) | (1ull << 52));
  const i128 N = (i128)r * ((i128)1 << k) - ((b >> 63) ? -mA : mA);
  if (N == 0) return false;
  const bool neg = N < 0;
  u128 M = neg ? (u128)(-N) : (u128)N;
  int nb = 0;
  for (u128 t = M; t; t >>= 1) nb++;
  int e = -k;
  if (nb > 24) {
    const int sh = nb - 24;
    u128 q = M >> sh;
    const u128 rem = M & (((u128)1 << sh) - 1), half = (u128)1 << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) q += 1;
    M = q;
    e += sh;
  }
  const double once = std::ldexp((double)(uint64_t)M, e) * (neg ? -1.0 : 1.0);
  return fbits((float)once) != fbits(got);
}

static void check_sub_fast(int32_t r, double A);
static void check_sub(int32_t r, double A) {
  check_sub_fast(r, A);
  const float want = (float)((double)r - A);
  float got;
  checked++;
  if (!f32_int_minus_f64(r, A, got)) {
    fallbacks++;
    return;
  }
  if (fbits(got) != fbits(want)) {
    if (mismatches < 5) printf("sub mismatch r=%d A=%.17g want=%.9g got=%.9g\n", r, A, want, got);
    mismatches++;
  }
  if (single_round_differs_sub(r, A, got)) dr_cases++;
}

// the per-pixel fast forms of the dense filter, where they apply
static long long fast_checked = 0;
static void check_sub_fast(int32_t r, double A) {
  const EmuSubPrep q = emu_sub_prep(A);
  if (q.c0 == INT32_MIN) return;
  const int64_t n = (int64_t)r - q.c0;
  if (n < 1 || n >= (1 << 24)) return;
  const float want = (float)((double)r - A);
  const float got = f32_sub_fast((int32_t)n, q.G);
  fast_checked++;
  if (fbits(got) != fbits(want)) {
    if (mismatches < 5) printf("sub_fast mismatch r=%d A=%.17g want=%.9g got=%.9g\n", r, A, want, got);
    mismatches++;
  }
}

static void check_mul_fast(float v, double g) {
  const EmuMulPrep q = emu_mul_prep(g);
  if (q.eg == INT32_MIN || !(v > 0.f)) return;
  float got;
  if (!f32_mul_fast(v, q, got)) return;
  const float want = (float)((double)v * g);
  fast_checked++;
  if (fbits(got) != fbits(want)) {
    if (mismatches < 5) printf("mul_fast mismatch v=%.9g g=%.17g want=%.9g got=%.9g\n", v, g, want, got);
    mismatches++;
  }
}

static void check_mul(float v, double g) {
  check_mul_fast(v, g);
  const float want = (float)((double)v * g);
  float got;
  checked++;
  if (!f32_mul_f64(v, g, got)) {
    fallbacks++;
    return;
  }
  if (fbits(got) != fbits(want)) {
    if (mismatches < 5) printf("mul mismatch v=%.9g g=%.17g want=%.9g got=%.9g\n", v, g, want, got);
    mismatches++;
  }
}

int main() {
  // dark levels: typical, wide exponents, near integers, negative, zero
  for (int t = 0; t < 600; t++) {
    double A;
    switch (t % 6) {
      case 0: A = 100.0 + 8.0 * (uniform() * 2 - 1) * 3; break;
      case 1: A = std::ldexp(uniform() + 1.0, (int)(uniform() * 42) - 12); break;
      case 2: A = std::floor(uniform() * 4000) + (uniform() < 0.5 ? 1 : -1) * std::ldexp(1.0, -(int)(uniform() * 40) - 1); break;
      case 3: A = -(uniform() * 500); break;
      case 4: A = (double)(float)(uniform() * 300); break;
      default: A = uniform() * 65536.0; break;
    }
    if (t == 0) A = 0.0;
    if (t == 6) A = -0.0;
    for (int32_t r = -32768; r <= 32767; r++) check_sub(r, A);
  }
  // dark levels outside the handled range: the caller's double evaluation
  // takes these (a result, if any, must still be right)
  {
    const long long fb0 = fallbacks;
    const double odd[] = {std::ldexp(1.0, -13), 1e-300, 5e-324, std::ldexp(1.0, 30), 3e9, 1e300,
                          -std::ldexp(1.0, 31)};
    for (double A : odd)
      for (int32_t r = -32768; r <= 32767; r += 7) check_sub(r, A);
    if (fallbacks == fb0) printf("out-of-range dark levels were not refused\n");
    fallbacks = fb0;
  }
  // r - A within a fraction of a double ulp beside a float midpoint
  for (int t = 0; t < 2000000; t++) {
    const int32_t r = (int32_t)(next_u64() % 65536) - 32768;
    const float f = (float)(uniform() * 60000.0 - 30000.0);
    if (f == 0.f || !std::isfinite(f)) continue;
    const double ulp = std::ldexp(1.0, std::ilogb((double)f) - 23);
    const double mid = (double)f + ulp / 2;  // exact in double
    const double delta = std::ldexp(ulp, -30 - (int)(uniform() * 20)) * (uniform() < 0.5 ? 1 : -1);
    const double A = ((double)r - mid) - delta;
    check_sub(r, A);
  }
  // products: gains near 1, wide exponents, and near-midpoint products
  for (int t = 0; t < 40000000; t++) {
    float v;
    double g;
    const int kind = t % 4;
    if (kind == 0) {
      v = (float)((double)((int)(next_u64() % 4096)) - (100.0 + uniform()));
      g = 0.9 + 0.2 * uniform();
    } else if (kind == 1) {
      v = (float)std::ldexp(uniform() + 0.5, (int)(uniform() * 120) - 60);
      g = std::ldexp(uniform() + 0.5, (int)(uniform() * 120) - 60);
    } else if (kind == 2) {
      v = (float)(int)(next_u64() % 64 + 1);
      const float f = (float)std::ldexp(uniform() + 1.0, (int)(uniform() * 30) - 10);
      const double mid = (double)f + std::ldexp(1.0, std::ilogb((double)f) - 24);
      g = mid / (double)v;
    } else {
      v = (float)(next_u64() % 32768);
      g = (double)(float)(0.5 + uniform());
    }
    check_mul(v, g);
  }
  check_mul(0.f, 1.25);
  check_mul(-0.f, 1.25);
  check_mul(3.f, -0.0);
  if (fast_checked < 10000000) printf("fast forms checked on %lld operands only\n", fast_checked);
  printf("%lld %lld %lld %lld\n", mismatches, fallbacks, dr_cases, checked);
  return mismatches != 0;
}
