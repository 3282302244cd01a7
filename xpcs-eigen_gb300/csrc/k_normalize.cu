// K-d: per-partition normalisation of G2/IP/IF into g2 and its standard error.
//
// Replaces Corr::normalizeG2s (src/xpcs/corr.cpp:927-1091).  BuildQMap's
// q -> sbin -> pixel mapping is flattened into entries (one per (q, sbin): q
// ascending, sbin ascending, pixels in raster order) and every entry's pixel
// range is cut into chunks of at most NCH pixels.
//
// float64 result (the reported one):
//   k_norm_chunk   one block per (chunk, tau) reads G2/IP/IF of the chunk's
//                  pixels once and produces, for the chunk: sum G2, sum IP,
//                  sum IF, sum x and sum (x - mean_chunk)^2 with
//                  x = G2 / (IP IF), NaN -> 0 and still counted (quirk Q8).
//                  Per-element arithmetic is double-word ("float-float") on
//                  the FP32 pipes -- TwoSum, FMA-based TwoProd, the quotient
//                  of a float by a double-word, and Sum2 compensated sums of
//                  Ogita, Rump & Oishi (2005) for the per-thread totals --
//                  because GB300's FP64 rate is a small fraction of its FP32
//                  rate; the block reductions use the double-word addition of
//                  Joldes, Muller & Popescu (ACM TOMS 2017), and the block
//                  totals and everything after are FP64.
//   k_norm_finish  one thread per (q, tau): entry ratio (G2/n)/((IP/n)(IF/n))
//                  (:966-1013), g2 = mean of the non-NaN ratios (:1018-1040),
//                  and the chunks' (n, mean, M2) merged in order with Chan's
//                  pairwise update; stderr = sqrt(1/n) sqrt(M2/n) (:1043-1087).
// float32 result (optional, bit-identical to the reference's float output):
//   k_f32_transpose / k_entry_f32 / k_q_f32 replay the reference's sequential
//   float operations in its order, including the running-mean/M2 update of
//   every pixel.
#include <algorithm>
#include <vector>

#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int NB = 256;          // threads per chunk block
constexpr int NIPT = 16;         // pixels per thread
constexpr int NCH = NB * NIPT;   // pixels per chunk

// ------------------------------------------------ double-word arithmetic

struct dw {
  float h, l;
};

__device__ __forceinline__ dw two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ dw fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dw two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
// double-word + double-word (AccurateDWPlusDW)
__device__ __forceinline__ dw dw_add(dw x, dw y) {
  dw s = two_sum(x.h, y.h), t = two_sum(x.l, y.l);
  dw v = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
  return fast_two_sum(v.h, __fadd_rn(t.l, v.l));
}
// float / double-word: a quotient from the reciprocal of the high word, then
// the quotient of the FMA remainder a - q (bh + bl) as the low word
// (relative error a few 2^-48)
__device__ __forceinline__ dw f_div_dw(float a, dw b) {
  if (a == 0.f) return {0.f, 0.f};  // 0 / b is 0 or NaN, and NaN counts as 0
  const float rb = __frcp_rn(b.h);
  float q = __fmul_rn(a, rb);
  if (!isfinite(q) || q == 0.f) return {__fdiv_rn(a, b.h), 0.f};
  float r = __fmaf_rn(-q, b.h, a);
  r = __fmaf_rn(-q, b.l, r);
  return fast_two_sum(q, __fmul_rn(r, rb));
}
// Sum2 (Ogita, Rump & Oishi, SIAM J. Sci. Comput. 26(6), 2005): a running
// float sum and, beside it, the float sum of every addition's exact rounding
// error; as accurate as summing in twice the precision, at one TwoSum and one
// addition per term.
struct sum2 {
  float s, c;
};
__device__ __forceinline__ void s2_add(sum2 &a, float x) {
  const dw t = two_sum(a.s, x);
  a.s = t.h;
  a.c = __fadd_rn(a.c, t.l);
}
// a double-word term: its low word joins the error sum
__device__ __forceinline__ void s2_add(sum2 &a, dw x) {
  s2_add(a, x.h);
  a.c = __fadd_rn(a.c, x.l);
}
__device__ __forceinline__ dw s2_value(const sum2 &a) { return two_sum(a.s, a.c); }
__device__ __forceinline__ dw dw_from_double(double x) {
  float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double to_double(dw x) { return (double)x.h + (double)x.l; }

// Block sum of N double-word values: warp reduction in double-word arithmetic
// on the FP32 pipes, FP64 only for the per-warp partials, which thread 0 adds
// up: out is valid in thread 0 only (FP64 runs at a small fraction of the FP32
// rate here, so the other threads do not repeat those additions).
template <int N>
__device__ __forceinline__ void block_sum_dw(dw (&x)[N], double (&out)[N], double *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; k++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dw y{__shfl_down_sync(0xffffffffu, x[k].h, o), __shfl_down_sync(0xffffffffu, x[k].l, o)};
      x[k] = dw_add(x[k], y);
    }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; k++) sh[k * (NB / 32) + w] = to_double(x[k]);
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) {
      double r = 0.0;
#pragma unroll
      for (int ww = 0; ww < NB / 32; ww++) r += sh[k * (NB / 32) + ww];
      out[k] = r;
    }
  }
  __syncthreads();
}

// part layout: [chunk][tau][5] = sum G2, sum IP, sum IF, sum x, M2 about the chunk mean
__global__ void __launch_bounds__(NB)
k_norm_chunk(int D, int P, const int32_t *__restrict__ ch_k0, const int32_t *__restrict__ ch_k1,
             const int32_t *__restrict__ pix, const float *__restrict__ G2,
             const float *__restrict__ IP, const float *__restrict__ IF, double *__restrict__ part) {
  __shared__ double sh[4 * (NB / 32) + 1];
  __shared__ float s_mean[2];
  __shared__ float xh[NCH], xl[NCH];
  const int c = blockIdx.x, t = blockIdx.y;
  const int k0 = ch_k0[c], k1 = ch_k1[c];
  const size_t o = (size_t)t * P;
  sum2 sg{0.f, 0.f}, si{0.f, 0.f}, sf{0.f, 0.f}, sx{0.f, 0.f};
#pragma unroll
  for (int j = 0; j < NIPT; j++) {
    const int k = k0 + j * NB + threadIdx.x;
    if (k < k1) {
      const int p = pix[k];
      const float g = G2[o + p], a = IP[o + p], b = IF[o + p];
      s2_add(sg, g);
      s2_add(si, a);
      s2_add(sf, b);
      dw x = f_div_dw(g, two_prod(a, b));
      if (isnan(x.h) || isnan(x.l)) x = {0.f, 0.f};
      s2_add(sx, x);
      xh[j * NB + threadIdx.x] = x.h;
      xl[j * NB + threadIdx.x] = x.l;
    }
  }
  const double n = (double)(k1 - k0);
  dw parts[4] = {s2_value(sg), s2_value(si), s2_value(sf), s2_value(sx)};
  double sums[4];
  block_sum_dw<4>(parts, sums, sh);  // thread 0 holds the sums
  if (threadIdx.x == 0) {
    const dw mu = dw_from_double(sums[3] / n);
    s_mean[0] = mu.h;
    s_mean[1] = mu.l;
  }
  __syncthreads();
  const float mh = -s_mean[0], ml = -s_mean[1];
  sum2 m2{0.f, 0.f};
#pragma unroll
  for (int j = 0; j < NIPT; j++) {
    const int k = k0 + j * NB + threadIdx.x;
    if (k < k1) {
      // d = x - mean as an exact high difference and a low remainder; d^2
      // as the exact square of the high part and the rest by FMA
      const dw d0 = two_sum(xh[j * NB + threadIdx.x], mh);
      const float dl = __fadd_rn(__fadd_rn(d0.l, xl[j * NB + threadIdx.x]), ml);
      const dw q = two_prod(d0.h, d0.h);
      s2_add(m2, dw{q.h, __fmaf_rn(__fmul_rn(2.f, d0.h), dl, __fmaf_rn(dl, dl, q.l))});
    }
  }
  dw mparts[1] = {s2_value(m2)};
  double msum[1];
  block_sum_dw<1>(mparts, msum, sh);
  if (threadIdx.x == 0) {
    double *q = part + ((size_t)c * D + t) * 5;
    q[0] = sums[0];
    q[1] = sums[1];
    q[2] = sums[2];
    q[3] = sums[3];
    q[4] = msum[0];
  }
}

__global__ void k_norm_finish(int NQ, int D, const int32_t *__restrict__ qep,
                              const int32_t *__restrict__ qrow,
                              const int32_t *__restrict__ e_chunk_ptr,
                              const int32_t *__restrict__ ch_k0, const int32_t *__restrict__ ch_k1,
                              const double *__restrict__ part, double *__restrict__ g2,
                              double *__restrict__ se) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= NQ * D) return;
  const int qi = idx / D, t = idx - qi * D;
  double gacc = 0.0, gcnt = 0.0;
  double n = 0.0, mean = 0.0, M2 = 0.0;
  for (int e = qep[qi]; e < qep[qi + 1]; e++) {
    double sg = 0.0, si = 0.0, sf = 0.0, ne = 0.0;
    for (int c = e_chunk_ptr[e]; c < e_chunk_ptr[e + 1]; c++) {
      const double *q = part + ((size_t)c * D + t) * 5;
      const double nc = (double)(ch_k1[c] - ch_k0[c]);
      sg += q[0];
      si += q[1];
      sf += q[2];
      ne += nc;
      // Chan et al.: merge (n, mean, M2) of the chunk into the running one
      const double mc = q[3] / nc;
      const double nn = n + nc;
      const double delta = mc - mean;
      mean = n == 0.0 ? mc : mean + delta * (nc / nn);
      M2 = n == 0.0 ? q[4] : M2 + q[4] + delta * delta * (n * nc / nn);
      n = nn;
    }
    const double r = (sg / ne) / ((si / ne) * (sf / ne));
    gacc += isnan(r) ? 0.0 : r;
    gcnt += isnan(r) ? 0.0 : 1.0;
  }
  const int row = qrow[qi];
  g2[(size_t)t * NQ + row] = gacc / gcnt;
  se[(size_t)t * NQ + row] = sqrt(1.0 / n) * sqrt(M2 / n);
}

// ------------------------------------------------ float32, reference order
//
// Every float sum below runs in the reference's order; what changes is where
// its operands come from.  k_f32_transpose writes G2, IP, IF and the per-pixel
// ratio x = G2 / (IP IF) (NaN -> 0) in q-ordered, pixel-major layout
// [mapped pixel][tau], so the sequential sums of neighbouring taus (adjacent
// threads) read adjacent words.  The running mean's division by the sample
// count uses the correctly rounded reciprocal of the count (__frcp_rn) and
// one FMA residual correction (Markstein; Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 4), which gives the IEEE quotient for every
// float numerator and every integer count up to 2^20 (checked exhaustively
// against __fdiv_rn on the GPU: every significand, every count); larger
// counts, zeros and non-finite numerators use __fdiv_rn.

constexpr int TR_K = 32, TR_T = 32;  // transpose tile: mapped pixels x taus

__global__ void __launch_bounds__(256)
k_f32_transpose(int NK, int D, int Dp, int P, const int32_t *__restrict__ pix,
                const float *__restrict__ G2, const float *__restrict__ IP,
                const float *__restrict__ IF, float *__restrict__ Tg, float *__restrict__ Ti,
                float *__restrict__ Tf, float *__restrict__ X, int32_t *__restrict__ unsafe) {
  __shared__ float sg[TR_T][TR_K + 1], si[TR_T][TR_K + 1], sf[TR_T][TR_K + 1];
  const int k0 = blockIdx.x * TR_K, t0 = blockIdx.y * TR_T;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  // read: lanes over mapped pixels (pixels of a ring run in raster order)
  const int k = k0 + tx;
  const int p = k < NK ? pix[k] : 0;
  for (int r = ty; r < TR_T; r += 8) {
    const int t = t0 + r;
    if (k < NK && t < D) {
      const size_t o = (size_t)t * P + p;
      sg[r][tx] = G2[o];
      si[r][tx] = IP[o];
      sf[r][tx] = IF[o];
    }
  }
  __syncthreads();
  // write: lanes over taus
  const int t = t0 + tx;
  for (int r = ty; r < TR_K; r += 8) {
    const int kk = k0 + r;
    bool bad = false;
    if (kk < NK && t < D) {
      const float g = sg[tx][r], a = si[tx][r], b = sf[tx][r];
      const size_t o = (size_t)kk * Dp + t;
      Tg[o] = g;
      Ti[o] = a;
      Tf[o] = b;
      float x = __fdiv_rn(g, __fmul_rn(a, b));
      x = isnan(x) ? 0.f : x;
      X[o] = x;
      bad = !(x == 0.f || (x >= 0x1p-20f && x <= 0x1p20f));
    }
    // any ratio outside the range where the q-ring replay's running mean
    // needs no special case (k_q_f32)
    if (__any_sync(0xffffffffu, bad) && tx == 0) atomicOr(unsafe, 1);
  }
}

// a / n for the running mean: n is the (integer-valued) sample count and y
// = __frcp_rn(n) its correctly rounded reciprocal, which depends on the count
// only and so stays off the chain of dependent operations
__device__ __forceinline__ float div_count(float a, float n, int ni, float y) {
  if (ni > (1 << 20) || a == 0.f || !isfinite(a) || fabsf(a) < 1e-30f) return __fdiv_rn(a, n);
  const float q0 = __fmul_rn(a, y);
  return __fmaf_rn(__fmaf_rn(-q0, n, a), y, q0);
}

// The replay kernels below run one block per q ring (or per entry) and one
// thread per tau.  The rows [k][0..Dp) of the block's pixel range (Dp: the
// delays padded to a multiple of 4, so that every row range is a 16-byte
// aligned, contiguous span) are brought into shared memory in chunks of up to
// 256 rows by 1-D bulk copies (cp.async.bulk, one per array, issued by one
// thread and completing on an mbarrier), double-buffered: chunk c+1 is in
// flight while the threads step through chunk c, so each thread's sequential
// chain reads shared memory instead of waiting on global loads.
constexpr int FR_SMEM = 200 * 1024;  // shared memory budget of a replay block
constexpr uint32_t FR_WAIT_LIMIT = 1u << 22;  // polls before a wait is given up

__device__ __forceinline__ uint32_t fr_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void fr_bar_init(uint64_t *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fr_u32(bar)));
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fr_u32(bar + 1)));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Waits for the phase of the given parity; false after FR_WAIT_LIMIT polls.
__device__ __forceinline__ bool fr_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = fr_u32(bar);
  for (uint32_t it = 0; it < FR_WAIT_LIMIT; it++) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// One thread: rows [r0, r0 + nrow) of each row-major [k][Dp] array into
// dst[a], completing on bar.
__device__ __forceinline__ void fr_bulk(const float *const *src, float *const *dst, int narr,
                                        int64_t r0, int nrow, int Dp, uint64_t *bar) {
  const uint32_t bytes = (uint32_t)nrow * (uint32_t)Dp * 4u;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fr_u32(bar)),
               "r"(bytes * (uint32_t)narr)
               : "memory");
  for (int a = 0; a < narr; a++)
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(fr_u32(dst[a])), "l"(src[a] + (size_t)r0 * Dp), "r"(bytes), "r"(fr_u32(bar))
        : "memory");
}

// The chunk loop shared by the replay kernels: `narr` arrays of the rows
// [k0, k0 + n) streamed through the two buffers of `buf` ([2][narr][ch][Dp]),
// `step(b, rows, row0)` called by every thread for each chunk in order (b:
// the chunk's buffer, row0: its first row in the range).  Returns false, after setting DEVERR_WAIT, if a copy's
// wait expired; the copies still in flight are then waited for (again with a
// limit) before the block leaves.
template <class Step>
__device__ __forceinline__ bool fr_stream(const float *const *src, int narr, int64_t k0, int n,
                                          int ch, int Dp, float *buf, uint64_t *bar,
                                          int32_t *err, Step step) {
  const int t = threadIdx.x, nch = (n + ch - 1) / ch;
  const size_t bw = (size_t)narr * ch * Dp;
  auto issue = [&](int c) {
    float *dst[3];
    for (int a = 0; a < narr; a++) dst[a] = buf + (size_t)(c & 1) * bw + (size_t)a * ch * Dp;
    fr_bulk(src, dst, narr, k0 + (int64_t)c * ch, min(ch, n - c * ch), Dp, &bar[c & 1]);
  };
  if (t == 0) fr_bar_init(bar);
  __syncthreads();
  if (t == 0) {
    if (nch > 0) issue(0);
    if (nch > 1) issue(1);
  }
  bool ok = true;
  int c = 0;
  for (; c < nch; c++) {
    ok = __syncthreads_and(fr_wait(&bar[c & 1], (uint32_t)(c >> 1) & 1u)) != 0;
    if (!ok) break;
    step(c & 1, min(ch, n - c * ch), c * ch);
    __syncthreads();  // every thread is done with the buffer before it is refilled
    if (t == 0 && c + 2 < nch) issue(c + 2);
  }
  if (!ok && t == 0) {
    atomicOr(err, DEVERR_WAIT);
    // the copies issued for chunks c and c + 1, if any, before the block goes
    for (int d = c; d < min(c + 2, nch); d++) fr_wait(&bar[d & 1], (uint32_t)(d >> 1) & 1u);
  }
  return ok;
}

// One block per entry, thread tau: the entry's sums of G2, IP, IF in pixel
// order, / pixels, ratio (corr.cpp:966-1013).
__global__ void k_entry_f32(int NE, int D, int Dp, int FR_CH, const int32_t *__restrict__ epp,
                            const float *__restrict__ Tg, const float *__restrict__ Ti,
                            const float *__restrict__ Tf, float *__restrict__ ratio,
                            int32_t *__restrict__ err) {
  extern __shared__ __align__(16) float fr_buf[];  // [2][3][FR_CH][Dp], then 2 mbarriers
  uint64_t *bar = (uint64_t *)(fr_buf + (size_t)2 * 3 * FR_CH * Dp);
  const int e = blockIdx.x, t = threadIdx.x;
  const int k0 = epp[e], n = epp[e + 1] - k0;
  const float *src[3] = {Tg, Ti, Tf};
  float sg = 0.f, si = 0.f, sf = 0.f;
  const size_t aw = (size_t)FR_CH * Dp;
  const bool ok = fr_stream(src, 3, k0, n, FR_CH, Dp, fr_buf, bar, err, [&](int b, int rows, int) {
    if (t >= D) return;
    const float *bg = fr_buf + (size_t)b * 3 * aw, *bi = bg + aw, *bf = bg + 2 * aw;
#pragma unroll 4
    for (int r = 0; r < rows; r++) {
      sg = __fadd_rn(sg, bg[r * Dp + t]);
      si = __fadd_rn(si, bi[r * Dp + t]);
      sf = __fadd_rn(sf, bf[r * Dp + t]);
    }
  });
  if (ok && t < D) {
    const float cnt = (float)n;
    sg = __fdiv_rn(sg, cnt);
    si = __fdiv_rn(si, cnt);
    sf = __fdiv_rn(sf, cnt);
    ratio[(size_t)e * D + t] = __fdiv_rn(sg, __fmul_rn(si, sf));
  }
}

// One block per q ring, thread tau: g2 = mean of the non-NaN entry ratios
// (corr.cpp:1018-1040); stderr from the running mean / M2 over the ring's
// pixels in order, NaN counted as 0 (corr.cpp:1043-1087).
__global__ void k_q_f32(int NQ, int D, int Dp, int FR_CH, const int32_t *__restrict__ qep,
                        const int32_t *__restrict__ qrow, const int32_t *__restrict__ epp,
                        const float *__restrict__ ratio, const float *__restrict__ X,
                        float *__restrict__ g2, float *__restrict__ se,
                        const int32_t *__restrict__ unsafe, int32_t *__restrict__ err) {
  extern __shared__ __align__(16) float fr_buf[];  // [2][FR_CH][Dp], then 2 mbarriers
  const bool all_safe = *unsafe == 0;
  uint64_t *bar = (uint64_t *)(fr_buf + (size_t)2 * FR_CH * Dp);
  const int qi = blockIdx.x, t = threadIdx.x;
  const int row = qrow[qi];
  if (t < D) {
    float acc = 0.f, cnt = 0.f;
    for (int e = qep[qi]; e < qep[qi + 1]; e++) {
      float r = ratio[(size_t)e * D + t];
      acc = __fadd_rn(acc, isnan(r) ? 0.f : r);
      cnt = __fadd_rn(cnt, isnan(r) ? 0.f : 1.f);
    }
    g2[(size_t)t * NQ + row] = __fdiv_rn(acc, cnt);
  }
  // The reference's sample count (samples += 1.0f per pixel) is the exact
  // count below 2^24 and stays at 2^24 from there on.  Its correctly rounded
  // reciprocal depends on the count only: the block computes each chunk's
  // into a table, off the chain of dependent operations that each tau's
  // running mean is.
  __shared__ float rtab[256];
  float avg = 0.f, sd = 0.f;
  const int k0 = epp[qep[qi]], n = epp[qep[qi + 1]] - k0;
  const float *src[1] = {X};
  const bool ok = fr_stream(src, 1, k0, n, FR_CH, Dp, fr_buf, bar, err, [&](int b, int rows,
                                                                          int row0) {
    for (int r = t; r < rows; r += blockDim.x) rtab[r] = __frcp_rn((float)(row0 + r + 1));
    __syncthreads();
    if (t >= D) return;
    const float *bx = fr_buf + (size_t)b * FR_CH * Dp;
    // When every ratio of the series is 0 or in [2^-20, 2^20] (flagged by
    // k_f32_transpose), the running mean of non-negative values over at most
    // 2^20 counts stays 0 or about [2^-40, 2^20] (checked at each chunk):
    // every difference a is then 0 (which leaves the mean as it is however it
    // is divided) or finite and at least about 2^-64 in size (the spacing of
    // floats near 2^-41), far inside the range where the reciprocal-and-
    // residual quotient is the IEEE one; the quotient is never NaN, and the
    // chain runs without a branch.
    if (all_safe && row0 + rows <= (1 << 20) &&
        (avg == 0.f || (avg >= 0x1p-40f && avg <= 0x1p20f))) {
      float cnt = (float)row0;
#pragma unroll 4
      for (int r = 0; r < rows; r++) {
        const float x = bx[r * Dp + t];
        cnt = __fadd_rn(cnt, 1.f);  // exact: counts below 2^24
        const float a = __fsub_rn(x, avg);
        const float q0 = __fmul_rn(a, rtab[r]);
        avg = __fadd_rn(avg, __fmaf_rn(__fmaf_rn(-q0, cnt, a), rtab[r], q0));
        sd = __fadd_rn(sd, __fmul_rn(a, __fsub_rn(x, avg)));
      }
    } else if (row0 + rows <= (1 << 20)) {
#pragma unroll 4
      for (int r = 0; r < rows; r++) {
        const float x = bx[r * Dp + t];
        const float cnt = (float)(row0 + r + 1);
        const float a = __fsub_rn(x, avg);
        // a / cnt by the reciprocal and one FMA residual correction: the IEEE
        // quotient for counts up to 2^20 and 1e-30 <= |a| <= FLT_MAX; zero,
        // tiny, infinite and NaN operands take the division itself
        const float q0 = __fmul_rn(a, rtab[r]);
        float tmp00 = __fmaf_rn(__fmaf_rn(-q0, cnt, a), rtab[r], q0);
        if (!(fabsf(a) >= 1e-30f && fabsf(a) <= 3.40282347e38f)) tmp00 = __fdiv_rn(a, cnt);
        tmp00 = isnan(tmp00) ? 0.f : tmp00;
        avg = __fadd_rn(avg, tmp00);
        sd = __fadd_rn(sd, __fmul_rn(a, __fsub_rn(x, avg)));
      }
    } else {
      for (int r = 0; r < rows; r++) {
        const float x = bx[r * Dp + t];
        const int k = row0 + r + 1;
        const float cnt = (float)min(k, 1 << 24);
        const float a = __fsub_rn(x, avg);
        float tmp00 = k <= (1 << 20) ? div_count(a, cnt, k, rtab[r]) : __fdiv_rn(a, cnt);
        tmp00 = isnan(tmp00) ? 0.f : tmp00;
        avg = __fadd_rn(avg, tmp00);
        sd = __fadd_rn(sd, __fmul_rn(a, __fsub_rn(x, avg)));
      }
    }
  });
  if (ok && t < D) {
    const float samples = (float)min(n, 1 << 24);
    const float stdNorm = __fdiv_rn(sd, samples);
    const float inv = __fdiv_rn(1.f, samples);
    se[(size_t)t * NQ + row] = __fmul_rn(__fsqrt_rn(inv), __fsqrt_rn(stdNorm));
  }
}

}  // namespace

void build_norm_chunks(Series &s) {
  const QMap &q = s.qmap;
  std::vector<int32_t> k0, k1, eptr(1, 0);
  for (int e = 0; e < q.nentries(); e++) {
    for (int a = q.entry_pix_ptr[e]; a < q.entry_pix_ptr[e + 1]; a += NCH) {
      k0.push_back(a);
      k1.push_back(std::min(a + NCH, q.entry_pix_ptr[e + 1]));
    }
    eptr.push_back((int32_t)k0.size());
  }
  s.n_chunks = (int32_t)k0.size();
  cudaStream_t st = s.stream;
  auto up = [&](DBuf<int32_t> &b, const std::vector<int32_t> &v) {
    b.reserve(v.size() ? v.size() : 1, st);
    if (!v.empty())
      XG_CUDA(cudaMemcpyAsync(b.p, v.data(), 4 * v.size(), cudaMemcpyHostToDevice, st));
  };
  up(s.n_ch_k0, k0);
  up(s.n_ch_k1, k1);
  up(s.n_e_chunk_ptr, eptr);
}

void run_normalize(Series &s, bool want64, bool want32) {
  cudaStream_t st = s.stream;
  const int D = s.D, P = s.P, NQ = s.qmap.nq(), NE = s.qmap.nentries();
  if (D == 0 || NQ == 0) return;
  if (want64) {
    s.n_g2.reserve((size_t)NQ * D, st);
    s.n_se.reserve((size_t)NQ * D, st);
    const int NC = s.n_chunks;
    s.n_part.reserve((size_t)(NC > 0 ? NC : 1) * D * 5, st);
    if (NC > 0) {
      k_norm_chunk<<<dim3(NC, D), NB, 0, st>>>(D, P, s.n_ch_k0.p, s.n_ch_k1.p, s.n_pix.p, s.G2.p,
                                              s.IP.p, s.IF.p, s.n_part.p);
      XG_CHECK_LAUNCH();
    }
    const int bs = 128;
    k_norm_finish<<<(NQ * D + bs - 1) / bs, bs, 0, st>>>(NQ, D, s.n_q_entry_ptr.p, s.n_q_row.p,
                                                        s.n_e_chunk_ptr.p, s.n_ch_k0.p,
                                                        s.n_ch_k1.p, s.n_part.p, s.n_g2.p,
                                                        s.n_se.p);
    XG_CHECK_LAUNCH();
  }
  if (want32) {
    const QMap &qm = s.qmap;
    const int NK = qm.entry_pix_ptr.empty() ? 0 : qm.entry_pix_ptr.back();
    s.n_ratio32.reserve((size_t)(NE > 0 ? NE : 1) * D, st);
    s.n_g2f.reserve((size_t)NQ * D, st);
    s.n_sef.reserve((size_t)NQ * D, st);
    // rows of the transposed arrays padded to a multiple of 4 delays: 16-byte
    // aligned row ranges for the replay kernels' bulk copies
    const int Dp = (D + 3) & ~3;
    const size_t nt = (size_t)(NK > 0 ? NK : 1) * Dp;
    s.n_tg.reserve(nt, st);
    s.n_ti.reserve(nt, st);
    s.n_tf.reserve(nt, st);
    s.n_tx.reserve(nt, st);
    s.n_unsafe.reserve(1, st);
    XG_CUDA(cudaMemsetAsync(s.n_unsafe.p, 0, sizeof(int32_t), st));
    if (NK > 0) {
      k_f32_transpose<<<dim3((NK + TR_K - 1) / TR_K, (D + TR_T - 1) / TR_T), 256, 0, st>>>(
          NK, D, Dp, P, s.n_pix.p, s.G2.p, s.IP.p, s.IF.p, s.n_tg.p, s.n_ti.p, s.n_tf.p,
          s.n_tx.p, s.n_unsafe.p);
      XG_CHECK_LAUNCH();
    }
    if (D > 1024) throw Error(XPCS_ERR_INVALID_ARGUMENT, "more than 1024 delays");
    const int bs = (D + 31) / 32 * 32;
    const int ch_e = std::max(1, std::min(256, (FR_SMEM - 64) / (24 * Dp)));
    const int ch_q = std::max(1, std::min(256, (FR_SMEM - 64) / (8 * Dp)));
    const size_t sm_e = sizeof(float) * 2 * 3 * (size_t)ch_e * Dp + 2 * sizeof(uint64_t);
    const size_t sm_q = sizeof(float) * 2 * (size_t)ch_q * Dp + 2 * sizeof(uint64_t);
    XG_CUDA(cudaFuncSetAttribute(k_entry_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm_e));
    XG_CUDA(cudaFuncSetAttribute(k_q_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm_q));
    if (NE > 0) {
      k_entry_f32<<<NE, bs, sm_e, st>>>(NE, D, Dp, ch_e, s.n_entry_pix_ptr.p, s.n_tg.p,
                                        s.n_ti.p, s.n_tf.p, s.n_ratio32.p, &s.stats.p->error);
      XG_CHECK_LAUNCH();
    }
    k_q_f32<<<NQ, bs, sm_q, st>>>(NQ, D, Dp, ch_q, s.n_q_entry_ptr.p, s.n_q_row.p,
                                  s.n_entry_pix_ptr.p, s.n_ratio32.p, s.n_tx.p, s.n_g2f.p,
                                  s.n_sef.p, s.n_unsafe.p, &s.stats.p->error);
    XG_CHECK_LAUNCH();
  }
}

}  // namespace xg
