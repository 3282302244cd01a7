// K-d: per-partition normalisation of G2/IP/IF into g2 and its standard error.
//
// Replaces Corr::normalizeG2s (src/xpcs/corr.cpp:927-1091).  The q -> sbin ->
// pixel mapping of BuildQMap is flattened into entries (one per (q, sbin),
// q ascending, sbin ascending, pixels in raster order).
//
// float64 evaluation (the reported result):
//   k_entry_f64: one block per (entry, tau) reduces sum G2, sum IP, sum IF over
//                the entry's pixels; ratio = (G2/n) / ((IP/n) (IF/n)) (:966-1013).
//   k_q_f64:     one block per (q, tau): g2 = mean of the non-NaN entry ratios
//                (:1018-1040); stderr over the q's pixels of x = G2/(IP IF) with
//                NaN -> 0 still counted (quirk Q8), two passes (mean, then sum
//                of squared deviations), sqrt(1/n) sqrt(M2/n) (:1043-1087).
// float32 evaluation (bit-identical to the reference's float output):
//   k_entry_f32 / k_q_f32: one thread per (entry or q, tau) replays the
//   reference's sequential float operations in its order, including the
//   running-mean / M2 update of every pixel.
#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int NB = 256;

__device__ __forceinline__ double block_sum(double x, double *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if (lane == 0) sh[w] = x;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < NB / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (threadIdx.x == 0) sh[0] = r;
  }
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(NB)
k_entry_f64(int D, int P, const int32_t *__restrict__ epp, const int32_t *__restrict__ pix,
            const float *__restrict__ G2, const float *__restrict__ IP,
            const float *__restrict__ IF, double *__restrict__ ratio) {
  __shared__ double sh[NB / 32];
  const int e = blockIdx.x / D, t = blockIdx.x - e * D;
  const int k0 = epp[e], k1 = epp[e + 1];
  const size_t o = (size_t)t * P;
  double sg = 0, si = 0, sf = 0;
  for (int k = k0 + threadIdx.x; k < k1; k += NB) {
    int p = pix[k];
    sg += (double)G2[o + p];
    si += (double)IP[o + p];
    sf += (double)IF[o + p];
  }
  sg = block_sum(sg, sh);
  si = block_sum(si, sh);
  sf = block_sum(sf, sh);
  if (threadIdx.x == 0) {
    double c = (double)(k1 - k0);
    sg /= c;
    si /= c;
    sf /= c;
    ratio[(size_t)e * D + t] = sg / (si * sf);
  }
}

__global__ void __launch_bounds__(NB)
k_q_f64(int D, int P, int NQ, const int32_t *__restrict__ qep, const int32_t *__restrict__ qrow,
        const int32_t *__restrict__ epp, const int32_t *__restrict__ pix,
        const double *__restrict__ ratio, const float *__restrict__ G2,
        const float *__restrict__ IP, const float *__restrict__ IF, double *__restrict__ g2,
        double *__restrict__ se) {
  __shared__ double sh[NB / 32];
  const int qi = blockIdx.x / D, t = blockIdx.x - qi * D;
  const int e0 = qep[qi], e1 = qep[qi + 1];
  const int k0 = epp[e0], k1 = epp[e1];
  const size_t o = (size_t)t * P;
  const int row = qrow[qi];
  if (threadIdx.x == 0) {
    double acc = 0.0, cnt = 0.0;
    for (int e = e0; e < e1; e++) {
      double r = ratio[(size_t)e * D + t];
      acc += isnan(r) ? 0.0 : r;
      cnt += isnan(r) ? 0.0 : 1.0;
    }
    g2[(size_t)t * NQ + row] = acc / cnt;
  }
  double s = 0.0;
  for (int k = k0 + threadIdx.x; k < k1; k += NB) {
    int p = pix[k];
    double x = (double)G2[o + p] / ((double)IP[o + p] * (double)IF[o + p]);
    s += isnan(x) ? 0.0 : x;
  }
  const double n = (double)(k1 - k0);
  const double mean = block_sum(s, sh) / n;
  double m2 = 0.0;
  for (int k = k0 + threadIdx.x; k < k1; k += NB) {
    int p = pix[k];
    double x = (double)G2[o + p] / ((double)IP[o + p] * (double)IF[o + p]);
    x = isnan(x) ? 0.0 : x;
    m2 += (x - mean) * (x - mean);
  }
  m2 = block_sum(m2, sh);
  if (threadIdx.x == 0) se[(size_t)t * NQ + row] = sqrt(1.0 / n) * sqrt(m2 / n);
}

__global__ void k_entry_f32(int NE, int D, int P, const int32_t *__restrict__ epp,
                            const int32_t *__restrict__ pix, const float *__restrict__ G2,
                            const float *__restrict__ IP, const float *__restrict__ IF,
                            float *__restrict__ ratio) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= NE * D) return;
  const int e = idx / D, t = idx - e * D;
  const size_t o = (size_t)t * P;
  float sg = 0.f, si = 0.f, sf = 0.f;
  for (int k = epp[e]; k < epp[e + 1]; k++) {
    int p = pix[k];
    sg = __fadd_rn(sg, G2[o + p]);
    si = __fadd_rn(si, IP[o + p]);
    sf = __fadd_rn(sf, IF[o + p]);
  }
  const float c = (float)(epp[e + 1] - epp[e]);
  sg = __fdiv_rn(sg, c);
  si = __fdiv_rn(si, c);
  sf = __fdiv_rn(sf, c);
  ratio[(size_t)e * D + t] = __fdiv_rn(sg, __fmul_rn(si, sf));
}

__global__ void k_q_f32(int NQ_, int D, int P, int NQ, const int32_t *__restrict__ qep,
                        const int32_t *__restrict__ qrow, const int32_t *__restrict__ epp,
                        const int32_t *__restrict__ pix, const float *__restrict__ ratio,
                        const float *__restrict__ G2, const float *__restrict__ IP,
                        const float *__restrict__ IF, float *__restrict__ g2,
                        float *__restrict__ se) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= NQ_ * D) return;
  const int qi = idx / D, t = idx - qi * D;
  const int row = qrow[qi];
  const size_t o = (size_t)t * P;
  float acc = 0.f, cnt = 0.f;
  for (int e = qep[qi]; e < qep[qi + 1]; e++) {
    float r = ratio[(size_t)e * D + t];
    acc = __fadd_rn(acc, isnan(r) ? 0.f : r);
    cnt = __fadd_rn(cnt, isnan(r) ? 0.f : 1.f);
  }
  g2[(size_t)t * NQ + row] = __fdiv_rn(acc, cnt);
  float avg = 0.f, sd = 0.f, samples = 0.f;
  for (int k = epp[qep[qi]]; k < epp[qep[qi + 1]]; k++) {
    int p = pix[k];
    float tmpAvg = avg;
    float x = __fdiv_rn(G2[o + p], __fmul_rn(IP[o + p], IF[o + p]));
    x = isnan(x) ? 0.f : x;
    samples = __fadd_rn(samples, 1.f);
    float tmp0 = __fsub_rn(x, tmpAvg);
    float tmp00 = __fdiv_rn(tmp0, samples);
    tmp00 = isnan(tmp00) ? 0.f : tmp00;
    avg = __fadd_rn(avg, tmp00);
    float tmp3 = __fmul_rn(__fsub_rn(x, tmpAvg), __fsub_rn(x, avg));
    sd = __fadd_rn(sd, tmp3);
  }
  float stdNorm = __fdiv_rn(sd, samples);
  float inv = __fdiv_rn(1.f, samples);
  se[(size_t)t * NQ + row] = __fmul_rn(__fsqrt_rn(inv), __fsqrt_rn(stdNorm));
}

}  // namespace

void run_normalize(Series &s, bool want64, bool want32) {
  cudaStream_t st = s.stream;
  const int D = s.D, P = s.P, NQ = s.qmap.nq(), NE = s.qmap.nentries();
  if (D == 0 || NQ == 0) return;
  if (want64) {
    s.n_ratio64.reserve((size_t)(NE > 0 ? NE : 1) * D, st);
    s.n_g2.reserve((size_t)NQ * D, st);
    s.n_se.reserve((size_t)NQ * D, st);
    if (NE > 0) {
      k_entry_f64<<<NE * D, NB, 0, st>>>(D, P, s.n_entry_pix_ptr.p, s.n_pix.p, s.G2.p, s.IP.p,
                                         s.IF.p, s.n_ratio64.p);
      XG_CHECK_LAUNCH();
    }
    k_q_f64<<<NQ * D, NB, 0, st>>>(D, P, NQ, s.n_q_entry_ptr.p, s.n_q_row.p, s.n_entry_pix_ptr.p,
                                   s.n_pix.p, s.n_ratio64.p, s.G2.p, s.IP.p, s.IF.p, s.n_g2.p,
                                   s.n_se.p);
    XG_CHECK_LAUNCH();
  }
  if (want32) {
    s.n_ratio32.reserve((size_t)(NE > 0 ? NE : 1) * D, st);
    s.n_g2f.reserve((size_t)NQ * D, st);
    s.n_sef.reserve((size_t)NQ * D, st);
    const int bs = 64;
    if (NE > 0) {
      k_entry_f32<<<(NE * D + bs - 1) / bs, bs, 0, st>>>(NE, D, P, s.n_entry_pix_ptr.p, s.n_pix.p,
                                                         s.G2.p, s.IP.p, s.IF.p, s.n_ratio32.p);
      XG_CHECK_LAUNCH();
    }
    k_q_f32<<<(NQ * D + bs - 1) / bs, bs, 0, st>>>(NQ, D, P, NQ, s.n_q_entry_ptr.p, s.n_q_row.p,
                                                  s.n_entry_pix_ptr.p, s.n_pix.p, s.n_ratio32.p,
                                                  s.G2.p, s.IP.p, s.IF.p, s.n_g2f.p, s.n_sef.p);
    XG_CHECK_LAUNCH();
  }
}

}  // namespace xg
