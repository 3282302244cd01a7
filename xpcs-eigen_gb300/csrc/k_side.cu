// F1: side statistics of the filters, bit-identical to the reference.
//
// SparseFilter::Apply / DenseFilter::Apply accumulate, per filter frame and
// in ascending pixel order (sparse_filter.cpp:160-192, dense_filter.cpp:176-
// 208), with float adds:
//   pixels_sum_[pix]                       += v   (frame order per pixel)
//   f_sum                                  += v   -> frames_sum_[F + k] = f_sum / P
//   partitions_mean_[sbin]                 += v   (frame-major, pixel order)
//   partial_partitions_mean_[win][sbin]    += v
// and main.cpp:321-411 divides pixelSum by the frame count and the partition
// means by pixels_per_bin * window (or * frames).  The float sums depend on
// the order, so they are replayed in it: pixel sums come from the merge pass
// (rows are in frame order); the event lists are stably re-sorted by frame
// (giving frame-major, pixel-ascending order), summed per frame, then stably
// re-sorted by static bin (keeping that order inside each bin) and summed per
// bin and per (window, bin).  Pixel-major dense series, whose finishing pass
// skips the pixel sums, get them here from their rows.
#include <vector>

#include "xpcs_internal.h"

namespace xg {
namespace {

__device__ __forceinline__ int64_t lower_bound_u32(const uint32_t *a, int64_t n, uint32_t x) {
  int64_t first = 0, len = n;
  while (len > 0) {
    int64_t half = len >> 1;
    if (a[first + half] < x) {
      first += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return first;
}

// rows (pixel-major) -> compact triples (key = frame, a = pixel, b = value)
__global__ void k_side_build(int32_t P, const int64_t *__restrict__ row_ptr,
                             const int32_t *__restrict__ row_len, const int64_t *__restrict__ cpos,
                             const int32_t *__restrict__ fr, const float *__restrict__ val,
                             uint32_t *__restrict__ key, int32_t *__restrict__ a,
                             float *__restrict__ b) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int64_t src = row_ptr[p], dst = cpos[p];
  for (int i = 0; i < row_len[p]; i++) {
    key[dst + i] = (uint32_t)fr[src + i];
    a[dst + i] = p;
    b[dst + i] = val[src + i];
  }
}

__global__ void k_frame_sums(int32_t F, int32_t P, int64_t n, const uint32_t *__restrict__ key,
                             const float *__restrict__ b, float *__restrict__ frame_sum) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= F) return;
  const int64_t lo = lower_bound_u32(key, n, (uint32_t)k), hi = lower_bound_u32(key, n, (uint32_t)k + 1);
  float f = 0.f;
  for (int64_t i = lo; i < hi; i++) f = __fadd_rn(f, b[i]);
  frame_sum[k] = (float)(k + 1.0);
  frame_sum[F + k] = __fdiv_rn(f, (float)P);
}

// key <- static bin of the pixel in a; a <- frame (the old key)
__global__ void k_sbin_keys(int64_t n, const int32_t *__restrict__ sbin, uint32_t *__restrict__ key,
                            int32_t *__restrict__ a) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t f = key[i];
  key[i] = (uint32_t)sbin[a[i]];
  a[i] = (int32_t)f;
}

// one thread per static bin: the whole-series sum, in event order
__global__ void k_part_total(int32_t S, int64_t n, const uint32_t *__restrict__ key,
                             const float *__restrict__ b, const int32_t *__restrict__ ppb,
                             int32_t F, float *__restrict__ total) {
  const int sb = blockIdx.x * blockDim.x + threadIdx.x;
  if (sb >= S) return;
  const int64_t lo = lower_bound_u32(key, n, (uint32_t)sb), hi = lower_bound_u32(key, n, (uint32_t)sb + 1);
  float acc = 0.f;
  int64_t i = lo;
  for (; i + 8 <= hi; i += 8) {
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = b[i + j];
#pragma unroll
    for (int j = 0; j < 8; j++) acc = __fadd_rn(acc, x[j]);
  }
  for (; i < hi; i++) acc = __fadd_rn(acc, b[i]);
  total[sb] = __fdiv_rn(acc, __fmul_rn((float)ppb[sb], (float)F));
}

// one thread per (window, static bin): the window's sum, in event order
__global__ void k_part_partial(int32_t S, int32_t nwin, int32_t sw, int64_t n,
                               const uint32_t *__restrict__ key, const int32_t *__restrict__ frame,
                               const float *__restrict__ b, const int32_t *__restrict__ ppb,
                               float *__restrict__ partial) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= S * nwin) return;
  const int w = idx / S, sb = idx - w * S;
  const int64_t lo = lower_bound_u32(key, n, (uint32_t)sb), hi = lower_bound_u32(key, n, (uint32_t)sb + 1);
  // frames ascend inside the bin's segment
  int64_t a = lo, len = hi - lo;
  while (len > 0) {
    int64_t h = len >> 1;
    if (frame[a + h] < w * sw) {
      a += h + 1;
      len -= h + 1;
    } else {
      len = h;
    }
  }
  float acc = 0.f;
  for (int64_t i = a; i < hi && frame[i] < (w + 1) * sw; i++) acc = __fadd_rn(acc, b[i]);
  const float den = __fmul_rn((float)ppb[sb], (float)sw);
  partial[(size_t)w * S + sb] = __fdiv_rn(acc, den);
}

// pixels_sum_[pix] += v over a row in frame order, for rows whose finishing
// pass does not form the sums (pixel-major dense series).
__global__ void k_row_sums(int32_t P, const int64_t *__restrict__ row_ptr,
                           const int32_t *__restrict__ row_len, const float *__restrict__ val,
                           float *__restrict__ ps) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int64_t b = row_ptr[p];
  float a = 0.f;
  for (int32_t i = 0; i < row_len[p]; i++) a = __fadd_rn(a, val[b + i]);
  ps[p] = a;
}

__global__ void k_pixel_sums(int32_t P, int32_t F, const float *__restrict__ ps,
                             float *__restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < P) out[p] = __fdiv_rn(ps[p], (float)F);
}

}  // namespace

void run_side_stats(Series &s, const SideOut &out) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P, F = s.F, S = s.qmap.total_static;
  const int32_t sw = s.desc.static_window, nwin = sw > 0 ? F / sw : 0;
  XG_CUDA(cudaStreamSynchronize(st));
  DevStats stats{};
  XG_CUDA(cudaMemcpy(&stats, s.stats.p, sizeof(stats), cudaMemcpyDeviceToHost));
  const int64_t n = (int64_t)stats.events;
  // device results: [P] pixel sums, [2F] frame sums, [S] totals, [nwin*S] partials
  const size_t nout = (size_t)P + 2 * (size_t)F + S + (size_t)nwin * S;
  s.side_out.reserve(nout ? nout : 1, st);
  float *d_pix = s.side_out.p, *d_fs = d_pix + P, *d_tot = d_fs + 2 * (size_t)F,
        *d_part = d_tot + S;
  XG_CUDA(cudaMemsetAsync(s.side_out.p, 0, sizeof(float) * nout, st));
  const int bs = 256;
  if (s.dense_px) {
    k_row_sums<<<(P + bs - 1) / bs, bs, 0, st>>>(P, s.row_ptr.p, s.row_len.p, s.ev_val.p,
                                                  s.pixels_sum.p);
    XG_CHECK_LAUNCH();
  }
  k_pixel_sums<<<(P + bs - 1) / bs, bs, 0, st>>>(P, F, s.pixels_sum.p, d_pix);
  XG_CHECK_LAUNCH();
  if (n > 0) {
    s.side_pos.reserve((size_t)P + 1, st);
    s.scan_tmp.reserve(scan_workspace_bytes(P), st);
    exclusive_scan_i32_i64(s.row_len.p, s.side_pos.p, P, s.scan_tmp.p, st);
    s.keyA.reserve(n, st);
    s.frA.reserve(n, st);
    s.vA.reserve(n, st);
    s.keyB.reserve(n, st);
    s.frB.reserve(n, st);
    s.vB.reserve(n, st);
    k_side_build<<<(P + bs - 1) / bs, bs, 0, st>>>(P, s.row_ptr.p, s.row_len.p, s.side_pos.p,
                                                    s.ev_frame.p, s.ev_val.p, s.keyA.p, s.frA.p,
                                                    s.vA.p);
    XG_CHECK_LAUNCH();
    const int fbits = 32 - __builtin_clz((unsigned)(F > 1 ? F - 1 : 1));
    const bool in_b = radix_sort_triples(s, s.keyA.p, s.frA.p, s.vA.p, s.keyB.p, s.frB.p, s.vB.p, n,
                                         fbits);
    uint32_t *k1 = in_b ? s.keyB.p : s.keyA.p, *k2 = in_b ? s.keyA.p : s.keyB.p;
    int32_t *a1 = in_b ? s.frB.p : s.frA.p, *a2 = in_b ? s.frA.p : s.frB.p;
    float *b1 = in_b ? s.vB.p : s.vA.p, *b2 = in_b ? s.vA.p : s.vB.p;
    k_frame_sums<<<(F + bs - 1) / bs, bs, 0, st>>>(F, P, n, k1, b1, d_fs);
    XG_CHECK_LAUNCH();
    k_sbin_keys<<<(unsigned)((n + bs - 1) / bs), bs, 0, st>>>(n, s.d_sbin.p, k1, a1);
    XG_CHECK_LAUNCH();
    const int sbits = 32 - __builtin_clz((unsigned)(S > 1 ? S - 1 : 1));
    const bool in2 = radix_sort_triples(s, k1, a1, b1, k2, a2, b2, n, sbits);
    uint32_t *kk = in2 ? k2 : k1;
    int32_t *ff = in2 ? a2 : a1;
    float *vv = in2 ? b2 : b1;
    k_part_total<<<(S + 63) / 64, 64, 0, st>>>(S, n, kk, vv, s.d_ppb.p, F, d_tot);
    XG_CHECK_LAUNCH();
    if (nwin > 0) {
      k_part_partial<<<(S * nwin + 63) / 64, 64, 0, st>>>(S, nwin, sw, n, kk, ff, vv, s.d_ppb.p,
                                                          d_part);
      XG_CHECK_LAUNCH();
    }
  } else {
    // no events: frame numbers still fill the first row of frameSum
    std::vector<float> fs(2 * (size_t)F, 0.f);
    for (int k = 0; k < F; k++) fs[k] = (float)(k + 1.0);
    if (F) XG_CUDA(cudaMemcpyAsync(d_fs, fs.data(), sizeof(float) * fs.size(), cudaMemcpyHostToDevice, st));
    XG_CUDA(cudaStreamSynchronize(st));
  }
  if (out.pixel_sum)
    XG_CUDA(cudaMemcpyAsync(out.pixel_sum, d_pix, sizeof(float) * P, cudaMemcpyDeviceToHost, st));
  if (out.frame_sum)
    XG_CUDA(cudaMemcpyAsync(out.frame_sum, d_fs, sizeof(float) * 2 * (size_t)F, cudaMemcpyDeviceToHost, st));
  if (out.part_total)
    XG_CUDA(cudaMemcpyAsync(out.part_total, d_tot, sizeof(float) * S, cudaMemcpyDeviceToHost, st));
  if (out.part_partial && nwin)
    XG_CUDA(cudaMemcpyAsync(out.part_partial, d_part, sizeof(float) * (size_t)nwin * S,
                            cudaMemcpyDeviceToHost, st));
  XG_CUDA(cudaStreamSynchronize(st));
}

// normalize_by_framesum (main.cpp:314-337): divisor frameSum[F+f] / mean per
// frame, mean = the float sum of frameSum[F..2F) in frame order / F, computed
// in float on the host exactly as the reference does; the float multi-tau
// kernel divides every value by it when it loads the rows.
void prepare_framesum_scale(Series &s) {
  const int32_t F = s.F;
  std::vector<float> fs(2 * (size_t)F + 1);
  run_side_stats(s, SideOut{nullptr, fs.data(), nullptr, nullptr});
  float acc = 0.f;
  for (int32_t f = 0; f < F; f++) acc += fs[(size_t)F + f];
  const float mean = acc / (float)F;
  std::vector<float> q((size_t)F + 1, 1.f);
  for (int32_t f = 0; f < F; f++) q[f] = fs[(size_t)F + f] / mean;
  s.d_fscale.reserve(q.size(), s.stream);
  XG_CUDA(cudaMemcpyAsync(s.d_fscale.p, q.data(), sizeof(float) * q.size(),
                          cudaMemcpyHostToDevice, s.stream));
  XG_CUDA(cudaStreamSynchronize(s.stream));
}

}  // namespace xg
