// K-b: dense (CCD) frames -> frame-major events, the input of the K-a transpose.
//
// Replaces DarkImage::Compute (src/xpcs/data_structure/dark_image.cpp:81-106)
// and the per-pixel part of DenseFilter::Apply
// (src/xpcs/filter/dense_filter.cpp:150-174):
//   v = (float)raw; if darks: v = (float)(v - dark_avg); v = max(v, 0);
//   thresh = (float)(lld + sigma * dark_std); keep if v > thresh;
//   v = (float)(v * flatfield).
// Every step of v is a non-decreasing function of the raw value and thresh
// is fixed per pixel, so "kept" is equivalent to raw >= R_min(pixel).  A
// one-off kernel finds R_min by bisection over the int16 range with the
// reference's own double/float operations; the streaming kernels then compare
// int16 values only and evaluate the exact float arithmetic for kept pixels.
//
// Streaming is two passes over each chunk of frames, tile by tile (a block
// keeps its pixels' R_min in registers across the chunk's frames): count the
// kept pixels per (frame, tile), scan, then write (pixel, value) at the
// scanned offsets, in pixel order within a frame.  Events stay frame-major,
// as sparse frames are, and sub-frames that stride skips are not emitted.
#include <algorithm>
#include <vector>

#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int KB_THREADS = 256;
constexpr int KB_PPT = 4;                         // pixels per thread
constexpr int KB_TILE = KB_THREADS * KB_PPT;      // pixels per tile
constexpr int32_t KB_NEVER = 32768;               // R_min of a pixel that never passes

// DarkImage::Compute: running mean and M2 in double over the dark frames of
// raw*flat; std = sqrt(M2 / n).  One thread per pixel, frames in order.
__global__ void k_dark(int32_t P, int32_t nd, const int16_t *__restrict__ dark,
                       const double *__restrict__ flat, double *__restrict__ avg,
                       double *__restrict__ sd) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const double f = flat ? flat[p] : 1.0;
  double a = 0.0, s = 0.0;
  for (int i = 0; i < nd; i++) {
    const double tmp = a;
    const double pix = __dmul_rn((double)(float)dark[(size_t)i * P + p], f);
    a = __dadd_rn(a, __ddiv_rn(__dsub_rn(pix, a), (double)(i + 1)));
    s = __dadd_rn(s, __dmul_rn(__dsub_rn(pix, tmp), __dsub_rn(pix, a)));
  }
  avg[p] = a;
  sd[p] = __dsqrt_rn(__ddiv_rn(s, (double)nd));
}

__device__ __forceinline__ float dense_value(int32_t raw, bool dark, double avg) {
  float v = (float)raw;
  if (dark) {
    v = __double2float_rn(__dsub_rn((double)v, avg));
    v = v > 0.0f ? v : 0.0f;  // std::max(v, 0.0f)
  }
  return v;
}

// Smallest raw value (int16 range) that the filter keeps, per pixel.
__global__ void k_rmin(int32_t P, const uint8_t *__restrict__ mask, int32_t has_dark,
                       const double *__restrict__ avg, const double *__restrict__ sd, float lld,
                       float sigma, int32_t *__restrict__ rmin) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  if (!mask[p]) {
    rmin[p] = KB_NEVER;
    return;
  }
  const double a = has_dark ? avg[p] : 0.0;
  const float thresh =
      has_dark ? __double2float_rn(__dadd_rn((double)lld, __dmul_rn((double)sigma, sd[p]))) : 0.0f;
  int lo = -32768, hi = KB_NEVER;  // answer in [lo, hi]; hi == KB_NEVER: none
  if (dense_value(32767, has_dark, a) <= thresh) {
    rmin[p] = KB_NEVER;
    return;
  }
  hi = 32767;
  while (lo < hi) {
    const int mid = lo + ((hi - lo) >> 1);
    if (dense_value(mid, has_dark, a) > thresh)
      hi = mid;
    else
      lo = mid + 1;
  }
  rmin[p] = lo;
}

struct ChunkCfg {
  const int16_t *raw;     // [n][P] frames of this chunk
  int32_t n, P, T;        // frames, pixels, tiles
  int32_t r0;             // raw index of the chunk's first frame
  int32_t R_in, stride, F;
  const int32_t *rmin;
};

__device__ __forceinline__ bool frame_used(const ChunkCfg &c, int f) {
  const int r = c.r0 + f;
  const int k = r / c.R_in;
  return k < c.F && ((r - k * c.R_in) % c.stride) == 0;
}

__global__ void __launch_bounds__(KB_THREADS)
k_dense_count(ChunkCfg c, int32_t *__restrict__ counts) {
  __shared__ int32_t wsum[KB_THREADS / 32];
  const int t = blockIdx.x;
  const int p0 = t * KB_TILE + threadIdx.x * KB_PPT;
  int32_t rm[KB_PPT];
#pragma unroll
  for (int j = 0; j < KB_PPT; j++) rm[j] = p0 + j < c.P ? c.rmin[p0 + j] : KB_NEVER;
  for (int f = 0; f < c.n; f++) {
    int cnt = 0;
    if (frame_used(c, f)) {
      const int16_t *row = c.raw + (size_t)f * c.P;
#pragma unroll
      for (int j = 0; j < KB_PPT; j++)
        if (p0 + j < c.P && (int32_t)row[p0 + j] >= rm[j]) cnt++;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
      int s = 0;
      for (int w = 0; w < KB_THREADS / 32; w++) s += wsum[w];
      counts[(size_t)f * c.T + t] = s;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(KB_THREADS)
k_dense_write(ChunkCfg c, const int64_t *__restrict__ offsets, int64_t base,
              const double *__restrict__ avg, const double *__restrict__ flat, int32_t has_dark,
              int32_t *__restrict__ out_idx, float *__restrict__ out_val) {
  __shared__ int32_t wsum[KB_THREADS / 32];
  const int t = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int p0 = t * KB_TILE + threadIdx.x * KB_PPT;
  int32_t rm[KB_PPT];
#pragma unroll
  for (int j = 0; j < KB_PPT; j++) rm[j] = p0 + j < c.P ? c.rmin[p0 + j] : KB_NEVER;
  for (int f = 0; f < c.n; f++) {
    if (!frame_used(c, f)) continue;  // block-uniform
    const int16_t *row = c.raw + (size_t)f * c.P;
    int16_t rv[KB_PPT];
    int cnt = 0;
#pragma unroll
    for (int j = 0; j < KB_PPT; j++) {
      rv[j] = p0 + j < c.P ? row[p0 + j] : (int16_t)0;
      if (p0 + j < c.P && (int32_t)rv[j] >= rm[j]) cnt++;
    }
    // exclusive prefix of counts over the block (pixel order)
    int x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    int before = 0;
    for (int ww = 0; ww < w; ww++) before += wsum[ww];
    int64_t o = base + offsets[(size_t)f * c.T + t] + before + x - cnt;
#pragma unroll
    for (int j = 0; j < KB_PPT; j++) {
      const int p = p0 + j;
      if (p < c.P && (int32_t)rv[j] >= rm[j]) {
        float v = dense_value(rv[j], has_dark, has_dark ? avg[p] : 0.0);
        if (flat) v = __double2float_rn(__dmul_rn((double)v, flat[p]));
        out_idx[o] = p;
        out_val[o] = v;
        o++;
      }
    }
    __syncthreads();
  }
}

}  // namespace

void dense_set_dark(Series &s, const int16_t *dark_host, int32_t nd) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P;
  s.dark_avg.reserve(P, st);
  s.dark_std.reserve(P, st);
  s.rmin.reserve(P, st);
  s.has_dark = nd > 0;
  if (nd > 0) {
    DBuf<int16_t> tmp;
    tmp.reserve((size_t)nd * P, st);
    XG_CUDA(cudaMemcpyAsync(tmp.p, dark_host, sizeof(int16_t) * (size_t)nd * P,
                            cudaMemcpyHostToDevice, st));
    k_dark<<<(P + 255) / 256, 256, 0, st>>>(P, nd, tmp.p, s.has_flat ? s.d_flat.p : nullptr,
                                             s.dark_avg.p, s.dark_std.p);
    XG_CHECK_LAUNCH();
    tmp.release(st);
  }
  k_rmin<<<(P + 255) / 256, 256, 0, st>>>(P, s.d_mask.p, s.has_dark ? 1 : 0, s.dark_avg.p,
                                           s.dark_std.p, s.desc.lld, s.desc.sigma, s.rmin.p);
  XG_CHECK_LAUNCH();
  s.rmin_ready = true;
}

void dense_ingest(Series &s, const int16_t *frames, int32_t nframes, bool on_device) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P, T = (P + KB_TILE - 1) / KB_TILE;
  if (!s.rmin_ready) dense_set_dark(s, nullptr, 0);
  const int32_t chunk = std::max(1, std::min(nframes, (int32_t)std::max<int64_t>(1, (256ll << 20) / (2ll * P))));
  DBuf<int16_t> staging;
  if (!on_device) staging.reserve((size_t)chunk * P, st);
  s.dn_counts.reserve((size_t)chunk * T, st);
  s.dn_offsets.reserve((size_t)chunk * T + 1, st);
  s.scan_tmp.reserve(scan_workspace_bytes((int64_t)chunk * T), st);
  std::vector<int64_t> offs((size_t)chunk * T + 1);
  for (int32_t f0 = 0; f0 < nframes; f0 += chunk) {
    const int32_t n = std::min(chunk, nframes - f0);
    const int16_t *src = frames + (size_t)f0 * P;
    const int16_t *raw = src;
    if (!on_device) {
      XG_CUDA(cudaMemcpyAsync(staging.p, src, sizeof(int16_t) * (size_t)n * P,
                              cudaMemcpyHostToDevice, st));
      raw = staging.p;
    }
    ChunkCfg c{raw, n, P, T, s.raw_frames, s.R_in, s.desc.stride_frames, s.F, s.rmin.p};
    k_dense_count<<<T, KB_THREADS, 0, st>>>(c, s.dn_counts.p);
    XG_CHECK_LAUNCH();
    exclusive_scan_i32_i64(s.dn_counts.p, s.dn_offsets.p, (int64_t)n * T, s.scan_tmp.p, st);
    XG_CUDA(cudaMemcpyAsync(offs.data(), s.dn_offsets.p, sizeof(int64_t) * ((size_t)n * T + 1),
                            cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaStreamSynchronize(st));
    const int64_t add = offs[(size_t)n * T];
    const int64_t old = s.raw_events, tot = old + add;
    if (tot >= ((int64_t)1 << 32))
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "more than 2^32 events in one series");
    s.raw_idx.grow((size_t)(tot ? tot : 1), (size_t)old, st);
    s.raw_valf.grow((size_t)(tot ? tot : 1), (size_t)old, st);
    k_dense_write<<<T, KB_THREADS, 0, st>>>(c, s.dn_offsets.p, old, s.dark_avg.p,
                                            s.has_flat ? s.d_flat.p : nullptr, s.has_dark ? 1 : 0,
                                            s.raw_idx.p, s.raw_valf.p);
    XG_CHECK_LAUNCH();
    for (int32_t f = 0; f < n; f++) s.frame_off.push_back(old + offs[(size_t)(f + 1) * T]);
    s.raw_events = tot;
    s.raw_frames += n;
    s.frame_off_dirty = true;
  }
  if (!on_device) staging.release(st);
  s.have_multitau = false;
}

void dense_get_dark(Series &s, double *avg, double *sd) {
  if (!s.has_dark) throw Error(XPCS_ERR_STATE, "no dark frames were set");
  if (avg)
    XG_CUDA(cudaMemcpyAsync(avg, s.dark_avg.p, sizeof(double) * s.P, cudaMemcpyDeviceToHost, s.stream));
  if (sd)
    XG_CUDA(cudaMemcpyAsync(sd, s.dark_std.p, sizeof(double) * s.P, cudaMemcpyDeviceToHost, s.stream));
  XG_CUDA(cudaStreamSynchronize(s.stream));
}

}  // namespace xg
