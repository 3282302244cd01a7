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
// Streaming is two passes over each chunk of frames.  A warp owns a tile of
// 256 pixels (8 per lane, one 16-byte load per frame, R_min in registers) and
// walks a slice of the chunk's frames, 4 frames in flight: the first pass
// counts the kept pixels per (frame, tile), a scan turns the counts into
// offsets, and the second pass writes (pixel, value) at the offsets, in pixel
// order within a frame.  Events stay frame-major, as sparse frames are, and
// frames that the stride skips are not emitted.
#include <algorithm>
#include <climits>
#include <vector>

#include "f64emu.cuh"
#include "xpcs_internal.h"

namespace xg {
namespace {

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

// Per-pixel forms of the dark level and the gain (f64emu.cuh).
struct DensePrep {
  EmuSubPrep sub;
  EmuMulPrep mul;
};

// dense_value followed by the flatfield, as the reference forms a kept
// event's value: the two double-rounded steps in integer arithmetic
// (f64emu.cuh), by the per-pixel short forms where they apply, else by the
// general ones, and in double precision only outside their range
__device__ __forceinline__ float dense_event_value(int32_t raw, bool dark, const double *avg,
                                                   const double *flat, const DensePrep *prep,
                                                   int p) {
  float v = (float)raw;
  if (dark) {
    const EmuSubPrep q = prep[p].sub;
    const int64_t n = (int64_t)raw - q.c0;
    if (q.c0 != INT32_MIN && n >= 1 && n < (1 << 24)) {
      v = f32_sub_fast((int32_t)n, q.G);
    } else {
      const double A = avg[p];
      if (!f32_int_minus_f64(raw, A, v)) v = __double2float_rn(__dsub_rn((double)v, A));
    }
    v = v > 0.0f ? v : 0.0f;  // std::max(v, 0.0f)
  }
  if (flat) {
    const EmuMulPrep q = prep[p].mul;
    float w;
    if (!(q.eg != INT32_MIN && v > 0.f && f32_mul_fast(v, q, w))) {
      const double g = flat[p];
      if (!f32_mul_f64(v, g, w)) w = __double2float_rn(__dmul_rn((double)v, g));
    }
    v = w;
  }
  return v;
}

// Smallest raw value (int16 range) that the filter keeps, per pixel.
__global__ void k_rmin(int32_t P, const uint8_t *__restrict__ mask, int32_t has_dark,
                       const double *__restrict__ avg, const double *__restrict__ sd, float lld,
                       float sigma, const double *__restrict__ flat, int32_t *__restrict__ rmin,
                       DensePrep *__restrict__ prep) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  prep[p].sub = has_dark ? emu_sub_prep(avg[p]) : EmuSubPrep{INT32_MIN, 0};
  prep[p].mul = flat ? emu_mul_prep(flat[p]) : EmuMulPrep{INT32_MIN, 0};
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
  int32_t n, P, T;        // frames, pixels, warp tiles of KB_WPIX pixels
  int32_t r0;             // raw index of the chunk's first frame
  int32_t R_in, stride, F;
  int32_t vec;            // rows are 16-byte aligned and P % 8 == 0
  int32_t fslice;         // frames per block row of the grid
  const int32_t *rmin;
};

constexpr int KB_LPIX = 8;                 // pixels per lane (one 16-byte load)
constexpr int KB_WPIX = 32 * KB_LPIX;      // pixels per warp tile
constexpr int KB_WARPS = 8;                // warps (tiles) per block
constexpr int KB_FU = 4;                   // frames a lane loads ahead (k_dense_write
                                           // selects among exactly 4)

__device__ __forceinline__ bool frame_used(const ChunkCfg &c, int f) {
  const int r = c.r0 + f;
  const int k = r / c.R_in;
  return k < c.F && ((r - k * c.R_in) % c.stride) == 0;
}

// the lane's 8 raw values of frame f (pixels p0 .. p0+7, zero past P), two
// int16 per word
__device__ __forceinline__ uint4 load8(const ChunkCfg &c, int f, int p0) {
  const int16_t *row = c.raw + (size_t)f * c.P;
  if (c.vec && p0 + KB_LPIX <= c.P) {
    const int4 u = __ldcs((const int4 *)(row + p0));
    return make_uint4((uint32_t)u.x, (uint32_t)u.y, (uint32_t)u.z, (uint32_t)u.w);
  }
  uint32_t h[KB_LPIX];
#pragma unroll
  for (int j = 0; j < KB_LPIX; j++)
    h[j] = p0 + j < c.P ? (uint32_t)(uint16_t)__ldcs(row + p0 + j) : 0u;
  return make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16),
                    h[6] | (h[7] << 16));
}

// raw value j (0..7) of a packed group
__device__ __forceinline__ int32_t raw_at(const uint4 &x, int j) {
  const uint32_t w = (j >> 1) == 0 ? x.x : ((j >> 1) == 1 ? x.y : ((j >> 1) == 2 ? x.z : x.w));
  return (j & 1) ? ((int32_t)w >> 16) : ((int32_t)(w << 16) >> 16);
}

__device__ __forceinline__ unsigned keep_mask(const uint4 &x, const int32_t (&rm)[KB_LPIX]) {
  unsigned m = 0;
#pragma unroll
  for (int j = 0; j < KB_LPIX; j++) m |= (raw_at(x, j) >= rm[j] ? 1u : 0u) << j;
  return m;
}

// Grid: x = groups of KB_WARPS warp tiles, y = slices of c.fslice frames.
// counts[f * T + t] = kept pixels of frame f in warp tile t (0 for frames the
// stride skips).
__global__ void __launch_bounds__(KB_WARPS * 32)
k_dense_count(ChunkCfg c, int32_t *__restrict__ counts) {
  constexpr int FU = 2 * KB_FU;  // frames in flight: the count pass is load-bound
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * KB_WARPS + (threadIdx.x >> 5);
  if (t >= c.T) return;
  const int p0 = t * KB_WPIX + lane * KB_LPIX;
  int32_t rm[KB_LPIX];
#pragma unroll
  for (int j = 0; j < KB_LPIX; j++) rm[j] = p0 + j < c.P ? c.rmin[p0 + j] : KB_NEVER;
  const int f0 = blockIdx.y * c.fslice, f1 = min(c.n, f0 + c.fslice);
  for (int fb = f0; fb < f1; fb += FU) {
    uint4 x[FU];
    bool used[FU];
#pragma unroll
    for (int u = 0; u < FU; u++) {
      used[u] = fb + u < f1 && frame_used(c, fb + u);
      if (used[u]) x[u] = load8(c, fb + u, p0);
    }
#pragma unroll
    for (int u = 0; u < FU; u++) {
      const int k = used[u] ? __popc(keep_mask(x[u], rm)) : 0;
      const int n = __reduce_add_sync(0xffffffffu, k);
      if (lane == 0 && fb + u < f1) counts[(size_t)(fb + u) * c.T + t] = n;
    }
  }
}

// Writes (pixel, value) of every kept pixel at its scanned offset, in pixel
// order within a frame, with value (float)((float)(raw - avg) * flat) as the
// reference forms it.  The warp first gathers the kept pixels of its frames
// in flight into shared memory (tile-local pixel, raw value), then all lanes
// evaluate them in order, so the per-event arithmetic runs on full warps and
// the stores are contiguous.
__global__ void __launch_bounds__(KB_WARPS * 32, 3)
k_dense_write(ChunkCfg c, const int64_t *__restrict__ offsets, int64_t base,
              const double *__restrict__ avg, const double *__restrict__ flat, int32_t has_dark,
              const DensePrep *__restrict__ prep, int32_t *__restrict__ out_idx,
              float *__restrict__ out_val) {
  __shared__ uint8_t s_loc[KB_WARPS][KB_FU * KB_WPIX];
  __shared__ int16_t s_raw[KB_WARPS][KB_FU * KB_WPIX];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int t = blockIdx.x * KB_WARPS + w;
  if (t >= c.T) return;
  const int tile0 = t * KB_WPIX, p0 = tile0 + lane * KB_LPIX;
  int32_t rm[KB_LPIX];
#pragma unroll
  for (int j = 0; j < KB_LPIX; j++) rm[j] = p0 + j < c.P ? c.rmin[p0 + j] : KB_NEVER;
  const int f0 = blockIdx.y * c.fslice, f1 = min(c.n, f0 + c.fslice);
  for (int fb = f0; fb < f1; fb += KB_FU) {
    uint4 x[KB_FU];
    int64_t o0[KB_FU];
    bool used[KB_FU];
#pragma unroll
    for (int u = 0; u < KB_FU; u++) {
      used[u] = fb + u < f1 && frame_used(c, fb + u);
      o0[u] = used[u] ? offsets[(size_t)(fb + u) * c.T + t] : 0;
      if (used[u]) x[u] = load8(c, fb + u, p0);
    }
    int start[KB_FU + 1];
    start[0] = 0;
#pragma unroll
    for (int u = 0; u < KB_FU; u++) {
      const unsigned m = used[u] ? keep_mask(x[u], rm) : 0u;
      const int cnt = __popc(m);
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      int k = start[u] + incl - cnt;
#pragma unroll
      for (int j = 0; j < KB_LPIX; j++) {
        if ((m >> j) & 1u) {
          s_loc[w][k] = (uint8_t)(lane * KB_LPIX + j);
          s_raw[w][k] = (int16_t)raw_at(x[u], j);
          k++;
        }
      }
      start[u + 1] = start[u] + __shfl_sync(0xffffffffu, incl, 31);
    }
    __syncwarp();
    const int total = start[KB_FU];
    for (int i = lane; i < total; i += 32) {
      const int u = (i >= start[1]) + (i >= start[2]) + (i >= start[3]);
      const int64_t ob = u == 0 ? o0[0] : (u == 1 ? o0[1] : (u == 2 ? o0[2] : o0[3]));
      const int su = u == 0 ? 0 : (u == 1 ? start[1] : (u == 2 ? start[2] : start[3]));
      const int p = tile0 + s_loc[w][i];
      const int64_t o = base + ob + (i - su);
      out_idx[o] = p;
      out_val[o] = dense_event_value(s_raw[w][i], has_dark, avg, flat, prep, p);
    }
    __syncwarp();
  }
}

// frame_end[f] = offsets[(f + 1) * T]: the end of frame f's events in the chunk
__global__ void k_frame_ends(int32_t n, int32_t T, const int64_t *__restrict__ offsets,
                             int64_t *__restrict__ frame_end) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < n) frame_end[f] = offsets[(size_t)(f + 1) * T];
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
  s.dn_prep.reserve(sizeof(DensePrep) * (size_t)P, st);
  k_rmin<<<(P + 255) / 256, 256, 0, st>>>(P, s.d_mask.p, s.has_dark ? 1 : 0, s.dark_avg.p,
                                           s.dark_std.p, s.desc.lld, s.desc.sigma,
                                           s.has_flat ? s.d_flat.p : nullptr, s.rmin.p,
                                           (DensePrep *)s.dn_prep.p);
  XG_CHECK_LAUNCH();
  s.rmin_ready = true;
}

void dense_ingest(Series &s, const int16_t *frames, int32_t nframes, bool on_device) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P, T = (P + KB_WPIX - 1) / KB_WPIX;
  if (!s.rmin_ready) dense_set_dark(s, nullptr, 0);
  // frames per pass: host frames go through a 256 MB staging buffer; frames
  // already on the device are taken up to 4096 at a time (one host sync each)
  const int64_t by_bytes = std::max<int64_t>(1, (256ll << 20) / (2ll * P));
  const int32_t chunk = std::max(1, std::min(nframes, (int32_t)(on_device ? 4096 : by_bytes)));
  DBuf<int16_t> staging;
  if (!on_device) staging.reserve((size_t)chunk * P, st);
  s.dn_counts.reserve((size_t)chunk * T, st);
  s.dn_offsets.reserve((size_t)chunk * T + 1, st);
  s.dn_frame_end.reserve((size_t)chunk, st);
  s.scan_tmp.reserve(scan_workspace_bytes((int64_t)chunk * T), st);
  std::vector<int64_t> ends((size_t)chunk);
  int sms = 0;
  XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s.device));
  const int gx = (T + KB_WARPS - 1) / KB_WARPS;
  for (int32_t f0 = 0; f0 < nframes; f0 += chunk) {
    const int32_t n = std::min(chunk, nframes - f0);
    const int16_t *src = frames + (size_t)f0 * P;
    const int16_t *raw = src;
    if (!on_device) {
      XG_CUDA(cudaMemcpyAsync(staging.p, src, sizeof(int16_t) * (size_t)n * P,
                              cudaMemcpyHostToDevice, st));
      raw = staging.p;
    }
    // slices of up to 256 frames: many blocks per SM, R_min loaded once per slice
    const int slices = std::max((n + 255) / 256, std::min((n + 15) / 16, (8 * sms + gx - 1) / gx));
    const int fslice = (n + slices - 1) / slices;
    const int vec = (P % KB_LPIX == 0) && ((uintptr_t)raw % 16 == 0);
    ChunkCfg c{raw, n, P, T, s.raw_frames, s.R_in, s.desc.stride_frames, s.F, vec, fslice,
               s.rmin.p};
    const dim3 grid(gx, (n + fslice - 1) / fslice);
    k_dense_count<<<grid, KB_WARPS * 32, 0, st>>>(c, s.dn_counts.p);
    XG_CHECK_LAUNCH();
    exclusive_scan_i32_i64(s.dn_counts.p, s.dn_offsets.p, (int64_t)n * T, s.scan_tmp.p, st);
    k_frame_ends<<<(n + 255) / 256, 256, 0, st>>>(n, T, s.dn_offsets.p, s.dn_frame_end.p);
    XG_CHECK_LAUNCH();
    XG_CUDA(cudaMemcpyAsync(ends.data(), s.dn_frame_end.p, sizeof(int64_t) * n,
                            cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaStreamSynchronize(st));
    const int64_t add = ends[(size_t)n - 1];
    const int64_t old = s.raw_events, tot = old + add;
    if (tot >= ((int64_t)1 << 32))
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "more than 2^32 events in one series");
    s.raw_idx.grow((size_t)(tot ? tot : 1), (size_t)old, st);
    s.raw_valf.grow((size_t)(tot ? tot : 1), (size_t)old, st);
    k_dense_write<<<grid, KB_WARPS * 32, 0, st>>>(c, s.dn_offsets.p, old, s.dark_avg.p,
                                                  s.has_flat ? s.d_flat.p : nullptr,
                                                  s.has_dark ? 1 : 0,
                                                  (const DensePrep *)s.dn_prep.p, s.raw_idx.p,
                                                  s.raw_valf.p);
    XG_CHECK_LAUNCH();
    for (int32_t f = 0; f < n; f++) s.frame_off.push_back(old + ends[f]);
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
