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

#include "classify.cuh"
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

// ------------------------------------------------------- pixel-major blocks
//
// Series without stride or frame averaging (every raw frame is its own filter
// frame, so a pixel never has two events of one frame): a run of at most
// 65,536 frames goes straight to pixel-major rows, one block of the series'
// block store, with no frame-major stream and no transpose.
//   count   each pixel's kept frames per slice of the run;
//   prefix  per pixel, the slice counts become offsets within its row; the
//           rows are padded to whole 32-byte sectors (8 entries) and a scan
//           over the pixels places them in the block;
//   write   each lane appends its 8 pixels' kept frames as packed words
//           ((frame - run start) << 16 | raw value) to per-pixel sectors in
//           shared memory and stores every completed sector as one aligned
//           32-byte write.  Only completed sectors reach memory, so no partly
//           written line waits in L2 for the rest of its row (every pixel's
//           row grows at once: their open lines would not fit in L2).
//   gather  (when the series finishes) one warp per pixel reads its packed
//           rows of every block and forms the values with the pixel's dark
//           level and gain held in registers, as the reference forms them.
// A row's events come out in frame order, the order a stable transpose of the
// frame-major stream gives them, so the event lists are the same bit for bit.

// counts[y * P + p] = kept frames of pixel p in slice y of the run.
__global__ void __launch_bounds__(KB_WARPS * 32)
k_dense_count_px(ChunkCfg c, int32_t *__restrict__ counts) {
  constexpr int FU = 2 * KB_FU;  // frames in flight: the count pass is load-bound
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * KB_WARPS + (threadIdx.x >> 5);
  if (t >= c.T) return;
  const int p0 = t * KB_WPIX + lane * KB_LPIX;
  int32_t rm[KB_LPIX], k[KB_LPIX];
#pragma unroll
  for (int j = 0; j < KB_LPIX; j++) {
    rm[j] = p0 + j < c.P ? c.rmin[p0 + j] : KB_NEVER;
    k[j] = 0;
  }
  // every raw frame is its own filter frame: frames from F on are not used
  const int f0 = blockIdx.y * c.fslice, f1 = min(min(c.n, f0 + c.fslice), c.F - c.r0);
  for (int fb = f0; fb < f1; fb += FU) {
    uint4 x[FU];
    bool used[FU];
#pragma unroll
    for (int u = 0; u < FU; u++) {
      used[u] = fb + u < f1;
      if (used[u]) x[u] = load8(c, fb + u, p0);
    }
#pragma unroll
    for (int u = 0; u < FU; u++) {
      if (used[u]) {
#pragma unroll
        for (int j = 0; j < KB_LPIX; j++) k[j] += raw_at(x[u], j) >= rm[j] ? 1 : 0;
      }
    }
  }
  int32_t *dst = counts + (size_t)blockIdx.y * c.P + p0;
  if (c.vec && p0 + KB_LPIX <= c.P) {  // P % 8 == 0: 32-byte aligned
    ((int4 *)dst)[0] = make_int4(k[0], k[1], k[2], k[3]);
    ((int4 *)dst)[1] = make_int4(k[4], k[5], k[6], k[7]);
  } else {
#pragma unroll
    for (int j = 0; j < KB_LPIX; j++)
      if (p0 + j < c.P) dst[j] = k[j];
  }
}

constexpr int KB_SECTOR = 8;  // packed 4-byte entries per 32-byte sector

// Per pixel: its slice counts become exclusive offsets within its row of the
// block; len[p] = the row's length, padded[p] = the length rounded up to
// whole sectors (the row's room in the block); *sum += the lengths.
__global__ void k_dense_prefix_px(int32_t P, int32_t ns, int32_t *__restrict__ counts,
                                  int32_t *__restrict__ padded, int32_t *__restrict__ len,
                                  unsigned long long *__restrict__ sum) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p - (int)(threadIdx.x & 31) >= P) return;  // whole warp past the end
  int32_t run = 0;
  if (p < P) {
    for (int y = 0; y < ns; y++) {
      int32_t *c = counts + (size_t)y * P + p;
      const int32_t k = *c;
      *c = run;
      run += k;
    }
    len[p] = run;
    padded[p] = (run + KB_SECTOR - 1) & ~(KB_SECTOR - 1);
  }
  const unsigned w = __reduce_add_sync(0xffffffffu, (unsigned)run);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(sum, (unsigned long long)w);
}

// Shared memory of the write pass, per warp: one open sector (8 entries) for
// each of its 256 pixels, laid out [pixel j of the lane][slot][lane] so that
// the lanes' stores of one j fall in distinct banks, then each pixel's next
// entry in the block, [j][lane].  Every word is private to its lane: shared
// memory serves as storage that a lane can index by the pixel it is on.
// After those, per warp, the raw words of the frames in flight, [frame][lane].
constexpr size_t KB_PX_WARP =
    (size_t)KB_WPIX * (KB_SECTOR + 1) * 4 + (size_t)2 * KB_FU * 32 * sizeof(uint4);
constexpr size_t KB_PX_SMEM = (size_t)KB_WARPS * KB_PX_WARP;

// Stores entries [lo, hi) of the open sector of the lane's pixel j at sector
// address dst (32-byte aligned): the whole sector at once when lo = 0 and
// hi = 8, else entry by entry (the first sector of a run that starts inside
// it, shared with the previous slice, and the last, partly filled one).
__device__ __forceinline__ void px_flush(const uint32_t *stg, int j, int lane, uint32_t *dst,
                                         int lo, int hi) {
  const uint32_t *q = stg + (size_t)j * KB_SECTOR * 32 + lane;
  if (lo == 0 && hi == KB_SECTOR) {
    const uint4 a = make_uint4(q[0], q[32], q[64], q[96]);
    const uint4 b = make_uint4(q[128], q[160], q[192], q[224]);
    ((uint4 *)dst)[0] = a;
    ((uint4 *)dst)[1] = b;
  } else {
    for (int e = lo; e < hi; e++) dst[e] = q[e * 32];
  }
}

// rp: the rows' starts in the block ([P + 1], from the scan of the padded
// lengths), pre: each (slice, pixel) run's offset within its row, out: the
// block's packed entries.  The slice-0 blocks also record each row's start.
// A lane visits only the kept pixels of its frames in flight (7 % of them on
// a CCD at 0.02 photons/pixel/frame): one compare per pixel and frame sets a
// bit of a 64-bit mask (frame-major), and the lane then walks the mask's set
// bits in order, so the warp waits on the lane with the most kept pixels over
// 8 frames rather than over each frame.  A bit's frame addresses the raw
// words kept in shared memory, its pixel the lane's open sector and offset;
// a pixel's frames come in frame order.
__global__ void __launch_bounds__(KB_WARPS * 32, 2)
k_dense_write_px(ChunkCfg c, const int32_t *__restrict__ pre, const int64_t *__restrict__ rp,
                 uint32_t *__restrict__ out, int32_t *__restrict__ blk_off) {
  extern __shared__ __align__(16) uint32_t px_stg[];
  constexpr int FU = 2 * KB_FU;
  static_assert(FU * KB_LPIX <= 64, "one bit of the kept mask per pixel and frame in flight");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int t = blockIdx.x * KB_WARPS + w;
  if (t >= c.T) return;
  uint8_t *wb = (uint8_t *)px_stg + (size_t)w * KB_PX_WARP;
  uint32_t *stg = (uint32_t *)wb;
  int32_t *so = (int32_t *)(wb + (size_t)KB_WPIX * KB_SECTOR * 4) + lane;  // so[j * 32]: pixel j's next entry
  uint4 *rawb = (uint4 *)(wb + (size_t)KB_WPIX * (KB_SECTOR + 1) * 4);  // [frame][lane]
  const int p0 = t * KB_WPIX + lane * KB_LPIX;
  const int32_t *pre_y = pre + (size_t)blockIdx.y * c.P;
  int32_t rm[KB_LPIX];
  uint32_t first = 0;  // 3 bits per pixel: where its run starts in its first sector
#pragma unroll
  for (int j = 0; j < KB_LPIX; j++) {
    const int p = p0 + j;
    int32_t o = 0;
    if (p < c.P) {
      rm[j] = c.rmin[p];
      const int64_t r = rp[p];
      o = (int32_t)r + pre_y[p];
      if (blockIdx.y == 0) blk_off[p] = (int32_t)r;
    } else {
      rm[j] = KB_NEVER;
    }
    so[j * 32] = o;
    first |= (uint32_t)(o & (KB_SECTOR - 1)) << (3 * j);
  }
  uint32_t open_first = (1u << KB_LPIX) - 1u;  // bit j: pixel j's open sector is its run's first
  // every raw frame is its own filter frame: frames from F on are not used
  const int f0 = blockIdx.y * c.fslice, f1 = min(min(c.n, f0 + c.fslice), c.F - c.r0);
  for (int fb = f0; fb < f1; fb += FU) {
    uint4 x[FU];
    bool used[FU];
#pragma unroll
    for (int u = 0; u < FU; u++) {
      used[u] = fb + u < f1;
      if (used[u]) x[u] = load8(c, fb + u, p0);
    }
    uint64_t m = 0;  // bit 8u + j: pixel j kept in frame fb + u
#pragma unroll
    for (int u = 0; u < FU; u++) {
      if (used[u]) {
        rawb[u * 32 + lane] = x[u];
        m |= (uint64_t)keep_mask(x[u], rm) << (8 * u);
      }
    }
    while (m) {
      const int b = __ffsll((long long)m) - 1;
      m &= m - 1u;
      const int u = b >> 3, j = b & 7;
      const uint32_t wd = ((const uint32_t *)&rawb[u * 32 + lane])[j >> 1];
      const uint32_t raw16 = (j & 1) ? (wd >> 16) : (wd & 0xffffu);
      const int32_t o = so[j * 32];
      const int slot = o & (KB_SECTOR - 1);
      stg[(j * KB_SECTOR + slot) * 32 + lane] = ((uint32_t)(fb + u) << 16) | raw16;
      so[j * 32] = o + 1;
      if (slot == KB_SECTOR - 1) {
        const int lo = ((open_first >> j) & 1u) ? (int)((first >> (3 * j)) & 7u) : 0;
        px_flush(stg, j, lane, out + (o + 1 - KB_SECTOR), lo, KB_SECTOR);
        open_first &= ~(1u << j);
      }
    }
  }
  // the last, partly filled sector of every run
#pragma unroll
  for (int j = 0; j < KB_LPIX; j++) {
    const int32_t o = so[j * 32];
    const int hi = o & (KB_SECTOR - 1);
    if (hi != 0) {
      const int lo = ((open_first >> j) & 1u) ? (int)((first >> (3 * j)) & 7u) : 0;
      px_flush(stg, j, lane, out + (o - hi), lo, hi);
    }
  }
}

// Per pixel: its row length summed over the blocks.
__global__ void k_px_totals(int32_t P, int32_t nblk, const int32_t *__restrict__ blk_len,
                            int32_t *__restrict__ tot) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int32_t t = 0;
  for (int32_t k = 0; k < nblk; k++) t += blk_len[(size_t)k * P + p];
  tot[p] = t;
}

constexpr int KB_VT = 128;  // raw values from a pixel's threshold up in its value table

struct PxGather {
  int32_t P, F, tcap, force_float, nblk, has_dark;
  const int64_t *blk_base;
  const int32_t *blk_r0, *blk_off, *blk_len;
  const uint32_t *pk;
  const int64_t *row_ptr;
  const uint8_t *mask;
  const int32_t *rmin;
  const double *avg, *flat;
  const DensePrep *prep;
  int32_t *fr;
  float *val;
  int32_t *row_len;
  uint8_t *pclass;
  ClassLists cl;
  DevStats *stats;
};

// One block per 32 pixels, each warp taking 4 of them in turn: a pixel's
// packed entries of every block, in block order, become (frame, value) in its
// row of the event lists.  For a given pixel the value is a function of the
// raw value alone: the warp first forms it, as the frame-major write does,
// for the 128 raw values from the pixel's threshold up (where nearly all kept
// values lie) and looks those up; others are formed directly.  The row's
// length, whether every value is an integer and sum |v| are collected on the
// way, and the block's first warp classifies the 32 pixels as the merge pass
// does for transposed rows (no row has two events of one frame here).
__global__ void __launch_bounds__(256)
k_dense_gather_px(PxGather g) {
  __shared__ float s_tab[KB_WARPS][KB_VT];
  __shared__ int32_t s_n[32], s_nonint[32];
  __shared__ long long s_tot[32];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int pb = blockIdx.x * 32;
  for (int q = 0; q < 32 / KB_WARPS; q++) {
    const int loc = q * KB_WARPS + w, p = pb + loc;
    if (p >= g.P) break;
    const int32_t rlo = g.rmin[p];
    int32_t n = 0;
    bool nonint = false;
    long long tot = 0;
    if (rlo < KB_NEVER) {
      for (int i = lane; i < KB_VT; i += 32)
        s_tab[w][i] = rlo + i <= 32767
                          ? dense_event_value(rlo + i, g.has_dark, g.avg, g.flat, g.prep, p)
                          : 0.f;
      __syncwarp();
      int64_t d = g.row_ptr[p];
      for (int32_t k = 0; k < g.nblk; k++) {
        const int32_t nk = g.blk_len[(size_t)k * g.P + p];
        const int64_t src = g.blk_base[k] + g.blk_off[(size_t)k * g.P + p];
        const int32_t r0 = g.blk_r0[k];
        // four 32-entry chunks' loads in flight before any is used
        for (int32_t i0 = 0; i0 < nk; i0 += 4 * 32) {
          uint32_t e[4];
#pragma unroll
          for (int h = 0; h < 4; h++) {
            const int32_t i = i0 + h * 32 + lane;
            e[h] = i < nk ? __ldcs(g.pk + src + i) : 0u;
          }
#pragma unroll
          for (int h = 0; h < 4; h++) {
            if (i0 + h * 32 >= nk) break;  // the same for every lane
            const int32_t i = i0 + h * 32 + lane;
            bool ni = false;
            unsigned a = 0;
            if (i < nk) {
              const int32_t raw = (int16_t)(e[h] & 0xffffu);
              const int32_t t = raw - rlo;  // >= 0: kept values pass the threshold
              const float v = t < KB_VT ? s_tab[w][t]
                                        : dense_event_value(raw, g.has_dark, g.avg, g.flat,
                                                            g.prep, p);
              g.fr[d + i] = r0 + (int32_t)(e[h] >> 16);
              g.val[d + i] = v;
              ni = !(v == truncf(v) && fabsf(v) < 16777216.f);
              a = ni ? 0u : (unsigned)fabsf(v);
            }
            nonint = nonint || __any_sync(FULL, ni);
            tot += __reduce_add_sync(FULL, a);
          }
        }
        d += nk;
        n += nk;
      }
      __syncwarp();  // the table is rebuilt for the warp's next pixel
    }
    if (lane == 0) {
      s_n[loc] = n;
      s_nonint[loc] = nonint ? 1 : 0;
      s_tot[loc] = tot;
      g.row_len[p] = n;
    }
  }
  __syncthreads();
  if (w == 0) {
    const int p = pb + lane;
    const bool has = p < g.P;
    const int32_t n = has ? s_n[lane] : 0;
    uint8_t c = has && g.mask[p] ? pixel_class(n, s_nonint[lane] == 0, s_tot[lane], g.F, g.tcap)
                                 : (uint8_t)PCLASS_EMPTY;
    if (g.force_float && c != PCLASS_EMPTY) c = PCLASS_FLOAT;  // values rescaled later
    record_class_warp(has, p, c, n, g.pclass, g.cl, g.stats);
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
  s.dn_prep.reserve(sizeof(DensePrep) * (size_t)P, st);
  k_rmin<<<(P + 255) / 256, 256, 0, st>>>(P, s.d_mask.p, s.has_dark ? 1 : 0, s.dark_avg.p,
                                           s.dark_std.p, s.desc.lld, s.desc.sigma,
                                           s.has_flat ? s.d_flat.p : nullptr, s.rmin.p,
                                           (DensePrep *)s.dn_prep.p);
  XG_CHECK_LAUNCH();
  s.rmin_ready = true;
}

namespace {

// Raw frames r0 .. r0+n-1, at raw on the device, as the next block of the
// block store; runs longer than 65,536 frames (the packed frame field), or
// whose padded rows would not fit the block's 32-bit row offsets, are split
// in halves (one frame holds at most P < 2^31 events).
void dense_px_block(Series &s, const int16_t *raw, int32_t n, int32_t r0) {
  if (n <= 0) return;
  cudaStream_t st = s.stream;
  const int32_t P = s.P, T = (P + KB_WPIX - 1) / KB_WPIX;
  if (n > 65536) {
    const int32_t h = n / 2;
    dense_px_block(s, raw, h, r0);
    dense_px_block(s, raw + (size_t)h * P, n - h, r0 + h);
    return;
  }
  int sms = 0;
  XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s.device));
  const int gx = (T + KB_WARPS - 1) / KB_WARPS;
  // slices of at least 64 frames, enough of them for 4 blocks per SM
  const int want = std::max(1, std::min((n + 63) / 64, (4 * sms + gx - 1) / gx));
  const int fslice = (n + want - 1) / want;
  const int ns = (n + fslice - 1) / fslice;
  const int vec = (P % KB_LPIX == 0) && ((uintptr_t)raw % 16 == 0);
  ChunkCfg c{raw, n, P, T, r0, s.R_in, s.desc.stride_frames, s.F, vec, fslice, s.rmin.p};
  const size_t k = s.blk_base.size();
  s.dn_counts.reserve((size_t)ns * P, st);
  s.dn_tot.reserve(P, st);
  s.blk_rp.reserve((size_t)P + 1, st);
  s.scan_tmp.reserve(scan_workspace_bytes(P), st);
  s.blk_off.grow((k + 1) * (size_t)P, k * (size_t)P, st);
  s.blk_len.grow((k + 1) * (size_t)P, k * (size_t)P, st);
  const dim3 grid(gx, ns);
  k_dense_count_px<<<grid, KB_WARPS * 32, 0, st>>>(c, s.dn_counts.p);
  XG_CHECK_LAUNCH();
  s.dn_sum.reserve(1, st);
  XG_CUDA(cudaMemsetAsync(s.dn_sum.p, 0, sizeof(unsigned long long), st));
  k_dense_prefix_px<<<(P + 255) / 256, 256, 0, st>>>(P, ns, s.dn_counts.p, s.dn_tot.p,
                                                      s.blk_len.p + k * P, s.dn_sum.p);
  XG_CHECK_LAUNCH();
  exclusive_scan_i32_i64(s.dn_tot.p, s.blk_rp.p, P, s.scan_tmp.p, st);
  int64_t total = 0;  // padded entries of the block
  unsigned long long events = 0;
  XG_CUDA(cudaMemcpyAsync(&total, s.blk_rp.p + P, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  XG_CUDA(cudaMemcpyAsync(&events, s.dn_sum.p, sizeof(events), cudaMemcpyDeviceToHost, st));
  XG_CUDA(cudaStreamSynchronize(st));
  if (total > (int64_t)INT32_MAX) {
    const int32_t h = n / 2;
    dense_px_block(s, raw, h, r0);
    dense_px_block(s, raw + (size_t)h * P, n - h, r0 + h);
    return;
  }
  // sector-aligned block start: rows and their sectors are 32-byte aligned
  const int64_t base = s.blk_events;
  s.blk_pk.grow((size_t)(base + std::max<int64_t>(total, KB_SECTOR)), (size_t)base, st);
  XG_CUDA(cudaFuncSetAttribute(k_dense_write_px, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)KB_PX_SMEM));
  k_dense_write_px<<<grid, KB_WARPS * 32, KB_PX_SMEM, st>>>(c, s.dn_counts.p, s.blk_rp.p,
                                                          s.blk_pk.p + base, s.blk_off.p + k * P);
  XG_CHECK_LAUNCH();
  s.blk_base.push_back(base);
  s.blk_r0.push_back(r0);
  // the device copies of the block tables are kept current here, so that
  // finishing the series (graph-captured in batches) uploads nothing
  s.d_blk_base.grow(k + 1, k, st);
  s.d_blk_r0.grow(k + 1, k, st);
  XG_CUDA(cudaMemcpyAsync(s.d_blk_base.p + k, &s.blk_base[k], sizeof(int64_t),
                          cudaMemcpyHostToDevice, st));
  XG_CUDA(cudaMemcpyAsync(s.d_blk_r0.p + k, &s.blk_r0[k], sizeof(int32_t),
                          cudaMemcpyHostToDevice, st));
  s.blk_events = base + total;  // a multiple of KB_SECTOR
  s.blk_raw_done = r0 + n;
  s.raw_events += (int64_t)events;
  if (s.raw_events >= ((int64_t)1 << 32))
    throw Error(XPCS_ERR_INVALID_ARGUMENT, "more than 2^32 events in one series");
}

// Frames per block of the pixel-major form: runs shorter than this wait in the
// pending buffer, so that each block's per-pixel tables (8 B per pixel) stay
// small beside its events.
int32_t px_block_frames(int32_t P) {
  return (int32_t)std::max<int64_t>(1, std::min<int64_t>(256, (512ll << 20) / (2ll * P)));
}

void dense_px_ingest(Series &s, const int16_t *frames, int32_t nframes, bool on_device) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P, bf = px_block_frames(P);
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  DBuf<int16_t> staging;
  int32_t f = 0;
  while (f < nframes) {
    const int32_t left = nframes - f;
    const int16_t *src = frames + (size_t)f * P;
    if (s.dn_pend_n == 0 && left >= bf) {
      // a long run: straight to blocks (host frames through a staging buffer
      // of up to 1 GB)
      int32_t m = left;
      const int16_t *raw = src;
      if (!on_device) {
        m = (int32_t)std::min<int64_t>(left, std::max<int64_t>(bf, (1ll << 30) / (2ll * P)));
        staging.reserve((size_t)m * P, st);
        XG_CUDA(cudaMemcpyAsync(staging.p, src, sizeof(int16_t) * (size_t)m * P,
                                cudaMemcpyHostToDevice, st));
        raw = staging.p;
      }
      dense_px_block(s, raw, m, s.raw_frames);
      s.raw_frames += m;
      f += m;
    } else {
      // a short run waits for more frames
      const int32_t m = std::min(left, bf - s.dn_pend_n);
      s.dn_pend.reserve((size_t)bf * P, st);
      if (s.dn_pend_n == 0) s.dn_pend_r0 = s.raw_frames;
      XG_CUDA(cudaMemcpyAsync(s.dn_pend.p + (size_t)s.dn_pend_n * P, src,
                              sizeof(int16_t) * (size_t)m * P, kind, st));
      s.dn_pend_n += m;
      s.raw_frames += m;
      f += m;
      if (s.dn_pend_n == bf) dense_px_flush(s);
    }
  }
  // host frames: the copies are done before the staging buffer goes back
  if (!on_device) XG_CUDA(cudaStreamSynchronize(st));
  staging.release(st);
}

}  // namespace

void dense_px_flush(Series &s) {
  if (!s.dense_px || s.dn_pend_n == 0) return;
  const int32_t n = s.dn_pend_n;
  s.dn_pend_n = 0;
  dense_px_block(s, s.dn_pend.p, n, s.dn_pend_r0);
}

void dense_px_gather(Series &s) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P, nblk = (int32_t)s.blk_base.size();
  s.blk_tot.reserve(P, st);
  if (nblk > 0) {
    k_px_totals<<<(P + 255) / 256, 256, 0, st>>>(P, nblk, s.blk_len.p, s.blk_tot.p);
    XG_CHECK_LAUNCH();
  } else {
    XG_CUDA(cudaMemsetAsync(s.blk_tot.p, 0, sizeof(int32_t) * (size_t)P, st));
  }
  exclusive_scan_i32_i64(s.blk_tot.p, s.row_ptr.p, P, s.scan_tmp.p, st);
  PxGather g{P, s.F, s.thread_cap, s.desc.normalize_by_framesum, nblk, s.has_dark ? 1 : 0,
             s.d_blk_base.p, s.d_blk_r0.p, s.blk_off.p, s.blk_len.p, s.blk_pk.p, s.row_ptr.p,
             s.d_mask.p, s.rmin.p, s.dark_avg.p, s.has_flat ? s.d_flat.p : nullptr,
             (const DensePrep *)s.dn_prep.p, s.ev_frame.p, s.ev_val.p, s.row_len.p, s.pclass.p,
             ClassLists{s.wlist.p, s.llist.p, s.flist.p}, s.stats.p};
  k_dense_gather_px<<<(P + 31) / 32, KB_WARPS * 32, 0, st>>>(g);
  XG_CHECK_LAUNCH();
}

void dense_ingest(Series &s, const int16_t *frames, int32_t nframes, bool on_device) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P, T = (P + KB_WPIX - 1) / KB_WPIX;
  if (!s.rmin_ready) dense_set_dark(s, nullptr, 0);
  if (s.dense_px) {
    dense_px_ingest(s, frames, nframes, on_device);
    s.have_multitau = false;
    return;
  }
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
