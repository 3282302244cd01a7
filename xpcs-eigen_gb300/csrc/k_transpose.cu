// K-a: sparse-frame filter and pixel-major transpose.
//
// Replaces SparseFilter::Apply (src/xpcs/filter/sparse_filter.cpp:115-193),
// which walks every frame and pushes (frame, value) onto per-pixel std::vector
// rows.  Here the raw frame-major event stream (int32 pixel index, int16 value)
// is filtered and stably sorted by pixel with an LSD radix sort, so that every
// pixel's events come out contiguous and in stream order (frame order).
//
//   pass 0   reads the raw events directly: per event it derives the filter
//            frame (raw frame / (stride*avg), from a per-warp-chunk table of
//            raw frames and a per-raw-frame table of filter frames), drops
//            unused stride sub-frames and frames past the end (key = P, sorts
//            last), and forms v = (float)(value * flatfield) as the reference
//            does (sparse_filter.cpp:149-153).
//   pass k   8-bit digit k of the pixel index: tile histograms -> digit-major
//            exclusive scan -> stable scatter.  Ranking inside a tile uses
//            per-bit warp ballots + per-warp digit counters, so equal digits
//            keep stream order (tile, warp, round, lane).
//   merge    one warp per 32 pixels: events of the same filter frame are
//            summed in stream order and divided by avg (sparse_filter.cpp:
//            160-172), pixelSum is accumulated in frame order, pixels outside
//            the mask (sparse_filter.cpp:147) get empty rows, and every pixel
//            is classified for the multi-tau kernels.
#include <algorithm>
#include <cstddef>

#include "f64emu.cuh"
#include "classify.cuh"
#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
// Items per lane: 8 (tiles of 2048) keeps more blocks resident; above
// RS_BIG_N events 16 (tiles of 4096) halves the tile histograms.
constexpr int64_t RS_BIG_N = (int64_t)1 << 27;
constexpr int RS_DIGITS = 256;
static_assert(RS_THREADS == RS_DIGITS, "one digit per thread in the downsweep scan");

// The raw frames [r0, r0 + nframes) of a series: idx/val/valf start at their
// first event e0, frame_off/frame_map at r0, and frame_off holds absolute
// event offsets, so an event's index relative to e0 is compared with
// frame_off[r] - e0.
struct RawCfg {
  const int32_t *idx;
  const int16_t *val;   // sparse series: raw values (flatfield applied here)
  const float *valf;    // dense series: values already filtered by K-b
  const int64_t *frame_off;  // [nframes+1]
  const int32_t *frame_map;  // [nframes]: filter frame of a raw frame, -1 if unused
  const int32_t *chunk_frame;  // [ceil(n / chunk)]: raw frame of item chunk * c
  int32_t nframes;
  int64_t e0;
  int64_t n;
  int32_t P, F, R_in, stride;
  const double *flat;  // may be null
  DevStats *stats;
};

struct PassCfg {
  const uint32_t *key_in;
  const int32_t *fr_in;
  const float *v_in;
  uint32_t *key_out;  // null on the last pass
  int32_t *fr_out;
  float *v_out;
  int64_t n;
  int shift;
  int ntiles;
  uint32_t sentinel;
};

// Raw frame of the first item of every chunk of 32 * IPT items (one warp's
// share of a tile): chunk c starts in frame r when off[r] - e0 <= chunk c <
// off[r + 1] - e0.
__global__ void k_chunk_frames(int32_t nframes, const int64_t *__restrict__ off, int64_t e0,
                               int64_t nchunks, int32_t chunk, int32_t *__restrict__ chunk_frame) {
  const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nframes) return;
  const int64_t c0 = (off[r] - e0 + chunk - 1) / chunk;
  const int64_t c1 = min((off[r + 1] - e0 + chunk - 1) / chunk, nchunks);
  for (int64_t c = c0; c < c1; c++) chunk_frame[c] = r;
}

// The raw loads of item i (pixel index and value), issued before any of the
// per-item work so that a lane's loads are in flight together.
__device__ __forceinline__ void raw_load(const RawCfg &c, int64_t i, int32_t &p, float &v) {
  p = c.idx[i];
  v = c.valf ? c.valf[i] : (float)c.val[i];
}

// Filter frame, sort key and filtered value of item i.  r is the raw frame of
// this lane's previous item, nb = frame_off[r + 1] and k = frame_map[r], kept
// in registers so that the common case (no frame boundary crossed) loads
// nothing.  Masked pixels keep their own key here; their rows are emptied by
// the merge, which reads the mask once per pixel instead of once per event.
__device__ __forceinline__ bool raw_frame_key(const RawCfg &c, int64_t i, int32_t &r, int64_t &nb,
                                              int32_t &k, int32_t p, uint32_t &key,
                                              int32_t &frame) {
  while (nb <= i) {
    r++;
    nb = c.frame_off[r + 1] - c.e0;
    k = c.frame_map[r];
  }
  frame = k;
  if (p < 0 || p >= c.P) {
    c.stats->error |= DEVERR_PIXEL_INDEX;
    key = (uint32_t)c.P;
    return false;
  }
  key = k >= 0 ? (uint32_t)p : (uint32_t)c.P;
  return true;
}

// (float)((double)v * g) as the reference forms a flat-fielded value,
// exactly, in integer arithmetic (f64emu.cuh)
__device__ __forceinline__ float flat_value(float v, double g) {
  float w;
  return f32_mul_f64(v, g, w) ? w : __double2float_rn(__dmul_rn((double)v, g));
}

__device__ __forceinline__ void raw_key(const RawCfg &c, int64_t i, int32_t &r, int64_t &nb,
                                        int32_t &k, int32_t p, float &v, uint32_t &key,
                                        int32_t &frame) {
  if (!raw_frame_key(c, i, r, nb, k, p, key, frame)) {
    v = 0.f;
    return;
  }
  if (!c.valf && c.flat) v = flat_value(v, c.flat[p]);
}

// Packed items (sparse series with fewer than 65,536 filter frames): filter
// frame in the high half, the raw int16 value in the low half.  The flatfield
// is applied when the last pass writes the events out.
__device__ __forceinline__ int32_t pack_item(int32_t frame, float raw) {
  return (int32_t)(((uint32_t)frame << 16) | ((uint32_t)(int32_t)raw & 0xffffu));
}

// Item i of a tile in warp-striped order: warp w owns [w*32*IPT, (w+1)*32*IPT),
// round k, lane l -> w*32*IPT + k*32 + l.
template <int IPT>
__device__ __forceinline__ int64_t item_index(int tile, int w, int k, int lane) {
  return (int64_t)tile * (RS_THREADS * IPT) + (int64_t)w * 32 * IPT + k * 32 + lane;
}

template <int IPT, bool FIRST>
__global__ void __launch_bounds__(RS_THREADS)
k_upsweep(RawCfg rc, PassCfg pc, uint32_t *__restrict__ hist) {
  __shared__ uint32_t h[RS_DIGITS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, tile = blockIdx.x;
  for (int d = threadIdx.x; d < RS_DIGITS; d += RS_THREADS) h[d] = 0;
  __syncthreads();
  uint32_t key[IPT];
  // all loads first, so that they are in flight together
  if (FIRST) {
    const int64_t nch = (rc.n + 32 * IPT - 1) / (32 * IPT);
    int32_t r = rc.chunk_frame[min((int64_t)tile * RS_WARPS + w, nch - 1)];
    int64_t nb = rc.frame_off[r + 1] - rc.e0;
    int32_t kf = rc.frame_map[r];
    int32_t pix[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      const int64_t i = item_index<IPT>(tile, w, k, lane);
      pix[k] = i < pc.n ? rc.idx[i] : 0;
    }
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      int64_t i = item_index<IPT>(tile, w, k, lane);
      key[k] = 0xffffffffu;
      if (i < pc.n) {
        while (nb <= i) {
          r++;
          nb = rc.frame_off[r + 1] - rc.e0;
          kf = rc.frame_map[r];
        }
        const int32_t p = pix[k];
        key[k] = (p < 0 || p >= rc.P || kf < 0) ? (uint32_t)rc.P : (uint32_t)p;
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      int64_t i = item_index<IPT>(tile, w, k, lane);
      key[k] = i < pc.n ? pc.key_in[i] : 0xffffffffu;
    }
  }
  int dropped = 0;  // items that sort last: their count gives the kept total
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    if (key[k] == 0xffffffffu) continue;
    if (FIRST && key[k] == pc.sentinel) dropped++;
    atomicAdd(&h[(key[k] >> pc.shift) & (RS_DIGITS - 1)], 1u);
  }
  if (FIRST) {
    dropped = __reduce_add_sync(0xffffffffu, dropped);
    if (lane == 0 && dropped) atomicAdd(&rc.stats->dropped, (unsigned long long)dropped);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RS_DIGITS; d += RS_THREADS)
    hist[(int64_t)d * pc.ntiles + tile] = h[d];
}

// Shared memory of the downsweep: per-warp digit counters, the tile's global
// and local digit offsets, and the tile staged in digit order.
template <int IPT, bool PK>
struct DsSmem {
  uint32_t wcnt[RS_WARPS][RS_DIGITS];
  uint32_t toff[RS_DIGITS];
  uint32_t tstart[RS_DIGITS];
  uint32_t wtot[RS_THREADS / 32];
  uint32_t key[RS_THREADS * IPT];
  int32_t fr[RS_THREADS * IPT];      // frame, or the packed item
  float v[PK ? 1 : RS_THREADS * IPT];
};

template <int IPT, bool FIRST, bool LAST, bool PK>
__global__ void __launch_bounds__(RS_THREADS)
k_downsweep(RawCfg rc, PassCfg pc, const uint32_t *__restrict__ offsets) {
  extern __shared__ __align__(16) uint8_t ds_raw[];
  DsSmem<IPT, PK> &sm = *reinterpret_cast<DsSmem<IPT, PK> *>(ds_raw);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, tile = blockIdx.x;
  for (int d = lane; d < RS_DIGITS; d += 32) sm.wcnt[w][d] = 0;
  for (int d = threadIdx.x; d < RS_DIGITS; d += RS_THREADS)
    sm.toff[d] = offsets[(int64_t)d * pc.ntiles + tile];
  __syncwarp();

  uint32_t key[IPT];
  int32_t fr[IPT];
  float v[IPT];
  uint32_t rank[IPT];
  const unsigned lt = (1u << lane) - 1u;
  // all loads first, so that they are in flight together
  if (FIRST) {
    const int64_t nch = (rc.n + 32 * IPT - 1) / (32 * IPT);
    int32_t r = rc.chunk_frame[min((int64_t)tile * RS_WARPS + w, nch - 1)];
    int64_t nb = rc.frame_off[r + 1] - rc.e0;
    int32_t kf = rc.frame_map[r];
    int32_t pix[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      const int64_t i = item_index<IPT>(tile, w, k, lane);
      pix[k] = 0;
      v[k] = 0.f;
      if (i < pc.n) raw_load(rc, i, pix[k], v[k]);
    }
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      const int64_t i = item_index<IPT>(tile, w, k, lane);
      key[k] = 0xffffffffu;
      fr[k] = 0;
      if (i < pc.n) {
        if (PK) {
          raw_frame_key(rc, i, r, nb, kf, pix[k], key[k], fr[k]);
          fr[k] = pack_item(fr[k], v[k]);
        } else {
          raw_key(rc, i, r, nb, kf, pix[k], v[k], key[k], fr[k]);
        }
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      int64_t i = item_index<IPT>(tile, w, k, lane);
      key[k] = 0xffffffffu;
      fr[k] = 0;
      v[k] = 0.f;
      if (i < pc.n) {
        key[k] = pc.key_in[i];
        fr[k] = pc.fr_in[i];
        if (!PK) v[k] = pc.v_in[i];
      }
    }
  }
  // stable rank within the warp: equal digits keep (round, lane) order
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    const bool ok = key[k] != 0xffffffffu;
    uint32_t d = ok ? ((key[k] >> pc.shift) & (RS_DIGITS - 1)) : RS_DIGITS;
    // lanes with the same digit (9 bits with the invalid marker), one ballot
    // per bit: cheaper here than match_any
    unsigned peers = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < 9; b++) {
      const bool bit = (d >> b) & 1u;
      const unsigned bal = __ballot_sync(0xffffffffu, bit);
      peers &= bit ? bal : ~bal;
    }
    int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (ok && lane == leader) {
      base = sm.wcnt[w][d];
      sm.wcnt[w][d] = base + __popc(peers);
    }
    base = __shfl_sync(0xffffffffu, base, leader);
    rank[k] = base + __popc(peers & lt);
  }
  __syncthreads();
  // per digit: exclusive over warps; tile total -> tile-local digit starts
  {
    const int d = threadIdx.x;  // RS_THREADS == RS_DIGITS
    uint32_t run = 0;
#pragma unroll
    for (int ww = 0; ww < RS_WARPS; ww++) {
      uint32_t c = sm.wcnt[ww][d];
      sm.wcnt[ww][d] = run;
      run += c;
    }
    uint32_t x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sm.wtot[w] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int ww = 0; ww < w; ww++) before += sm.wtot[ww];
    sm.tstart[d] = before + x - run;
  }
  __syncthreads();
  // stage the tile in digit order
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    if (key[k] == 0xffffffffu) continue;
    const uint32_t d = (key[k] >> pc.shift) & (RS_DIGITS - 1);
    const uint32_t q = sm.tstart[d] + sm.wcnt[w][d] + rank[k];
    sm.key[q] = key[k];
    sm.fr[q] = fr[k];
    if (!PK) sm.v[q] = v[k];
  }
  __syncthreads();
  // write out: consecutive staged elements of a digit go to consecutive addresses
  uint32_t nvalid = 0;
#pragma unroll
  for (int ww = 0; ww < RS_THREADS / 32; ww++) nvalid += sm.wtot[ww];
  for (uint32_t q = threadIdx.x; q < nvalid; q += RS_THREADS) {
    const uint32_t kq = sm.key[q];
    if (LAST && kq == pc.sentinel) continue;
    const uint32_t d = (kq >> pc.shift) & (RS_DIGITS - 1);
    const uint32_t pos = sm.toff[d] + (q - sm.tstart[d]);
    if (!LAST || pc.key_out) pc.key_out[pos] = kq;
    if (PK && LAST) {
      const uint32_t it = (uint32_t)sm.fr[q];
      const float raw = (float)(int16_t)(it & 0xffffu);
      pc.fr_out[pos] = (int32_t)(it >> 16);
      pc.v_out[pos] = rc.flat ? flat_value(raw, rc.flat[kq]) : raw;
    } else {
      pc.fr_out[pos] = sm.fr[q];
      if (!PK) pc.v_out[pos] = sm.v[q];
    }
  }
}

// Row pointers from the sorted keys: row_ptr[p] = first position whose key
// is >= p (std::lower_bound over the kept items), row_ptr[P] = the kept total.
// One thread per pixel; neighbouring pixels share the upper search steps.
__global__ void k_row_ptr(const uint32_t *__restrict__ keys, int64_t n,
                          const DevStats *__restrict__ stats, int32_t P,
                          int64_t *__restrict__ row_ptr) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p > P) return;
  const int64_t nv = n - (int64_t)stats->dropped;
  int64_t first = 0, len = nv;
  while (len > 0) {
    const int64_t half = len >> 1;
    if ((int64_t)keys[first + half] < p) {
      first += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  row_ptr[p] = first;
}

// Per-lane merge of one pixel's row: events of the same filter frame summed in
// stream order as pixels_value_[pix] += v, then / avg (sparse_filter.cpp:
// 146-172); pixelSum accumulated in frame order.
__device__ void merge_row(int32_t p, int32_t n, int64_t b, float favg, int32_t *fr, float *val,
                          int32_t &out, bool &integral, long long &total, float &psum) {
  int32_t i = 0;
  out = 0;
  integral = true;
  total = 0;
  psum = 0.f;
  while (i < n) {
    int32_t f = fr[b + i];
    float acc = 0.f;
    do {
      acc = __fadd_rn(acc, val[b + i]);
      i++;
    } while (i < n && fr[b + i] == f);
    float x = __fdiv_rn(acc, favg);
    fr[b + out] = f;
    val[b + out] = x;
    out++;
    psum = __fadd_rn(psum, x);
    if (integral) {
      if (x == truncf(x) && fabsf(x) < 16777216.f)
        total += llabs((long long)x);
      else
        integral = false;
    }
  }
}

// One warp per 32 consecutive pixels (their rows are contiguous): events are
// read coalesced to detect duplicate frames and to collect, per pixel, whether
// every value is an integer, sum |v| and sum v.  Without duplicates and with
// avg == 1 the rows are final as sorted, and for integer rows with sum |v| <
// 2^24 every float partial sum of pixelSum is exact, so pixelSum = (float)sum v;
// otherwise each lane merges its own row / sums it in frame order.  Pixels
// outside the mask get empty rows.
__global__ void __launch_bounds__(256, 6)
k_merge_classify(int32_t P, int32_t F, int32_t avg, int32_t tcap, int32_t force_float,
                 const int64_t *__restrict__ row_ptr, const uint8_t *__restrict__ mask,
                 int32_t *__restrict__ fr, float *__restrict__ val, int32_t *__restrict__ row_len,
                 uint8_t *__restrict__ pclass, ClassLists cl, float *__restrict__ pixels_sum,
                 DevStats *__restrict__ stats) {
  __shared__ long long s_total[8][32];
  __shared__ long long s_sum[8][32];
  __shared__ int32_t s_nonint[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int p0 = (blockIdx.x * 8 + w) * 32;
  if (p0 >= P) return;
  const int p = p0 + lane;
  const bool has = p < P;
  const int plast = min(p0 + 32, P);
  const int64_t e0 = row_ptr[p0], e1 = row_ptr[plast];
  const int64_t my_b = has ? row_ptr[p] : e1;
  const int32_t my_n = has ? (int32_t)(row_ptr[p + 1] - my_b) : 0;
  const bool keep = has && mask[p] != 0;
  s_total[w][lane] = 0;
  s_sum[w][lane] = 0;
  s_nonint[w][lane] = 0;
  __syncwarp();
  bool dup = false;
  // The chunks of the warp's rows, in positions relative to e0 of type T:
  // 32-bit when the rows span less than 2^30 events (one shuffle and one
  // compare per step of the owner search), else 64-bit.  Each 32-event chunk
  // is loaded one chunk ahead; the previous chunk's last frame carries over
  // to lane 0.
  auto chunks = [&](auto zero) {
    using T = decltype(zero);
    const int32_t *frw = fr + e0;
    const float *valw = val + e0;
    const T n_all = (T)(e1 - e0), my_bt = (T)(my_b - e0);
    int32_t f_nx = lane < n_all ? frw[lane] : 0;
    float x_nx = lane < n_all ? valw[lane] : 0.f;
    int32_t carry_f = 0;
    for (T base = 0; base < n_all; base += 32) {
      const T e = base + lane;
      const int32_t f = f_nx;
      const float x = x_nx;
      const bool in_nx = base + 32 + lane < n_all;
      f_nx = in_nx ? frw[base + 32 + lane] : 0;
      x_nx = in_nx ? valw[base + 32 + lane] : 0.f;
      int owner = 0;  // last lane whose row starts at or before e
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const int cand = owner + o;  // at most 31
        const T cb = __shfl_sync(0xffffffffu, my_bt, cand);
        if (cb <= e) owner = cand;
      }
      const T ob = __shfl_sync(0xffffffffu, my_bt, owner);
      const bool in = e < n_all;
      int32_t fprev = __shfl_up_sync(0xffffffffu, f, 1);
      if (lane == 0) fprev = carry_f;  // e > 0: the previous chunk's last frame
      carry_f = __shfl_sync(0xffffffffu, f, 31);
      if (in && e > ob && f == fprev) dup = true;
      const bool nonint = in && !(x == truncf(x) && fabsf(x) < 16777216.f);
      // a row's lanes are one run (owners do not decrease across the lanes)
      const int ow = in ? owner : 32;
      const int oprev = __shfl_up_sync(0xffffffffu, ow, 1);
      const unsigned starts = __ballot_sync(0xffffffffu, lane == 0 || ow != oprev);
      const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
      const int rs = 31 - __clz(starts & upto);
      const unsigned after = starts & ~upto;
      const unsigned peers =
          (after ? ((1u << (__ffs(after) - 1)) - 1u) : 0xffffffffu) & ~((1u << rs) - 1u);
      const unsigned a = in ? (unsigned)fminf(fabsf(x), 16777216.f) : 0u;
      const int xi = (in && !nonint) ? (int)x : 0;
      const unsigned sum = __reduce_add_sync(peers, a);
      const int ssum = __reduce_add_sync(peers, xi);
      const unsigned anynon = __reduce_or_sync(peers, nonint ? 1u : 0u);
      if (in && lane == __ffs(peers) - 1) {
        s_total[w][owner] += sum;
        s_sum[w][owner] += ssum;
        s_nonint[w][owner] |= (int)anynon;
      }
      __syncwarp();
    }
  };
  if (e1 - e0 < ((int64_t)1 << 30))
    chunks(int32_t{0});
  else
    chunks(int64_t{0});
  dup = __any_sync(0xffffffffu, dup);
  int32_t out = keep ? my_n : 0;
  bool integral = s_nonint[w][lane] == 0;
  long long total = s_total[w][lane];
  float psum = 0.f;
  if (keep) {
    if (dup || avg != 1) {
      merge_row(p, my_n, my_b, (float)avg, fr, val, out, integral, total, psum);
    } else if (integral && total < 16777216) {
      psum = (float)s_sum[w][lane];
    } else {
      for (int32_t i = 0; i < my_n; i++) psum = __fadd_rn(psum, val[my_b + i]);
    }
  }
  if (has) {
    row_len[p] = out;
    pixels_sum[p] = psum;
  }
  uint8_t c = keep ? pixel_class(out, integral, total, F, tcap) : (uint8_t)PCLASS_EMPTY;
  if (force_float && c != PCLASS_EMPTY) c = PCLASS_FLOAT;  // values rescaled after the filter
  record_class_warp(has, p, c, out, pclass, cl, stats);
}

template <int IPT, bool FIRST, bool LAST, bool PK>
void launch_downsweep(int ntiles, cudaStream_t st, const RawCfg &rc, const PassCfg &pc,
                      const uint32_t *offsets) {
  const size_t smem = sizeof(DsSmem<IPT, PK>);
  XG_CUDA(cudaFuncSetAttribute(k_downsweep<IPT, FIRST, LAST, PK>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_downsweep<IPT, FIRST, LAST, PK><<<ntiles, RS_THREADS, smem, st>>>(rc, pc, offsets);
}

// One radix pass: tile histograms, digit-major scan, stable scatter.
template <int IPT>
void radix_pass(Series &s, bool first, bool last, bool packed, int ntiles, const RawCfg &rc,
                const PassCfg &pc) {
  cudaStream_t st = s.stream;
  if (first)
    k_upsweep<IPT, true><<<ntiles, RS_THREADS, 0, st>>>(rc, pc, s.hist.p);
  else
    k_upsweep<IPT, false><<<ntiles, RS_THREADS, 0, st>>>(rc, pc, s.hist.p);
  XG_CHECK_LAUNCH();
  exclusive_scan_u32(s.hist.p, s.hist_scan.p, (int64_t)RS_DIGITS * ntiles, s.scan_tmp.p, st);
  if (packed) {
    if (first && last)
      launch_downsweep<IPT, true, true, true>(ntiles, st, rc, pc, s.hist_scan.p);
    else if (first)
      launch_downsweep<IPT, true, false, true>(ntiles, st, rc, pc, s.hist_scan.p);
    else if (last)
      launch_downsweep<IPT, false, true, true>(ntiles, st, rc, pc, s.hist_scan.p);
    else
      launch_downsweep<IPT, false, false, true>(ntiles, st, rc, pc, s.hist_scan.p);
  } else {
    if (first && last)
      launch_downsweep<IPT, true, true, false>(ntiles, st, rc, pc, s.hist_scan.p);
    else if (first)
      launch_downsweep<IPT, true, false, false>(ntiles, st, rc, pc, s.hist_scan.p);
    else if (last)
      launch_downsweep<IPT, false, true, false>(ntiles, st, rc, pc, s.hist_scan.p);
    else
      launch_downsweep<IPT, false, false, false>(ntiles, st, rc, pc, s.hist_scan.p);
  }
  XG_CHECK_LAUNCH();
}

int items_per_lane(int64_t n) { return n >= RS_BIG_N ? 16 : 8; }

}  // namespace

// Stable LSD radix sort of (key, a, b) triples by the low `key_bits` bits of
// key, with the passes above; (key2, a2, b2) is scratch of the same length.
// Returns true when the sorted triples ended in the scratch arrays.
bool radix_sort_triples(Series &s, uint32_t *key, int32_t *a, float *b, uint32_t *key2,
                        int32_t *a2, float *b2, int64_t n, int key_bits) {
  cudaStream_t st = s.stream;
  if (n <= 0 || key_bits <= 0) return false;
  const int passes = (key_bits + 7) / 8;
  const int ipt = items_per_lane(n);
  const int ntiles = (int)((n + RS_THREADS * ipt - 1) / (RS_THREADS * ipt));
  s.hist.reserve((size_t)RS_DIGITS * ntiles, st);
  s.hist_scan.reserve((size_t)RS_DIGITS * ntiles, st);
  s.scan_tmp.reserve(scan_workspace_bytes((int64_t)RS_DIGITS * ntiles), st);
  RawCfg rc{};
  uint32_t *kb[2] = {key, key2};
  int32_t *ab[2] = {a, a2};
  float *bb[2] = {b, b2};
  for (int pass = 0; pass < passes; pass++) {
    PassCfg pc{};
    pc.n = n;
    pc.shift = 8 * pass;
    pc.ntiles = ntiles;
    pc.sentinel = 0xfffffffeu;
    pc.key_in = kb[pass & 1];
    pc.fr_in = ab[pass & 1];
    pc.v_in = bb[pass & 1];
    pc.key_out = kb[(pass + 1) & 1];
    pc.fr_out = ab[(pass + 1) & 1];
    pc.v_out = bb[(pass + 1) & 1];
    if (ipt == 16)
      radix_pass<16>(s, false, false, false, ntiles, rc, pc);
    else
      radix_pass<8>(s, false, false, false, ntiles, rc, pc);
  }
  return (passes & 1) != 0;
}

namespace {

// Device copies of the per-raw-frame tables (event offsets, filter frame of
// every raw frame) after frames were ingested.
void upload_frame_tables(Series &s) {
  cudaStream_t st = s.stream;
  if (!s.frame_off_dirty) return;
  s.d_frame_off.reserve(s.frame_off.size(), st);
  XG_CUDA(cudaMemcpyAsync(s.d_frame_off.p, s.frame_off.data(),
                          sizeof(int64_t) * s.frame_off.size(), cudaMemcpyHostToDevice, st));
  s.frame_map.resize(s.raw_frames);
  for (int32_t r = 0; r < s.raw_frames; r++) {  // stride*avg raw frames per filter frame
    const int32_t k = r / s.R_in;
    s.frame_map[r] = (k < s.F && ((r - k * s.R_in) % s.desc.stride_frames) == 0) ? k : -1;
  }
  s.d_frame_map.reserve(s.frame_map.size() ? s.frame_map.size() : 1, st);
  if (!s.frame_map.empty())
    XG_CUDA(cudaMemcpyAsync(s.d_frame_map.p, s.frame_map.data(),
                            sizeof(int32_t) * s.frame_map.size(), cudaMemcpyHostToDevice, st));
  s.frame_off_dirty = false;
}

// Filter and stable radix transpose of the raw frames [r0, r1): pixel-major
// events into ev_fr / ev_val and their row pointers (relative to ev_fr) into
// row_ptr [P+1].  Needs the frame tables on the device.
void transpose_range(Series &s, int32_t r0, int32_t r1, int32_t *ev_fr, float *ev_val,
                     int64_t *row_ptr) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P;
  const int64_t e0 = s.frame_off[r0], n = s.frame_off[r1] - e0;
  s.scan_tmp.reserve(scan_workspace_bytes(P), st);
  if (n <= 0) {
    XG_CUDA(cudaMemsetAsync(row_ptr, 0, sizeof(int64_t) * ((size_t)P + 1), st));
    return;
  }
  // the count of items sorted last, read by the row pointers, is per range
  XG_CUDA(cudaMemsetAsync(&s.stats.p->dropped, 0, sizeof(unsigned long long), st));
  const int nbits = 32 - __builtin_clz((unsigned)P);  // bits to hold P (the drop key)
  const int passes = (nbits + 7) / 8;
  const int ipt = s.radix_ipt == 8 || s.radix_ipt == 16 ? s.radix_ipt : items_per_lane(n);
  const int ntiles = (int)((n + RS_THREADS * ipt - 1) / (RS_THREADS * ipt));
  s.hist.reserve((size_t)RS_DIGITS * ntiles, st);
  s.hist_scan.reserve((size_t)RS_DIGITS * ntiles, st);
  const size_t ws = scan_workspace_bytes((int64_t)RS_DIGITS * ntiles);
  s.scan_tmp.reserve(std::max(ws, scan_workspace_bytes(P)), st);
  // sparse series below 65,536 filter frames carry one packed word per item
  // (frame, raw value) through the passes instead of a frame and a value
  const bool dense = s.desc.dense != 0;
  const bool packed = !dense && s.F <= 65536;
  // the last pass also writes the kept items' keys, for the row pointers
  s.keyA.reserve(n, st);
  if (passes > 1) {
    s.keyB.reserve(n, st);
    s.frA.reserve(n, st);
    if (!packed) s.vA.reserve(n, st);
  }
  if (passes > 2) {
    s.frB.reserve(n, st);
    if (!packed) s.vB.reserve(n, st);
  }
  const int chunk = 32 * ipt;
  const int64_t nch = (n + chunk - 1) / chunk;
  const int32_t nfr = r1 - r0;
  s.d_chunk_frame.reserve((size_t)nch, st);
  k_chunk_frames<<<(nfr + 255) / 256, 256, 0, st>>>(nfr, s.d_frame_off.p + r0, e0, nch, chunk,
                                                     s.d_chunk_frame.p);
  XG_CHECK_LAUNCH();
  RawCfg rc{s.raw_idx.p + e0, dense ? nullptr : s.raw_val.p + e0,
            dense ? s.raw_valf.p + e0 : nullptr, s.d_frame_off.p + r0, s.d_frame_map.p + r0,
            s.d_chunk_frame.p, nfr, e0, n, P, s.F, s.R_in, s.desc.stride_frames,
            s.has_flat ? s.d_flat.p : nullptr, s.stats.p};
  uint32_t *kbuf[2] = {s.keyA.p, s.keyB.p};
  int32_t *fbuf[2] = {s.frA.p, s.frB.p};
  float *vbuf[2] = {s.vA.p, s.vB.p};
  for (int pass = 0; pass < passes; pass++) {
    bool first = pass == 0, last = pass == passes - 1;
    PassCfg pc{};
    pc.n = n;
    pc.shift = 8 * pass;
    pc.ntiles = ntiles;
    pc.sentinel = (uint32_t)P;
    if (!first) {
      pc.key_in = kbuf[(pass - 1) & 1];
      pc.fr_in = fbuf[(pass - 1) & 1];
      pc.v_in = vbuf[(pass - 1) & 1];
    }
    if (last) {
      pc.key_out = kbuf[pass & 1];  // not the pass's input
      pc.fr_out = ev_fr;
      pc.v_out = ev_val;
    } else {
      pc.key_out = kbuf[pass & 1];
      pc.fr_out = fbuf[pass & 1];
      pc.v_out = vbuf[pass & 1];
    }
    if (ipt == 16)
      radix_pass<16>(s, first, last, packed, ntiles, rc, pc);
    else
      radix_pass<8>(s, first, last, packed, ntiles, rc, pc);
  }
  const uint32_t *keys = (passes % 2 == 0) ? s.keyB.p : s.keyA.p;  // written by the last pass
  k_row_ptr<<<(unsigned)(((int64_t)P + 1 + 255) / 256), 256, 0, st>>>(keys, n, s.stats.p, P,
                                                                      row_ptr);
  XG_CHECK_LAUNCH();
}

void reserve_lists(Series &s) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P;
  s.row_ptr.reserve((size_t)P + 1, st);
  s.row_len.reserve(P, st);
  s.pclass.reserve(P, st);
  s.flist.reserve(P, st);
  s.wlist.reserve(P, st);
  s.llist.reserve(P, st);
  s.pixels_sum.reserve(P, st);
  s.stats.reserve(1, st);
}

void merge_classify(Series &s, int32_t avg) {
  const int pix_per_block = 256;
  k_merge_classify<<<(s.P + pix_per_block - 1) / pix_per_block, 256, 0, s.stream>>>(
      s.P, s.F, avg, s.thread_cap, s.desc.normalize_by_framesum, s.row_ptr.p, s.d_mask.p,
      s.ev_frame.p, s.ev_val.p, s.row_len.p, s.pclass.p,
      ClassLists{s.wlist.p, s.llist.p, s.flist.p}, s.pixels_sum.p, s.stats.p);
  XG_CHECK_LAUNCH();
}

}  // namespace

// ----------------------------------------------------- incremental transposes
//
// With a block size set (xpcs_series_set_block_frames), the frames are
// transposed as they are ingested, block by block (block_frames filter frames
// = block_frames * stride * avg raw frames, so that a filter frame's raw
// frames never straddle two blocks), into a store of block-local pixel-major
// rows that stays on the device.  Each block's rows are merged (events of one
// filter frame summed in stream order, then / avg; masked pixels emptied) as
// the whole-series merge does.  Finishing the series transposes the last,
// partial block and gathers every pixel's segments in block order -- blocks
// follow each other in time, so a row's segments concatenate in frame order --
// into the series' event lists, which are then classified as usual.  The
// result is the same event lists, bit for bit, as one transpose of every frame.

namespace {

// Block merge: one warp per 32 pixels; each lane merges its pixel's row of the
// block in place (when the block's rows hold a repeated frame or avg > 1) and
// records the row's start in the block and its merged length.
__global__ void __launch_bounds__(256)
k_merge_block(int32_t P, int32_t avg, const int64_t *__restrict__ row_ptr,
              const uint8_t *__restrict__ mask, int32_t *__restrict__ fr,
              float *__restrict__ val, int32_t *__restrict__ blk_off,
              int32_t *__restrict__ blk_len) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p - (int)(threadIdx.x & 31) >= P) return;  // whole warp past the end
  const bool has = p < P;
  const int64_t b = has ? row_ptr[p] : 0;
  const int32_t n = has ? (int32_t)(row_ptr[p + 1] - b) : 0;
  int32_t out = 0;
  if (has && mask[p]) {
    bool dup = false;
    for (int32_t i = 1; i < n && !dup; i++) dup = fr[b + i] == fr[b + i - 1];
    if (dup || avg != 1) {
      const float favg = (float)avg;
      int32_t i = 0;
      while (i < n) {
        const int32_t f = fr[b + i];
        float acc = 0.f;
        do {
          acc = __fadd_rn(acc, val[b + i]);
          i++;
        } while (i < n && fr[b + i] == f);
        fr[b + out] = f;
        val[b + out] = __fdiv_rn(acc, favg);
        out++;
      }
    } else {
      out = n;
    }
  }
  if (has) {
    blk_off[p] = (int32_t)b;
    blk_len[p] = out;
  }
}

// Merged row lengths of every block summed per pixel.
__global__ void k_block_totals(int32_t P, int32_t nblk, const int32_t *__restrict__ blk_len,
                               int32_t *__restrict__ tot) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int32_t t = 0;
  for (int32_t k = 0; k < nblk; k++) t += blk_len[(size_t)k * P + p];
  tot[p] = t;
}

// Each pixel's block segments, in block order, copied to its row of the
// series' event lists.
__global__ void k_gather_blocks(int32_t P, int32_t nblk, const int64_t *__restrict__ blk_base,
                                const int32_t *__restrict__ blk_off,
                                const int32_t *__restrict__ blk_len,
                                const int32_t *__restrict__ bfr, const float *__restrict__ bval,
                                const int64_t *__restrict__ row_ptr, int32_t *__restrict__ fr,
                                float *__restrict__ val) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t d = row_ptr[p];
  for (int32_t k = 0; k < nblk; k++) {
    const int32_t n = blk_len[(size_t)k * P + p];
    const int64_t src = blk_base[k] + blk_off[(size_t)k * P + p];
    for (int32_t i = 0; i < n; i++) {
      fr[d + i] = bfr[src + i];
      val[d + i] = bval[src + i];
    }
    d += n;
  }
}

// Every pixel's block segments gathered into its row of the series' event
// lists (d_blk_base on the device already), then classified (the rows are
// merged already: avg 1 leaves nothing to merge).
void gather_blocks(Series &s) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P, nblk = (int32_t)s.blk_base.size();
  s.blk_tot.reserve(P, st);
  if (nblk > 0) {
    k_block_totals<<<(P + 255) / 256, 256, 0, st>>>(P, nblk, s.blk_len.p, s.blk_tot.p);
    XG_CHECK_LAUNCH();
    exclusive_scan_i32_i64(s.blk_tot.p, s.row_ptr.p, P, s.scan_tmp.p, st);
    k_gather_blocks<<<(P + 255) / 256, 256, 0, st>>>(P, nblk, s.d_blk_base.p, s.blk_off.p,
                                                     s.blk_len.p, s.blk_fr.p, s.blk_val.p,
                                                     s.row_ptr.p, s.ev_frame.p, s.ev_val.p);
    XG_CHECK_LAUNCH();
  } else {
    XG_CUDA(cudaMemsetAsync(s.row_ptr.p, 0, sizeof(int64_t) * ((size_t)P + 1), st));
  }
  merge_classify(s, 1);
}

// Transposes the next block, ending at raw frame r1, into the block store.
void transpose_block(Series &s, int32_t r1) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P, r0 = s.blk_raw_done;
  const int64_t n = s.frame_off[r1] - s.frame_off[r0];
  const int64_t base = s.blk_events;
  s.blk_fr.grow((size_t)(base + std::max<int64_t>(n, 1)), (size_t)base, st);
  s.blk_val.grow((size_t)(base + std::max<int64_t>(n, 1)), (size_t)base, st);
  const size_t k = s.blk_base.size();
  s.blk_off.grow((k + 1) * (size_t)P, k * (size_t)P, st);
  s.blk_len.grow((k + 1) * (size_t)P, k * (size_t)P, st);
  s.blk_rp.reserve((size_t)P + 1, st);
  transpose_range(s, r0, r1, s.blk_fr.p + base, s.blk_val.p + base, s.blk_rp.p);
  k_merge_block<<<(P + 255) / 256, 256, 0, st>>>(P, s.desc.avg_frames, s.blk_rp.p, s.d_mask.p,
                                                  s.blk_fr.p + base, s.blk_val.p + base,
                                                  s.blk_off.p + k * (size_t)P,
                                                  s.blk_len.p + k * (size_t)P);
  XG_CHECK_LAUNCH();
  s.blk_base.push_back(base);
  s.blk_events = base + n;
  s.blk_raw_done = r1;
}

}  // namespace

void transpose_ready_blocks(Series &s) {
  // pixel-major dense series write their blocks as frames arrive
  if (s.block_frames <= 0 || s.dense_px) return;
  const int32_t step = s.block_frames * s.R_in;
  // raw frames past the series' last filter frame are never used
  const int32_t limit = std::min<int64_t>(s.raw_frames, (int64_t)s.F * s.R_in);
  if (s.blk_raw_done + step > limit) return;
  s.stats.reserve(1, s.stream);
  if (s.blk_base.empty())  // the first block of the series: a clean error word
    XG_CUDA(cudaMemsetAsync(s.stats.p, 0, sizeof(DevStats), s.stream));
  upload_frame_tables(s);
  while (s.blk_raw_done + step <= limit) transpose_block(s, s.blk_raw_done + step);
}

void reset_blocks(Series &s) {
  s.blk_base.clear();
  s.blk_r0.clear();
  s.blk_events = 0;
  s.blk_raw_done = 0;
  s.dn_pend_n = 0;
}

// The thread kernel's row capacity for a series nobody tuned: the smallest
// capacity of at least 1.5 mean rows, which the autotuner also picks for mean
// rows of 25, 52 and 100 events (1 Mi pixels, 5,000-20,000 frames), and the
// extra scratch words it picks from 16,384 frames on.
void default_knobs(Series &s) {
  if (s.knobs_set) return;
  if (s.valid_pixels < 0) {
    s.valid_pixels = 0;
    for (uint8_t v : s.qmap.valid) s.valid_pixels += v;
  }
  const double mean =
      (double)s.raw_events / ((double)std::max<int64_t>(s.valid_pixels, 1) * s.R_in);
  int32_t cap = MT_THREAD_CAPS[MT_THREAD_NCAPS - 1];
  for (int c : MT_THREAD_CAPS)
    if (c >= 1.5 * mean) {
      cap = c;
      break;
    }
  s.thread_cap = cap;
  s.scr_extra = s.F >= 16384 ? 8 : 0;
}

void run_filter_transpose(Series &s) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P;
  dense_px_flush(s);  // frames still pending become the last block
  default_knobs(s);
  reserve_lists(s);
  const size_t nalloc = s.raw_events > 0 ? (size_t)s.raw_events : 1;
  s.ev_frame.reserve(nalloc, st);
  s.ev_val.reserve(nalloc, st);
  s.scan_tmp.reserve(scan_workspace_bytes(P), st);
  if (s.dense_px) {
    XG_CUDA(cudaMemsetAsync(s.stats.p, 0, sizeof(DevStats), st));
    dense_px_gather(s);  // gathers and classifies
    return;
  }
  if (s.block_frames <= 0) {
    XG_CUDA(cudaMemsetAsync(s.stats.p, 0, sizeof(DevStats), st));
    upload_frame_tables(s);
    transpose_range(s, 0, s.raw_frames, s.ev_frame.p, s.ev_val.p, s.row_ptr.p);
    merge_classify(s, s.desc.avg_frames);
    return;
  }
  // the error word keeps what earlier block transposes found; the counters restart
  if (s.blk_base.empty())
    XG_CUDA(cudaMemsetAsync(s.stats.p, 0, sizeof(DevStats), st));
  else
    XG_CUDA(cudaMemsetAsync(&s.stats.p->nfloat, 0,
                            sizeof(DevStats) - offsetof(DevStats, nfloat), st));
  upload_frame_tables(s);
  if (s.blk_raw_done < s.raw_frames) transpose_block(s, s.raw_frames);  // the last block
  const int32_t nblk = (int32_t)s.blk_base.size();
  s.d_blk_base.reserve((size_t)std::max(nblk, 1), st);
  if (nblk > 0)
    XG_CUDA(cudaMemcpyAsync(s.d_blk_base.p, s.blk_base.data(), sizeof(int64_t) * nblk,
                            cudaMemcpyHostToDevice, st));
  gather_blocks(s);
}

}  // namespace xg

namespace xg {
namespace {

// Caller-held rows (xpcs_multitau2): rows stay as given; a pixel takes the
// integer path only if its frames are strictly increasing within [0, F), its
// values are integers and sum |v| < 4096.
__global__ void k_classify_rows(int32_t P, int32_t F, int32_t tcap, const int64_t *__restrict__ row_ptr,
                                const int32_t *__restrict__ fr, const float *__restrict__ val,
                                int32_t *__restrict__ row_len, uint8_t *__restrict__ pclass,
                                ClassLists cl, DevStats *__restrict__ stats) {
  const int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p - (int32_t)(threadIdx.x & 31) >= P) return;  // whole warp past the end
  const bool has = p < P;
  const int64_t b = has ? row_ptr[p] : 0;
  const int32_t n = has ? (int32_t)(row_ptr[p + 1] - b) : 0;
  if (has) row_len[p] = n;
  bool ok = n <= MT_LONG_CAP;
  long long total = 0;
  int32_t prev = -1;
  for (int32_t i = 0; i < n && ok; i++) {
    int32_t f = fr[b + i];
    float x = val[b + i];
    ok = f > prev && f < F && x == truncf(x) && fabsf(x) < 16777216.f;
    if (ok) total += llabs((long long)x);
    prev = f;
  }
  const uint8_t c = n == 0 ? (uint8_t)PCLASS_EMPTY : pixel_class(n, ok, total, F, tcap);
  record_class_warp(has, p, c, n, pclass, cl, stats);
}

}  // namespace

void multitau_rows_upload(Series &s, const int64_t *row_ptr, const int32_t *frame,
                          const float *value, int64_t events) {
  cudaStream_t st = s.stream;
  const int32_t P = s.P;
  size_t ne = events > 0 ? (size_t)events : 1;
  s.row_ptr.reserve((size_t)P + 1, st);
  s.row_len.reserve(P, st);
  s.pclass.reserve(P, st);
  s.flist.reserve(P, st);
  s.wlist.reserve(P, st);
  s.llist.reserve(P, st);
  s.stats.reserve(1, st);
  s.ev_frame.reserve(ne, st);
  s.ev_val.reserve(ne, st);
  s.raw_events = events;
  XG_CUDA(cudaMemsetAsync(s.stats.p, 0, sizeof(DevStats), st));
  XG_CUDA(cudaMemcpyAsync(s.row_ptr.p, row_ptr, sizeof(int64_t) * ((size_t)P + 1),
                          cudaMemcpyHostToDevice, st));
  if (events > 0) {
    XG_CUDA(cudaMemcpyAsync(s.ev_frame.p, frame, sizeof(int32_t) * events, cudaMemcpyHostToDevice, st));
    XG_CUDA(cudaMemcpyAsync(s.ev_val.p, value, sizeof(float) * events, cudaMemcpyHostToDevice, st));
  }
  default_knobs(s);
  const int bs = 256;
  k_classify_rows<<<(P + bs - 1) / bs, bs, 0, st>>>(P, s.F, s.thread_cap, s.row_ptr.p, s.ev_frame.p,
                                                     s.ev_val.p, s.row_len.p, s.pclass.p,
                                                     ClassLists{s.wlist.p, s.llist.p, s.flist.p},
                                                     s.stats.p);
  XG_CHECK_LAUNCH();
}

}  // namespace xg
