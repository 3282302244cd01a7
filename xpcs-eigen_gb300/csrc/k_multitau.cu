// K-c: per-pixel multi-tau G2 / IP / IF.
//
// Replaces Corr::multiTau2 (src/xpcs/corr.cpp:315-431).  For every pixel with
// events and every delay (level L, tau):
//   on a level change lastframe halves (odd -> -1 first) and the row is
//   compacted in place: index/2, equal neighbours merged by addition, indices
//   >= lastframe dropped, every live value halved (:349-390);
//   IP  = sum of v over events with t < lastframe - tau,
//   G2  = sum of v(t) * v(t + tau), the partner found by std::lower_bound over
//         the row buffer (:406),
//   IF  = sum of v over events with tau <= t < lastframe,
//   each divided by (lastframe - tau) (:420-424).
//
// Integer paths (values are integers, sum |v| < 4096): a level-L value is an
// integer numerator N over 2^L, every float partial sum of the reference is
// exact, so integer sums scaled by 2^-L (2^-2L for G2) followed by one IEEE
// division reproduce the reference bit for bit.
//   * IP and IF do not depend on the compaction: level L keeps exactly the
//     events with frame < lastframe << L, so IP(tau) = S(t_ip) and
//     IF(tau) = S(lastframe << L) - S(tau_frames), S(T) = sum of v over
//     original events with frame < T.  Two merge sweeps over the sorted row
//     and the (monotone) per-delay thresholds give all of them.
//   * G2 needs the compacted rows: per level the row is compacted in place
//     (the same buffer the reference keeps, stale tail included) and the
//     pairs whose bin distance lies in the level's delay window are summed.
//     In REFERENCE mode a pair counts only when lower_bound over the whole
//     buffer lands on the partner; that always holds while the buffer is
//     globally sorted, which is tracked per level from the junction between
//     the new prefix and the stale tail.
// k_mt_thread: one thread per pixel, rows packed (frame << 16 | int16 value)
//   in shared memory with a lane-interleaved layout (conflict-free), outputs
//   written straight to [D][P] (32 consecutive pixels per warp = coalesced).
//   Levels of few bins find pairs from an occupancy bitmask of the row in the
//   thread's scratch words; sparse levels check each source's next two
//   entries without branching.  Pixels of other classes get zeros here and
//   are rewritten by the kernels below.
// k_mt_warp:   one warp per pixel, rows packed in shared memory: rows of up
//   to 256 events (8 warps per block), up to 1024 (4 warps per block) and up
//   to 4096 (2 warps per block).
// k_mt_float:  one thread per pixel replaying the reference's float
//   operations in its order (no fused multiply-add) on a scratch copy.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include "mt_replay.cuh"
#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int MT_WARPS = 2;  // warps per block of the thread-per-pixel kernel
constexpr int WP_WARPS = 8;  // warps per block of the warp-per-pixel kernel
constexpr int MT_MID_CAP = 1024;  // long rows up to this length: 4 warps per block
constexpr int MID_WARPS = 4;
constexpr int LONG_WARPS = 2;  // warps per block for rows of up to MT_LONG_CAP events

// std::lower_bound as libstdc++ implements it (halving the remaining length),
// over lane-interleaved packed words (frame in the high half).
__device__ __forceinline__ int lower_bound_packed(const uint32_t *row, int n, int32_t x) {
  int first = 0, len = n;
  while (len > 0) {
    int half = len >> 1;
    if ((int32_t)(row[(first + half) * 32] >> 16) < x) {
      first += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return first;
}

__device__ __forceinline__ float pow2_neg(int e) { return __int_as_float((127 - e) << 23); }

// (float)num * 2^-shift / den as the reference's float arithmetic produces it
// (num is an integer below 2^24, den an integer below 2^16 as a float).  The
// IEEE quotient comes from the correctly rounded reciprocal by one residual
// correction (Markstein 1990; Muller et al., Handbook of Floating-Point
// Arithmetic, ch. 4): q0 = x*y, r = x - q0*den (exact by FMA), q = q0 + r*y.
// It equals the IEEE division for every 24-bit significand x and every integer
// den in [1, 65536] (checked exhaustively on the GPU against __fdiv_rn).
__device__ __forceinline__ float scaled_quotient(int num, int shift, float den, float rcp) {
  if (num == 0) return 0.f;
  const float x = __fmul_rn((float)num, pow2_neg(shift));
  if (!(den > 0.f)) return x;
  const float q0 = __fmul_rn(x, rcp);
  return __fmaf_rn(__fmaf_rn(-q0, den, x), rcp, q0);
}

// The same without branches, for divisors prepared by div_prep: num = 0 gives
// +0 through the correction steps, and a delay without division carries
// (den, rcp) = (1, 1), for which the steps return x unchanged.
__device__ __forceinline__ float scaled_quotient_nb(int num, int shift, float den, float rcp) {
  const float x = __fmul_rn((float)num, pow2_neg(shift));
  const float q0 = __fmul_rn(x, rcp);
  return __fmaf_rn(__fmaf_rn(-q0, den, x), rcp, q0);
}
__device__ __forceinline__ void div_prep(float &den, float &rcp) {
  if (!(den > 0.f)) {
    den = 1.f;
    rcp = 1.f;
  }
}

__device__ __forceinline__ int32_t pk_t(uint32_t w) { return (int32_t)(w >> 16); }
__device__ __forceinline__ int32_t pk_v(uint32_t w) { return (int32_t)(int16_t)(w & 0xffffu); }
__device__ __forceinline__ uint32_t pk(int32_t t, int32_t v) {
  return ((uint32_t)t << 16) | ((uint32_t)v & 0xffffu);
}

__device__ __forceinline__ void copy_plan(uint8_t *dst, const uint8_t *src, size_t bytes) {
  for (int k = threadIdx.x; k < (int)(bytes / 4); k += blockDim.x)
    ((int32_t *)dst)[k] = ((const int32_t *)src)[k];
}

// ------------------------------------------------------ thread per pixel

// Levels of at most 32 x (scratch words) bins: the thread keeps its row's
// occupied bins as a bitmask in its scratch words (lane-interleaved, one
// 32-bit word per 32 bins).  Bins in a row's live prefix are distinct and
// increasing, so the entry at bin b sits at position popcount(bits below b):
// one 64-bit window of the mask after a source's bin gives both the position
// of its first partner and which of the level's delays have one.  The KM >=
// count accumulators stay in registers and overwrite the mask once the
// sources are done; sources stop at the first bin whose first partner would
// be past lastframe.
template <int KM>
__device__ __forceinline__ void bins_pairs(const uint32_t *row, int m, int lf, int tlo,
                                                int count, int32_t *acc) {
  const uint32_t *mk = (const uint32_t *)acc;
  const int nw = (lf + 31) >> 5;
  int a[KM];
#pragma unroll
  for (int k = 0; k < KM; k++) a[k] = 0;
  const uint64_t gap = (1ull << (tlo - 1)) - 1ull;
  const uint32_t cmask = (1u << count) - 1u;
  for (int i = 0; i < m; i++) {
    const uint32_t wi = row[i * 32];
    const int ti = pk_t(wi);
    if (ti + tlo >= lf) break;
    const int s = ti + 1, q = s >> 5, sh = s & 31;  // s < lf: word q exists
    const uint32_t m0 = mk[q * 32];
    const uint32_t m1 = q + 1 < nw ? mk[(q + 1) * 32] : 0u;
    const uint32_t m2 = q + 2 < nw ? mk[(q + 2) * 32] : 0u;
    const uint64_t W = ((uint64_t)__funnelshift_r(m1, m2, sh) << 32) | __funnelshift_r(m0, m1, sh);
    int j = i + 1 + __popcll(W & gap);
    const uint32_t w = (uint32_t)(W >> (tlo - 1)) & cmask;
    const int vi = pk_v(wi);
#pragma unroll
    for (int k = 0; k < KM; k++) {
      if (w & (1u << k)) {
        a[k] += vi * pk_v(row[j * 32]);
        j++;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < KM; k++)
    if (k < count) acc[k * 32] = a[k];
}

// One warp's 32 consecutive pixels p0 .. p0+31 of a series: the body of the
// thread-per-pixel kernel, shared by its per-series launch and by the batch's
// work-queue launch.  wbase: the warp's (CAP + scratch words) x 32 words of
// shared memory.
template <int CAP>
__device__ __forceinline__ void mt_thread_warp(const uint8_t *__restrict__ plan_g,
                                               const int64_t *__restrict__ row_ptr,
                                               const int32_t *__restrict__ row_len,
                                               const uint8_t *__restrict__ pclass,
                                               const int32_t *__restrict__ ev_frame,
                                               const float *__restrict__ ev_val,
                                               float *__restrict__ G2, float *__restrict__ IP,
                                               float *__restrict__ IF, int p0,
                                               uint32_t *wbase) {
  // the plan is read from global memory: every lane of a warp reads the same
  // words (one L1-cached broadcast), and shared memory is left to the rows
  const McPlan *pl = (const McPlan *)plan_g;
  const int D = pl->D;
  const McArrays ar = mc_arrays(plan_g, D);
  const int P = pl->P, nlev = pl->nlev, mode = pl->mode;
  const int scr = pl->scr;
  const int lane = threadIdx.x & 31;
  uint32_t *row = wbase + lane;
  int32_t *acc = (int32_t *)(row + CAP * 32);  // scratch, also S(t_end) per level

  if (p0 >= P) return;
  const int p = p0 + lane;
  const bool mine = p < P && pclass[p] == PCLASS_THREAD;
  const int n0 = mine ? row_len[p] : 0;

  // cooperative, coalesced load of the warp's rows (consecutive pixels have
  // consecutive rows), scattered to the owning lane's slots; four chunks of
  // 32 events in flight per lane.  Positions are relative to the warp's first
  // event: when a lane owns a packed row every frame is below 65536, so the
  // 32 rows span fewer than 2^21 events.
  if (__any_sync(0xffffffffu, n0 > 0)) {
    const unsigned FULL = 0xffffffffu;
    const int plast = min(p0 + 32, P);
    const int64_t e0 = row_ptr[p0];
    const int nw = (int)(row_ptr[plast] - e0);
    const int my_b = p < P ? (int)(row_ptr[p] - e0) : nw;
    const int lo = __reduce_min_sync(FULL, n0 > 0 ? my_b : INT_MAX);
    const int hi = __reduce_max_sync(FULL, n0 > 0 ? my_b + n0 : 0);
    for (int base = lo; base < hi; base += 128) {
      int dst[4], fr[4];
      float vl[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int e = base + u * 32 + lane;
        int owner = 0;  // last lane whose row starts at or before e
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const int cand = owner + o;
          const int cb = __shfl_sync(FULL, my_b, cand & 31);
          if (cand < 32 && cb <= e) owner = cand;
        }
        const int slot = e - __shfl_sync(FULL, my_b, owner);
        const int olen = __shfl_sync(FULL, n0, owner);
        dst[u] = (e < hi && slot < olen) ? slot * 32 + owner : -1;
        if (dst[u] >= 0) {
          fr[u] = ev_frame[e0 + e];
          vl[u] = ev_val[e0 + e];
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (dst[u] >= 0) wbase[dst[u]] = pk(fr[u], __float2int_rn(vl[u]));
    }
  }
  __syncwarp();

  // total and S(t_end) per level (sweep from the end; t_end non-increasing)
  int total = 0;
  for (int i = 0; i < n0; i++) total += pk_v(row[i * 32]);
  {
    int j = n0 - 1, rsum = 0;
    for (int g = 0; g < nlev; g++) {
      const int te = pl->lv[g].t_end;
      while (j >= 0 && pk_t(row[j * 32]) >= te) {
        rsum += pk_v(row[j * 32]);
        j--;
      }
      acc[g * 32] = total - rsum;
    }
  }
  // IP and IF in one sweep over the delays, level group by level group: the
  // IP thresholds t_ip decrease with the delay index (a pointer from the end
  // of the row), the IF thresholds tau (in frames) increase (one from the
  // start).  Lane k loads the thresholds and divisor of the chunk's k-th
  // delay, and they are broadcast by shuffle.
  {
    const unsigned FULL = 0xffffffffu;
    int jp = n0 - 1, rsum = 0, jf = 0, ssum = 0;
    uint32_t wp = n0 > 0 ? row[(n0 - 1) * 32] : 0u;  // word at jp
    uint32_t wf = n0 > 0 ? row[0] : 0u;              // word at jf
    for (int g = 0; g < nlev; g++) {
      const McLevel L = pl->lv[g];
      const int lvl = L.level, s_end = acc[g * 32];
      for (int d0 = L.first; d0 < L.first + L.count; d0 += 32) {
        const int nd = min(32, L.first + L.count - d0);
        int tp_l = 0, tf_l = 0;
        float den_l = 0.f, rc_l = 0.f;
        if (lane < nd) {
          tp_l = ar.t_ip[d0 + lane];
          tf_l = ar.tau_abs[d0 + lane];
          den_l = ar.denom[d0 + lane];
          rc_l = ar.rcp[d0 + lane];
          div_prep(den_l, rc_l);
        }
        for (int k = 0; k < nd; k++) {
          const int Tp = __shfl_sync(FULL, tp_l, k), Tf = __shfl_sync(FULL, tf_l, k);
          const float den = __shfl_sync(FULL, den_l, k), rc = __shfl_sync(FULL, rc_l, k);
          // one step of each pointer without a branch (lanes step at different
          // delays), then a loop for the lanes that need more
          bool ap = jp >= 0 && pk_t(wp) >= Tp, af = jf < n0 && pk_t(wf) < Tf;
          {
            const uint32_t np = row[max(jp - 1, 0) * 32], nf = row[min(jf + 1, CAP - 1) * 32];
            rsum += ap ? pk_v(wp) : 0;
            ssum += af ? pk_v(wf) : 0;
            jp -= ap ? 1 : 0;
            jf += af ? 1 : 0;
            wp = ap ? (jp >= 0 ? np : 0u) : wp;
            wf = af ? (jf < n0 ? nf : 0u) : wf;
          }
          ap = jp >= 0 && pk_t(wp) >= Tp;
          af = jf < n0 && pk_t(wf) < Tf;
          if (__any_sync(FULL, ap || af)) {
            while (jp >= 0 && pk_t(wp) >= Tp) {
              rsum += pk_v(wp);
              jp--;
              wp = jp >= 0 ? row[jp * 32] : 0u;
            }
            while (jf < n0 && pk_t(wf) < Tf) {
              ssum += pk_v(wf);
              jf++;
              wf = jf < n0 ? row[jf * 32] : 0u;
            }
          }
          // lanes without a row of this kernel have n0 = 0: both numerators are 0
          if (p < P) {
            const size_t o = (size_t)(d0 + k) * P + p;
            IP[o] = scaled_quotient_nb(total - rsum, lvl, den, rc);
            IF[o] = scaled_quotient_nb(s_end - ssum, lvl, den, rc);
          }
        }
      }
    }
  }

  // G2: level by level on the compacted buffer
  int m = n0;
  bool J = true, U = true;  // junction at m sorted; stale suffix [m, n0) sorted
  for (int g = 0; g < nlev; g++) {
    const McLevel L = pl->lv[g];
    if (L.compact && m > 0) {
      const int lf = L.lastframe;
      int index = -1, prev = INT_MIN;
      uint32_t wnext = row[0];
      for (int i = 0; i < m; i++) {
        const uint32_t w = wnext;
        wnext = row[min(i + 1, CAP - 1) * 32];  // ahead of the writes (index <= i)
        const int t = pk_t(w) >> 1;
        if (t >= lf) break;
        if (t == prev) {
          const uint32_t h = row[index * 32];
          row[index * 32] = pk(t, pk_v(h) + pk_v(w));
        } else {
          row[++index * 32] = pk(t, pk_v(w));
          prev = t;
        }
      }
      const int m2 = index + 1;
      U = (m2 < m) ? (J && U) : U;
      J = (m2 == 0 || m2 >= n0) ? true : (pk_t(row[(m2 - 1) * 32]) <= pk_t(row[m2 * 32]));
      m = m2;
    }
    const bool sorted = mode != XPCS_MODE_REFERENCE || (J && U);
    const int tlo = L.tau_lo, thi = L.tau_lo + L.count - 1;
    // warp-uniform: every lane of the warp sees the same level
    const bool bins = tlo >= 1 && thi <= 64 && L.count <= 16 && L.lastframe <= 32 * scr;
    if (bins && sorted) {
      // mask words in the scratch: zeroed, then one store per word that holds
      // an entry (the bins increase along the prefix)
      const int nw = (L.lastframe + 31) >> 5;
      for (int q = 0; q < nw; q++) acc[q * 32] = 0;
      int cq = -1;
      uint32_t cb = 0u;
      for (int i = 0; i < m; i++) {
        const int t = pk_t(row[i * 32]);
        if ((t >> 5) != cq) {
          if (cq >= 0) acc[cq * 32] = (int32_t)cb;
          cq = t >> 5;
          cb = 0u;
        }
        cb |= 1u << (t & 31);
      }
      if (cq >= 0) acc[cq * 32] = (int32_t)cb;
      if (L.count <= 8)
        bins_pairs<8>(row, m, L.lastframe, tlo, L.count, acc);
      else
        bins_pairs<16>(row, m, L.lastframe, tlo, L.count, acc);
    } else if (sorted) {
      for (int k = 0; k < L.count; k++) acc[k * 32] = 0;
      // per source the next two entries are checked without a branch (lanes
      // stay together); a loop runs only while the second one is still short
      // of the window's end
      uint32_t wi = m > 0 ? row[0] : 0u;
      uint32_t w1 = m > 1 ? row[32] : 0u;
      for (int i = 0; i < m - 1; i++) {
        const uint32_t w2 = i + 2 < m ? row[(i + 2) * 32] : 0xffff0000u;  // frame 65535, value 0
        const int ti = pk_t(wi), vi = pk_v(wi);
        const int d1 = pk_t(w1) - ti, d2 = pk_t(w2) - ti;
        if (d1 >= tlo && d1 <= thi) acc[(d1 - tlo) * 32] += vi * pk_v(w1);
        if (d2 >= tlo && d2 <= thi) acc[(d2 - tlo) * 32] += vi * pk_v(w2);
        if (d2 < thi && i + 3 < m) {
          for (int j = i + 3; j < m; j++) {
            const uint32_t wj = row[j * 32];
            const int d = pk_t(wj) - ti;
            if (d > thi) break;
            if (d >= tlo) acc[(d - tlo) * 32] += vi * pk_v(wj);
          }
        }
        wi = w1;
        w1 = w2;
      }
    } else {
      // the buffer is not globally sorted: a pair counts only when the
      // reference's lower_bound over the whole buffer lands on the partner
      for (int k = 0; k < L.count; k++) acc[k * 32] = 0;
      for (int i = 0; i < m; i++) {
        const uint32_t wi = row[i * 32];
        const int ti = pk_t(wi);
        for (int j = i + 1; j < m; j++) {
          const uint32_t wj = row[j * 32];
          const int d = pk_t(wj) - ti;
          if (d > thi) break;
          if (d >= tlo && lower_bound_packed(row, n0, pk_t(wj)) == j)
            acc[(d - tlo) * 32] += pk_v(wi) * pk_v(wj);
        }
      }
    }
    // divisors broadcast by shuffle as in the IP/IF sweep; lanes without a
    // row of this kernel have zero sums
    for (int d0 = L.first; d0 < L.first + L.count; d0 += 32) {
      const int nd = min(32, L.first + L.count - d0);
      float den_l = 0.f, rc_l = 0.f;
      if (lane < nd) {
        den_l = ar.denom[d0 + lane];
        rc_l = ar.rcp[d0 + lane];
        div_prep(den_l, rc_l);
      }
      for (int k = 0; k < nd; k++) {
        const float den = __shfl_sync(0xffffffffu, den_l, k), rc = __shfl_sync(0xffffffffu, rc_l, k);
        if (p < P)
          G2[(size_t)(d0 + k) * P + p] =
              scaled_quotient_nb(acc[(d0 - L.first + k) * 32], 2 * L.level, den, rc);
      }
    }
  }
}

template <int CAP>
__global__ void __launch_bounds__(MT_WARPS * 32, 8)
k_mt_thread(const uint8_t *__restrict__ plan_g, const int64_t *__restrict__ row_ptr,
            const int32_t *__restrict__ row_len, const uint8_t *__restrict__ pclass,
            const int32_t *__restrict__ ev_frame, const float *__restrict__ ev_val,
            float *__restrict__ G2, float *__restrict__ IP, float *__restrict__ IF) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int scr = ((const McPlan *)plan_g)->scr;
  const int warp = threadIdx.x >> 5;
  uint32_t *wbase = (uint32_t *)smem + (size_t)warp * (CAP + scr) * 32;
  mt_thread_warp<CAP>(plan_g, row_ptr, row_len, pclass, ev_frame, ev_val, G2, IP, IF,
                      (blockIdx.x * MT_WARPS + warp) * 32, wbase);
}

// ------------------------------------------------------- warp per pixel

// lower_bound over a contiguous packed row (frame in the high half)
__device__ __forceinline__ int lower_bound_row(const uint32_t *row, int n, int32_t x) {
  int first = 0, len = n;
  while (len > 0) {
    int half = len >> 1;
    if ((int32_t)(row[first + half] >> 16) < x) {
      first += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return first;
}

// In-place compaction of the live prefix row[0, m) for the next level
// (warp-cooperative): frame/2, equal neighbours merged, frames >= lastframe
// dropped.  Entries at and beyond the returned length are left untouched
// (the reference's stale tail).
__device__ int compact_row(uint32_t *row, int m, int lastframe, int lane) {
  const unsigned FULL = 0xffffffffu, lt = (1u << lane) - 1u;
  int gbase = 0;
  int prev = INT_MIN;  // halved frame of the entry before the current chunk
  for (int c0 = 0; c0 < m; c0 += 32) {
    const int i = c0 + lane;
    const bool in = i < m;
    const uint32_t w = in ? row[i] : 0u;
    const int ti = in ? (pk_t(w) >> 1) : INT_MAX;
    int vi = in ? pk_v(w) : 0;
    if (i + 1 < m) {
      const uint32_t w2 = row[i + 1];
      if ((pk_t(w2) >> 1) == ti) vi += pk_v(w2);  // rows hold distinct frames: pairs at most
    }
    int tp = __shfl_up_sync(FULL, ti, 1);
    if (lane == 0) tp = prev;
    const bool head = in && ti != tp && ti < lastframe;
    const unsigned hm = __ballot_sync(FULL, head);
    prev = __shfl_sync(FULL, ti, 31);
    __syncwarp();
    if (head) row[gbase + __popc(hm & lt)] = pk(ti, vi);
    gbase += __popc(hm);
    __syncwarp();
    if (prev >= lastframe) break;
  }
  return gbase;
}

// One warp per pixel of `list` (count at *count_p) whose row holds more than
// min_n and at most `cap` events, packed (frame << 16 | int16 value) in the warp's shared memory, with
// the row's inclusive prefix sums and per-lane accumulators beside it.
//   IP / IF: from the original row, as in the thread kernel: lanes take the
//     delays and look the thresholds up in the prefix sums.
//   G2: per level, warp-cooperative compaction, then every lane takes the
//     sources lane, lane+32, ... in one flat loop over (source, partner)
//     visits into its own accumulators, summed over the warp at the end of
//     the level.  On sorted levels where a fifth of the bins hold an entry,
//     the prefix-sum array (done with after IP/IF) holds the values by bin
//     and a source finds each partner by one lookup.  On other sorted levels
//     of delays <= 64 where the row could reach every delay (m x (thi + 1) >=
//     lastframe), the same words hold the row's occupancy bitmask: a source
//     reads the 64 bins after it, finds its first partner's index by a
//     population count over the bins below tau_lo and visits only the
//     occupied bins of the delay window.
// One pixel p of a series with a row of n0 events (min_n < n0 <= cap): the
// body of the warp-per-pixel kernel, shared by its per-series launches and by
// the batch's work-queue launches.  pl / ar: the plan (shared or global
// memory); row, S: the warp's 2 x cap words; acc: this lane's accumulators
// (acc[k * 32]).
__device__ __forceinline__ void mt_warp_pixel(const McPlan *pl, const McArrays &ar, int p,
                                              const int64_t *__restrict__ row_ptr,
                                              const int32_t *__restrict__ row_len,
                                              const int32_t *__restrict__ ev_frame,
                                              const float *__restrict__ ev_val,
                                              float *__restrict__ G2, float *__restrict__ IP,
                                              float *__restrict__ IF, int cap, uint32_t *row,
                                              int32_t *S, int32_t *acc) {
  const int P = pl->P, mode = pl->mode, D = pl->D;
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  const int n0 = row_len[p];
  const int64_t b = row_ptr[p];
  int carry = 0;
  for (int c0 = 0; c0 < n0; c0 += 32) {
    const int i = c0 + lane;
    int x = 0;
    if (i < n0) {
      x = __float2int_rn(ev_val[b + i]);
      row[i] = pk(ev_frame[b + i], x);
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (i < n0) S[i] = x + carry;
    carry += __shfl_sync(FULL, x, 31);
  }
  __syncwarp();
  // IP(d) = S(t_ip[d]); IF(d) = S(t_end of its level) - S(tau_abs[d]); S(T) = sum of
  // v over frames < T
  for (int d = lane; d < D; d += 32) {
    const int g = ar.gi[d];
    const int lvl = pl->lv[g].level;
    const int c_ip = lower_bound_row(row, n0, ar.t_ip[d]);
    const int c_end = lower_bound_row(row, n0, pl->lv[g].t_end);
    const int c_tau = lower_bound_row(row, n0, ar.tau_abs[d]);
    const int ip = c_ip ? S[c_ip - 1] : 0;
    const int iff = (c_end ? S[c_end - 1] : 0) - (c_tau ? S[c_tau - 1] : 0);
    IP[(size_t)d * P + p] = scaled_quotient(ip, lvl, ar.denom[d], ar.rcp[d]);
    IF[(size_t)d * P + p] = scaled_quotient(iff, lvl, ar.denom[d], ar.rcp[d]);
  }
  int m = n0;
  bool J = true, U = true;  // junction at m sorted; stale suffix [m, n0) sorted
  for (int gi = 0; gi < pl->nlev; gi++) {
    const McLevel L = pl->lv[gi];
    if (L.compact && m > 0) {
      const int m2 = compact_row(row, m, L.lastframe, lane);
      U = (m2 < m) ? (J && U) : U;
      J = (m2 == 0 || m2 >= n0) ? true : (pk_t(row[m2 - 1]) <= pk_t(row[m2]));
      m = m2;
    }
    const bool sorted = mode != XPCS_MODE_REFERENCE || (J && U);
    const int tlo = L.tau_lo, thi = L.tau_lo + L.count - 1;
    for (int k = 0; k < L.count; k++) acc[k * 32] = 0;
    const int lf = L.lastframe;
    if (sorted && tlo >= 1 && lf <= cap && 5 * m >= lf) {
      // at least a fifth of the level's bins hold an entry: the prefix sums
      // S are done with, and S becomes the row's values by bin, so that each
      // source finds its partner for every delay with one lookup (a missing
      // bin reads 0, which adds nothing)
      for (int bq = lane; bq < lf; bq += 32) S[bq] = 0;
      __syncwarp();
      for (int k = lane; k < m; k += 32) S[pk_t(row[k])] = pk_v(row[k]);
      __syncwarp();
      for (int i = lane; i < m; i += 32) {
        const uint32_t wi = row[i];
        const int ti = pk_t(wi), vi = pk_v(wi);
        for (int k = 0; k < L.count; k++) {
          const int tb = ti + tlo + k;
          if (tb < lf) acc[k * 32] += vi * S[tb];
        }
      }
    } else if (sorted && tlo >= 1 && thi <= 64 && lf <= 32 * cap && m * (thi + 1) >= lf) {
      // about one entry or more per delay window: S (done with after IP/IF)
      // becomes the level's occupancy bitmask.  Bins of the prefix are distinct
      // and increasing, so the entry at bin b is at position popcount(bits
      // below b): one 64-bit window of the mask after a source's bin gives the
      // position of its first partner (entries closer than the smallest delay
      // are counted, not visited) and which delays have a partner
      uint32_t *mk = (uint32_t *)S;
      const int nw = (lf + 31) >> 5;
      for (int q = lane; q < nw; q += 32) mk[q] = 0u;
      __syncwarp();
      for (int k = lane; k < m; k += 32) {
        const int t = pk_t(row[k]);
        atomicOr(&mk[t >> 5], 1u << (t & 31));
      }
      __syncwarp();
      const uint64_t gap = (1ull << (tlo - 1)) - 1ull;
      const uint32_t cmask = L.count >= 32 ? 0xffffffffu : ((1u << L.count) - 1u);
      for (int i = lane; i < m; i += 32) {
        const uint32_t wi = row[i];
        const int ti = pk_t(wi);
        if (ti + tlo >= lf) break;  // this and later sources have no partner below lastframe
        const int s0 = ti + 1, q = s0 >> 5, sh = s0 & 31;  // s0 < lf: word q exists
        const uint32_t m0 = mk[q];
        const uint32_t m1 = q + 1 < nw ? mk[q + 1] : 0u;
        const uint32_t m2 = q + 2 < nw ? mk[q + 2] : 0u;
        const uint64_t W =
            ((uint64_t)__funnelshift_r(m1, m2, sh) << 32) | __funnelshift_r(m0, m1, sh);
        int j = i + 1 + __popcll(W & gap);
        uint32_t w = (uint32_t)(W >> (tlo - 1)) & cmask;
        const int vi = pk_v(wi);
        while (w) {
          const int k = __ffs(w) - 1;
          acc[k * 32] += vi * pk_v(row[j]);
          j++;
          w &= w - 1u;
        }
      }
      __syncwarp();
    } else {
      int i = lane, j = lane + 1;
      uint32_t wi = i < m ? row[i] : 0u;
      uint32_t wj = j < m ? row[j] : 0u;
      while (i < m) {
        const int d = pk_t(wj) - pk_t(wi);
        if (j < m && d <= thi) {
          if (d >= tlo && (sorted || lower_bound_row(row, n0, pk_t(wj)) == j))
            acc[(d - tlo) * 32] += pk_v(wi) * pk_v(wj);
          j++;
        } else {
          i += 32;
          if (i >= m) break;
          wi = row[i];
          j = i + 1;
        }
        wj = j < m ? row[j] : 0u;
      }
    }
    int mine = 0;
    for (int k = 0; k < L.count; k++) {
      const int tot = __reduce_add_sync(FULL, acc[k * 32]);
      if (lane == k) mine = tot;
    }
    if (lane < L.count) {
      const int d = L.first + lane;
      G2[(size_t)d * P + p] = scaled_quotient(mine, 2 * L.level, ar.denom[d], ar.rcp[d]);
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(256)
k_mt_warp(const uint8_t *__restrict__ plan_g, const int32_t *__restrict__ list,
          const int32_t *__restrict__ count_p, int32_t min_n, int32_t cap,
          const int64_t *__restrict__ row_ptr, const int32_t *__restrict__ row_len,
          const int32_t *__restrict__ ev_frame, const float *__restrict__ ev_val,
          float *__restrict__ G2, float *__restrict__ IP, float *__restrict__ IF) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int D = ((const McPlan *)plan_g)->D;
  const size_t pb = mc_plan_bytes(D);
  copy_plan(smem, plan_g, pb);
  __syncthreads();
  const McPlan *pl = (const McPlan *)smem;
  const McArrays ar = mc_arrays(smem, D);
  const int ACC = max(pl->acc, pl->nlev);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  uint32_t *row = (uint32_t *)(smem + pb) + (size_t)warp * (2 * cap + 32 * ACC);
  int32_t *S = (int32_t *)(row + cap);
  int32_t *acc = S + cap + lane;  // acc[k * 32]: this lane's accumulator k
  const int nw = *count_p;
  for (int q = blockIdx.x * nwb + warp; q < nw; q += gridDim.x * nwb) {
    const int p = list[q];
    const int n0 = row_len[p];
    if (n0 <= min_n || n0 > cap) continue;  // another launch's share of the list
    mt_warp_pixel(pl, ar, p, row_ptr, row_len, ev_frame, ev_val, G2, IP, IF, cap, row, S, acc);
  }
}

// ------------------------------------------------ batch work-queue launches
//
// The multi-tau of every member of a batch as persistent grids that pull work
// items from a device counter: 32-pixel groups of every member with the same
// thread-kernel row capacity in one launch, the warp-per-pixel rows of every
// member in one launch per row tier.  Small members' items run beside large
// members' items, and no member's kernel leaves a tail of idle SMs.

// Thread-per-pixel items: group g of the queue is group g - first of the
// member whose range holds it.  wbase strides by the batch's largest scratch.
template <int CAP>
__global__ void __launch_bounds__(MT_WARPS * 32, 8)
k_mt_thread_queue(const MtQueueMember *__restrict__ tab, int32_t n, int32_t total,
                  int32_t scr_max, int32_t *__restrict__ next) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t *wbase = (uint32_t *)smem + (size_t)warp * (CAP + scr_max) * 32;
  for (;;) {
    int g = 0;
    if (lane == 0) g = atomicAdd(next, 1);
    g = __shfl_sync(0xffffffffu, g, 0);
    if (g >= total) break;
    int lo = 0, hi = n - 1;  // the last member whose first group is <= g
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tab[mid].first <= g) lo = mid;
      else hi = mid - 1;
    }
    const MtQueueMember &m = tab[lo];
    mt_thread_warp<CAP>(m.plan, m.row_ptr, m.row_len, m.pclass, m.ev_frame, m.ev_val, m.G2, m.IP,
                        m.IF, (g - m.first) * 32, wbase);
    __syncwarp();
  }
}

// Warp-per-pixel items: entry q of the members' warp lists (use_long = 0) or
// long-row lists, concatenated in table order; rows outside (min_n, cap]
// belong to another tier's launch.  The plan is read from global memory.
__global__ void __launch_bounds__(256)
k_mt_warp_queue(const MtQueueMember *__restrict__ tab, int32_t n, int32_t use_long,
                int32_t min_n, int32_t cap, int32_t acc_max, int32_t *__restrict__ next) {
  extern __shared__ __align__(16) uint8_t smem[];
  int32_t *pref = (int32_t *)smem;  // [n + 1]: first entry of each member's list
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    int32_t t = 0;
    for (int i = 0; i < n; i++) {
      pref[i] = t;
      t += use_long ? tab[i].stats->nlong : tab[i].stats->nwarp;
    }
    pref[n] = t;
  }
  __syncthreads();
  const int total = pref[n];
  const size_t pref_bytes = mc_align16(sizeof(int32_t) * (size_t)(n + 1));
  uint32_t *row = (uint32_t *)(smem + pref_bytes) + (size_t)warp * (2 * cap + 32 * acc_max);
  int32_t *S = (int32_t *)(row + cap);
  int32_t *acc = S + cap + lane;
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(next, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= total) break;
    int lo = 0, hi = n - 1;  // the last member whose list starts at or before q
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (pref[mid] <= q) lo = mid;
      else hi = mid - 1;
    }
    const MtQueueMember &m = tab[lo];
    const int p = (use_long ? m.llist : m.wlist)[q - pref[lo]];
    const int n0 = m.row_len[p];
    if (n0 <= min_n || n0 > cap) continue;
    const McPlan *pl = (const McPlan *)m.plan;
    const McArrays ar = mc_arrays(m.plan, pl->D);
    mt_warp_pixel(pl, ar, p, m.row_ptr, m.row_len, m.ev_frame, m.ev_val, m.G2, m.IP, m.IF, cap,
                  row, S, acc);
  }
}

// --------------------------------------------------------- float replay

__global__ void __launch_bounds__(128)
k_mt_float(const uint8_t *__restrict__ plan_g, const int32_t *__restrict__ flist,
           const DevStats *__restrict__ stats, const int64_t *__restrict__ row_ptr,
           const int32_t *__restrict__ row_len, const int32_t *__restrict__ ev_frame,
           const float *__restrict__ ev_val, const float *__restrict__ fscale,
           int32_t *__restrict__ sc_frame, float *__restrict__ sc_val, float *__restrict__ G2,
           float *__restrict__ IP, float *__restrict__ IF) {
  const McPlan *pl = (const McPlan *)plan_g;
  const int D = pl->D, P = pl->P;
  const McArrays ar = mc_arrays(plan_g, D);
  const int nf = stats->nfloat;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nf; q += gridDim.x * blockDim.x) {
    const int p = flist[q];
    const int64_t b = row_ptr[p];
    const int n0 = row_len[p];
    int32_t *idx = sc_frame + b;
    float *val = sc_val + b;
    for (int i = 0; i < n0; i++) {
      idx[i] = ev_frame[b + i];
      // normalize_by_framesum: v / (frameSum[f] / mean) (main.cpp:330-333)
      val[i] = fscale ? __fdiv_rn(ev_val[b + i], fscale[idx[i]]) : ev_val[b + i];
    }
    replay_pixel(pl, ar, P, p, idx, val, n0, G2, IP, IF);
  }
}

// ------------------------------------------------ float rows, warp per pixel
//
// The same operations as k_mt_float, in the same order per sum, with the work
// of one pixel spread over a warp:
//   * the row is compacted in place in the scratch buffer exactly as the
//     reference does it (so the stale tail is the reference's), 32 entries per
//     step: each entry's half index, a ballot of the group starts and the pair
//     sum (v[i] + v[i+1]) / 2 of merged neighbours;
//   * lower_bound over the whole buffer lands on a prefix entry j exactly when
//     lower_bound(idx[j]) == j ("findable"); the search result is monotone in
//     its argument, so a pair (r, j) counts iff idx[j] == idx[r] + tau and j is
//     findable.  While the buffer is sorted (tracked per level from the
//     junctions between the prefix and the older segments) every entry is
//     findable; otherwise each lane runs the reference's search for its entry;
//   * each float sum (G2, IP, IF of every delay of the level) is a chain that
//     one lane accumulates in the reference's order: per 32 entries the lanes
//     first write their terms (v*v' of the pair with distance tau, or v inside
//     the IP / IF ranges, else +0, which leaves a sum unchanged) to shared
//     memory, then each chain's lane adds its 32 terms in entry order.
// Partners lie at most tau entries ahead (distinct ascending indices), so a
// ring of two 32-entry tiles holds every partner of the current tile.
constexpr int FW_WARPS = 4;
constexpr int FW_MAXC = 32;  // delays per level and largest delay in level units
// Term rows of 36 floats: 16-byte aligned, so a chain's lane reads its 32
// terms as 8 float4 loads; lanes 0-7 of such a load (chains 0-7) touch banks
// 4*chain .. 4*chain+3, distinct, so the loads stay free of bank conflicts.
constexpr int FW_TSTRIDE = 36;
constexpr int FW_WIN = 128;  // bins of the per-warp partner window

// Shared memory of one warp: ring idx[64], val[64]; the bin window's values
// [FW_WIN]; terms [3 * acc][FW_TSTRIDE] and the shared IP/IF row
// [FW_TSTRIDE]; rounded up to 16 bytes.  (The ring's findable flags are a
// register mask: at 16 delays in a level this makes 8,080 bytes, and 4 warps
// per block fit 7 blocks on an SM.)
__host__ __device__ constexpr size_t fw_warp_bytes(int acc_max) {
  return (64 * 8 + FW_WIN * 4 + (3 * (size_t)acc_max + 1) * FW_TSTRIDE * 4 + 15) & ~(size_t)15;
}

__device__ __forceinline__ int lower_bound_g(const int32_t *a, int n, int32_t x) {
  int first = 0, len = n;
  while (len > 0) {
    const int half = len >> 1;
    if (a[first + half] < x) {
      first += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return first;
}

// Entry tb + lane of the level's row with its findable flag, fetched into
// registers (fw_fetch) some time before it goes into its ring slot (fw_put),
// so that the load's latency passes while a tile is processed.
struct FwEntry {
  int32_t x;
  float v;
  uint8_t f;
};

__device__ __forceinline__ FwEntry fw_fetch(int tb, int lane, int L, int n0, bool all_find,
                                            const int32_t *idx, const float *val) {
  FwEntry e{0, 0.f, 0};
  const int j = tb + lane;
  if (j < L) {
    e.x = idx[j];
    e.v = val[j];
    e.f = all_find ? 1 : (lower_bound_g(idx, n0, e.x) == j);
  }
  return e;
}

// The ring's findable flags are one 64-bit mask, the same in every lane: tb is
// a multiple of 32, so a tile fills one half of the ring, bits (tb & 32) on.
__device__ __forceinline__ void fw_put(int tb, int lane, int L, const FwEntry &e, int32_t *ridx,
                                       float *rval, uint64_t &fmask) {
  const int j = tb + lane, slot = j & 63;
  if (j < L) {
    ridx[slot] = e.x;
    rval[slot] = e.v;
  }
  const uint64_t b = __ballot_sync(0xffffffffu, j < L && e.f);
  const int sh = tb & 32;
  fmask = (fmask & ~(0xffffffffull << sh)) | (b << sh);
}

__device__ __forceinline__ bool fw_findable(uint64_t fmask, int j) {
  return (fmask >> (j & 63)) & 1u;
}

__global__ void __launch_bounds__(FW_WARPS * 32, 7)
k_mt_fwarp(const uint8_t *__restrict__ plan_g, const int32_t *__restrict__ flist,
           DevStats *__restrict__ stats, const int64_t *__restrict__ row_ptr,
           const int32_t *__restrict__ row_len, const int32_t *__restrict__ ev_frame,
           const float *__restrict__ ev_val, const float *__restrict__ fscale,
           int32_t *__restrict__ sc_frame, float *__restrict__ sc_val, float *__restrict__ G2,
           float *__restrict__ IP, float *__restrict__ IF) {
  extern __shared__ __align__(16) uint8_t fw_smem[];
  const McPlan *pl = (const McPlan *)plan_g;
  const int D = pl->D, P = pl->P, nlev = pl->nlev, acc_max = pl->acc;
  const bool ref = pl->mode == XPCS_MODE_REFERENCE;
  const McArrays ar = mc_arrays(plan_g, D);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint8_t *wb = fw_smem + (size_t)w * fw_warp_bytes(acc_max);
  int32_t *ridx = (int32_t *)wb;
  float *rval = (float *)(wb + 256);
  // bin b of the window: the value of the entry at b0 + b when it is
  // findable, else 0; the G2 term v * 0 = +-0 then leaves its chain
  // unchanged (the chains start at +0 and x + -x is +0, so no chain is ever
  // -0, and a + +-0 == a for every other a)
  float *bval = (float *)(wb + 512);
  float *terms = (float *)(wb + 512 + FW_WIN * 4);
  float *vrow = terms + (size_t)3 * acc_max * FW_TSTRIDE;
  const int nf = stats->nfloat;
  // pixels are handed out one per warp from a counter: rows differ in length
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(&stats->fnext, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= nf) break;
    const int p = flist[q];
    const int64_t b = row_ptr[p];
    const int n0 = row_len[p];
    int32_t *idx = sc_frame + b;
    float *val = sc_val + b;
    for (int i0 = 0; i0 < n0; i0 += 4 * 32) {
      int32_t f[4];
      float x[4];
#pragma unroll
      for (int h = 0; h < 4; h++) {  // the loads first, in flight together
        const int i = i0 + h * 32 + lane;
        if (i < n0) {
          f[h] = ev_frame[b + i];
          x[h] = ev_val[b + i];
        }
      }
#pragma unroll
      for (int h = 0; h < 4; h++) {
        const int i = i0 + h * 32 + lane;
        if (i < n0) {
          idx[i] = f[h];
          // normalize_by_framesum: v / (frameSum[f] / mean) (main.cpp:330-333)
          val[i] = fscale ? __fdiv_rn(x[h], fscale[f[h]]) : x[h];
        }
      }
    }
    __syncwarp();
    int L = n0;
    bool tail_sorted = true, dead = false;
    for (int gi = 0; gi < nlev; gi++) {
      const McLevel lv = pl->lv[gi];
      const int lastframe = lv.lastframe, cnt = lv.count, t0 = lv.tau_lo;
      if (lv.compact && !dead) {
        const int prevL = L;
        // the junction between the previous prefix and the older tail
        bool junction_ok = true;
        if (prevL < n0) junction_ok = idx[prevL - 1] <= idx[prevL];
        if ((idx[0] >> 1) >= lastframe) {
          dead = true;  // nothing is kept: lastIndex becomes 1 on a stale entry
        } else {
          int out = 0, carry_h = -1;
          // chunks of 32 entries, each loaded two chunks ahead: a chunk's
          // pass writes only below its own end, so the entries in flight
          // are never overwritten before they are used
          int32_t ia = lane < prevL ? idx[lane] : INT_MAX;
          float va = lane < prevL ? val[lane] : 0.f;
          int32_t ia1 = 32 + lane < prevL ? idx[32 + lane] : INT_MAX;
          float va1 = 32 + lane < prevL ? val[32 + lane] : 0.f;
          for (int base = 0; base < prevL; base += 32) {
            const int a2 = base + 64 + lane;
            const int32_t ia2 = a2 < prevL ? idx[a2] : INT_MAX;
            const float va2 = a2 < prevL ? val[a2] : 0.f;
            const int a = base + lane;
            const bool in = a < prevL;
            const bool has_b = a + 1 < prevL;
            // the next entry: the lane above's, or the next chunk's first
            int32_t ib = __shfl_down_sync(0xffffffffu, ia, 1);
            float vb = __shfl_down_sync(0xffffffffu, va, 1);
            const int32_t ib1 = __shfl_sync(0xffffffffu, ia1, 0);
            const float vb1 = __shfl_sync(0xffffffffu, va1, 0);
            if (lane == 31) {
              ib = ib1;
              vb = vb1;
            }
            const int h = ia >> 1, hb = ib >> 1;
            int hp = __shfl_up_sync(0xffffffffu, h, 1);
            if (lane == 0) hp = carry_h;
            const bool keep = in && (a == 0 || h != hp) && h < lastframe;
            const bool merge = keep && has_b && hb == h;
            float sv = va;
            if (merge) sv = __fadd_rn(va, vb);
            sv = __fmul_rn(sv, 0.5f);  // == sv / 2 (exact scaling)
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            const bool stop = __any_sync(0xffffffffu, in && h >= lastframe);
            carry_h = __shfl_sync(0xffffffffu, h, 31);
            __syncwarp();
            if (keep) {
              const int o = out + __popc(bal & ((1u << lane) - 1u));
              idx[o] = h;
              val[o] = sv;
            }
            out += __popc(bal);
            __syncwarp();
            if (stop) break;
            ia = ia1;
            va = va1;
            ia1 = ia2;
            va1 = va2;
          }
          L = out;
          tail_sorted = tail_sorted && (L >= prevL || junction_ok);
        }
      }
      if (dead) {
        for (int c = lane; c < cnt; c += 32) {
          const size_t o = (size_t)(lv.first + c) * P + p;
          G2[o] = 0.f;
          IP[o] = 0.f;
          IF[o] = 0.f;
        }
        continue;
      }
      // every prefix entry is findable unless the reference searches a buffer
      // that is out of order
      const bool all_find = !ref || (tail_sorted && (L >= n0 || idx[L - 1] <= idx[L]));
      const int kmax = t0 + cnt - 1;
      const int nchain = 3 * cnt;
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      // ring slots past the row end are never read (partners stop at L)
      uint64_t fmask = 0;
      fw_put(0, lane, L, fw_fetch(0, lane, L, n0, all_find, idx, val), ridx, rval, fmask);
      fw_put(32, lane, L, fw_fetch(32, lane, L, n0, all_find, idx, val), ridx, rval, fmask);
      for (int base = 0; base < L; base += 32) {
        // the tile after next, in flight while this one is processed
        const FwEntry nx = fw_fetch(base + 64, lane, L, n0, all_find, idx, val);
        __syncwarp();
        const int r = base + lane;
        const bool valid = r < L;
        const int nt = min(32, L - base);  // entries in this tile
        const int32_t src = valid ? ridx[r & 63] : 0;
        const float v = valid ? rval[r & 63] : 0.f;
        // partners: when the tile and its partners span fewer than FW_WIN
        // bins, through a per-warp bin array (one lookup per delay), else by
        // scanning the following entries
        const int32_t b0 = ridx[base & 63];
        const bool use_bins = ridx[(base + nt - 1) & 63] + kmax - b0 < FW_WIN;
        if (use_bins) {
          ((float4 *)bval)[lane] = make_float4(0.f, 0.f, 0.f, 0.f);  // FW_WIN = 128 bins
          __syncwarp();
          if (valid) bval[src - b0] = fw_findable(fmask, r) ? v : 0.f;
          const int q2 = base + 32 + lane;
          if (lane < kmax && q2 < L) {
            const int tb = ridx[q2 & 63] - b0;
            if (tb < FW_WIN) bval[tb] = fw_findable(fmask, q2) ? rval[q2 & 63] : 0.f;
          }
          __syncwarp();
        }
        // inside [kmax, lastframe - kmax) every IP and IF term of the tile is v:
        // the IP/IF chains then read one shared row
        const bool bulk = b0 >= kmax && ridx[(base + nt - 1) & 63] < lastframe - kmax;
        if (valid) {
          if (bulk) {
            vrow[lane] = v;
          } else {
            float *tp = terms + (size_t)cnt * FW_TSTRIDE + lane;
            float *tf = tp + (size_t)cnt * FW_TSTRIDE;
#pragma unroll
            for (int c = 0; c < FW_MAXC; c++) {
              if (c >= cnt) break;
              const int tau = t0 + c;
              tp[c * FW_TSTRIDE] = src < lastframe - tau ? v : 0.f;
              tf[c * FW_TSTRIDE] = (src >= tau && src < lastframe) ? v : 0.f;
            }
          }
          // a partner is a prefix entry, so it lies below lastframe and the
          // reference's src < lastframe - tau test holds for every pair found
          if (use_bins) {
            const float *bw = bval + (src + t0 - b0);  // + c <= src - b0 + kmax < FW_WIN
            float *tg = terms + lane;
            if ((cnt & 3) == 0) {  // e.g. every level of 8 delays: one test per 4 delays
#pragma unroll
              for (int c = 0; c < FW_MAXC; c += 4) {
                if (c >= cnt) break;
#pragma unroll
                for (int u = 0; u < 4; u++) tg[(c + u) * FW_TSTRIDE] = __fmul_rn(v, bw[c + u]);
              }
            } else {
#pragma unroll
              for (int c = 0; c < FW_MAXC; c++) {
                if (c >= cnt) break;
                tg[c * FW_TSTRIDE] = __fmul_rn(v, bw[c]);
              }
            }
          } else {
            for (int c = 0; c < cnt; c++) terms[(size_t)c * FW_TSTRIDE + lane] = 0.f;
            for (int k = t0 > 0 ? 1 : 0; k <= kmax; k++) {
              const int qk = r + k;
              if (qk >= L) break;
              const int d = ridx[qk & 63] - src;
              if (d > kmax) break;
              if (d >= t0 && fw_findable(fmask, qk))
                terms[(size_t)(d - t0) * FW_TSTRIDE + lane] = __fmul_rn(v, rval[qk & 63]);
            }
          }
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int ch = lane + 32 * j;
          if (ch < nchain) {
            const float *tr = (bulk && ch >= cnt) ? vrow : terms + (size_t)ch * FW_TSTRIDE;
            float a = acc[j];
            if (nt == 32) {
              const float4 *t4 = (const float4 *)tr;
#pragma unroll
              for (int i = 0; i < 8; i++) {
                const float4 y = t4[i];
                a = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(a, y.x), y.y), y.z), y.w);
              }
            } else {
#pragma unroll
              for (int i = 0; i < 32; i++) {
                if (i >= nt) break;
                a = __fadd_rn(a, tr[i]);
              }
            }
            acc[j] = a;
          }
        }
        __syncwarp();
        // the tile after next replaces this one in the ring
        fw_put(base + 64, lane, L, nx, ridx, rval, fmask);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int ch = lane + 32 * j;
        if (ch < nchain) {
          const int type = ch / cnt, c = ch - type * cnt;
          const int d = lv.first + c;
          const float den = ar.denom[d];
          const float x = den > 0.f ? __fdiv_rn(acc[j], den) : acc[j];
          float *dst = type == 0 ? G2 : (type == 1 ? IP : IF);
          dst[(size_t)d * P + p] = x;
        }
      }
    }
    __syncwarp();
  }
}

// Host-side plan: level groups of the delay schedule with the lastframe each
// sees and whether the reference compacts before it (corr.cpp:341-391).
std::vector<uint8_t> make_plan(const Series &s, int mode) {
  const int D = s.D;
  std::vector<uint8_t> buf(mc_plan_bytes(D), 0);
  McPlan *pl = (McPlan *)buf.data();
  int32_t *base = (int32_t *)(buf.data() + sizeof(McPlan));
  int32_t *tau_lvl = base;
  float *denom = (float *)(base + D);
  int32_t *tau_abs = base + 2 * D, *t_ip = base + 3 * D, *gi = base + 4 * D;
  float *rcp = (float *)(base + 5 * D);
  pl->P = s.P;
  pl->D = D;
  pl->F = s.F;
  pl->mode = mode;
  int ll = 0, lastframe = s.F, nlev = 0, acc = 1;
  for (int k = 0; k < D; k++) {
    int level = s.delays.level[k];
    bool newgroup = (k == 0) || level != s.delays.level[k - 1];
    int compact = 0;
    if (ll != level) {
      if (lastframe % 2) lastframe -= 1;
      lastframe = lastframe / 2;
      compact = 1;
    }
    // tau / pow(2, level) truncated to int (corr.cpp:393-394)
    int tau = level > 0 ? (int)(s.delays.tau[k] / std::pow(2.0, level)) : s.delays.tau[k];
    tau_lvl[k] = tau;
    tau_abs[k] = s.delays.tau[k];
    denom[k] = (lastframe - tau) > 0 ? (float)(lastframe - tau) : 0.f;
    rcp[k] = denom[k] > 0.f ? recip_rn((int32_t)(lastframe - tau)) : 0.f;
    t_ip[k] = (int32_t)std::max<int64_t>(0, (int64_t)(lastframe - tau) << level);
    if (newgroup) {
      if (nlev >= MAX_LEVELS) throw Error(XPCS_ERR_INVALID_ARGUMENT, "too many multi-tau levels");
      McLevel &L = pl->lv[nlev++];
      L.level = level;
      L.first = k;
      L.count = 0;
      L.lastframe = lastframe;
      L.tau_lo = tau;
      L.compact = compact;
      L.t_end = (int32_t)((int64_t)lastframe << level);
    }
    McLevel &L = pl->lv[nlev - 1];
    if (tau != L.tau_lo + L.count)
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "non-consecutive delays within a level");
    L.count++;
    acc = std::max(acc, L.count);
    gi[k] = nlev - 1;
    ll = level;
  }
  pl->nlev = nlev;
  pl->acc = acc;
  pl->scr = std::max(acc, nlev) + std::max(0, s.scr_extra);
  for (int k = 1; k < D; k++)
    if (t_ip[k] >= t_ip[k - 1] || tau_abs[k] <= tau_abs[k - 1])
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "delay thresholds are not monotone");
  for (int g = 1; g < nlev; g++)
    if (pl->lv[g].t_end > pl->lv[g - 1].t_end)
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "level end thresholds are not monotone");
  return buf;
}

size_t thread_smem(int scr, int cap) {
  return (size_t)MT_WARPS * (cap + scr) * 32 * sizeof(uint32_t);
}

using ThreadKernel = void (*)(const uint8_t *, const int64_t *, const int32_t *, const uint8_t *,
                              const int32_t *, const float *, float *, float *, float *);

ThreadKernel thread_kernel(int cap) {
  switch (cap) {
    case 32: return k_mt_thread<32>;
    case 48: return k_mt_thread<48>;
    case 64: return k_mt_thread<64>;
    case 80: return k_mt_thread<80>;
    case 112: return k_mt_thread<112>;
  }
  throw Error(XPCS_ERR_INVALID_ARGUMENT, "unsupported thread-kernel row capacity");
}
size_t warp_smem(int D, int acc, int cap, int warps) {
  return mc_plan_bytes(D) + (size_t)warps * (2 * cap + 32 * acc) * sizeof(int32_t);
}

// The float rows of a series (flatfield, average, hot pixels, dense data,
// normalize_by_framesum) on st: the warp-per-row replay when the schedule
// allows it, else the thread-per-row one.
void launch_float_rows(Series &s, const McPlan &hp, cudaStream_t st, int sms) {
  const int P = s.P;
  size_t ne = s.raw_events > 0 ? (size_t)s.raw_events : 1;
  s.sc_frame.reserve(ne, st);
  s.sc_val.reserve(ne, st);
  int grid = std::max(1, std::min((P + 127) / 128, sms * 8));
  const float *fscale = nullptr;
  if (s.desc.normalize_by_framesum) {
    prepare_framesum_scale(s);
    fscale = s.d_fscale.p;
  }
  int kmax = 0;
  for (int g = 0; g < hp.nlev; g++) kmax = std::max(kmax, hp.lv[g].tau_lo + hp.lv[g].count - 1);
  if (kmax <= FW_MAXC && hp.acc <= FW_MAXC) {
    const size_t smf = FW_WARPS * fw_warp_bytes(hp.acc);
    XG_CUDA(cudaFuncSetAttribute(k_mt_fwarp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smf));
    int per_sm = 0;
    XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mt_fwarp, FW_WARPS * 32,
                                                          smf));
    XG_CUDA(cudaMemsetAsync(&s.stats.p->fnext, 0, sizeof(int32_t), st));
    k_mt_fwarp<<<sms * std::max(1, per_sm), FW_WARPS * 32, smf, st>>>(
        s.plan.p, s.flist.p, s.stats.p, s.row_ptr.p, s.row_len.p, s.ev_frame.p, s.ev_val.p,
        fscale, s.sc_frame.p, s.sc_val.p, s.G2.p, s.IP.p, s.IF.p);
  } else {
    k_mt_float<<<grid, 128, 0, st>>>(s.plan.p, s.flist.p, s.stats.p, s.row_ptr.p, s.row_len.p,
                                     s.ev_frame.p, s.ev_val.p, fscale, s.sc_frame.p, s.sc_val.p,
                                     s.G2.p, s.IP.p, s.IF.p);
  }
  XG_CHECK_LAUNCH();
}

}  // namespace

// The float nearest to 1/b (ties to even) for an integer b in [1, 2^24]:
// candidates around the double quotient compared by their exact residuals
// (g*b has at most 48 significant bits, so 1 - g*b is exact in double).
float recip_rn(int32_t b) {
  const float f = (float)(1.0 / (double)b);
  float best = f;
  double be = std::fabs(1.0 - (double)f * b);
  for (float g : {std::nextafter(f, 0.f), std::nextafter(f, 2.f * f)}) {
    const double e = std::fabs(1.0 - (double)g * b);
    uint32_t gb, bb;
    std::memcpy(&gb, &g, 4);
    std::memcpy(&bb, &best, 4);
    if (e < be || (e == be && (gb & 1u) == 0 && (bb & 1u) != 0)) {
      best = g;
      be = e;
    }
  }
  return best;
}

void run_multitau(Series &s, int mode) {
  cudaStream_t st = s.stream;
  const int D = s.D, P = s.P;
  // the plan depends on the series' shape and the mode only; it is uploaded
  // once per mode (a captured batch graph must not copy from host memory)
  std::vector<uint8_t> plan = make_plan(s, mode);
  const McPlan *hp = (const McPlan *)plan.data();
  if (s.plan_mode != mode || s.plan_scr != hp->scr) {
    s.plan.reserve(plan.size(), st);
    XG_CUDA(cudaMemcpyAsync(s.plan.p, plan.data(), plan.size(), cudaMemcpyHostToDevice, st));
    XG_CUDA(cudaStreamSynchronize(st));
    s.plan_mode = mode;
    s.plan_scr = hp->scr;
  }
  const size_t nD = (size_t)D * P;
  s.G2.reserve(nD ? nD : 1, st);
  s.IP.reserve(nD ? nD : 1, st);
  s.IF.reserve(nD ? nD : 1, st);
  if (D == 0 || P == 0) return;
  const int scr = std::max(hp->acc, hp->nlev);
  const ThreadKernel ktt = thread_kernel(s.thread_cap);
  const size_t smt = thread_smem(hp->scr, s.thread_cap),
               smw = warp_smem(D, scr, MT_WARP_CAP, WP_WARPS);
  const size_t smm = warp_smem(D, scr, MT_MID_CAP, MID_WARPS);
  const size_t sml = warp_smem(D, scr, MT_LONG_CAP, LONG_WARPS);
  if (smt > 227 * 1024 || smw > 227 * 1024 || smm > 227 * 1024 || sml > 227 * 1024)
    throw Error(XPCS_ERR_INVALID_ARGUMENT, "delay schedule too large for the multi-tau kernels");
  XG_CUDA(cudaFuncSetAttribute(ktt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smt));
  XG_CUDA(cudaFuncSetAttribute(k_mt_warp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)std::max(std::max(smw, smm), sml)));
  int sms = 0;
  XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s.device));
  XG_CUDA(cudaEventRecord(s.ev[4], st));
  const int per_block = MT_WARPS * 32;
  ktt<<<(P + per_block - 1) / per_block, per_block, smt, st>>>(
      s.plan.p, s.row_ptr.p, s.row_len.p, s.pclass.p, s.ev_frame.p, s.ev_val.p, s.G2.p, s.IP.p,
      s.IF.p);
  XG_CHECK_LAUNCH();
  const DevStats *ds = s.stats.p;
  // rows of 81-256 events; long rows in two launches over one list: up to 1024
  // events with 4 warps per block, longer ones with 2 warps per block
  k_mt_warp<<<sms * (int)((227 * 1024) / smw), WP_WARPS * 32, smw, st>>>(
      s.plan.p, s.wlist.p, &ds->nwarp, 0, MT_WARP_CAP, s.row_ptr.p, s.row_len.p, s.ev_frame.p,
      s.ev_val.p, s.G2.p, s.IP.p, s.IF.p);
  XG_CHECK_LAUNCH();
  k_mt_warp<<<sms * (int)((227 * 1024) / smm), MID_WARPS * 32, smm, st>>>(
      s.plan.p, s.llist.p, &ds->nlong, MT_WARP_CAP, MT_MID_CAP, s.row_ptr.p, s.row_len.p,
      s.ev_frame.p, s.ev_val.p, s.G2.p, s.IP.p, s.IF.p);
  XG_CHECK_LAUNCH();
  k_mt_warp<<<sms * (int)((227 * 1024) / sml), LONG_WARPS * 32, sml, st>>>(
      s.plan.p, s.llist.p, &ds->nlong, MT_MID_CAP, MT_LONG_CAP, s.row_ptr.p, s.row_len.p,
      s.ev_frame.p, s.ev_val.p, s.G2.p, s.IP.p, s.IF.p);
  XG_CHECK_LAUNCH();
  XG_CUDA(cudaEventRecord(s.ev[5], st));
  launch_float_rows(s, *hp, st, sms);
  XG_CUDA(cudaEventRecord(s.ev[6], st));
}

void mt_queue_build(const std::vector<Series *> &ss, MtQueue &q, cudaStream_t st) {
  std::vector<MtQueueMember> tab;
  q.cap_first.assign(MT_THREAD_NCAPS, 0);
  q.cap_count.assign(MT_THREAD_NCAPS, 0);
  q.cap_groups.assign(MT_THREAD_NCAPS, 0);
  q.scr_max = q.acc_max = 1;
  for (int c = 0; c < MT_THREAD_NCAPS; c++) {
    q.cap_first[c] = (int32_t)tab.size();
    int32_t groups = 0;
    for (Series *sp : ss) {
      Series &s = *sp;
      if (s.thread_cap != MT_THREAD_CAPS[c] || s.D == 0 || s.P == 0) continue;
      const McPlan hp = *(const McPlan *)make_plan(s, s.plan_mode).data();
      q.scr_max = std::max(q.scr_max, hp.scr);
      q.acc_max = std::max(q.acc_max, std::max(hp.acc, hp.nlev));
      MtQueueMember m{s.plan.p, s.row_ptr.p, s.row_len.p, s.pclass.p, s.ev_frame.p, s.ev_val.p,
                      s.G2.p, s.IP.p, s.IF.p, s.wlist.p, s.llist.p, s.stats.p, groups,
                      (s.P + 31) / 32};
      groups += m.groups;
      tab.push_back(m);
    }
    q.cap_count[c] = (int32_t)tab.size() - q.cap_first[c];
    q.cap_groups[c] = groups;
  }
  q.tab.reserve(std::max<size_t>(tab.size(), 1), st);
  if (!tab.empty())
    XG_CUDA(cudaMemcpyAsync(q.tab.p, tab.data(), sizeof(MtQueueMember) * tab.size(),
                            cudaMemcpyHostToDevice, st));
  q.next.reserve(MT_THREAD_NCAPS + 3, st);
  XG_CUDA(cudaStreamSynchronize(st));
}

void mt_queue_run(const std::vector<Series *> &ss, MtQueue &q, cudaStream_t st) {
  const int32_t n = q.cap_first.empty() ? 0 : q.cap_first.back() + q.cap_count.back();
  if (n == 0) return;
  int dev = 0, sms = 0;
  XG_CUDA(cudaGetDevice(&dev));
  XG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  XG_CUDA(cudaMemsetAsync(q.next.p, 0, sizeof(int32_t) * (MT_THREAD_NCAPS + 3), st));
  using QueueKernel = void (*)(const MtQueueMember *, int32_t, int32_t, int32_t, int32_t *);
  const QueueKernel kq[MT_THREAD_NCAPS] = {k_mt_thread_queue<32>, k_mt_thread_queue<48>,
                                           k_mt_thread_queue<64>, k_mt_thread_queue<80>,
                                           k_mt_thread_queue<112>};
  for (int c = 0; c < MT_THREAD_NCAPS; c++) {
    if (!q.cap_count[c]) continue;
    const size_t smt = thread_smem(q.scr_max, MT_THREAD_CAPS[c]);
    if (smt > 227 * 1024)
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "delay schedule too large for the multi-tau kernels");
    XG_CUDA(cudaFuncSetAttribute(kq[c], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smt));
    int per_sm = 0;
    XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kq[c], MT_WARPS * 32, smt));
    const int blocks = std::min(sms * std::max(1, per_sm), (q.cap_groups[c] + MT_WARPS - 1) /
                                                               MT_WARPS);
    kq[c]<<<std::max(1, blocks), MT_WARPS * 32, smt, st>>>(q.tab.p + q.cap_first[c],
                                                           q.cap_count[c], q.cap_groups[c],
                                                           q.scr_max, q.next.p + c);
    XG_CHECK_LAUNCH();
  }
  // the warp-per-pixel tiers over every member: rows of 81-256, 257-1024 and
  // 1025-4096 events (the thread kernels above wrote zeros for those pixels)
  const int tiers[3][4] = {{0, 0, MT_WARP_CAP, WP_WARPS},
                           {1, MT_WARP_CAP, MT_MID_CAP, MID_WARPS},
                           {1, MT_MID_CAP, MT_LONG_CAP, LONG_WARPS}};
  const size_t pref_bytes = mc_align16(sizeof(int32_t) * (size_t)(n + 1));
  for (int t = 0; t < 3; t++) {
    const int cap = tiers[t][2], warps = tiers[t][3];
    const size_t sm = pref_bytes + (size_t)warps * (2 * cap + 32 * q.acc_max) * sizeof(int32_t);
    if (sm > 227 * 1024)
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "delay schedule too large for the multi-tau kernels");
    XG_CUDA(cudaFuncSetAttribute(k_mt_warp_queue, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm));
    int per_sm = 0;
    XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mt_warp_queue, warps * 32,
                                                          sm));
    k_mt_warp_queue<<<sms * std::max(1, per_sm), warps * 32, sm, st>>>(
        q.tab.p, n, tiers[t][0], tiers[t][1], cap, q.acc_max, q.next.p + MT_THREAD_NCAPS + t);
    XG_CHECK_LAUNCH();
  }
  for (Series *sp : ss) {  // float rows, member by member (none in integer data)
    Series &s = *sp;
    if (s.D == 0 || s.P == 0) continue;
    const McPlan hp = *(const McPlan *)make_plan(s, s.plan_mode).data();
    launch_float_rows(s, hp, st, sms);
  }
}

}  // namespace xg
