// The reference's per-pixel multi-tau loop replayed with its own float
// operations, in its order, on a working copy of one pixel's row.
//
// Corr::multiTau2 (src/xpcs/corr.cpp:340-425): on every level change the row
// is compacted in place (index / 2 truncated toward zero, equal neighbours
// merged by float addition, indices >= lastframe dropped, every live value
// halved), then for each delay of the level
//   IP += v           over r < lastIndex with idx[r] < lastframe - tau,
//   G2 += v * v'      when std::lower_bound over the search range finds
//                     idx[r] + tau inside the live prefix,
//   IF += v           over r < lastIndex with tau <= idx[r] < lastframe,
// each divided by (lastframe - tau).  In REFERENCE mode the search range is
// the whole buffer including the stale tail the compaction leaves behind
// (:406); in EXACT mode it is the live prefix only.  No fused multiply-add:
// every operation is an explicitly rounded one.
//
// Shared by the thread-per-pixel float kernel (k_multitau.cu) and the
// allocation-free entry point (noalloc.cu), so that the two cannot drift.
#pragma once

#include "xpcs_internal.h"

namespace xg {

// std::lower_bound as libstdc++ implements it (halving the remaining length).
__device__ __forceinline__ int replay_lower_bound(const int32_t *a, int n, int32_t x) {
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

// One pixel p of P: idx/val hold its n0 events (frames ascending) and are
// destroyed; G2/IP/IF [D][P] receive every delay of the plan.
__device__ inline void replay_pixel(const McPlan *pl, const McArrays &ar, int P, int p,
                                    int32_t *idx, float *val, int n0, float *G2, float *IP,
                                    float *IF) {
  const int mode = pl->mode;
  int lastIndex = n0;
  for (int gi = 0; gi < pl->nlev; gi++) {
    const McLevel L = pl->lv[gi];
    const int lastframe = L.lastframe;
    if (L.compact && n0 > 0) {
      int index = 0, cnt = 0;
      int i0 = idx[0] / 2, i1;  // (int)(idx / 2.0): truncation toward zero
      if (lastIndex > 0 && i0 < lastframe) {
        idx[index] = i0;
        cnt = 1;
      }
      while (cnt < lastIndex) {
        i1 = idx[cnt] / 2;
        if (i1 >= lastframe) break;
        if (i1 == i0) {
          val[index] = __fadd_rn(val[index], val[cnt]);
        } else {
          idx[++index] = i1;
          val[index] = val[cnt];
        }
        i0 = i1;
        cnt++;
      }
      lastIndex = index + 1;
      for (int r = 0; r < lastIndex; r++) val[r] = __fdiv_rn(val[r], 2.0f);
    }
    const int sn = mode == XPCS_MODE_REFERENCE ? n0 : lastIndex;
    for (int k = 0; k < L.count; k++) {
      const int d = L.first + k;
      const int tau = ar.tau_lvl[d];
      float g2 = 0.f, ip = 0.f, iff = 0.f;
      for (int r = 0; r < lastIndex; r++) {
        const int src = idx[r];
        if (src < lastframe - tau) {
          ip = __fadd_rn(ip, val[r]);
          const int pos = replay_lower_bound(idx, sn, src + tau);
          if (pos != sn && pos < lastIndex && idx[pos] == src + tau)
            g2 = __fadd_rn(g2, __fmul_rn(val[r], val[pos]));
        }
        if (src >= tau && src < lastframe) iff = __fadd_rn(iff, val[r]);
      }
      const float den = ar.denom[d];
      if (den > 0.f) {
        g2 = __fdiv_rn(g2, den);
        ip = __fdiv_rn(ip, den);
        iff = __fdiv_rn(iff, den);
      }
      G2[(size_t)d * P + p] = g2;
      IP[(size_t)d * P + p] = ip;
      IF[(size_t)d * P + p] = iff;
    }
  }
}

}  // namespace xg
