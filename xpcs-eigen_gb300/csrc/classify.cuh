// Pixel classification shared by the filters' finishing passes: the pixel
// class of every row and the work lists of the multi-tau kernels.
#pragma once

#include "xpcs_internal.h"

namespace xg {

// Work lists of the multi-tau kernels (pixel indices per class).
struct ClassLists {
  int32_t *wlist, *llist, *flist;
};

// Classification of the pixels of one warp (all 32 lanes call it; lanes
// without a pixel pass has = false): pclass, the float/warp work lists and the
// counters, one atomic per warp and counter.
__device__ __forceinline__ void record_class_warp(bool has, int32_t p, uint8_t c, int32_t n,
                                                  uint8_t *pclass, const ClassLists &cl,
                                                  DevStats *stats) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  if (has) pclass[p] = c;
  const bool live = has && c != PCLASS_EMPTY;
  const unsigned mv = __ballot_sync(FULL, live);
  const unsigned mw = __ballot_sync(FULL, live && c == PCLASS_WARP);
  const unsigned ml = __ballot_sync(FULL, live && c == PCLASS_LONG);
  const unsigned mf = __ballot_sync(FULL, live && c == PCLASS_FLOAT);
  const unsigned ev = __reduce_add_sync(FULL, live ? (unsigned)n : 0u);
  int bw = 0, bl = 0, bf = 0;
  if (lane == 0) {
    if (mv) {
      atomicAdd(&stats->nvalid, __popc(mv));
      atomicAdd(&stats->events, (unsigned long long)ev);
    }
    if (mw) bw = atomicAdd(&stats->nwarp, __popc(mw));
    if (ml) bl = atomicAdd(&stats->nlong, __popc(ml));
    if (mf) bf = atomicAdd(&stats->nfloat, __popc(mf));
  }
  bw = __shfl_sync(FULL, bw, 0);
  bl = __shfl_sync(FULL, bl, 0);
  bf = __shfl_sync(FULL, bf, 0);
  if (live && c == PCLASS_WARP) cl.wlist[bw + __popc(mw & lt)] = p;
  if (live && c == PCLASS_LONG) cl.llist[bl + __popc(ml & lt)] = p;
  if (live && c == PCLASS_FLOAT) cl.flist[bf + __popc(mf & lt)] = p;
}

}  // namespace xg
