// K-c: per-pixel multi-tau G2 / IP / IF.
//
// Replaces Corr::multiTau2 (src/xpcs/corr.cpp:315-431).  For every pixel with
// events and every delay (level L, tau):
//   on a level change, lastframe halves (odd -> -1 first) and the row is
//   compacted in place: index/2, equal neighbours merged by addition, indices
//   >= lastframe dropped, every live value halved (:349-390);
//   IP  = sum of v over events with t < lastframe - tau,
//   G2  = sum of v(t) * v(t + tau) with the partner found by std::lower_bound
//         over the row buffer (:406),
//   IF  = sum of v over events with tau <= t < lastframe,
//   each divided by (lastframe - tau) (:420-424).
//
// Integer path (pixels whose values are integers with sum |v| < 4096): one
// warp per pixel keeps the row in shared memory as integer numerators
// (value at level L = N / 2^L).  Every float partial sum of the reference is
// then exact, so integer sums scaled by 2^-L (2^-2L for G2) and one IEEE
// division reproduce the reference bit for bit.  IP and IF come from a prefix
// sum and two binary searches per delay; G2 from an event-parallel scan of
// the pairs within the level's delay window.  In REFERENCE mode a pair counts
// only if lower_bound over the whole row buffer (live prefix + the stale tail
// the in-place compaction leaves behind) lands on the partner, exactly as in
// the reference; when the buffer is globally sorted that always holds.
// Results are staged per 32-pixel tile in shared memory and written as
// coalesced 128-byte rows of the [D][P] outputs.
//
// Float path (all other pixels): one thread per pixel replays the reference's
// float operations in the reference's order (no fused multiply-add), on a
// scratch copy of its row.
#include <algorithm>
#include <climits>
#include <cmath>

#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int MC_WARPS = 8;
constexpr int MC_THREADS = MC_WARPS * 32;
constexpr int MC_TILE = 32;
constexpr int MC_ACC = 64;  // max delays per level on the integer path (2*dpl <= 64)
constexpr int MC_CAP = 256; // max events per pixel on the integer path

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }
__host__ __device__ inline size_t plan_bytes(int D) {
  return align16(sizeof(McPlan) + (size_t)D * sizeof(int32_t) + (size_t)D * sizeof(float));
}
__host__ __device__ inline size_t warp_bytes(int cap) { return (size_t)(3 * cap + MC_ACC) * sizeof(int32_t); }
inline size_t int_smem_bytes(int D, int cap) {
  return plan_bytes(D) + MC_WARPS * warp_bytes(cap) + (size_t)3 * D * MC_TILE * sizeof(float);
}

// std::lower_bound as libstdc++ implements it (halving the remaining length).
__device__ __forceinline__ int lower_bound_i32(const int32_t *a, int n, int32_t x) {
  int first = 0, len = n;
  while (len > 0) {
    int half = len >> 1;
    if (a[first + half] < x) {
      first += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return first;
}

__device__ __forceinline__ float pow2_neg(int e) { return __int_as_float((127 - e) << 23); }

// In-place compaction of the live prefix t[0..m), v[0..m) (warp-cooperative).
// Returns the new live length; entries at and beyond it are left untouched.
__device__ int compact_warp(int32_t *t, int32_t *v, int m, int lastframe, int lane) {
  const unsigned FULL = 0xffffffffu, lt = (1u << lane) - 1u;
  int gbase = 0;
  int prev = INT_MIN;  // halved index of the element before the current chunk
  for (int c0 = 0; c0 < m; c0 += 32) {
    int i = c0 + lane;
    bool in = i < m;
    int ti = in ? (t[i] >> 1) : INT_MAX;
    int vi = in ? v[i] : 0;
    bool pair = (i + 1 < m) && ((t[i + 1] >> 1) == ti);
    int vn = pair ? v[i + 1] : 0;
    int tp = __shfl_up_sync(FULL, ti, 1);
    if (lane == 0) tp = prev;
    bool head = in && ti != tp && ti < lastframe;
    unsigned hm = __ballot_sync(FULL, head);
    prev = __shfl_sync(FULL, ti, 31);
    __syncwarp();
    if (head) {
      int g = gbase + __popc(hm & lt);
      t[g] = ti;
      v[g] = vi + vn;
    }
    gbase += __popc(hm);
    __syncwarp();
    if (prev >= lastframe) break;
  }
  return gbase;
}

__global__ void __launch_bounds__(MC_THREADS)
k_multitau_int(const uint8_t *__restrict__ plan_g, const int64_t *__restrict__ row_ptr,
               const int32_t *__restrict__ row_len, const uint8_t *__restrict__ pclass,
               const int32_t *__restrict__ ev_frame, const float *__restrict__ ev_val,
               float *__restrict__ G2, float *__restrict__ IP, float *__restrict__ IF) {
  extern __shared__ __align__(16) uint8_t smem[];
  const McPlan *gp = (const McPlan *)plan_g;
  const int D = gp->D, P = gp->P, cap = gp->cap, mode = gp->mode;
  const size_t pb = plan_bytes(D);
  {
    const int32_t *src = (const int32_t *)plan_g;
    int32_t *dst = (int32_t *)smem;
    for (int k = threadIdx.x; k < (int)(pb / 4); k += MC_THREADS) dst[k] = src[k];
  }
  const McPlan *pl = (const McPlan *)smem;
  const int32_t *tau_lvl = (const int32_t *)(smem + sizeof(McPlan));
  const float *denom = (const float *)(tau_lvl + D);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t *t = (int32_t *)(smem + pb + warp * warp_bytes(cap));
  int32_t *v = t + cap;
  int32_t *S = v + cap;
  int32_t *acc = S + cap;
  float *stg = (float *)(smem + pb + MC_WARPS * warp_bytes(cap));
  const int nst = 3 * D * MC_TILE;
  for (int k = threadIdx.x; k < nst; k += MC_THREADS) stg[k] = 0.f;
  __syncthreads();

  const int tile0 = blockIdx.x * MC_TILE;
  const unsigned FULL = 0xffffffffu;
  for (int lp = warp; lp < MC_TILE; lp += MC_WARPS) {
    const int p = tile0 + lp;
    if (p >= P || pclass[p] != PCLASS_INT) continue;
    const int64_t b = row_ptr[p];
    const int n0 = row_len[p];
    for (int i = lane; i < n0; i += 32) {
      t[i] = ev_frame[b + i];
      v[i] = __float2int_rn(ev_val[b + i]);
    }
    __syncwarp();
    int m = n0;
    for (int gi = 0; gi < pl->nlev; gi++) {
      const McLevel L = pl->lv[gi];
      const int lastframe = L.lastframe;
      if (L.compact) m = compact_warp(t, v, m, lastframe, lane);
      if (m == 0) break;  // nothing live: every remaining output stays 0
      bool sorted = true;
      if (mode == XPCS_MODE_REFERENCE) {
        bool ok = true;
        for (int i = lane; i + 1 < n0; i += 32) ok &= t[i] <= t[i + 1];
        sorted = __all_sync(FULL, ok);
      }
      // inclusive prefix sums of the live values
      int carry = 0;
      for (int c0 = 0; c0 < m; c0 += 32) {
        int i = c0 + lane;
        int x = i < m ? v[i] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(FULL, x, o);
          if (lane >= o) x += y;
        }
        if (i < m) S[i] = x + carry;
        carry += __shfl_sync(FULL, x, 31);
      }
      for (int k = lane; k < L.count; k += 32) acc[k] = 0;
      __syncwarp();
      const int tlo = L.tau_lo, thi = L.tau_lo + L.count - 1;
      for (int i = lane; i < m; i += 32) {
        const int ti = t[i], vi = v[i];
        for (int j = i + 1; j < m; j++) {
          const int tj = t[j];
          const int d = tj - ti;
          if (d > thi) break;
          if (d >= tlo) {
            if (!sorted && lower_bound_i32(t, n0, tj) != j) continue;
            atomicAdd(&acc[d - tlo], vi * v[j]);
          }
        }
      }
      __syncwarp();
      const float s1 = pow2_neg(L.level), s2 = pow2_neg(2 * L.level);
      const int total = S[m - 1];
      for (int k = lane; k < L.count; k += 32) {
        const int tau = tlo + k;
        const int cip = lower_bound_i32(t, m, lastframe - tau);
        const int cif = lower_bound_i32(t, m, tau);
        const int ip = cip ? S[cip - 1] : 0;
        const int iff = total - (cif ? S[cif - 1] : 0);
        float fg = __fmul_rn((float)acc[k], s2);
        float fi = __fmul_rn((float)ip, s1);
        float ff = __fmul_rn((float)iff, s1);
        const float den = denom[L.first + k];
        if (den > 0.f) {
          fg = __fdiv_rn(fg, den);
          fi = __fdiv_rn(fi, den);
          ff = __fdiv_rn(ff, den);
        }
        const int o = (L.first + k) * MC_TILE + lp;
        stg[o] = fg;
        stg[D * MC_TILE + o] = fi;
        stg[2 * D * MC_TILE + o] = ff;
      }
      __syncwarp();
    }
    __syncwarp();
  }
  __syncthreads();
  // coalesced write-out of the tile: rows of 32 consecutive pixels
  for (int k = threadIdx.x; k < nst; k += MC_THREADS) {
    const int a = k / (D * MC_TILE);
    const int rem = k - a * D * MC_TILE;
    const int d = rem / MC_TILE, lp = rem - d * MC_TILE;
    const int p = tile0 + lp;
    if (p < P) {
      float *dst = a == 0 ? G2 : (a == 1 ? IP : IF);
      dst[(size_t)d * P + p] = stg[k];
    }
  }
}

// Order-preserving float replay of Corr::multiTau2 for one pixel per thread.
__global__ void __launch_bounds__(128)
k_multitau_float(const uint8_t *__restrict__ plan_g, const int32_t *__restrict__ flist,
                 const DevStats *__restrict__ stats, const int64_t *__restrict__ row_ptr,
                 const int32_t *__restrict__ row_len, const int32_t *__restrict__ ev_frame,
                 const float *__restrict__ ev_val, int32_t *__restrict__ sc_frame,
                 float *__restrict__ sc_val, float *__restrict__ G2, float *__restrict__ IP,
                 float *__restrict__ IF) {
  const McPlan *pl = (const McPlan *)plan_g;
  const int D = pl->D, P = pl->P, mode = pl->mode;
  const int32_t *tau_lvl = (const int32_t *)(plan_g + sizeof(McPlan));
  const float *denom = (const float *)(tau_lvl + D);
  const int nf = stats->nfloat;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nf; q += gridDim.x * blockDim.x) {
    const int p = flist[q];
    const int64_t b = row_ptr[p];
    const int n0 = row_len[p];
    int32_t *idx = sc_frame + b;
    float *val = sc_val + b;
    for (int i = 0; i < n0; i++) {
      idx[i] = ev_frame[b + i];
      val[i] = ev_val[b + i];
    }
    int lastIndex = n0;
    for (int gi = 0; gi < pl->nlev; gi++) {
      const McLevel L = pl->lv[gi];
      const int lastframe = L.lastframe;
      if (L.compact) {
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
        const int tau = tau_lvl[d];
        float g2 = 0.f, ip = 0.f, iff = 0.f;
        for (int r = 0; r < lastIndex; r++) {
          const int src = idx[r];
          if (src < lastframe - tau) {
            ip = __fadd_rn(ip, val[r]);
            const int pos = lower_bound_i32(idx, sn, src + tau);
            if (pos != sn && pos < lastIndex && idx[pos] == src + tau)
              g2 = __fadd_rn(g2, __fmul_rn(val[r], val[pos]));
          }
          if (src >= tau && src < lastframe) iff = __fadd_rn(iff, val[r]);
        }
        const float den = denom[d];
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
}

}  // namespace

int multitau_cap(int) { return MC_CAP; }

// Host-side plan: level groups of the delay schedule with the lastframe each
// sees and whether the reference compacts before it (corr.cpp:341-391).
static std::vector<uint8_t> make_plan(const Series &s, int mode) {
  const int D = s.D;
  std::vector<uint8_t> buf(plan_bytes(D), 0);
  McPlan *pl = (McPlan *)buf.data();
  int32_t *tau_lvl = (int32_t *)(buf.data() + sizeof(McPlan));
  float *denom = (float *)(tau_lvl + D);
  pl->P = s.P;
  pl->D = D;
  pl->F = s.F;
  pl->mode = mode;
  pl->cap = s.cap;
  int ll = 0, lastframe = s.F, nlev = 0;
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
    denom[k] = (lastframe - tau) > 0 ? (float)(lastframe - tau) : 0.f;
    if (newgroup) {
      if (nlev >= MAX_LEVELS) throw Error(XPCS_ERR_INVALID_ARGUMENT, "too many multi-tau levels");
      McLevel &L = pl->lv[nlev++];
      L.level = level;
      L.first = k;
      L.count = 0;
      L.lastframe = lastframe;
      L.tau_lo = tau;
      L.compact = compact;
    }
    McLevel &L = pl->lv[nlev - 1];
    if (tau != L.tau_lo + L.count)
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "non-consecutive delays within a level");
    L.count++;
    ll = level;
  }
  pl->nlev = nlev;
  return buf;
}

void run_multitau(Series &s, int mode) {
  cudaStream_t st = s.stream;
  const int D = s.D, P = s.P;
  std::vector<uint8_t> plan = make_plan(s, mode);
  int maxcount = 0;
  for (int g = 0; g < ((McPlan *)plan.data())->nlev; g++)
    maxcount = std::max(maxcount, ((McPlan *)plan.data())->lv[g].count);
  s.plan.reserve(plan.size(), st);
  XG_CUDA(cudaMemcpyAsync(s.plan.p, plan.data(), plan.size(), cudaMemcpyHostToDevice, st));
  const size_t nD = (size_t)D * P;
  s.G2.reserve(nD ? nD : 1, st);
  s.IP.reserve(nD ? nD : 1, st);
  s.IF.reserve(nD ? nD : 1, st);
  if (D == 0 || P == 0) return;
  size_t smem = int_smem_bytes(D, s.cap);
  if (smem > 227 * 1024 || maxcount > MC_ACC)
    throw Error(XPCS_ERR_INVALID_ARGUMENT, "delay schedule too large for the multi-tau kernel");
  XG_CUDA(cudaFuncSetAttribute(k_multitau_int, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  XG_CUDA(cudaEventRecord(s.ev[4], st));
  k_multitau_int<<<(P + MC_TILE - 1) / MC_TILE, MC_THREADS, smem, st>>>(
      s.plan.p, s.row_ptr.p, s.row_len.p, s.pclass.p, s.ev_frame.p, s.ev_val.p, s.G2.p, s.IP.p,
      s.IF.p);
  XG_CHECK_LAUNCH();
  XG_CUDA(cudaEventRecord(s.ev[5], st));
  size_t ne = s.raw_events > 0 ? (size_t)s.raw_events : 1;
  s.sc_frame.reserve(ne, st);
  s.sc_val.reserve(ne, st);
  int dev_sms = 0;
  XG_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, s.device));
  int grid = std::max(1, std::min((P + 127) / 128, dev_sms * 8));
  k_multitau_float<<<grid, 128, 0, st>>>(s.plan.p, s.flist.p, s.stats.p, s.row_ptr.p,
                                         s.row_len.p, s.ev_frame.p, s.ev_val.p, s.sc_frame.p,
                                         s.sc_val.p, s.G2.p, s.IP.p, s.IF.p);
  XG_CHECK_LAUNCH();
  XG_CUDA(cudaEventRecord(s.ev[6], st));
}

}  // namespace xg
