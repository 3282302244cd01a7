// F3 EXACT mode: the two-time Gram products of the integer photon counts on
// the 5th-generation tensor cores, then the reference's smoothing applied in
// float64.
//
// For every smoothing group g (a static bin with the static-map method, a q
// bin with the symmetric one) the raw counts X_g [pixels][F] give
//   G_g(t1, t2) = sum_p X_g[p][t1] X_g[p][t2]          (exact integers)
//   S_g(t)      = sum_p X_g[p][t]                      (exact integers)
// and, since every value of g is divided by sg_g(t) = S_g(t) / pixels_g (or
// its mean over frames with the average filter) before the products,
//   C_q(t1, t2) = sum_{g in q} G_g(t1, t2) / (sg_g(t1) sg_g(t2)) / pixels_q.
// G_g runs as fp16 x fp16 -> fp32 tcgen05 MMAs (kind::f16): counts up to
// 2048 are exact in fp16, and when sum_p max_t X_g[p][t]^2 < 2^24 every
// partial sum is an integer below 2^24, exact in fp32.  A group outside that
// range takes an int64 CUDA-core Gram instead.  Operands are loaded by TMA
// (128-byte swizzle, 128 x 64 and 256 x 64 fp16 tiles, 4 stages), one thread
// issues M=128, N=256 MMAs into a 128 x 256 fp32 accumulator in tensor
// memory, and four warps read it back with tcgen05.ld.  Only tiles that meet
// the upper triangle are computed.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int TC_BM = 128;  // tile rows (frames t1), = tensor-memory lanes
constexpr int TC_BN = 256;  // tile columns (frames t2), = tensor-memory columns
constexpr int TC_BK = 64;   // pixels per stage: 64 fp16 = one 128-byte swizzle row
constexpr int TC_STAGES = 4;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;  // 16 KB
constexpr int TC_B_BYTES = TC_BN * TC_BK * 2;  // 32 KB
constexpr uint32_t TC_WAIT_LIMIT = 1u << 20;      // bounded mbarrier waits

struct TcSmem {
  uint8_t a[TC_STAGES][TC_A_BYTES];
  uint8_t b[TC_STAGES][TC_B_BYTES];
  uint64_t full[TC_STAGES], empty[TC_STAGES], done;
  uint32_t tmem;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}

// Waits for the phase with the given parity; false after TC_WAIT_LIMIT polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity) {
  const uint32_t a = smem_u32(b);
  for (uint32_t it = 0; it < TC_WAIT_LIMIT; it++) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)tm), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand in the 128-byte swizzle
// layout (rows of 128 bytes, 8-row groups 1024 bytes apart).
__device__ __forceinline__ uint64_t smem_desc_sw128(const void *p) {
  const uint32_t a = smem_u32(p);
  uint64_t d = (uint64_t)((a & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                          // leading byte offset (unused here)
  d |= (uint64_t)(1024 >> 4) << 32;                // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                          // descriptor version
  d |= (uint64_t)2 << 61;                          // swizzle: 128 bytes
  return d;
}

// Instruction descriptor of kind::f16: A, B fp16, D fp32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_f16_f32(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// One CTA (4 warps) per 128 x 256 tile of G = X^T X that meets the upper
// triangle, X^T given as an fp16 tensor [Fp][Kp] (K-major, Fp a multiple of
// 256), read through two tensor maps (128- and 256-row boxes).  Thread 0 loads
// by TMA, thread 32 issues the MMAs, all four warps read the accumulator back.
// G: [Fp][Fp]; tile row bi covers frames [128 bi, 128 bi + 128), tile column
// bj frames [256 bj, 256 bj + 256), bj >= bi / 2.
__global__ void __launch_bounds__(128)
k_gram_tc(const __grid_constant__ CUtensorMap tma, const __grid_constant__ CUtensorMap tmb,
          int32_t nkt, int32_t nrow, int32_t ncol, float *__restrict__ G, int64_t ldg,
          int32_t *__restrict__ err) {
  extern __shared__ uint8_t tc_raw[];
  TcSmem &sm = *reinterpret_cast<TcSmem *>(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int id = blockIdx.x, bi = 0;
  while (bi < nrow && id >= ncol - bi / 2) {
    id -= ncol - bi / 2;
    bi++;
  }
  const int bj = bi / 2 + id;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; s++) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    mbar_init(&sm.done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&sm.tmem)),
                 "r"(TC_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = sm.tmem;
  bool ok = true;
  if (threadIdx.x == 0) {  // TMA producer
    for (int kt = 0; kt < nkt && ok; kt++) {
      const int s = kt % TC_STAGES;
      if (kt >= TC_STAGES) ok = mbar_wait(&sm.empty[s], ((kt / TC_STAGES) - 1) & 1);
      if (!ok) break;
      mbar_expect_tx(&sm.full[s], TC_A_BYTES + TC_B_BYTES);
      tma_load_2d(sm.a[s], &tma, kt * TC_BK, bi * TC_BM, &sm.full[s]);
      tma_load_2d(sm.b[s], &tmb, kt * TC_BK, bj * TC_BN, &sm.full[s]);
    }
    if (!ok) atomicOr(err, 8);
  } else if (threadIdx.x == 32) {  // MMA issuer
    constexpr uint32_t idesc = idesc_f16_f32(TC_BM, TC_BN);
    for (int kt = 0; kt < nkt && ok; kt++) {
      const int s = kt % TC_STAGES;
      ok = mbar_wait(&sm.full[s], (kt / TC_STAGES) & 1);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t ad = smem_desc_sw128(sm.a[s]), bd = smem_desc_sw128(sm.b[s]);
#pragma unroll
      for (int k = 0; k < TC_BK / 16; k++)  // 16 fp16 per MMA = 32 bytes along the row
        umma_f16(tmem, ad + (uint64_t)(2 * k), bd + (uint64_t)(2 * k), idesc,
                 (kt > 0 || k > 0) ? 1u : 0u);
      umma_commit(&sm.empty[s]);
    }
    umma_commit(&sm.done);  // arrives when every MMA issued above has completed
    if (!ok) atomicOr(err, 16);
  }
  __syncwarp();
  const bool done = __all_sync(0xffffffffu, mbar_wait(&sm.done, 0));
  if (!done && lane == 0) atomicOr(err, 32);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (done) {
    const int row = bi * TC_BM + warp * 32 + lane;
    float *out = G + (size_t)row * ldg + (size_t)bj * TC_BN;
    for (int c = 0; c < TC_BN; c += 16) {
      uint32_t r[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, r);
#pragma unroll
      for (int j = 0; j < 16; j++) out[c + j] = __uint_as_float(r[j]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_BN));
}

// ---------------------------------------------------- integer group data

// rows of one group -> X^T [Fp][Kp] fp16 (counts), per-frame sums, row maxima
__global__ void k_xt_build(int32_t nrows, int32_t F, int64_t kp, int32_t r0,
                           const int32_t *__restrict__ row_pix, const int64_t *__restrict__ row_ptr,
                           const int32_t *__restrict__ row_len,
                           const int32_t *__restrict__ ev_frame, const float *__restrict__ ev_val,
                           __half *__restrict__ XT, long long *__restrict__ S,
                           unsigned long long *__restrict__ sq_bound,
                           int32_t *__restrict__ flags) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nrows) return;
  const int p = row_pix[r0 + k];
  const int64_t b = row_ptr[p];
  const int n = row_len[p];
  long long mx = 0;
  for (int i = 0; i < n; i++) {
    const int f = ev_frame[b + i];
    const float v = ev_val[b + i];
    if (f < 0 || f >= F) continue;
    if (v != truncf(v) || fabsf(v) > 65536.f) {
      atomicOr(flags, 1);  // not an integer count
      continue;
    }
    const long long c = (long long)v;
    if (c > 2048 || c < -2048) atomicOr(flags, 2);  // beyond exact fp16 integers
    XT[(size_t)f * kp + k] = __float2half_rn(v);
    atomicAdd((unsigned long long *)&S[f], (unsigned long long)c);
    mx = max(mx, c < 0 ? -c : c);
  }
  atomicAdd(sq_bound, (unsigned long long)(mx * mx));
}

// int64 CUDA-core Gram of the counts (groups outside the fp16/fp32-exact range)
__global__ void k_gram_i64(int32_t nrows, int32_t F, int32_t r0,
                           const int32_t *__restrict__ row_pix, const int64_t *__restrict__ row_ptr,
                           const int32_t *__restrict__ row_len,
                           const int32_t *__restrict__ ev_frame, const float *__restrict__ ev_val,
                           unsigned long long *__restrict__ Gi, int64_t ldg) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nrows) return;
  const int p = row_pix[r0 + k];
  const int64_t b = row_ptr[p];
  const int n = row_len[p];
  for (int i = 0; i < n; i++)
    for (int j = i; j < n; j++) {
      const int f0 = ev_frame[b + i], f1 = ev_frame[b + j];
      if (f0 < 0 || f1 >= F) continue;
      const long long c = (long long)ev_val[b + i] * (long long)ev_val[b + j];
      atomicAdd(&Gi[(size_t)f0 * ldg + f1], (unsigned long long)c);
    }
}

// The smoothing factors are reciprocals of sg (float64, one per frame, or one
// for the averaged form), so that a matrix element costs multiplications
// only: GB300 runs FP64 at a small fraction of its FP32 rate, and a float64
// division is several times the cost of a multiplication.

// C_acc[t1][t2] += G[t1][t2] * (1/sg[t1]) * (1/sg[t2]) on the upper triangle;
// block row t1 = blockIdx.y, columns t2 from blockIdx.x
template <bool I64>
__global__ void k_tc_accum(int32_t F, const void *__restrict__ Gv, int64_t ldg,
                           const double *__restrict__ isg, int32_t avg,
                           double *__restrict__ Cacc) {
  const int t1 = blockIdx.y, t2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (t2 >= F || t2 < t1) return;
  const double g = I64 ? (double)(long long)((const unsigned long long *)Gv)[(size_t)t1 * ldg + t2]
                       : (double)((const float *)Gv)[(size_t)t1 * ldg + t2];
  if (g == 0.0) return;
  const double a = avg ? isg[0] : isg[t1], b = avg ? isg[0] : isg[t2];
  Cacc[(size_t)t1 * F + t2] += g * a * b;
}

// A q bin of one smoothing group: C_q = G / (sg sg) / pixels in one pass (the
// same double operations as k_tc_accum into a zeroed C_acc and k_tc_final).
// Only the upper triangle of the float64 scratch Cq is read later.
template <bool I64>
__global__ void k_tc_single(int32_t F, const void *__restrict__ Gv, int64_t ldg,
                            const double *__restrict__ isg, int32_t avg, double inv_npix,
                            double *__restrict__ Cq, float *__restrict__ C) {
  const int t1 = blockIdx.y, t2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (t2 >= F) return;
  const size_t i = (size_t)t1 * F + t2;
  if (t2 < t1) {
    C[i] = 0.f;
    return;
  }
  const double g = I64 ? (double)(long long)((const unsigned long long *)Gv)[(size_t)t1 * ldg + t2]
                       : (double)((const float *)Gv)[(size_t)t1 * ldg + t2];
  double v = 0.0;
  if (g != 0.0) {
    const double a = avg ? isg[0] : isg[t1], b = avg ? isg[0] : isg[t2];
    v = (0.0 + g * a * b) * inv_npix;
  }
  Cq[i] = v;
  C[i] = (float)v;
}

__global__ void k_tc_final(int32_t F, double inv_npix, const double *__restrict__ Cacc,
                           double *__restrict__ Cq, float *__restrict__ C) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)F * F) return;
  const double v = Cacc[i] * inv_npix;
  Cq[i] = v;
  C[i] = (float)v;
}

// one block per diagonal ff: g2full = its mean; for ff < window, one thread
// per window w sums g2partials
__global__ void __launch_bounds__(256)
k_tc_diag(int32_t Q, int32_t q, int32_t F, int32_t window, int32_t tp,
          const double *__restrict__ Cq, float *__restrict__ g2full,
          float *__restrict__ g2part) {
  __shared__ double red[256];
  const int ff = blockIdx.x;
  double acc = 0.0;
  for (int fx = threadIdx.x; fx < F - ff; fx += blockDim.x) acc += Cq[(size_t)fx * F + fx + ff];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) g2full[(size_t)ff * Q + q] = (float)(red[0] / (F - ff));
  if (ff < window)
    for (int w = threadIdx.x; w < tp; w += blockDim.x) {
      double sw = 0.0;
      for (int fx = w * window; fx < (w + 1) * window && fx < F - ff; fx++)
        sw += Cq[(size_t)fx * F + fx + ff];
      g2part[((size_t)ff * tp + w) * Q + q] = (float)(sw / window);
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    XG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p)
      throw Error(XPCS_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    fn = (EncodeTiledFn)p;
  }
  return fn;
}

}  // namespace

// Groups and rows as run_twotime builds them; `force_i64` routes every group
// to the CUDA-core Gram (the check of the tensor-core one).
void run_twotime_exact(Series &s, const TwoTimeReq &req, const TwoTimeLayout &lay,
                       bool force_i64) {
  cudaStream_t st = s.stream;
  TwoTimeOut &o = s.tt;
  const int32_t F = s.F, G = (int32_t)lay.grp_ptr.size() - 1, Q = (int32_t)lay.q_ptr.size() - 1;
  if (F > 65535) throw Error(XPCS_ERR_INVALID_ARGUMENT, "EXACT two-time supports up to 65535 frames");
  const int64_t Fp = ((int64_t)F + TC_BN - 1) / TC_BN * TC_BN;
  const int nrow = (int)(Fp / TC_BM), ncol = (int)(Fp / TC_BN);
  int ntiles = 0;
  for (int bi = 0; bi < nrow; bi++) ntiles += ncol - bi / 2;
  s.tt_err.reserve(1, st);
  s.tt_flags.reserve(1, st);
  XG_CUDA(cudaMemsetAsync(s.tt_err.p, 0, sizeof(int32_t), st));
  s.tt_S.reserve((size_t)F + 1, st);
  s.tt_bound.reserve(2, st);
  s.tt_sgd.reserve((size_t)(G ? G : 1) * (F + 1), st);
  s.tt_Cacc.reserve((size_t)F * F + 1, st);
  s.tt_Cq.reserve((size_t)F * F + 1, st);
  std::vector<double> sg_host((size_t)G * (req.average ? 1 : F));
  const size_t smem = sizeof(TcSmem) + 1024;
  XG_CUDA(cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int32_t gq = 0;  // group index across q bins
  std::vector<cudaEvent_t> gram_ev;  // start/stop of every tensor-core Gram
  struct EvList {
    std::vector<cudaEvent_t> &v;
    ~EvList() {
      for (cudaEvent_t e : v) cudaEventDestroy(e);
    }
  } evl{gram_ev};
  for (int32_t q = 0; q < Q; q++) {
    const int32_t g_end = req.static_map ? lay.q_grp_end[q] : q + 1;
    const bool single = g_end - gq == 1;  // C_q straight from the one Gram
    const int32_t npix = lay.q_ptr[q + 1] - lay.q_ptr[q];
    const double inv_npix = npix ? 1.0 / npix : 0.0;
    float *Cout = s.tt_C.p + (size_t)q * F * F;
    if (!single) XG_CUDA(cudaMemsetAsync(s.tt_Cacc.p, 0, sizeof(double) * (size_t)F * F, st));
    for (; gq < g_end; gq++) {
      const int32_t r0 = lay.grp_ptr[gq], nr = lay.grp_ptr[gq + 1] - r0;
      const int64_t Kp = std::max<int64_t>(TC_BK, ((int64_t)nr + TC_BK - 1) / TC_BK * TC_BK);
      s.tt_XT.reserve((size_t)(Fp * Kp), st);
      XG_CUDA(cudaMemsetAsync(s.tt_XT.p, 0, sizeof(__half) * (size_t)(Fp * Kp), st));
      XG_CUDA(cudaMemsetAsync(s.tt_S.p, 0, sizeof(long long) * ((size_t)F + 1), st));
      XG_CUDA(cudaMemsetAsync(s.tt_bound.p, 0, sizeof(unsigned long long) * 2, st));
      XG_CUDA(cudaMemsetAsync(s.tt_flags.p, 0, sizeof(int32_t), st));
      k_xt_build<<<(nr + 127) / 128, 128, 0, st>>>(
          nr, F, Kp, r0, s.tt_row_pix.p, s.row_ptr.p, s.row_len.p, s.ev_frame.p, s.ev_val.p,
          (__half *)s.tt_XT.p, (long long *)s.tt_S.p, (unsigned long long *)s.tt_bound.p,
          s.tt_flags.p);
      XG_CHECK_LAUNCH();
      // per-frame sums and the exactness bound back on the host: sg in float64
      std::vector<long long> Sh((size_t)F);
      unsigned long long bound = 0;
      int32_t flags = 0;
      XG_CUDA(cudaMemcpyAsync(Sh.data(), s.tt_S.p, sizeof(long long) * F, cudaMemcpyDeviceToHost, st));
      XG_CUDA(cudaMemcpyAsync(&bound, s.tt_bound.p, sizeof(bound), cudaMemcpyDeviceToHost, st));
      XG_CUDA(cudaMemcpyAsync(&flags, s.tt_flags.p, sizeof(flags), cudaMemcpyDeviceToHost, st));
      XG_CUDA(cudaStreamSynchronize(st));
      if (flags & 1)
        throw Error(XPCS_ERR_INPUT, "EXACT two-time needs integer counts (no flatfield, dense "
                                    "or averaged frames)");
      double *sgd = sg_host.data() + (size_t)gq * (req.average ? 1 : F);
      double mean = 0.0;
      for (int32_t f = 0; f < F; f++) {
        const double v = (double)Sh[f] / nr;
        if (req.average)
          mean += v;
        else
          sgd[f] = v;
      }
      if (req.average) sgd[0] = mean / F;
      // every group has its own device copy of 1/sg, so no group waits for
      // the previous one's kernels
      const size_t nsg = req.average ? 1 : (size_t)F;
      std::vector<double> isg(nsg);
      for (size_t f = 0; f < nsg; f++) isg[f] = 1.0 / sgd[f];
      double *sgdev = s.tt_sgd.p + (size_t)gq * (F + 1);
      XG_CUDA(cudaMemcpyAsync(sgdev, isg.data(), sizeof(double) * nsg, cudaMemcpyHostToDevice,
                              st));
      const bool tensor = !force_i64 && !(flags & 2) && bound < (1ull << 24);
      const size_t nF2 = (size_t)F * F;
      if (tensor) {
        s.tt_Gf.reserve((size_t)(Fp * Fp), st);
        CUtensorMap tma, tmb;
        const cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)Fp};
        const cuuint64_t strides[1] = {(cuuint64_t)(Kp * 2)};
        const cuuint32_t boxa[2] = {TC_BK, TC_BM}, boxb[2] = {TC_BK, TC_BN};
        const cuuint32_t es[2] = {1, 1};
        for (int w = 0; w < 2; w++) {
          const CUresult cr = encode_fn()(w ? &tmb : &tma, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                                          s.tt_XT.p, dims, strides, w ? boxb : boxa, es,
                                          CU_TENSOR_MAP_INTERLEAVE_NONE,
                                          CU_TENSOR_MAP_SWIZZLE_128B,
                                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
          if (cr != CUDA_SUCCESS) throw Error(XPCS_ERR_CUDA, "tensor map encoding failed");
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        XG_CUDA(cudaEventCreate(&e0));
        gram_ev.push_back(e0);
        XG_CUDA(cudaEventCreate(&e1));
        gram_ev.push_back(e1);
        XG_CUDA(cudaEventRecord(e0, st));
        k_gram_tc<<<ntiles, 128, smem, st>>>(tma, tmb, (int32_t)(Kp / TC_BK), nrow, ncol,
                                             s.tt_Gf.p, Fp, s.tt_err.p);
        XG_CHECK_LAUNCH();
        XG_CUDA(cudaEventRecord(e1, st));
        o.gram_flop += (double)ntiles * 2.0 * TC_BM * TC_BN * (double)Kp;
        // the Gram's own work: the F(F+1)/2 upper-triangle cells (diagonal
        // included) over the group's nr rows, without tile and K padding
        o.gram_flop_alg += 2.0 * (double)nr * ((double)F * (F + 1) / 2.0);
        if (single)
          k_tc_single<false><<<dim3((F + 255) / 256, F), 256, 0, st>>>(
              F, s.tt_Gf.p, Fp, sgdev, req.average, inv_npix, s.tt_Cq.p, Cout);
        else
          k_tc_accum<false><<<dim3((F + 255) / 256, F), 256, 0, st>>>(
              F, s.tt_Gf.p, Fp, sgdev, req.average, s.tt_Cacc.p);
        XG_CHECK_LAUNCH();
      } else {
        s.tt_Gi.reserve(nF2 + 1, st);
        XG_CUDA(cudaMemsetAsync(s.tt_Gi.p, 0, sizeof(unsigned long long) * nF2, st));
        k_gram_i64<<<(nr + 127) / 128, 128, 0, st>>>(nr, F, r0, s.tt_row_pix.p,
                                                    s.row_ptr.p, s.row_len.p, s.ev_frame.p,
                                                    s.ev_val.p, s.tt_Gi.p, F);
        XG_CHECK_LAUNCH();
        if (single)
          k_tc_single<true><<<dim3((F + 255) / 256, F), 256, 0, st>>>(
              F, s.tt_Gi.p, F, sgdev, req.average, inv_npix, s.tt_Cq.p, Cout);
        else
          k_tc_accum<true><<<dim3((F + 255) / 256, F), 256, 0, st>>>(
              F, s.tt_Gi.p, F, sgdev, req.average, s.tt_Cacc.p);
        XG_CHECK_LAUNCH();
      }
    }
    if (!single) {
      k_tc_final<<<(unsigned)(((size_t)F * F + 255) / 256), 256, 0, st>>>(
          F, inv_npix, s.tt_Cacc.p, s.tt_Cq.p, Cout);
      XG_CHECK_LAUNCH();
    }
    k_tc_diag<<<F, 256, 0, st>>>(Q, q, F, req.window, o.partials, s.tt_Cq.p, s.tt_full.p,
                                 s.tt_part.p);
    XG_CHECK_LAUNCH();
  }
  // sg as float, [G][F] or [G][1]
  std::vector<float> sgf(sg_host.size());
  for (size_t i = 0; i < sgf.size(); i++) sgf[i] = (float)sg_host[i];
  float *dst = req.average ? s.tt_sga.p : s.tt_sg.p;
  if (!sgf.empty())
    XG_CUDA(cudaMemcpyAsync(dst, sgf.data(), 4 * sgf.size(), cudaMemcpyHostToDevice, st));
  int32_t err = 0;
  XG_CUDA(cudaMemcpyAsync(&err, s.tt_err.p, sizeof(err), cudaMemcpyDeviceToHost, st));
  XG_CUDA(cudaStreamSynchronize(st));
  for (size_t k = 0; k + 1 < gram_ev.size(); k += 2) {
    float ms = 0.f;
    XG_CUDA(cudaEventElapsedTime(&ms, gram_ev[k], gram_ev[k + 1]));
    o.gram_ms += ms;
  }
  if (err)  // a bounded wait of the tensor-core Gram expired
    throw Error(XPCS_ERR_CUDA, "tensor-core two-time: a pipeline wait timed out");
}

}  // namespace xg
