// Allocation-free multi-tau entry point (xpcs_multitau2_noalloc).
//
// Some callers cannot allocate device memory: code running inside another
// framework's memory pool, a process whose GPU memory budget is fixed up
// front, or a real-time acquisition loop that must never call cudaMalloc or
// cudaFree (they synchronise the device).  This entry point computes the same
// G2/IP/IF as Corr::multiTau2 (src/xpcs/corr.cpp:315-431) on rows the caller
// already holds in device memory, writing into device outputs the caller also
// provides, and uses no allocation of its own: its scratch (the plan, the
// working copy of the rows that the in-place level compaction destroys, and a
// status word) is one file-scope __device__ array of fixed size.
//
// Every pixel is replayed with the reference's own float operations in its
// order (the order-preserving path of k_multitau.cu), so the result is
// bit-identical to xpcs_multitau2 for any input rows.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "mt_replay.cuh"
#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr size_t NA_PLAN_BYTES = 16384;
static_assert(sizeof(McPlan) + (size_t)XPCS_NOALLOC_MAX_DELAYS * 6 * sizeof(int32_t) <=
                  NA_PLAN_BYTES,
              "the plan of the largest accepted delay schedule fits its scratch slot");
constexpr size_t NA_STATUS_BYTES = 256;
constexpr int64_t NA_MAX_EVENTS = XPCS_NOALLOC_MAX_EVENTS;
constexpr size_t NA_SCRATCH_BYTES =
    NA_PLAN_BYTES + NA_STATUS_BYTES + (size_t)NA_MAX_EVENTS * (sizeof(int32_t) + sizeof(float));

// The scratch.  Held by every GPU that loads this library until the process
// exits.  Its name is only a host-side handle: kernels get the device address
// obtained with cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
unsigned char *g_na_ptr[NA_MAX_DEVICES] = {};

struct NaView {
  const uint8_t *plan;
  int32_t *status;
  int32_t *frame;
  float *value;
};

__host__ __device__ inline NaView na_view(unsigned char *base) {
  return NaView{base, (int32_t *)(base + NA_PLAN_BYTES),
                (int32_t *)(base + NA_PLAN_BYTES + NA_STATUS_BYTES),
                (float *)(base + NA_PLAN_BYTES + NA_STATUS_BYTES +
                          (size_t)NA_MAX_EVENTS * sizeof(int32_t))};
}

__global__ void __launch_bounds__(128)
k_mt_float_noalloc(unsigned char *scratch, const int64_t *__restrict__ row_ptr,
                   const int32_t *__restrict__ frame, const float *__restrict__ value,
                   int32_t P, int64_t events, float *__restrict__ G2, float *__restrict__ IP,
                   float *__restrict__ IF) {
  const NaView v = na_view(scratch);
  const McPlan *pl = (const McPlan *)v.plan;
  const int D = pl->D;
  const McArrays ar = mc_arrays(v.plan, D);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int64_t b = row_ptr[p];
    const int64_t n64 = row_ptr[p + 1] - b;
    if (b < 0 || n64 < 0 || b + n64 > events) {
      atomicOr(v.status, 1);
      for (int d = 0; d < D; d++) {
        G2[(size_t)d * P + p] = 0.f;
        IP[(size_t)d * P + p] = 0.f;
        IF[(size_t)d * P + p] = 0.f;
      }
      continue;
    }
    const int n0 = (int)n64;
    int32_t *idx = v.frame + b;
    float *val = v.value + b;
    for (int i = 0; i < n0; i++) {
      idx[i] = frame[b + i];
      val[i] = value[b + i];
    }
    replay_pixel(pl, ar, P, p, idx, val, n0, G2, IP, IF);
  }
}

// Delay schedule and level plan (the same rules as delay_schedule / the
// multi-tau plan) written into a caller buffer, without heap use.
// Returns D, or -1 if the plan does not fit.
int na_build_plan(int32_t P, int32_t F, int32_t dpl, int32_t mode, uint8_t *buf, size_t cap) {
  std::memset(buf, 0, cap);
  McPlan *pl = (McPlan *)buf;
  const size_t head = sizeof(McPlan);
  // count the delays first
  int max_level = 0;
  if (F >= dpl * 2 && dpl > 0)
    max_level = (int)(std::floor(std::log2((double)F) - std::log2(1.0 + 1.0 / (double)dpl)) -
                      std::log2((double)dpl));
  int D = 0;
  {
    long long ll = 0;
    for (int i = 0; i <= max_level && i < 62 && dpl > 0 && F > 0; i++) {
      long long step = 1ll << i;
      int per = i == 0 ? 2 * dpl : dpl;
      for (int j = 0; j < per; j++) {
        if (ll + step + step > F) break;
        ll += step;
        D++;
      }
    }
  }
  if (D > XPCS_NOALLOC_MAX_DELAYS || head + (size_t)D * 6 * sizeof(int32_t) > cap) return -1;
  int32_t *base = (int32_t *)(buf + head);
  int32_t *tau_lvl = base;
  float *denom = (float *)(base + D);
  int32_t *tau_abs = base + 2 * D, *t_ip = base + 3 * D, *gi = base + 4 * D;
  pl->P = P;
  pl->D = D;
  pl->F = F;
  pl->mode = mode;
  int k = 0, ll_level = 0, lastframe = F, nlev = 0, prev_level = -1;
  long long ll = 0;
  for (int i = 0; i <= max_level && i < 62 && dpl > 0 && F > 0; i++) {
    long long step = 1ll << i;
    int per = i == 0 ? 2 * dpl : dpl;
    for (int j = 0; j < per; j++) {
      if (ll + step + step > F) break;
      ll += step;
      const int level = i, tau_frames = (int)ll;
      int compact = 0;
      if (ll_level != level) {
        if (lastframe % 2) lastframe -= 1;
        lastframe = lastframe / 2;
        compact = 1;
      }
      const int tau = level > 0 ? (int)(tau_frames / std::pow(2.0, level)) : tau_frames;
      tau_lvl[k] = tau;
      tau_abs[k] = tau_frames;
      denom[k] = (lastframe - tau) > 0 ? (float)(lastframe - tau) : 0.f;
      t_ip[k] = (int32_t)std::max<int64_t>(0, (int64_t)(lastframe - tau) << level);
      if (level != prev_level) {
        if (nlev >= MAX_LEVELS) return -1;
        McLevel &L = pl->lv[nlev++];
        L.level = level;
        L.first = k;
        L.count = 0;
        L.lastframe = lastframe;
        L.tau_lo = tau;
        L.compact = compact;
        L.t_end = (int32_t)((int64_t)lastframe << level);
        prev_level = level;
      }
      pl->lv[nlev - 1].count++;
      gi[k] = nlev - 1;
      ll_level = level;
      k++;
    }
  }
  pl->nlev = nlev;
  pl->acc = 1;
  pl->scr = nlev > 1 ? nlev : 1;
  return D;
}

}  // namespace
}  // namespace xg

using namespace xg;

extern "C" int xpcs_multitau2_noalloc(const int64_t *row_ptr, const int32_t *frame,
                                      const float *value, int32_t pixels, int64_t events,
                                      int32_t frames, int32_t delays_per_level, int32_t mode,
                                      float *G2, float *IP, float *IF, void *stream) {
  auto fail = [](int code, const char *msg) {
    xpcs_set_last_error(msg);
    return code;
  };
  if (!row_ptr || pixels <= 0 || frames < 0 || delays_per_level < 0 || events < 0 || !G2 ||
      !IP || !IF || (events > 0 && (!frame || !value)))
    return fail(XPCS_ERR_INVALID_ARGUMENT, "xpcs_multitau2_noalloc: bad argument");
  if (mode != XPCS_MODE_REFERENCE && mode != XPCS_MODE_EXACT)
    return fail(XPCS_ERR_INVALID_ARGUMENT, "xpcs_multitau2_noalloc: unknown mode");
  if (events > NA_MAX_EVENTS)
    return fail(XPCS_ERR_INVALID_ARGUMENT,
                "xpcs_multitau2_noalloc: more events than the fixed scratch holds "
                "(XPCS_NOALLOC_MAX_EVENTS)");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES)
    return fail(XPCS_ERR_NO_DEVICE, "xpcs_multitau2_noalloc: no current CUDA device");
  unsigned char *scratch = nullptr;
  {
    // once per device, with that device current: the scratch's device address
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
      void *ptr = nullptr;
      // under lazy module loading this first lookup also loads the module,
      // which is when the driver reserves the array on this device
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? XPCS_ERR_OUT_OF_MEMORY : XPCS_ERR_CUDA,
                    "xpcs_multitau2_noalloc: the fixed scratch array could not be set up on this "
                    "device (its first call loads the library's device code and reserves the "
                    "array; make that call at initialisation, with device memory to spare)");
      }
      g_na_ptr[dev] = (unsigned char *)ptr;
    }
    scratch = g_na_ptr[dev];
  }
  alignas(16) uint8_t plan[NA_PLAN_BYTES];
  const int D = na_build_plan(pixels, frames, delays_per_level, mode, plan, sizeof(plan));
  if (D < 0)
    return fail(XPCS_ERR_INVALID_ARGUMENT,
                "xpcs_multitau2_noalloc: more delays than the fixed scratch holds "
                "(XPCS_NOALLOC_MAX_DELAYS)");
  cudaStream_t st = (cudaStream_t)stream;
  const NaView v = na_view(scratch);
  if (cudaMemsetAsync(v.status, 0, sizeof(int32_t), st) != cudaSuccess ||
      cudaMemcpyAsync((void *)v.plan, plan, sizeof(plan), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail(XPCS_ERR_CUDA, "xpcs_multitau2_noalloc: copy to the scratch failed");
  if (D > 0) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = std::max(1, std::min((pixels + 127) / 128, std::max(sms, 1) * 8));
    k_mt_float_noalloc<<<grid, 128, 0, st>>>(scratch, row_ptr, frame, value, pixels, events, G2,
                                             IP, IF);
    if (cudaGetLastError() != cudaSuccess)
      return fail(XPCS_ERR_CUDA, "xpcs_multitau2_noalloc: kernel launch failed");
  }
  int32_t status = 0;
  if (cudaMemcpyAsync(&status, v.status, sizeof(status), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail(XPCS_ERR_CUDA, "xpcs_multitau2_noalloc: device error");
  if (status)
    return fail(XPCS_ERR_INPUT, "xpcs_multitau2_noalloc: row_ptr outside [0, events]");
  xpcs_set_last_error("");
  return XPCS_OK;
}
