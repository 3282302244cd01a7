// Device-wide exclusive prefix sums (reduce-then-scan, recursive over block
// totals).  Used for radix-sort digit offsets and for the pixel-major row
// offsets of the event lists.
#include "xpcs_internal.h"

namespace xg {
namespace {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_IPT;

template <class T>
__device__ T block_exclusive(T v, T *total) {
  __shared__ T warp_tot[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    T t = lane < SCAN_THREADS / 32 ? warp_tot[lane] : T(0);
    T s = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < SCAN_THREADS / 32) warp_tot[lane] = s - t;
    if (lane == SCAN_THREADS / 32 - 1) *total = s;
  }
  __syncthreads();
  T r = warp_tot[w] + x - v;
  __syncthreads();
  return r;
}

// in[g] for g < n_in, 0 for n_in <= g < n_out
template <class TI, class TO>
__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_reduce(const TI *__restrict__ in, int64_t n_in, int64_t n_out, TO *__restrict__ sums) {
  __shared__ TO total;
  const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
  TO acc = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    int64_t g = base + k * SCAN_THREADS + threadIdx.x;
    if (g < n_in && g < n_out) acc += (TO)in[g];
  }
  block_exclusive<TO>(acc, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <class TI, class TO>
__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_down(const TI *__restrict__ in, int64_t n_in, int64_t n_out,
            const TO *__restrict__ prefix, TO *__restrict__ out) {
  __shared__ TO total;
  const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK + (int64_t)threadIdx.x * SCAN_IPT;
  TO v[SCAN_IPT];
  TO sum = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    int64_t g = base + k;
    v[k] = (g < n_in && g < n_out) ? (TO)in[g] : TO(0);
    sum += v[k];
  }
  TO run = block_exclusive<TO>(sum, &total) + (prefix ? prefix[blockIdx.x] : TO(0));
#pragma unroll
  for (int k = 0; k < SCAN_IPT; k++) {
    int64_t g = base + k;
    if (g < n_out) out[g] = run;
    run += v[k];
  }
}

template <class TO>
size_t ws_bytes(int64_t n) {
  size_t b = 0;
  while (n > SCAN_CHUNK) {
    int64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
    b += 2 * ((sizeof(TO) * nb + 255) / 256 * 256);
    n = nb;
  }
  return b + 256;
}

template <class TI, class TO>
void scan_rec(const TI *in, int64_t n_in, int64_t n_out, TO *out, uint8_t *ws, cudaStream_t st) {
  if (n_out <= 0) return;
  int64_t nb = (n_out + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if (nb == 1) {
    k_scan_down<TI, TO><<<1, SCAN_THREADS, 0, st>>>(in, n_in, n_out, nullptr, out);
    XG_CHECK_LAUNCH();
    return;
  }
  size_t seg = (sizeof(TO) * nb + 255) / 256 * 256;
  TO *sums = (TO *)ws;
  TO *pref = (TO *)(ws + seg);
  k_scan_reduce<TI, TO><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n_in, n_out, sums);
  XG_CHECK_LAUNCH();
  scan_rec<TO, TO>(sums, nb, nb, pref, ws + 2 * seg, st);
  k_scan_down<TI, TO><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n_in, n_out, pref, out);
  XG_CHECK_LAUNCH();
}

}  // namespace

size_t scan_workspace_bytes(int64_t n) { return ws_bytes<int64_t>(n + 1); }

void exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, void *ws, cudaStream_t st) {
  scan_rec<uint32_t, uint32_t>(in, n, n, out, (uint8_t *)ws, st);
}

// out has n+1 entries; out[n] is the total.
void exclusive_scan_i32_i64(const int32_t *in, int64_t *out, int64_t n, void *ws,
                            cudaStream_t st) {
  scan_rec<int32_t, int64_t>(in, n, n + 1, out, (uint8_t *)ws, st);
}

}  // namespace xg
