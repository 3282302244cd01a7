// xpcs_synth_gpu — the sparse frames of xpcs_synth (xs_sparse) drawn on the
// GPU, for benchmark inputs too large to draw on the host in reasonable time
// (64 uneven series, 16 concurrent 1 Mpx streams).
//
// Same model and the same per-pixel random streams as the host generator: one
// thread per pixel runs its splitmix64 stream through the frames in order
// (two Irwin-Hall normals per AR(1) step, one uniform per Poisson draw), so
// the events are those of xs_sparse for the same parameters (the Poisson
// inversion evaluates exp() in double; a draw can differ only if its uniform
// falls within rounding of a cdf boundary).  Frames are produced in chunks:
// counts [chunk][P] -> per-(frame, 1024-pixel block) counts -> offsets on the
// host -> compaction in ascending pixel order, appended to device arrays.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "xpcs_synth.h"

namespace {

constexpr uint64_t STREAM_SPECKLE = 3;
constexpr int BLK = 1024;

__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ inline uint64_t next(uint64_t &s) {
  s += 0x9E3779B97F4A7C15ull;
  return mix64(s);
}

__device__ inline float normal(uint64_t &s) {
  const uint64_t r = next(s);
  float a = __fadd_rn(__fadd_rn(__fadd_rn((float)(r & 0xFFFF), (float)((r >> 16) & 0xFFFF)),
                                (float)((r >> 32) & 0xFFFF)),
                      (float)(r >> 48));
  return __fmul_rn(__fsub_rn(__fadd_rn(__fmul_rn(a, 1.0f / 65536.0f), 4.0f * (0.5f / 65536.0f)),
                             2.0f),
                   1.7320508f);
}

__device__ inline int poisson(uint64_t &s, double lambda) {
  const double u = (double)(next(s) >> 11) * (1.0 / 9007199254740992.0);
  if (u < 1.0 - lambda) return 0;
  double p = exp(-lambda), cdf = p;
  int k = 0;
  while (u >= cdf && k < 65535) {
    k++;
    p *= lambda / k;
    cdf += p;
    if (p == 0.0) break;
  }
  return k;
}

struct PixelState {
  float er, ei;
  uint64_t rng;
};

__global__ void k_init(int32_t P, uint64_t seed, PixelState *st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  st[i].rng = mix64(seed ^ mix64(STREAM_SPECKLE * 0x9E3779B97F4A7C15ull + (uint64_t)i + 1));
}

// frames [t0, t0 + nt) of every pixel -> counts[t - t0][P]
__global__ void k_draw(int32_t P, int32_t t0, int32_t nt, double mean,
                       const float *__restrict__ fa, const float *__restrict__ fs,
                       PixelState *__restrict__ st, uint16_t *__restrict__ counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  PixelState x = st[i];
  const float a = fa[i], sc = fs[i];
  for (int k = 0; k < nt; k++) {
    const int t = t0 + k;
    if (t == 0) {
      x.er = __fmul_rn(normal(x.rng), 0.70710678f);
      x.ei = __fmul_rn(normal(x.rng), 0.70710678f);
    } else {
      const float nr = __fmul_rn(normal(x.rng), 0.70710678f);
      const float ni = __fmul_rn(normal(x.rng), 0.70710678f);
      x.er = __fadd_rn(__fmul_rn(a, x.er), __fmul_rn(sc, nr));
      x.ei = __fadd_rn(__fmul_rn(a, x.ei), __fmul_rn(sc, ni));
    }
    const float inten = __fadd_rn(__fmul_rn(x.er, x.er), __fmul_rn(x.ei, x.ei));
    int c = poisson(x.rng, mean * (double)inten);
    counts[(size_t)k * P + i] = (uint16_t)(c > 65535 ? 65535 : c);
  }
  st[i] = x;
}

// per (frame k, block b): nonzero counts
__global__ void k_block_counts(int32_t P, const uint16_t *__restrict__ counts,
                               int32_t *__restrict__ bc) {
  __shared__ int s_w[BLK / 32];
  const int b = blockIdx.x, k = blockIdx.y, i = b * BLK + threadIdx.x;
  const bool nz = i < P && counts[(size_t)k * P + i] != 0;
  const unsigned m = __ballot_sync(0xffffffffu, nz);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    for (int w = 0; w < BLK / 32; w++) c += s_w[w];
    bc[(size_t)k * gridDim.x + b] = c;
  }
}

// compaction in ascending pixel order at the block's offset
__global__ void k_block_write(int32_t P, const uint16_t *__restrict__ counts,
                              const int64_t *__restrict__ boff, int32_t *__restrict__ idx,
                              int16_t *__restrict__ val) {
  __shared__ int s_w[BLK / 32];
  const int b = blockIdx.x, k = blockIdx.y, i = b * BLK + threadIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint16_t c = i < P ? counts[(size_t)k * P + i] : 0;
  const unsigned m = __ballot_sync(0xffffffffu, c != 0);
  if (lane == 0) s_w[w] = __popc(m);
  __syncthreads();
  int before = 0;
  for (int j = 0; j < w; j++) before += s_w[j];
  if (c != 0) {
    const int64_t o = boff[(size_t)k * gridDim.x + b] + before + __popc(m & ((1u << lane) - 1u));
    idx[o] = i;
    val[o] = (int16_t)c;
  }
}

bool grow(void **p, size_t &cap, size_t need, size_t used, size_t elem) {
  if (need <= cap) return true;
  size_t nc = cap ? cap : 1;
  while (nc < need) nc *= 2;
  void *q = nullptr;
  if (cudaMalloc(&q, nc * elem) != cudaSuccess) return false;
  if (used && cudaMemcpy(q, *p, used * elem, cudaMemcpyDeviceToDevice) != cudaSuccess) return false;
  if (*p) cudaFree(*p);
  *p = q;
  cap = nc;
  return true;
}

}  // namespace

extern "C" {

/* Sparse frames of xs_sparse drawn on the current CUDA device.  a/s: the
 * per-pixel field coefficients (xs_pixel_fields), host arrays.  nnz: host
 * [frames].  *idx_dev / *val_dev: device arrays (free with xsg_free).
 * Returns the total event count, or -1 on failure. */
int64_t xsg_sparse(const xs_params *p, const float *a, const float *s, uint32_t *nnz,
                   int32_t **idx_dev, int16_t **val_dev) {
  const int32_t P = p->width * p->height, F = p->frames;
  const int nb = (P + BLK - 1) / BLK;
  const int CH = std::max(1, std::min(256, (int)((size_t)256 * 1048576 / ((size_t)P * 2))));
  float *da = nullptr, *ds = nullptr;
  PixelState *st = nullptr;
  uint16_t *counts = nullptr;
  int32_t *bc = nullptr;
  int64_t *boff = nullptr;
  void *idx = nullptr, *val = nullptr;
  size_t cap_i = 0, cap_v = 0;
  int64_t total = 0;
  bool ok = cudaMalloc(&da, sizeof(float) * P) == cudaSuccess &&
            cudaMalloc(&ds, sizeof(float) * P) == cudaSuccess &&
            cudaMalloc(&st, sizeof(PixelState) * P) == cudaSuccess &&
            cudaMalloc(&counts, sizeof(uint16_t) * (size_t)CH * P) == cudaSuccess &&
            cudaMalloc(&bc, sizeof(int32_t) * (size_t)CH * nb) == cudaSuccess &&
            cudaMalloc(&boff, sizeof(int64_t) * (size_t)CH * nb) == cudaSuccess;
  ok = ok && cudaMemcpy(da, a, sizeof(float) * P, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(ds, s, sizeof(float) * P, cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    k_init<<<(P + 255) / 256, 256>>>(P, p->seed, st);
    std::vector<int32_t> hbc((size_t)CH * nb);
    std::vector<int64_t> hoff((size_t)CH * nb);
    for (int t0 = 0; ok && t0 < F; t0 += CH) {
      const int nt = std::min(CH, F - t0);
      k_draw<<<(P + 127) / 128, 128>>>(P, t0, nt, p->mean, da, ds, st, counts);
      k_block_counts<<<dim3(nb, nt), BLK>>>(P, counts, bc);
      ok = cudaMemcpy(hbc.data(), bc, sizeof(int32_t) * (size_t)nt * nb,
                      cudaMemcpyDeviceToHost) == cudaSuccess;
      if (!ok) break;
      int64_t run = total;
      for (int k = 0; k < nt; k++) {
        int64_t f0 = run;
        for (int b = 0; b < nb; b++) {
          hoff[(size_t)k * nb + b] = run;
          run += hbc[(size_t)k * nb + b];
        }
        nnz[t0 + k] = (uint32_t)(run - f0);
      }
      ok = grow(&idx, cap_i, (size_t)run, (size_t)total, sizeof(int32_t)) &&
           grow(&val, cap_v, (size_t)run, (size_t)total, sizeof(int16_t)) &&
           cudaMemcpy(boff, hoff.data(), sizeof(int64_t) * (size_t)nt * nb,
                      cudaMemcpyHostToDevice) == cudaSuccess;
      if (!ok) break;
      k_block_write<<<dim3(nb, nt), BLK>>>(P, counts, boff, (int32_t *)idx, (int16_t *)val);
      total = run;
    }
    ok = ok && cudaDeviceSynchronize() == cudaSuccess;
  }
  cudaFree(da);
  cudaFree(ds);
  cudaFree(st);
  cudaFree(counts);
  cudaFree(bc);
  cudaFree(boff);
  if (!ok) {
    cudaFree(idx);
    cudaFree(val);
    return -1;
  }
  if (!idx) ok = grow(&idx, cap_i, 1, 0, sizeof(int32_t)) && grow(&val, cap_v, 1, 0, sizeof(int16_t));
  *idx_dev = (int32_t *)idx;
  *val_dev = (int16_t *)val;
  return ok ? total : -1;
}

void xsg_free(void *dev) { cudaFree(dev); }

/* Device -> host copy of generated arrays. */
int xsg_to_host(void *host, const void *dev, uint64_t bytes) {
  return cudaMemcpy(host, dev, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : 1;
}

}  // extern "C"
