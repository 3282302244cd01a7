// xpcs_synth_gpu — the sparse frames of xpcs_synth (xs_sparse) and its dense
// CCD frames (xs_dense_next) drawn on the GPU, for benchmark inputs too large
// to draw on the host in reasonable time (64 uneven series, 16 concurrent
// 1 Mpx streams, 20,100 frames of 960x960).
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

constexpr uint64_t STREAM_DARK = 4, STREAM_NOISE = 6;

__device__ inline uint64_t stream_seed(uint64_t seed, uint64_t stream, uint64_t i) {
  return mix64(seed ^ mix64(stream * 0x9E3779B97F4A7C15ull + i + 1));
}

// dense frames: the dark level and the read-noise stream of every pixel
__global__ void k_dense_init(int32_t P, uint64_t seed, double dark_mean, double dark_sigma,
                             float *__restrict__ dark, uint64_t *__restrict__ noise,
                             PixelState *__restrict__ st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  uint64_t d = stream_seed(seed, STREAM_DARK, (uint64_t)i);
  dark[i] = __double2float_rn(__dadd_rn(dark_mean, __dmul_rn(dark_sigma, (double)normal(d))));
  noise[i] = stream_seed(seed, STREAM_NOISE, (uint64_t)i);
  st[i].rng = stream_seed(seed, STREAM_SPECKLE, (uint64_t)i);
}

// sequence frames [f0, f0 + nf) ("dark_frames" darks, then data frames) of
// every pixel: dark level + read noise, plus adu * photons / gain on data
// frames, rounded and clipped to [0, 65535], stored as the int16 bit pattern
__global__ void k_dense_draw(int32_t P, int64_t f0, int32_t nf, int32_t dark_frames, double mean,
                             double read_noise, double adu, const float *__restrict__ fa,
                             const float *__restrict__ fs, const float *__restrict__ dark,
                             const double *__restrict__ flat, uint64_t *__restrict__ noise,
                             PixelState *__restrict__ st, int16_t *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  PixelState x = st[i];
  uint64_t nz = noise[i];
  const float a = fa[i], sc = fs[i], dk = dark[i];
  const double g = flat[i];
  for (int k = 0; k < nf; k++) {
    const int64_t fr = f0 + k;
    double v = __dadd_rn((double)dk, __dmul_rn(read_noise, (double)normal(nz)));
    if (fr >= dark_frames) {
      if (fr == dark_frames) {
        x.er = __fmul_rn(normal(x.rng), 0.70710678f);
        x.ei = __fmul_rn(normal(x.rng), 0.70710678f);
      } else {
        const float nr = __fmul_rn(normal(x.rng), 0.70710678f);
        const float ni = __fmul_rn(normal(x.rng), 0.70710678f);
        x.er = __fadd_rn(__fmul_rn(a, x.er), __fmul_rn(sc, nr));
        x.ei = __fadd_rn(__fmul_rn(a, x.ei), __fmul_rn(sc, ni));
      }
      const float inten = __fadd_rn(__fmul_rn(x.er, x.er), __fmul_rn(x.ei, x.ei));
      const int n = poisson(x.rng, mean * (double)inten);
      v = __dadd_rn(v, __ddiv_rn(__dmul_rn(adu, (double)n), g));
    }
    double r = floor(__dadd_rn(v, 0.5));
    r = r < 0.0 ? 0.0 : (r > 65535.0 ? 65535.0 : r);
    out[(size_t)k * P + i] = (int16_t)(uint16_t)r;
  }
  st[i] = x;
  noise[i] = nz;
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

/* Dense frames of xs_dense_next drawn on the current CUDA device: the whole
 * sequence of dark_frames darks and then frames data frames, int16
 * [dark_frames + frames][P] in one device allocation (*out_dev, free with
 * xsg_free).  a/s: xs_pixel_fields; flat: the flatfield of xs_make_maps
 * (host arrays).  Returns 0, or 1 on failure. */
int xsg_dense(const xs_params *p, const float *a, const float *s, const double *flat,
              int16_t **out_dev) {
  const int32_t P = p->width * p->height;
  const int64_t NF = (int64_t)p->dark_frames + p->frames;
  float *da = nullptr, *ds = nullptr, *dark = nullptr;
  double *dflat = nullptr;
  uint64_t *noise = nullptr;
  PixelState *st = nullptr;
  int16_t *out = nullptr;
  bool ok = cudaMalloc(&da, sizeof(float) * P) == cudaSuccess &&
            cudaMalloc(&ds, sizeof(float) * P) == cudaSuccess &&
            cudaMalloc(&dark, sizeof(float) * P) == cudaSuccess &&
            cudaMalloc(&dflat, sizeof(double) * P) == cudaSuccess &&
            cudaMalloc(&noise, sizeof(uint64_t) * P) == cudaSuccess &&
            cudaMalloc(&st, sizeof(PixelState) * P) == cudaSuccess &&
            cudaMalloc(&out, sizeof(int16_t) * (size_t)(NF > 0 ? NF : 1) * P) == cudaSuccess;
  ok = ok && cudaMemcpy(da, a, sizeof(float) * P, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(ds, s, sizeof(float) * P, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(dflat, flat, sizeof(double) * P, cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    k_dense_init<<<(P + 255) / 256, 256>>>(P, p->seed, p->dark_mean, p->dark_sigma, dark, noise,
                                           st);
    for (int64_t f0 = 0; f0 < NF; f0 += 256) {
      const int32_t nf = (int32_t)(NF - f0 < 256 ? NF - f0 : 256);
      k_dense_draw<<<(P + 127) / 128, 128>>>(P, f0, nf, p->dark_frames, p->mean, p->read_noise,
                                             p->adu_per_photon, da, ds, dark, dflat, noise, st,
                                             out + (size_t)f0 * P);
    }
    ok = cudaDeviceSynchronize() == cudaSuccess;
  }
  cudaFree(da);
  cudaFree(ds);
  cudaFree(dark);
  cudaFree(dflat);
  cudaFree(noise);
  cudaFree(st);
  if (!ok) {
    cudaFree(out);
    return 1;
  }
  *out_dev = out;
  return 0;
}

void xsg_free(void *dev) { cudaFree(dev); }

/* Device -> host copy of generated arrays. */
int xsg_to_host(void *host, const void *dev, uint64_t bytes) {
  return cudaMemcpy(host, dev, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : 1;
}

}  // extern "C"
