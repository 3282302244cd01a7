// xpcs_synth — seeded synthetic XPCS acquisitions; see xpcs_synth.h.
//
// Random numbers: one splitmix64 stream per pixel (Steele, Lea & Flood 2014),
// seeded from (seed, stream id, pixel).  Normal deviates are Irwin-Hall sums of
// four 16-bit uniforms scaled to unit variance, which is enough for a speckle
// field whose second-order statistics are what matters.  Poisson deviates use
// inversion; the common "no photon" outcome is decided without evaluating
// exp() because exp(-lambda) >= 1 - lambda.
#include "xpcs_synth.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Rng {
  uint64_t s;
  Rng(uint64_t seed, uint64_t stream, uint64_t index)
      : s(mix64(seed ^ mix64(stream * 0x9E3779B97F4A7C15ull + index + 1))) {}
  inline uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    return mix64(s);
  }
  inline double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  inline float normal() {
    uint64_t r = next();
    float a = (float)(r & 0xFFFF) + (float)((r >> 16) & 0xFFFF) + (float)((r >> 32) & 0xFFFF) +
              (float)(r >> 48);
    // sum of four U(0,1) (midpoints of 16-bit cells) has mean 2, variance 1/3
    return (a * (1.0f / 65536.0f) + 4.0f * (0.5f / 65536.0f) - 2.0f) * 1.7320508f;
  }
};

inline int poisson(Rng &rng, double lambda) {
  double u = rng.uniform();
  if (u < 1.0 - lambda) return 0;  // u < 1 - lambda <= exp(-lambda)
  double p = std::exp(-lambda), cdf = p;
  int k = 0;
  while (u >= cdf && k < 65535) {
    k++;
    p *= lambda / k;
    cdf += p;
    if (p == 0.0) break;
  }
  return k;
}

enum : uint64_t { STREAM_MASK = 1, STREAM_TAU = 2, STREAM_SPECKLE = 3, STREAM_DARK = 4,
                  STREAM_GAIN = 5, STREAM_NOISE = 6 };

struct Geometry {
  std::vector<int32_t> ring;  // 0-based dynamic ring of every pixel (ignoring the mask)
  std::vector<double> tau;    // per dynamic ring
};

Geometry geometry(const xs_params *p, int32_t *dq, int32_t *sq) {
  const int W = p->width, H = p->height, P = W * H;
  Geometry g;
  g.ring.resize(P);
  double rmax = 0.0;
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      double r = std::sqrt((x - p->center_x) * (x - p->center_x) +
                           (y - p->center_y) * (y - p->center_y));
      if (r > rmax) rmax = r;
    }
  int per = p->n_static / p->n_dynamic;
  if (per < 1) per = 1;
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      int i = y * W + x;
      double r = std::sqrt((x - p->center_x) * (x - p->center_x) +
                           (y - p->center_y) * (y - p->center_y));
      int s = (int)std::floor(r / (rmax > 0 ? rmax : 1.0) * p->n_static) + 1;
      if (s > p->n_static) s = p->n_static;
      int q = (s - 1) / per + 1;
      if (q > p->n_dynamic) q = p->n_dynamic;
      g.ring[i] = q - 1;
      Rng m(p->seed, STREAM_MASK, (uint64_t)i);
      bool masked = m.uniform() < p->mask_fraction;
      if (dq) dq[i] = masked ? 0 : q;
      if (sq) sq[i] = masked ? 0 : s;
    }
  g.tau.resize(p->n_dynamic > 0 ? p->n_dynamic : 1);
  for (int q = 0; q < p->n_dynamic; q++) {
    Rng t(p->seed, STREAM_TAU, (uint64_t)q);
    double u = t.uniform();
    g.tau[q] = p->tau_max > p->tau_min
                   ? std::exp(std::log(p->tau_min) + u * (std::log(p->tau_max) - std::log(p->tau_min)))
                   : p->tau_min;
  }
  return g;
}

struct PixelField {
  float er, ei, a, s;
};

inline void field_init(PixelField &f, Rng &rng, double tau) {
  f.a = (float)std::exp(-1.0 / tau);
  f.s = (float)std::sqrt(1.0 - (double)f.a * f.a);
  f.er = rng.normal() * 0.70710678f;
  f.ei = rng.normal() * 0.70710678f;
}

inline float field_step(PixelField &f, Rng &rng, bool first) {
  if (!first) {
    float nr = rng.normal() * 0.70710678f, ni = rng.normal() * 0.70710678f;
    f.er = f.a * f.er + f.s * nr;
    f.ei = f.a * f.ei + f.s * ni;
  }
  return f.er * f.er + f.ei * f.ei;
}

}  // namespace

extern "C" int xs_make_maps(const xs_params *p, int32_t *dqmap, int32_t *sqmap, double *flat,
                            double *tau) {
  if (!p || p->width <= 0 || p->height <= 0 || p->n_static <= 0 || p->n_dynamic <= 0) return 1;
  Geometry g = geometry(p, dqmap, sqmap);
  const int P = p->width * p->height;
  if (flat) {
    for (int i = 0; i < P; i++) {
      Rng r(p->seed, STREAM_GAIN, (uint64_t)i);
      flat[i] = p->gain_max > p->gain_min
                    ? p->gain_min + r.uniform() * (p->gain_max - p->gain_min)
                    : 1.0;
    }
  }
  if (tau)
    for (int q = 0; q < p->n_dynamic; q++) tau[q] = g.tau[q];
  return 0;
}

extern "C" int xs_pixel_fields(const xs_params *p, float *a, float *s) {
  if (!p || p->width <= 0 || p->height <= 0 || p->n_static <= 0 || p->n_dynamic <= 0) return 1;
  Geometry g = geometry(p, nullptr, nullptr);
  const int P = p->width * p->height;
  for (int i = 0; i < P; i++) {
    const double tau = g.tau[g.ring[i]];
    a[i] = (float)std::exp(-1.0 / tau);
    s[i] = (float)std::sqrt(1.0 - (double)a[i] * a[i]);
  }
  return 0;
}

extern "C" int64_t xs_sparse(const xs_params *p, uint32_t *nnz, int32_t **idx_out,
                             int16_t **val_out) {
  const int P = p->width * p->height, F = p->frames;
  Geometry g = geometry(p, nullptr, nullptr);
  const int CH = 1024;
  const int nch = (P + CH - 1) / CH;
  struct Ev {
    int32_t frame, pixel;
    uint16_t count;
  };
  std::vector<std::vector<Ev>> chunks(nch);
#pragma omp parallel for schedule(dynamic, 4)
  for (int c = 0; c < nch; c++) {
    std::vector<Ev> &out = chunks[c];
    for (int i = c * CH; i < P && i < (c + 1) * CH; i++) {
      Rng rng(p->seed, STREAM_SPECKLE, (uint64_t)i);
      PixelField f;
      field_init(f, rng, g.tau[g.ring[i]]);
      for (int t = 0; t < F; t++) {
        float inten = field_step(f, rng, t == 0);
        int k = poisson(rng, p->mean * inten);
        if (k > 0) out.push_back(Ev{t, i, (uint16_t)(k > 65535 ? 65535 : k)});
      }
    }
  }
  std::vector<int64_t> off(F + 1, 0);
  for (auto &ch : chunks)
    for (auto &e : ch) off[e.frame + 1]++;
  for (int t = 0; t < F; t++) {
    nnz[t] = (uint32_t)off[t + 1];
    off[t + 1] += off[t];
  }
  int64_t total = off[F];
  int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(total ? total : 1));
  int16_t *val = (int16_t *)malloc(sizeof(int16_t) * (size_t)(total ? total : 1));
  if (!idx || !val) {
    free(idx);
    free(val);
    return -1;
  }
  std::vector<int64_t> cur(off.begin(), off.end() - 1);
  for (auto &ch : chunks)  // chunks in pixel order, so each frame stays pixel-sorted
    for (auto &e : ch) {
      int64_t k = cur[e.frame]++;
      idx[k] = e.pixel;
      val[k] = (int16_t)e.count;
    }
  *idx_out = idx;
  *val_out = val;
  return total;
}

struct xs_dense_state {
  xs_params p;
  Geometry g;
  std::vector<PixelField> field;
  std::vector<Rng> rng, noise;
  std::vector<float> dark;
  std::vector<double> flat;
  int64_t next_frame = 0;
};

extern "C" xs_dense_state *xs_dense_create(const xs_params *p) {
  xs_dense_state *s = new xs_dense_state();
  s->p = *p;
  s->g = geometry(p, nullptr, nullptr);
  const int P = p->width * p->height;
  s->field.resize(P);
  s->dark.resize(P);
  s->flat.resize(P);
  s->rng.reserve(P);
  s->noise.reserve(P);
  for (int i = 0; i < P; i++) {
    s->rng.emplace_back(p->seed, STREAM_SPECKLE, (uint64_t)i);
    s->noise.emplace_back(p->seed, STREAM_NOISE, (uint64_t)i);
    Rng d(p->seed, STREAM_DARK, (uint64_t)i);
    s->dark[i] = (float)(p->dark_mean + p->dark_sigma * d.normal());
    Rng r(p->seed, STREAM_GAIN, (uint64_t)i);
    s->flat[i] = p->gain_max > p->gain_min
                     ? p->gain_min + r.uniform() * (p->gain_max - p->gain_min)
                     : 1.0;
    field_init(s->field[i], s->rng[i], s->g.tau[s->g.ring[i]]);
  }
  return s;
}

extern "C" int xs_dense_next(xs_dense_state *s, int32_t count, int16_t *out) {
  const xs_params &p = s->p;
  const int P = p.width * p.height;
  for (int k = 0; k < count; k++) {
    int64_t fr = s->next_frame++;
    bool is_dark = fr < p.dark_frames;
    int64_t t = fr - p.dark_frames;
    int16_t *o = out + (size_t)k * P;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < P; i++) {
      double v = s->dark[i] + p.read_noise * s->noise[i].normal();
      if (!is_dark) {
        float inten = field_step(s->field[i], s->rng[i], t == 0);
        int n = poisson(s->rng[i], p.mean * inten);
        v += p.adu_per_photon * n / s->flat[i];
      }
      double r = std::floor(v + 0.5);
      if (r < 0) r = 0;
      if (r > 65535) r = 65535;
      o[i] = (int16_t)(uint16_t)r;
    }
  }
  return 0;
}

extern "C" void xs_dense_destroy(xs_dense_state *s) { delete s; }

extern "C" void xs_free(void *ptr) { free(ptr); }
