/*
 * xpcs_synth — seeded synthetic XPCS acquisitions (benchmark and test inputs).
 *
 * Speckle model: every pixel carries a complex Gaussian field E(t) evolving as
 * an AR(1) process E(t) = a E(t-1) + sqrt(1-a^2) n(t), a = exp(-1/tau_c), with
 * <|E|^2> = 1; the photon count of a frame is Poisson(mean * |E(t)|^2).
 * tau_c is drawn log-uniform in [tau_min, tau_max] per dynamic ring.  Rings are
 * annuli about (center_x, center_y): n_static equal-width static bins, each
 * group of n_static/n_dynamic consecutive static bins forms one dynamic bin.  A
 * random fraction of pixels is masked (dqmap = sqmap = 0).
 *
 * The output depends only on the parameters and the seed (per-pixel
 * counter-based random streams), not on the number of threads.
 */
#ifndef XPCS_SYNTH_H
#define XPCS_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int32_t width, height;   /* detector columns, rows */
  int32_t frames;          /* data frames */
  int32_t n_static, n_dynamic;
  double center_x, center_y;
  double mask_fraction;
  double mean;             /* photons per pixel per frame */
  double tau_min, tau_max; /* speckle correlation time (frames) */
  uint64_t seed;
  /* dense (CCD) frames only */
  int32_t dark_frames;
  double dark_mean, dark_sigma; /* per-pixel dark level ~ N(dark_mean, dark_sigma^2) */
  double read_noise;            /* per-frame read noise sigma (ADU) */
  double adu_per_photon;
  double gain_min, gain_max;    /* per-pixel flatfield ~ U[gain_min, gain_max] */
} xs_params;

/* q-partition maps, flatfield and per-dynamic-ring tau_c.
 * dqmap/sqmap/flat: [height*width]; tau: [n_dynamic] (may be NULL). */
int xs_make_maps(const xs_params *p, int32_t *dqmap, int32_t *sqmap, double *flat, double *tau);

/* Sparse (photon counting) frames.  Allocates the idx and val arrays (free with xs_free);
 * nnz: [frames].  Events of a frame are in ascending pixel order; values are
 * the uint16 counts stored as their int16 bit pattern.  Returns the total
 * event count, or -1 on allocation failure. */
int64_t xs_sparse(const xs_params *p, uint32_t *nnz, int32_t **idx, int16_t **val);

/* Dense (CCD) frames, streamed: frames [first, first+count) of the sequence
 * "dark_frames dark frames, then `frames` data frames" written to
 * out[count][height*width].  A state object carries the speckle field. */
typedef struct xs_dense_state xs_dense_state;
xs_dense_state *xs_dense_create(const xs_params *p);
int xs_dense_next(xs_dense_state *s, int32_t count, int16_t *out);
void xs_dense_destroy(xs_dense_state *s);

void xs_free(void *ptr);

/* The speckle field's AR(1) coefficients of every pixel (a = exp(-1/tau_c) of
 * its ring, s = sqrt(1-a^2)), masked pixels included: [height*width] each.
 * The GPU generator (xpcs_synth_gpu.cu) takes them to draw the same frames. */
int xs_pixel_fields(const xs_params *p, float *a, float *s);

#ifdef __cplusplus
}
#endif

#endif
