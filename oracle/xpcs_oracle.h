/*
 * xpcs_oracle — CPU restatement of xpcs-eigen's multi-tau correlation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation and the timed CPU baseline ("port") of the benchmark.  Only
 * tests, the smoke check and the benchmark's CPU-baseline leg may load it;
 * the product never links or calls it.
 *
 * Every function restates one reference routine (cited per function) with the
 * same arithmetic types and the same operation order, so that float results
 * are bit-identical to the reference built without floating-point
 * contraction.  Pinning: tests/test_oracle_golden.py checks it against
 * outputs of the reference `corr` itself (tests/golden/, generated by
 * tests/golden/make_golden.py from the reference built by oracle/ref_build).
 */
#ifndef XPCS_ORACLE_H
#define XPCS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Corr::calculateLevelMax, src/xpcs/corr.cpp:1156-1160 */
int xo_level_max(int frames, int dpl);

/* Corr::delaysPerLevel, src/xpcs/corr.cpp:1133-1154.  Writes up to `cap`
 * (level, tau) pairs; returns the number of delays D. */
int xo_delays(int frames, int dpl, int32_t *level, int32_t *tau, int cap);

/* Result of Configuration::BuildQMap (src/xpcs/configuration.cpp:244-381).
 * The q -> sbin -> pixel mapping is flattened in the reference's iteration
 * order: q ascending, sbin ascending within q, pixels in insertion order. */
typedef struct {
  int32_t pixels;
  int32_t total_static;   /* m_totalStaticPartitions (quirk Q5 kept) */
  int32_t total_dynamic;  /* m_totalDynamicPartitions */
  int32_t nq;             /* m_mapping.size() == rows of g2/stderr */
  int32_t nsb;            /* number of (q, sbin) entries in the mapping */
  int32_t npix;           /* pixels in the mapping (after quirk Q6 drops) */
  int16_t *valid;         /* [pixels] m_validPixelMask */
  int32_t *sbin_mask;     /* [pixels] m_sbin (1-based, 0 = none) */
  int32_t *pixels_per_bin;/* [total_static] over all valid pixels */
  int32_t *q_ids;         /* [nq] */
  int32_t *q_sb_ptr;      /* [nq+1] into sb_ids */
  int32_t *sb_ids;        /* [nsb] 1-based sbin of each entry */
  int32_t *sb_pix_ptr;    /* [nsb+1] into pix */
  int32_t *pix;           /* [npix] */
  int32_t error;          /* 1 if the reference would index out of bounds (Q5/Q7) */
} xo_qmap;

int xo_build_qmap(const int32_t *dqmap, const int32_t *sqmap, int32_t pixels, xo_qmap *out);
void xo_free_qmap(xo_qmap *q);

/* Parameters shared by the sparse and dense filters
 * (SparseFilter ctor src/xpcs/filter/sparse_filter.cpp:63-108,
 *  DenseFilter ctor src/xpcs/filter/dense_filter.cpp:63-111). */
typedef struct {
  int32_t pixels;        /* frame_width * frame_height */
  int32_t frames;        /* getFrameTodoCount() */
  int32_t real_frames;   /* getRealFrameTodoCount() */
  int32_t stride;        /* FrameStride() */
  int32_t average;       /* FrameAverage() */
  int32_t static_window; /* getStaticWindowSize() */
  int32_t total_static;  /* getTotalStaticPartitions() */
  const int16_t *pixel_mask;  /* getPixelMask() */
  const int32_t *sbin_mask;   /* getSbinMask() */
  const double *flatfield;    /* getFlatField() (all 1.0 when disabled) */
} xo_filter_params;

/* Pixel-major event lists (SparseData / Row, src/xpcs/data_structure). */
typedef struct {
  int32_t pixels;
  int64_t *row_ptr;  /* [pixels+1] */
  int32_t *frame;    /* indxPtr */
  float *value;      /* valPtr */
} xo_rows;

/* Side statistics produced by the filters. */
typedef struct {
  float *pixels_sum;          /* [pixels] */
  float *frames_sum;          /* [2*frames] */
  float *partitions_mean;     /* [total_static] */
  float *partial_mean;        /* [ceil(frames/static_window) * total_static] */
  double *timestamp_clock;    /* [2*real_frames] */
  double *timestamp_ticks;    /* [2*real_frames] */
} xo_side;

/* SparseFilter::Apply over the whole series, src/xpcs/filter/sparse_filter.cpp:115-193,
 * driven as main.cpp:258-268 does (read_in_count raw frames per Apply).
 * Raw frame r has nnz[r] events idx[off[r]..], val[off[r]..] with
 * off = exclusive prefix of nnz.  clock/ticks may be NULL. */
int xo_sparse_filter(const xo_filter_params *p, const int32_t *idx, const int16_t *val,
                     const uint32_t *nnz, const double *clock, const double *ticks,
                     xo_rows *rows, xo_side *side);

/* DarkImage::Compute, src/xpcs/data_structure/dark_image.cpp:81-106.
 * dark: [ndark][pixels] raw int16 values. */
void xo_dark_image(const int16_t *dark, int ndark, int pixels, const double *flatfield,
                   double *dark_avg, double *dark_std);

/* DenseFilter::Apply over the whole series, src/xpcs/filter/dense_filter.cpp:121-210.
 * raw: [raw frames][pixels] int16.  dark_avg/dark_std NULL = no dark. */
int xo_dense_filter(const xo_filter_params *p, const int16_t *raw, const double *dark_avg,
                    const double *dark_std, float lld, float sigma, const double *clock,
                    const double *ticks, xo_rows *rows, xo_side *side);

/* Post-processing of the side statistics done by main.cpp:321-411. */
void xo_finish_side(const xo_filter_params *p, const int32_t *pixels_per_bin, xo_side *side);

void xo_free_rows(xo_rows *r);
void xo_free_side(xo_side *s);

/* Corr::multiTau2, src/xpcs/corr.cpp:315-431, on a private copy of `rows`.
 * mode 0 = reference (lower_bound over the whole row, quirk Q1);
 * mode 1 = exact (lower_bound over the live prefix).
 * G2/IP/IF: [D][pixels], zeroed here.  threads <= 0: OpenMP default. */
int xo_multitau2(const xo_rows *rows, int frames, int dpl, int mode, int threads, float *G2,
                 float *IP, float *IF);

/* Corr::normalizeG2s, src/xpcs/corr.cpp:927-1091, float32 exactly as the
 * reference evaluates it.  g2/stderr: [D][nq]. */
int xo_normalize_f32(const xo_qmap *q, int D, const float *G2, const float *IP, const float *IF,
                     float *g2, float *stderr_);

/* The same formulas evaluated in double (sequential, reference order). */
int xo_normalize_f64(const xo_qmap *q, int D, const float *G2, const float *IP, const float *IF,
                     double *g2, double *stderr_);

#ifdef __cplusplus
}
#endif

#endif
