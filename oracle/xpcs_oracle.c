/*
 * xpcs_oracle — CPU restatement of xpcs-eigen's multi-tau correlation path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels and the timed CPU
 * baseline of the benchmark.  The product never links or calls this file.
 *
 * Build: gcc -std=c11 -O3 -fopenmp -ffp-contract=off -fPIC -shared
 * (-ffp-contract=off: every float expression is evaluated as the reference's
 * x86-64 build evaluates it, one rounding per operation, no fused multiply-add).
 *
 * Each function cites the reference routine it restates; the arithmetic types
 * and the order of every floating-point operation follow the reference.
 */
#include "xpcs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- delays */

/* Corr::calculateLevelMax, src/xpcs/corr.cpp:1156-1160 */
int xo_level_max(int frames, int dpl) {
  if (frames < dpl * 2) return 0;
  return (int)(floor(log2((double)frames) - log2(1.0 + 1.0 / (double)dpl)) - log2((double)dpl));
}

/* Corr::delaysPerLevel, src/xpcs/corr.cpp:1133-1154: level 0 has 2*dpl delays
 * of step 1, level i has dpl delays of step 2^i; a delay is kept while
 * ll + 2^i + 2^i <= frames.  tau is in frames (cumulative). */
int xo_delays(int frames, int dpl, int32_t *level, int32_t *tau, int cap) {
  int max_level = xo_level_max(frames, dpl);
  int n = 0, ll = 0;
  for (int i = 0; i <= max_level; i++) {
    int step = (int)pow(2.0, i);
    int dpll = i == 0 ? dpl * 2 : dpl;
    for (int j = 0; j < dpll; j++) {
      if ((ll + step + pow(2.0, i)) > frames) break;
      if (n < cap) {
        level[n] = i;
        tau[n] = ll + step;
      }
      n++;
      ll = ll + step;
    }
  }
  return n;
}

/* ------------------------------------------------------------------ qmap */

typedef struct {
  int32_t q, s, p;
} qsp_t;

static int cmp_qsp(const void *a, const void *b) {
  const qsp_t *x = (const qsp_t *)a, *y = (const qsp_t *)b;
  if (x->q != y->q) return x->q < y->q ? -1 : 1;
  if (x->s != y->s) return x->s < y->s ? -1 : 1;
  return x->p < y->p ? -1 : (x->p > y->p);
}

/* Configuration::BuildQMap, src/xpcs/configuration.cpp:244-381.
 * - valid pixel: dqmap >= 1 and sqmap >= 1 (:256-260)
 * - m_totalStaticPartitions grows only when the pixel's q is already in the
 *   mapping (:271-274, quirk Q5); m_totalDynamicPartitions = max q (:266-267)
 * - an sbin mapped to several q is kept only under the q holding most of its
 *   pixels (first such q in ascending order); the reference's merge copies the
 *   destination map by value (:327-328), so the other q's pixels of that sbin
 *   are dropped (quirk Q6)
 * - pixels_per_bin counts every valid pixel by sqmap (:349-356). */
int xo_build_qmap(const int32_t *dq, const int32_t *sq, int32_t pixels, xo_qmap *out) {
  memset(out, 0, sizeof(*out));
  out->pixels = pixels;
  out->valid = (int16_t *)calloc((size_t)pixels, sizeof(int16_t));
  out->sbin_mask = (int32_t *)calloc((size_t)pixels, sizeof(int32_t));
  int32_t maxq = 0, maxs = 0, nvalid = 0;
  for (int32_t i = 0; i < pixels; i++) {
    if (dq[i] < 1 || sq[i] < 1) continue;
    nvalid++;
    if (dq[i] > maxq) maxq = dq[i];
    if (sq[i] > maxs) maxs = sq[i];
  }
  char *q_seen = (char *)calloc((size_t)maxq + 2, 1);
  qsp_t *t = (qsp_t *)malloc(sizeof(qsp_t) * (size_t)(nvalid > 0 ? nvalid : 1));
  int32_t n = 0;
  for (int32_t i = 0; i < pixels; i++) {
    if (dq[i] < 1 || sq[i] < 1) continue;
    out->valid[i] = 1;
    out->sbin_mask[i] = sq[i];
    if (out->total_dynamic < dq[i]) out->total_dynamic = dq[i];
    if (q_seen[dq[i]]) {
      if (out->total_static < sq[i]) out->total_static = sq[i];
    }
    q_seen[dq[i]] = 1;
    t[n].q = dq[i];
    t[n].s = sq[i];
    t[n].p = i;
    n++;
  }
  qsort(t, (size_t)n, sizeof(qsp_t), cmp_qsp);

  /* groups (q, s) in (q asc, s asc) order */
  int32_t ng = 0;
  int32_t *g_start = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
  for (int32_t k = 0; k < n; k++)
    if (k == 0 || t[k].q != t[k - 1].q || t[k].s != t[k - 1].s) g_start[ng++] = k;
  g_start[ng] = n;
  char *erased = (char *)calloc((size_t)ng + 1, 1);

  /* duplicate sbin -> several q: keep the q with most pixels (strictly greater
   * wins, so the first maximum in ascending q order), erase the others */
  int32_t *first_g = (int32_t *)malloc(sizeof(int32_t) * ((size_t)maxs + 2));
  int32_t *cnt_q = (int32_t *)calloc((size_t)maxs + 2, sizeof(int32_t));
  for (int32_t s = 0; s <= maxs; s++) first_g[s] = -1;
  for (int32_t g = 0; g < ng; g++) cnt_q[t[g_start[g]].s]++;
  for (int32_t s = 1; s <= maxs; s++) {
    if (cnt_q[s] <= 1) continue;
    int32_t best_g = -1, best_n = 0;
    for (int32_t g = 0; g < ng; g++) {
      if (t[g_start[g]].s != s) continue;
      int32_t np = g_start[g + 1] - g_start[g];
      if (np > best_n) {
        best_n = np;
        best_g = g;
      }
    }
    for (int32_t g = 0; g < ng; g++)
      if (t[g_start[g]].s == s && g != best_g) erased[g] = 1;
  }

  /* flatten */
  out->q_ids = (int32_t *)malloc(sizeof(int32_t) * ((size_t)maxq + 1));
  out->q_sb_ptr = (int32_t *)malloc(sizeof(int32_t) * ((size_t)maxq + 2));
  out->sb_ids = (int32_t *)malloc(sizeof(int32_t) * ((size_t)ng + 1));
  out->sb_pix_ptr = (int32_t *)malloc(sizeof(int32_t) * ((size_t)ng + 2));
  out->pix = (int32_t *)malloc(sizeof(int32_t) * ((size_t)n + 1));
  int32_t nq = 0, nsb = 0, npix = 0;
  for (int32_t g = 0; g < ng; g++) {
    int32_t q = t[g_start[g]].q;
    if (nq == 0 || out->q_ids[nq - 1] != q) {
      out->q_ids[nq] = q;
      out->q_sb_ptr[nq] = nsb;
      nq++;
    }
    if (erased[g]) continue;
    out->sb_ids[nsb] = t[g_start[g]].s;
    out->sb_pix_ptr[nsb] = npix;
    for (int32_t k = g_start[g]; k < g_start[g + 1]; k++) out->pix[npix++] = t[k].p;
    nsb++;
  }
  out->q_sb_ptr[nq] = nsb;
  out->sb_pix_ptr[nsb] = npix;
  out->nq = nq;
  out->nsb = nsb;
  out->npix = npix;

  out->pixels_per_bin = (int32_t *)calloc((size_t)out->total_static + 1, sizeof(int32_t));
  for (int32_t i = 0; i < pixels; i++) {
    if (sq[i] < 1 || dq[i] < 1) continue;
    if (sq[i] > out->total_static) {
      out->error = 1; /* Q5: pixels_per_bin[sqmap-1] out of bounds */
      continue;
    }
    out->pixels_per_bin[sq[i] - 1]++;
  }
  for (int32_t k = 0; k < nq; k++)
    if (out->q_ids[k] > nq) out->error = 1; /* Q7: g2.row(q-1) out of bounds */

  free(q_seen);
  free(t);
  free(g_start);
  free(erased);
  free(first_g);
  free(cnt_q);
  return out->error ? 1 : 0;
}

void xo_free_qmap(xo_qmap *q) {
  free(q->valid);
  free(q->sbin_mask);
  free(q->pixels_per_bin);
  free(q->q_ids);
  free(q->q_sb_ptr);
  free(q->sb_ids);
  free(q->sb_pix_ptr);
  free(q->pix);
  memset(q, 0, sizeof(*q));
}

/* --------------------------------------------------------------- filters */

typedef struct {
  int32_t n, cap;
  int32_t *idx;
  float *val;
} xo_row;

static void row_push(xo_row *r, int32_t f, float v) {
  if (r->n == r->cap) {
    int32_t c = r->cap ? 2 * r->cap : 100; /* Row(100) reserve, row.h:66-70 */
    r->idx = (int32_t *)realloc(r->idx, sizeof(int32_t) * (size_t)c);
    r->val = (float *)realloc(r->val, sizeof(float) * (size_t)c);
    r->cap = c;
  }
  r->idx[r->n] = f;
  r->val[r->n] = v;
  r->n++;
}

static void rows_from_lists(int32_t pixels, xo_row *lists, xo_rows *rows) {
  rows->pixels = pixels;
  rows->row_ptr = (int64_t *)malloc(sizeof(int64_t) * ((size_t)pixels + 1));
  int64_t tot = 0;
  for (int32_t i = 0; i < pixels; i++) {
    rows->row_ptr[i] = tot;
    tot += lists[i].n;
  }
  rows->row_ptr[pixels] = tot;
  rows->frame = (int32_t *)malloc(sizeof(int32_t) * (size_t)(tot ? tot : 1));
  rows->value = (float *)malloc(sizeof(float) * (size_t)(tot ? tot : 1));
  for (int32_t i = 0; i < pixels; i++) {
    if (lists[i].n) {
      memcpy(rows->frame + rows->row_ptr[i], lists[i].idx, sizeof(int32_t) * (size_t)lists[i].n);
      memcpy(rows->value + rows->row_ptr[i], lists[i].val, sizeof(float) * (size_t)lists[i].n);
    }
    free(lists[i].idx);
    free(lists[i].val);
  }
  free(lists);
}

static void side_alloc(const xo_filter_params *p, xo_side *s) {
  int partitions = (int)ceil((double)p->frames / p->static_window);
  s->pixels_sum = (float *)calloc((size_t)p->pixels, sizeof(float));
  s->frames_sum = (float *)calloc(2 * (size_t)p->frames, sizeof(float));
  s->partitions_mean = (float *)calloc((size_t)p->total_static + 1, sizeof(float));
  s->partial_mean =
      (float *)calloc((size_t)p->total_static * (size_t)partitions + 1, sizeof(float));
  s->timestamp_clock = (double *)calloc(2 * (size_t)p->real_frames + 1, sizeof(double));
  s->timestamp_ticks = (double *)calloc(2 * (size_t)p->real_frames + 1, sizeof(double));
}

/* The per-filter-frame tail shared by SparseFilter::Apply
 * (sparse_filter.cpp:160-192) and DenseFilter::Apply (dense_filter.cpp:176-208):
 * ascending pixel order, v = sum / average, push (frame, v), side sums. */
static void filter_frame_tail(const xo_filter_params *p, int frame_index, int *partition_no,
                              const float *pixels_value, const int16_t *sparse_map,
                              xo_row *lists, xo_side *s) {
  if (frame_index > 0 && (frame_index % p->static_window) == 0) (*partition_no)++;
  float f_sum = 0.0f;
  for (int32_t i = 0; i < p->pixels; i++) {
    if (sparse_map[i] == 0) continue;
    float v = pixels_value[i] / (float)p->average;
    s->pixels_sum[i] += v;
    f_sum += v;
    row_push(&lists[i], frame_index, v);
    int sbin = p->sbin_mask[i] - 1;
    s->partitions_mean[sbin] += v;
    s->partial_mean[*partition_no * p->total_static + sbin] += v;
  }
  s->frames_sum[frame_index] = (float)(frame_index + 1.0);
  s->frames_sum[frame_index + p->frames] = f_sum / (float)p->pixels;
}

/* SparseFilter::Apply, src/xpcs/filter/sparse_filter.cpp:115-193, called once
 * per filter frame with stride*average raw frames (main.cpp:258-268). */
int xo_sparse_filter(const xo_filter_params *p, const int32_t *idx, const int16_t *val,
                     const uint32_t *nnz, const double *clock, const double *ticks,
                     xo_rows *rows, xo_side *side) {
  int read_in = p->stride > 1 ? p->stride : p->average;
  if (p->stride > 1 && p->average > 1) read_in = p->stride * p->average;
  xo_row *lists = (xo_row *)calloc((size_t)p->pixels, sizeof(xo_row));
  float *pixels_value = (float *)malloc(sizeof(float) * (size_t)p->pixels);
  int16_t *sparse_map = (int16_t *)malloc(sizeof(int16_t) * (size_t)p->pixels);
  side_alloc(p, side);
  int nraw = p->frames * read_in;
  int64_t *off = (int64_t *)malloc(sizeof(int64_t) * ((size_t)nraw + 1));
  off[0] = 0;
  for (int g = 0; g < nraw; g++) off[g + 1] = off[g] + nnz[g];
  int raw = 0, partition_no = 0, bad = 0;
  for (int f = 0; f < p->frames; f++) {
    for (int32_t j = 0; j < p->pixels; j++) {
      pixels_value[j] = 0.0f;
      sparse_map[j] = 0;
    }
    for (int i = 0; i < read_in; i++) {
      int g = raw + i;
      side->timestamp_clock[g] = g + 1;
      side->timestamp_clock[g + p->real_frames] = clock ? clock[g] : 0.0;
      side->timestamp_ticks[g] = g + 1;
      side->timestamp_ticks[g + p->real_frames] = ticks ? ticks[g] : 0.0;
    }
    for (int i = 0; i < read_in; i += p->stride) {
      int64_t b = off[raw + i];
      for (uint32_t j = 0; j < nnz[raw + i]; j++) {
        int32_t pix = idx[b + j];
        if (pix < 0 || pix >= p->pixels) {
          bad = 1; /* the reference reads out of bounds here */
          continue;
        }
        if (p->pixel_mask[pix] != 0) {
          float v = (float)((double)(float)val[b + j] * p->flatfield[pix]);
          pixels_value[pix] += v;
          sparse_map[pix] = 1;
        }
      }
    }
    filter_frame_tail(p, f, &partition_no, pixels_value, sparse_map, lists, side);
    raw += read_in;
  }
  free(off);
  rows_from_lists(p->pixels, lists, rows);
  free(pixels_value);
  free(sparse_map);
  return bad;
}

/* DarkImage::Compute, src/xpcs/data_structure/dark_image.cpp:81-106: running
 * mean and M2 in double of raw*flat over the dark frames; std = sqrt(M2/n). */
void xo_dark_image(const int16_t *dark, int ndark, int pixels, const double *flat,
                   double *avg, double *std) {
  for (int j = 0; j < pixels; j++) {
    avg[j] = 0.0;
    std[j] = 0.0;
  }
  for (int i = 0; i < ndark; i++) {
    for (int j = 0; j < pixels; j++) {
      double tmp = avg[j];
      double pix = (double)(float)dark[(size_t)i * pixels + j] * flat[j];
      avg[j] += ((pix - avg[j]) / (double)(i + 1));
      std[j] += ((pix - tmp) * (pix - avg[j]));
    }
  }
  for (int j = 0; j < pixels; j++) std[j] = sqrt(std[j] / ndark);
}

/* DenseFilter::Apply, src/xpcs/filter/dense_filter.cpp:121-210 (quirk Q4: the
 * frame is dark-subtracted with its raw value, the dark mean includes flat). */
int xo_dense_filter(const xo_filter_params *p, const int16_t *raw_frames, const double *dark_avg,
                    const double *dark_std, float lld, float sigma, const double *clock,
                    const double *ticks, xo_rows *rows, xo_side *side) {
  int read_in = p->stride > 1 ? p->stride : p->average;
  if (p->stride > 1 && p->average > 1) read_in = p->stride * p->average;
  xo_row *lists = (xo_row *)calloc((size_t)p->pixels, sizeof(xo_row));
  float *pixels_value = (float *)malloc(sizeof(float) * (size_t)p->pixels);
  int16_t *sparse_map = (int16_t *)malloc(sizeof(int16_t) * (size_t)p->pixels);
  side_alloc(p, side);
  int raw = 0, partition_no = 0;
  for (int f = 0; f < p->frames; f++) {
    for (int i = 0; i < read_in; i++) {
      int g = raw + i;
      side->timestamp_clock[g] = g + 1;
      side->timestamp_clock[g + p->real_frames] = clock ? clock[g] : 0.0;
      side->timestamp_ticks[g] = g + 1;
      side->timestamp_ticks[g + p->real_frames] = ticks ? ticks[g] : 0.0;
    }
    for (int32_t j = 0; j < p->pixels; j++) {
      pixels_value[j] = 0.0f;
      sparse_map[j] = 0;
    }
    for (int i = 0; i < read_in; i += p->stride) {
      const int16_t *value = raw_frames + (size_t)(raw + i) * p->pixels;
      for (int32_t j = 0; j < p->pixels; j++) {
        if (p->pixel_mask[j] != 0) {
          float v = (float)value[j];
          float thresh = 0.0f;
          if (dark_avg) {
            v = (float)((double)v - dark_avg[j]);
            v = v > 0.0f ? v : 0.0f; /* std::max(v, 0.0f) */
            thresh = (float)((double)lld + (double)sigma * dark_std[j]);
          }
          if (v <= thresh) continue;
          sparse_map[j] = 1;
          v = (float)((double)v * p->flatfield[j]);
          pixels_value[j] += v;
        }
      }
    }
    filter_frame_tail(p, f, &partition_no, pixels_value, sparse_map, lists, side);
    raw += read_in;
  }
  rows_from_lists(p->pixels, lists, rows);
  free(pixels_value);
  free(sparse_map);
  return 0;
}

/* main.cpp:321-411: pixelSum /= frames; partial means /= pixels_per_sbin *
 * swindow over the floor(frames/swindow) full windows; total means /=
 * pixels_per_sbin * frames. */
void xo_finish_side(const xo_filter_params *p, const int32_t *ppb, xo_side *s) {
  for (int32_t i = 0; i < p->pixels; i++) s->pixels_sum[i] /= p->frames;
  int partitions = (int)floor((double)p->frames / p->static_window);
  for (int i = 0; i < p->total_static; i++) {
    for (int j = 0; j < partitions; j++) {
      float denominator = (float)ppb[i] * p->static_window;
      s->partial_mean[j * p->total_static + i] /= denominator;
    }
  }
  for (int i = 0; i < p->total_static; i++) {
    float denominator = (float)ppb[i] * p->frames;
    s->partitions_mean[i] /= denominator;
  }
}

void xo_free_rows(xo_rows *r) {
  free(r->row_ptr);
  free(r->frame);
  free(r->value);
  memset(r, 0, sizeof(*r));
}

void xo_free_side(xo_side *s) {
  free(s->pixels_sum);
  free(s->frames_sum);
  free(s->partitions_mean);
  free(s->partial_mean);
  free(s->timestamp_clock);
  free(s->timestamp_ticks);
  memset(s, 0, sizeof(*s));
}

/* ------------------------------------------------------------- multi-tau */

/* std::lower_bound as libstdc++ implements it (binary search by halving the
 * remaining length); the reference calls it at src/xpcs/corr.cpp:406. */
static int32_t lower_bound_i32(const int32_t *a, int32_t n, int32_t x) {
  int32_t first = 0, len = n;
  while (len > 0) {
    int32_t half = len >> 1;
    if (a[first + half] < x) {
      first = first + half + 1;
      len = len - half - 1;
    } else {
      len = half;
    }
  }
  return first;
}

/* Corr::multiTau2, src/xpcs/corr.cpp:315-431.  For each pixel with events, for
 * each (level, tau): on a level change halve lastframe (odd -> -1 first) and
 * compact the row in place (idx/2, merge equal neighbours by float add, stop at
 * the first index >= lastframe, then every live value /= 2) (:349-390); then
 * accumulate IP, G2 (partner found by lower_bound over the WHOLE row buffer,
 * stale tail included: quirk Q1) and IF (:395-418) and divide by
 * (lastframe - tau) (:420-424). */
int xo_multitau2(const xo_rows *rows, int frames, int dpl, int mode, int threads, float *G2s,
                 float *IPs, float *IFs) {
  int cap = 4096;
  int32_t *dl = (int32_t *)malloc(sizeof(int32_t) * cap);
  int32_t *dt = (int32_t *)malloc(sizeof(int32_t) * cap);
  int D = xo_delays(frames, dpl, dl, dt, cap);
  int32_t pixels = rows->pixels;
  size_t tot = (size_t)D * pixels;
  memset(G2s, 0, sizeof(float) * tot);
  memset(IPs, 0, sizeof(float) * tot);
  memset(IFs, 0, sizeof(float) * tot);
  int32_t maxlen = 0, nvalid = 0;
  for (int32_t p = 0; p < pixels; p++) {
    int32_t n = (int32_t)(rows->row_ptr[p + 1] - rows->row_ptr[p]);
    if (n > maxlen) maxlen = n;
    if (n > 0) nvalid++;
  }
  int32_t *valid = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nvalid ? nvalid : 1));
  nvalid = 0;
  for (int32_t p = 0; p < pixels; p++)
    if (rows->row_ptr[p + 1] > rows->row_ptr[p]) valid[nvalid++] = p;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif

#pragma omp parallel
  {
    int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(maxlen ? maxlen : 1));
    float *val = (float *)malloc(sizeof(float) * (size_t)(maxlen ? maxlen : 1));
#pragma omp for schedule(dynamic, 20)
    for (int32_t i = 0; i < nvalid; i++) {
      int32_t pixel = valid[i];
      int32_t n0 = (int32_t)(rows->row_ptr[pixel + 1] - rows->row_ptr[pixel]);
      memcpy(idx, rows->frame + rows->row_ptr[pixel], sizeof(int32_t) * (size_t)n0);
      memcpy(val, rows->value + rows->row_ptr[pixel], sizeof(float) * (size_t)n0);
      int ll = 0;
      int lastframe = frames;
      int lastIndex = n0;
      for (int k = 0; k < D; k++) {
        int level = dl[k];
        int tau = dt[k];
        if (ll != level) {
          if (lastframe % 2) lastframe -= 1;
          lastframe = lastframe / 2;
          int index = 0, cnt = 0;
          int i0 = (int)(idx[cnt] / 2.0), i1;
          if (lastIndex > 0 && i0 < lastframe) {
            idx[index] = i0;
            cnt = 1;
          }
          while (cnt < lastIndex) {
            i1 = (int)(idx[cnt] / 2.0);
            if (i1 >= lastframe) break;
            if (i1 == i0) {
              val[index] += val[cnt];
            } else {
              idx[++index] = i1;
              val[index] = val[cnt];
            }
            i0 = i1;
            cnt++;
          }
          lastIndex = index + 1;
          for (int r = 0; r < lastIndex; r++) val[r] /= 2.0f;
        }
        if (level > 0) tau = (int)(tau / pow(2, level));
        size_t g = (size_t)k * pixels + pixel;
        int32_t search_n = mode == 0 ? n0 : lastIndex;
        for (int r = 0; r < lastIndex; r++) {
          int src = idx[r];
          if (src < (lastframe - tau)) {
            IPs[g] += val[r];
            int32_t pos = lower_bound_i32(idx, search_n, src + tau);
            if (pos != search_n) {
              if (pos < lastIndex && idx[pos] == (src + tau)) G2s[g] += val[r] * val[pos];
            }
          }
          if (src >= tau && src < lastframe) IFs[g] += val[r];
        }
        if ((lastframe - tau) > 0) {
          G2s[g] /= (lastframe - tau);
          IPs[g] /= (lastframe - tau);
          IFs[g] /= (lastframe - tau);
        }
        ll = level;
      }
    }
    free(idx);
    free(val);
  }
  free(valid);
  free(dl);
  free(dt);
  return D;
}

/* --------------------------------------------------------- normalisation */

/* Corr::normalizeG2s, src/xpcs/corr.cpp:927-1091, in float32 exactly as the
 * reference's Eigen expressions evaluate element-wise:
 *  - per sbin, sum G2/IP/IF rows over its pixels in mapping order (:966-991),
 *    divide each by the pixel count, then g2Sums /= (ipSums * ifSums) (:998-1013);
 *  - per q, add the non-NaN sbin ratios (ascending sbin) and divide by their
 *    count (:1018-1040);
 *  - per q, running mean / M2 over the pixels of G2/(IP*IF) with NaN -> 0 and
 *    still counted (quirk Q8), stderr = sqrt(1/n) * sqrt(M2/n) (:1043-1087). */
int xo_normalize_f32(const xo_qmap *q, int D, const float *G2, const float *IP, const float *IF,
                     float *g2, float *stderr_) {
  int S = q->total_static, P = q->pixels, NQ = q->nq;
  if (q->error) return 1;
  float *g2s = (float *)calloc((size_t)S * D + 1, sizeof(float));
  float *ips = (float *)calloc((size_t)S * D + 1, sizeof(float));
  float *ifs = (float *)calloc((size_t)S * D + 1, sizeof(float));
  int32_t *ppc = (int32_t *)calloc((size_t)S + 1, sizeof(int32_t));
  for (size_t k = 0; k < (size_t)D * NQ; k++) {
    g2[k] = 0.0f;
    stderr_[k] = 0.0f;
  }
  for (int qi = 0; qi < NQ; qi++) {
    for (int e = q->q_sb_ptr[qi]; e < q->q_sb_ptr[qi + 1]; e++) {
      int s = q->sb_ids[e] - 1;
      for (int k = q->sb_pix_ptr[e]; k < q->sb_pix_ptr[e + 1]; k++) {
        int p = q->pix[k];
        for (int t = 0; t < D; t++) {
          g2s[(size_t)s * D + t] += G2[(size_t)t * P + p];
          ips[(size_t)s * D + t] += IP[(size_t)t * P + p];
          ifs[(size_t)s * D + t] += IF[(size_t)t * P + p];
        }
        ppc[s] += 1;
      }
    }
  }
  for (int qi = 0; qi < NQ; qi++) {
    for (int e = q->q_sb_ptr[qi]; e < q->q_sb_ptr[qi + 1]; e++) {
      int s = q->sb_ids[e] - 1;
      float c = (float)ppc[s];
      for (int t = 0; t < D; t++) {
        size_t o = (size_t)s * D + t;
        g2s[o] /= c;
        ips[o] /= c;
        ifs[o] /= c;
        g2s[o] = g2s[o] / (ips[o] * ifs[o]);
      }
    }
  }
  float *counts = (float *)malloc(sizeof(float) * (size_t)D);
  for (int qi = 0; qi < NQ; qi++) {
    int row = q->q_ids[qi] - 1;
    for (int t = 0; t < D; t++) counts[t] = 0.0f;
    for (int e = q->q_sb_ptr[qi]; e < q->q_sb_ptr[qi + 1]; e++) {
      int s = q->sb_ids[e] - 1;
      for (int t = 0; t < D; t++) {
        float r = g2s[(size_t)s * D + t];
        g2[(size_t)t * NQ + row] += isnan(r) ? 0.0f : r;
        counts[t] += isnan(r) ? 0.0f : 1.0f;
      }
    }
    for (int t = 0; t < D; t++) g2[(size_t)t * NQ + row] = g2[(size_t)t * NQ + row] / counts[t];
  }
  float *avg = (float *)malloc(sizeof(float) * (size_t)D);
  float *stdv = (float *)malloc(sizeof(float) * (size_t)D);
  float *samples = (float *)malloc(sizeof(float) * (size_t)D);
  for (int qi = 0; qi < NQ; qi++) {
    int row = q->q_ids[qi] - 1;
    for (int t = 0; t < D; t++) {
      avg[t] = 0.0f;
      stdv[t] = 0.0f;
      samples[t] = 0.0f;
    }
    for (int e = q->q_sb_ptr[qi]; e < q->q_sb_ptr[qi + 1]; e++) {
      for (int k = q->sb_pix_ptr[e]; k < q->sb_pix_ptr[e + 1]; k++) {
        int p = q->pix[k];
        for (int t = 0; t < D; t++) {
          size_t o = (size_t)t * P + p;
          float tmpAvg = avg[t];
          float x = G2[o] / (IP[o] * IF[o]);
          x = isnan(x) ? 0.0f : x;
          samples[t] += 1.0f;
          float tmp0 = x - tmpAvg;
          float tmp00 = tmp0 / samples[t];
          tmp00 = isnan(tmp00) ? 0.0f : tmp00;
          avg[t] += tmp00;
          float tmp1 = x - tmpAvg;
          float tmp2 = x - avg[t];
          float tmp3 = tmp1 * tmp2;
          stdv[t] += tmp3;
        }
      }
    }
    for (int t = 0; t < D; t++) {
      float stdNorm = stdv[t] / samples[t];
      float inv = 1.0f / samples[t];
      stderr_[(size_t)t * NQ + row] = sqrtf(inv) * sqrtf(stdNorm);
    }
  }
  free(g2s);
  free(ips);
  free(ifs);
  free(ppc);
  free(counts);
  free(avg);
  free(stdv);
  free(samples);
  return 0;
}

/* The same normalisation evaluated in double precision, reference order. */
int xo_normalize_f64(const xo_qmap *q, int D, const float *G2, const float *IP, const float *IF,
                     double *g2, double *stderr_) {
  int S = q->total_static, P = q->pixels, NQ = q->nq;
  if (q->error) return 1;
  double *g2s = (double *)calloc((size_t)S * D + 1, sizeof(double));
  double *ips = (double *)calloc((size_t)S * D + 1, sizeof(double));
  double *ifs = (double *)calloc((size_t)S * D + 1, sizeof(double));
  int32_t *ppc = (int32_t *)calloc((size_t)S + 1, sizeof(int32_t));
  for (size_t k = 0; k < (size_t)D * NQ; k++) {
    g2[k] = 0.0;
    stderr_[k] = 0.0;
  }
  for (int qi = 0; qi < NQ; qi++)
    for (int e = q->q_sb_ptr[qi]; e < q->q_sb_ptr[qi + 1]; e++) {
      int s = q->sb_ids[e] - 1;
      for (int k = q->sb_pix_ptr[e]; k < q->sb_pix_ptr[e + 1]; k++) {
        int p = q->pix[k];
        for (int t = 0; t < D; t++) {
          g2s[(size_t)s * D + t] += G2[(size_t)t * P + p];
          ips[(size_t)s * D + t] += IP[(size_t)t * P + p];
          ifs[(size_t)s * D + t] += IF[(size_t)t * P + p];
        }
        ppc[s] += 1;
      }
    }
  for (int qi = 0; qi < NQ; qi++)
    for (int e = q->q_sb_ptr[qi]; e < q->q_sb_ptr[qi + 1]; e++) {
      int s = q->sb_ids[e] - 1;
      double c = (double)ppc[s];
      for (int t = 0; t < D; t++) {
        size_t o = (size_t)s * D + t;
        g2s[o] /= c;
        ips[o] /= c;
        ifs[o] /= c;
        g2s[o] = g2s[o] / (ips[o] * ifs[o]);
      }
    }
  double *counts = (double *)malloc(sizeof(double) * (size_t)D);
  for (int qi = 0; qi < NQ; qi++) {
    int row = q->q_ids[qi] - 1;
    for (int t = 0; t < D; t++) counts[t] = 0.0;
    for (int e = q->q_sb_ptr[qi]; e < q->q_sb_ptr[qi + 1]; e++) {
      int s = q->sb_ids[e] - 1;
      for (int t = 0; t < D; t++) {
        double r = g2s[(size_t)s * D + t];
        g2[(size_t)t * NQ + row] += isnan(r) ? 0.0 : r;
        counts[t] += isnan(r) ? 0.0 : 1.0;
      }
    }
    for (int t = 0; t < D; t++) g2[(size_t)t * NQ + row] = g2[(size_t)t * NQ + row] / counts[t];
  }
  double *avg = (double *)malloc(sizeof(double) * (size_t)D);
  double *stdv = (double *)malloc(sizeof(double) * (size_t)D);
  double *samples = (double *)malloc(sizeof(double) * (size_t)D);
  for (int qi = 0; qi < NQ; qi++) {
    int row = q->q_ids[qi] - 1;
    for (int t = 0; t < D; t++) avg[t] = stdv[t] = samples[t] = 0.0;
    for (int e = q->q_sb_ptr[qi]; e < q->q_sb_ptr[qi + 1]; e++)
      for (int k = q->sb_pix_ptr[e]; k < q->sb_pix_ptr[e + 1]; k++) {
        int p = q->pix[k];
        for (int t = 0; t < D; t++) {
          size_t o = (size_t)t * P + p;
          double tmpAvg = avg[t];
          double x = (double)G2[o] / ((double)IP[o] * (double)IF[o]);
          x = isnan(x) ? 0.0 : x;
          samples[t] += 1.0;
          double tmp00 = (x - tmpAvg) / samples[t];
          tmp00 = isnan(tmp00) ? 0.0 : tmp00;
          avg[t] += tmp00;
          stdv[t] += (x - tmpAvg) * (x - avg[t]);
        }
      }
    for (int t = 0; t < D; t++)
      stderr_[(size_t)t * NQ + row] = sqrt(1.0 / samples[t]) * sqrt(stdv[t] / samples[t]);
  }
  free(g2s);
  free(ips);
  free(ifs);
  free(ppc);
  free(counts);
  free(avg);
  free(stdv);
  free(samples);
  return 0;
}
