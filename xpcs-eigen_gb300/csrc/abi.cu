// C ABI of libxpcs_gpu (include/xpcs_gpu.h): series lifecycle, ingest,
// multi-tau, normalisation, results and the per-stage CUDA-event tracer.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <new>

#include "xpcs_internal.h"

using namespace xg;

namespace {
thread_local std::string g_last_error;
}

namespace xg {
thread_local int64_t tl_launches = 0;
void xpcs_set_last_error(const char *msg) { g_last_error.assign(msg); }

namespace {
constexpr int ACCT_DEVICES = 64;
std::atomic<uint64_t> g_dev_used[ACCT_DEVICES];
std::atomic<uint64_t> g_dev_limit[ACCT_DEVICES];  // 0: no limit

int acct_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= ACCT_DEVICES) return 0;
  return dev;
}
}  // namespace

void *dev_alloc(size_t bytes, cudaStream_t st) {
  const int dev = acct_device();
  const uint64_t lim = g_dev_limit[dev].load();
  const uint64_t was = g_dev_used[dev].fetch_add(bytes);
  if (lim && was + bytes > lim) {
    g_dev_used[dev].fetch_sub(bytes);
    throw Error(XPCS_ERR_OUT_OF_MEMORY,
                "device memory limit reached: " + std::to_string(was + bytes) + " bytes asked, " +
                    std::to_string(lim) + " allowed on device " + std::to_string(dev));
  }
  void *q = nullptr;
  const cudaError_t e = cudaMallocAsync(&q, bytes, st);
  if (e != cudaSuccess) {
    g_dev_used[dev].fetch_sub(bytes);
    cudaGetLastError();
    throw Error(e == cudaErrorMemoryAllocation ? XPCS_ERR_OUT_OF_MEMORY : XPCS_ERR_CUDA,
                std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
  }
  return q;
}

void dev_free(void *p, size_t bytes, cudaStream_t st) {
  if (!p) return;
  cudaFreeAsync(p, st);
  g_dev_used[acct_device()].fetch_sub(bytes);
}
}

namespace {

template <class F>
int guarded(F &&f) {
  try {
    f();
    g_last_error.clear();
    return XPCS_OK;
  } catch (const Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return XPCS_ERR_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return XPCS_ERR_INVALID_ARGUMENT;
  }
}

void need(bool ok, const char *msg) {
  if (!ok) throw Error(XPCS_ERR_INVALID_ARGUMENT, msg);
}

template <class T>
void upload(DBuf<T> &b, const std::vector<T> &v, cudaStream_t st) {
  b.reserve(v.size() ? v.size() : 1, st);
  if (!v.empty())
    XG_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
}

// Wait for the stream and turn device error words into a status.
void sync_and_check(Series &s) {
  XG_CUDA(cudaStreamSynchronize(s.stream));
  if (s.stats.p) {
    DevStats st{};
    XG_CUDA(cudaMemcpy(&st, s.stats.p, sizeof(DevStats), cudaMemcpyDeviceToHost));
    if (st.error & DEVERR_PIXEL_INDEX)
      throw Error(XPCS_ERR_INPUT, "a sparse frame holds a pixel index outside the detector");
    if (st.error & DEVERR_WAIT)
      throw Error(XPCS_ERR_CUDA, "an asynchronous copy did not complete within its wait limit");
  }
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) XG_CUDA(cudaSetDevice(dev));
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

void init_series(Series &s) {
  XG_CUDA(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
  for (auto &e : s.ev) XG_CUDA(cudaEventCreate(&e));
}

void free_series(Series *s) {
  if (!s) return;
  if (s->stream) {
    DeviceGuard g(s->device);
    cudaStream_t st = s->stream;
    cudaStreamSynchronize(st);
    DBuf<int32_t> *i32[] = {&s->raw_idx, &s->frA, &s->frB, &s->row_len,
                            &s->flist, &s->wlist, &s->llist, &s->ev_frame, &s->sc_frame,
                            &s->n_q_entry_ptr,
                            &s->n_entry_sbin, &s->n_entry_pix_ptr, &s->n_pix, &s->n_q_row,
                            &s->n_ch_k0, &s->n_ch_k1, &s->n_e_chunk_ptr, &s->d_sbin,
                            &s->d_ppb};
    for (auto *b : i32) b->release(st);
    DBuf<float> *f32[] = {&s->vA, &s->vB, &s->ev_val, &s->pixels_sum, &s->sc_val, &s->G2,
                          &s->IP, &s->IF, &s->n_ratio32, &s->n_g2f, &s->n_sef, &s->n_tg,
                          &s->n_ti, &s->n_tf, &s->n_tx};
    for (auto *b : f32) b->release(st);
    s->raw_val.release(st);
    s->raw_valf.release(st);
    s->dark_avg.release(st);
    s->dark_std.release(st);
    s->rmin.release(st);
    s->dn_counts.release(st);
    s->dn_offsets.release(st);
    s->dn_frame_end.release(st);
    s->dn_prep.release(st);
    s->dn_pend.release(st);
    s->dn_tot.release(st);
    s->dn_sum.release(st);
    s->blk_pk.release(st);
    s->d_blk_r0.release(st);
    s->d_frame_off.release(st);
    s->d_frame_map.release(st);
    s->d_chunk_frame.release(st);
    s->row_ptr.release(st);
    s->d_mask.release(st);
    s->pclass.release(st);
    s->scan_tmp.release(st);
    s->plan.release(st);
    s->d_flat.release(st);
    s->n_part.release(st);
    s->side_pos.release(st);
    s->side_out.release(st);
    DBuf<int32_t> *tti[] = {&s->tt_row_pix, &s->tt_row_grp, &s->tt_grp_ptr, &s->tt_order};
    for (auto *b : tti) b->release(st);
    DBuf<float> *ttf[] = {&s->tt_V, &s->tt_sg, &s->tt_sga, &s->tt_C, &s->tt_full, &s->tt_part};
    for (auto *b : ttf) b->release(st);
    s->d_fscale.release(st);
    s->n_unsafe.release(st);
    s->tt_err.release(st);
    s->tt_flags.release(st);
    s->tt_XT.release(st);
    s->tt_S.release(st);
    s->tt_bound.release(st);
    s->tt_Gi.release(st);
    s->tt_sgd.release(st);
    s->tt_Cacc.release(st);
    s->tt_Cq.release(st);
    s->tt_Gf.release(st);
    s->n_g2.release(st);
    s->n_se.release(st);
    s->keyA.release(st);
    s->keyB.release(st);
    s->hist.release(st);
    s->hist_scan.release(st);
    s->d_blk_base.release(st);
    s->blk_fr.release(st);
    s->blk_val.release(st);
    s->blk_off.release(st);
    s->blk_len.release(st);
    s->blk_rp.release(st);
    s->blk_tot.release(st);
    s->stats.release(st);
    cudaStreamSynchronize(st);
    for (auto &e : s->ev)
      if (e) cudaEventDestroy(e);
    cudaStreamDestroy(st);
  }
  delete s;
}

}  // namespace

extern "C" {

int xpcs_abi_version(void) { return XPCS_GPU_ABI_VERSION; }

const char *xpcs_last_error(void) { return g_last_error.c_str(); }

int xpcs_delay_schedule(int32_t frames, int32_t dpl, int32_t *level, int32_t *tau,
                        int32_t capacity, int32_t *count) {
  return guarded([&] {
    need(frames >= 0 && dpl >= 0 && capacity >= 0, "negative argument");
    DelaySchedule d = delay_schedule(frames, dpl);
    int n = (int)d.level.size();
    for (int k = 0; k < n && k < capacity; k++) {
      if (level) level[k] = d.level[k];
      if (tau) tau[k] = d.tau[k];
    }
    if (count) *count = n;
  });
}

int xpcs_series_create(const xpcs_series_desc *desc, xpcs_series **out) {
  Series *s = nullptr;
  int rc = guarded([&] {
    need(desc && out, "null argument");
    need(desc->width > 0 && desc->height > 0, "detector size must be positive");
    need((int64_t)desc->width * desc->height < (int64_t)1 << 30, "detector too large");
    need(desc->frames >= 0, "frame count must be non-negative");
    need(desc->delays_per_level >= 0, "delays_per_level must be non-negative");
    need(desc->stride_frames >= 1 && desc->avg_frames >= 1, "stride/avg must be >= 1");
    need(desc->static_window >= 1, "static_window must be >= 1");
    need(desc->dqmap && desc->sqmap, "dqmap and sqmap are required");
    need(desc->dense == 0 || desc->dense == 1, "dense must be 0 or 1");
    need(desc->normalize_by_framesum == 0 || desc->normalize_by_framesum == 1,
         "normalize_by_framesum must be 0 or 1");
    s = new Series();
    s->desc = *desc;
    s->desc.dqmap = nullptr;
    s->desc.sqmap = nullptr;
    s->desc.flatfield = nullptr;
    s->device = desc->device;
    s->P = desc->width * desc->height;
    s->F = desc->frames;
    s->R_in = desc->stride_frames * desc->avg_frames;
    s->dense_px = desc->dense && s->R_in == 1;
    s->delays = delay_schedule(s->F, desc->delays_per_level);
    s->D = (int32_t)s->delays.level.size();
    s->qmap = build_qmap(desc->dqmap, desc->sqmap, s->P);
    if (!s->qmap.error.empty()) throw Error(XPCS_ERR_QMAP, s->qmap.error);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      throw Error(XPCS_ERR_NO_DEVICE, "no CUDA device");
    need(desc->device >= 0 && desc->device < ndev, "device ordinal out of range");
    DeviceGuard g(s->device);
    init_series(*s);
    cudaStream_t st = s->stream;
    upload(s->d_mask, s->qmap.valid, st);
    if (desc->flatfield) {
      std::vector<double> flat(desc->flatfield, desc->flatfield + s->P);
      upload(s->d_flat, flat, st);
      s->has_flat = true;
    }
    const QMap &q = s->qmap;
    upload(s->n_q_entry_ptr, q.q_entry_ptr, st);
    upload(s->n_entry_sbin, q.entry_sbin, st);
    upload(s->n_entry_pix_ptr, q.entry_pix_ptr, st);
    upload(s->n_pix, q.pix, st);
    std::vector<int32_t> rows(q.q_ids.size());
    for (size_t k = 0; k < rows.size(); k++) rows[k] = q.q_ids[k] - 1;
    upload(s->n_q_row, rows, st);
    std::vector<int32_t> sb(s->P);
    for (int32_t i = 0; i < s->P; i++) sb[i] = q.valid[i] ? q.sbin[i] - 1 : -1;
    upload(s->d_sbin, sb, st);
    upload(s->d_ppb, q.pixels_per_bin, st);
    build_norm_chunks(*s);
    XG_CUDA(cudaStreamSynchronize(st));
    *out = (xpcs_series *)s;
  });
  if (rc != XPCS_OK && s) free_series(s);
  return rc;
}

void xpcs_series_destroy(xpcs_series *h) { free_series((Series *)h); }

int xpcs_series_reset(xpcs_series *h) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    XG_CUDA(cudaStreamSynchronize(s.stream));
    s.frame_off.assign(1, 0);
    reset_blocks(s);
    s.raw_events = 0;
    s.rmin_ready = s.rmin_ready && s.has_dark;
    s.raw_frames = 0;
    s.frame_off_dirty = true;
    s.have_multitau = false;
    s.have_norm64 = s.have_norm32 = false;
    s.tt.ready = false;
    s.timed_h2d = false;
    s.h2d_ms_acc = 0.f;
    s.generation++;
  });
}

int xpcs_series_set_block_frames(xpcs_series *h, int32_t block_frames) {
  return guarded([&] {
    need(h, "null handle");
    need(block_frames >= 0, "block_frames must be non-negative");
    Series &s = *(Series *)h;
    if (s.raw_frames > 0)
      throw Error(XPCS_ERR_STATE, "set the block size before ingesting frames");
    s.block_frames = block_frames;
  });
}

int xpcs_series_get_info(xpcs_series *h, xpcs_series_info *info) {
  return guarded([&] {
    need(h && info, "null argument");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    sync_and_check(s);
    std::memset(info, 0, sizeof(*info));
    info->pixels = s.P;
    info->delays = s.D;
    info->total_static = s.qmap.total_static;
    info->total_dynamic = s.qmap.total_dynamic;
    info->qbins = s.qmap.nq();
    info->raw_frames = s.raw_frames;
    info->raw_events = s.raw_events;
    if (s.have_multitau && s.stats.p) {
      DevStats st{};
      XG_CUDA(cudaMemcpy(&st, s.stats.p, sizeof(st), cudaMemcpyDeviceToHost));
      info->events = (int64_t)st.events;
      info->valid_pixels = st.nvalid;
      info->float_path_pixels = st.nfloat;
    }
  });
}

static void ingest_common(Series &s, const int32_t *idx, const int16_t *val, const uint32_t *nnz,
                          int32_t nframes, bool on_device) {
  need(nframes >= 0, "negative frame count");
  need(nnz || nframes == 0, "null nnz");
  DeviceGuard g(s.device);
  cudaStream_t st = s.stream;
  int64_t add = 0;
  for (int32_t r = 0; r < nframes; r++) add += nnz[r];
  need(add == 0 || (idx && val), "null event arrays");
  const int64_t old = s.raw_events, tot = old + add;
  need(tot < ((int64_t)1 << 32), "more than 2^32 raw events in one series");
  s.raw_idx.grow((size_t)(tot ? tot : 1), (size_t)old, st);
  s.raw_val.grow((size_t)(tot ? tot : 1), (size_t)old, st);
  if (!s.timed_h2d) {
    XG_CUDA(cudaEventRecord(s.ev[0], st));
    s.timed_h2d = true;
  }
  if (add) {
    cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    XG_CUDA(cudaMemcpyAsync(s.raw_idx.p + old, idx, sizeof(int32_t) * add, kind, st));
    XG_CUDA(cudaMemcpyAsync(s.raw_val.p + old, val, sizeof(int16_t) * add, kind, st));
  }
  XG_CUDA(cudaEventRecord(s.ev[1], st));
  for (int32_t r = 0; r < nframes; r++) s.frame_off.push_back(s.frame_off.back() + nnz[r]);
  s.raw_events = tot;
  s.raw_frames += nframes;
  s.frame_off_dirty = true;
  s.have_multitau = false;
  s.tt.ready = false;
  s.generation++;
  transpose_ready_blocks(s);
}

int xpcs_ingest_sparse(xpcs_series *h, const int32_t *idx, const int16_t *val,
                       const uint32_t *nnz, int32_t nframes) {
  return guarded([&] {
    need(h, "null handle");
    if (((Series *)h)->desc.dense) throw Error(XPCS_ERR_STATE, "series was created for dense frames");
    ingest_common(*(Series *)h, idx, val, nnz, nframes, false);
  });
}

int xpcs_ingest_sparse_device(xpcs_series *h, const int32_t *idx, const int16_t *val,
                              const uint32_t *nnz, int32_t nframes) {
  return guarded([&] {
    need(h, "null handle");
    if (((Series *)h)->desc.dense) throw Error(XPCS_ERR_STATE, "series was created for dense frames");
    ingest_common(*(Series *)h, idx, val, nnz, nframes, true);
  });
}

int xpcs_set_dark(xpcs_series *h, const int16_t *dark, int32_t ndark) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    if (!s.desc.dense) throw Error(XPCS_ERR_STATE, "darks apply to dense series only");
    if (s.raw_frames > 0) throw Error(XPCS_ERR_STATE, "set the darks before ingesting frames");
    need(ndark >= 0 && (ndark == 0 || dark), "bad dark frames");
    DeviceGuard g(s.device);
    dense_set_dark(s, dark, ndark);
    s.generation++;
  });
}

static int ingest_dense_common(xpcs_series *h, const int16_t *frames, int32_t nframes, bool dev) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    if (!s.desc.dense) throw Error(XPCS_ERR_STATE, "series was created for sparse frames");
    need(nframes >= 0 && (nframes == 0 || frames), "bad frames");
    DeviceGuard g(s.device);
    if (!s.timed_h2d) {
      XG_CUDA(cudaEventRecord(s.ev[0], s.stream));
      s.timed_h2d = true;
    }
    dense_ingest(s, frames, nframes, dev);
    s.generation++;
    s.have_multitau = false;
    s.tt.ready = false;
    transpose_ready_blocks(s);
    XG_CUDA(cudaEventRecord(s.ev[1], s.stream));
  });
}

int xpcs_ingest_dense(xpcs_series *h, const int16_t *frames, int32_t nframes) {
  return ingest_dense_common(h, frames, nframes, false);
}

int xpcs_ingest_dense_device(xpcs_series *h, const int16_t *frames, int32_t nframes) {
  return ingest_dense_common(h, frames, nframes, true);
}

int xpcs_get_dark(xpcs_series *h, double *avg, double *std_) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    dense_get_dark(s, avg, std_);
  });
}

int xpcs_multitau(xpcs_series *h, int32_t mode) {
  return guarded([&] {
    need(h, "null handle");
    need(mode == XPCS_MODE_REFERENCE || mode == XPCS_MODE_EXACT, "unknown mode");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    const int64_t l0 = tl_launches;
    XG_CUDA(cudaEventRecord(s.ev[2], s.stream));
    run_filter_transpose(s);
    XG_CUDA(cudaEventRecord(s.ev[3], s.stream));
    run_multitau(s, mode);
    s.launches = (int32_t)(tl_launches - l0);
    s.have_multitau = true;
    s.have_norm64 = s.have_norm32 = false;
    s.timed_h2d = false;
  });
}

int xpcs_get_g2ipif(xpcs_series *h, float *G2, float *IP, float *IF) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    if (!s.have_multitau) throw Error(XPCS_ERR_STATE, "xpcs_multitau has not run");
    DeviceGuard g(s.device);
    const size_t n = (size_t)s.D * s.P;
    XG_CUDA(cudaEventRecord(s.ev[9], s.stream));
    if (G2 && n) XG_CUDA(cudaMemcpyAsync(G2, s.G2.p, 4 * n, cudaMemcpyDeviceToHost, s.stream));
    if (IP && n) XG_CUDA(cudaMemcpyAsync(IP, s.IP.p, 4 * n, cudaMemcpyDeviceToHost, s.stream));
    if (IF && n) XG_CUDA(cudaMemcpyAsync(IF, s.IF.p, 4 * n, cudaMemcpyDeviceToHost, s.stream));
    XG_CUDA(cudaEventRecord(s.ev[10], s.stream));
    sync_and_check(s);
  });
}

int xpcs_normalize(xpcs_series *h, double *g2, double *se, float *g2f, float *sef) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    if (!s.have_multitau) throw Error(XPCS_ERR_STATE, "xpcs_multitau has not run");
    DeviceGuard g(s.device);
    cudaStream_t st = s.stream;
    const bool w64 = g2 || se, w32 = g2f || sef;
    const int64_t l0 = tl_launches;
    XG_CUDA(cudaEventRecord(s.ev[7], st));
    run_normalize(s, w64, w32);
    s.have_norm64 = w64;
    s.have_norm32 = w32;
    s.launches += (int32_t)(tl_launches - l0);
    XG_CUDA(cudaEventRecord(s.ev[8], st));
    const size_t n = (size_t)s.D * s.qmap.nq();
    if (n) {
      if (g2) XG_CUDA(cudaMemcpyAsync(g2, s.n_g2.p, 8 * n, cudaMemcpyDeviceToHost, st));
      if (se) XG_CUDA(cudaMemcpyAsync(se, s.n_se.p, 8 * n, cudaMemcpyDeviceToHost, st));
      if (g2f) XG_CUDA(cudaMemcpyAsync(g2f, s.n_g2f.p, 4 * n, cudaMemcpyDeviceToHost, st));
      if (sef) XG_CUDA(cudaMemcpyAsync(sef, s.n_sef.p, 4 * n, cudaMemcpyDeviceToHost, st));
    }
    XG_CUDA(cudaEventRecord(s.ev[11], st));
    sync_and_check(s);
  });
}

int xpcs_get_normalized(xpcs_series *h, double *g2, double *se, float *g2f, float *sef) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    if ((g2 || se) && !s.have_norm64)
      throw Error(XPCS_ERR_STATE, "no float64 normalisation has run since the last change");
    if ((g2f || sef) && !s.have_norm32)
      throw Error(XPCS_ERR_STATE, "no float32 normalisation has run since the last change");
    DeviceGuard g(s.device);
    cudaStream_t st = s.stream;
    const size_t n = (size_t)s.D * s.qmap.nq();
    if (n) {
      if (g2) XG_CUDA(cudaMemcpyAsync(g2, s.n_g2.p, 8 * n, cudaMemcpyDeviceToHost, st));
      if (se) XG_CUDA(cudaMemcpyAsync(se, s.n_se.p, 8 * n, cudaMemcpyDeviceToHost, st));
      if (g2f) XG_CUDA(cudaMemcpyAsync(g2f, s.n_g2f.p, 4 * n, cudaMemcpyDeviceToHost, st));
      if (sef) XG_CUDA(cudaMemcpyAsync(sef, s.n_sef.p, 4 * n, cudaMemcpyDeviceToHost, st));
    }
    sync_and_check(s);
  });
}

int xpcs_side_stats(xpcs_series *h, float *pixel_sum, float *frame_sum,
                    float *partition_mean_total, float *partition_mean_partial) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    if (!s.have_multitau && !s.tt.ready)
      throw Error(XPCS_ERR_STATE, "neither xpcs_multitau nor xpcs_twotime has run");
    DeviceGuard g(s.device);
    sync_and_check(s);
    run_side_stats(s, SideOut{pixel_sum, frame_sum, partition_mean_total, partition_mean_partial});
  });
}

int xpcs_twotime(xpcs_series *h, const xpcs_twotime_desc *d, int32_t mode,
                 xpcs_twotime_info *info) {
  return guarded([&] {
    need(h && d, "null argument");
    need(mode == XPCS_MODE_REFERENCE || mode == XPCS_MODE_EXACT ||
             mode == XPCS_TWOTIME_EXACT_CUDA_CORES,
         "unknown two-time mode");
    need(d->nqbins >= 0 && (d->nqbins == 0 || d->qbins), "bad q-bin list");
    need(d->window >= 1, "window must be >= 1");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    TwoTimeReq req;
    req.qbins.assign(d->qbins, d->qbins + d->nqbins);
    req.static_map = d->static_map != 0;
    req.average = d->average != 0;
    req.window = d->window;
    req.frame_threading = d->frame_threading != 0;
    run_filter_transpose(s);
    run_twotime(s, req, mode == XPCS_MODE_REFERENCE ? XPCS_MODE_REFERENCE : XPCS_MODE_EXACT,
                mode == XPCS_TWOTIME_EXACT_CUDA_CORES);
    sync_and_check(s);
    if (info) {
      info->qbins = (int32_t)s.tt.qbins.size();
      info->frames = s.tt.frames;
      info->window = s.tt.window;
      info->partials = s.tt.partials;
      info->sg_rows = s.tt.sg_rows;
      info->sg_cols = s.tt.sg_cols;
      info->gram_ms = s.tt.gram_ms;
      info->gram_flop = s.tt.gram_flop;
      info->gram_flop_algorithmic = s.tt.gram_flop_alg;
    }
  });
}

int xpcs_get_twotime(xpcs_series *h, int32_t *qbins, float *sg, float *c2t, float *g2full,
                     float *g2partials) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    if (!s.tt.ready) throw Error(XPCS_ERR_STATE, "xpcs_twotime has not run");
    DeviceGuard g(s.device);
    get_twotime(s, qbins, sg, c2t, g2full, g2partials);
  });
}

int xpcs_autotune(xpcs_series *h, int32_t mode, int32_t *thread_cap) {
  return guarded([&] {
    need(h, "null handle");
    need(mode == XPCS_MODE_REFERENCE || mode == XPCS_MODE_EXACT, "unknown mode");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    const int32_t c = autotune(s, mode);
    if (thread_cap) *thread_cap = c;
  });
}

int xpcs_series_get_tuning(xpcs_series *h, xpcs_tuning *t) {
  return guarded([&] {
    need(h && t, "null argument");
    Series &s = *(Series *)h;
    t->thread_cap = s.thread_cap;
    t->scratch_extra = s.scr_extra;
    t->radix_items_per_lane = s.radix_ipt;
  });
}

int xpcs_series_set_tuning(xpcs_series *h, const xpcs_tuning *t) {
  return guarded([&] {
    need(h && t, "null argument");
    bool cap_ok = false;
    for (int c : MT_THREAD_CAPS) cap_ok = cap_ok || c == t->thread_cap;
    need(cap_ok, "thread_cap must be 32, 48, 64, 80 or 112");
    need(t->scratch_extra == 0 || t->scratch_extra == 8, "scratch_extra must be 0 or 8");
    need(t->radix_items_per_lane == 0 || t->radix_items_per_lane == 8 ||
             t->radix_items_per_lane == 16,
         "radix_items_per_lane must be 0, 8 or 16");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    XG_CUDA(cudaStreamSynchronize(s.stream));
    s.thread_cap = t->thread_cap;
    s.scr_extra = t->scratch_extra;
    s.radix_ipt = t->radix_items_per_lane;
    s.knobs_set = true;
    s.have_multitau = false;
    s.have_norm64 = s.have_norm32 = false;
    s.generation++;
  });
}

int xpcs_batch_create(xpcs_series *const *series, int32_t count, xpcs_batch **out) {
  return guarded([&] {
    need(series && out && count > 0, "bad batch arguments");
    *out = nullptr;
    DeviceGuard g(((Series *)series[0])->device);
    *out = (xpcs_batch *)batch_create((Series *const *)series, count);
  });
}

int xpcs_batch_run(xpcs_batch *h, int32_t mode, uint32_t flags) {
  return guarded([&] {
    need(h, "null batch");
    need(mode == XPCS_MODE_REFERENCE || mode == XPCS_MODE_EXACT, "unknown mode");
    need((flags & ~(XPCS_BATCH_F64 | XPCS_BATCH_F32 | XPCS_BATCH_AUTOTUNE)) == 0,
         "unknown batch flags");
    Batch &b = *(Batch *)h;
    DeviceGuard g(b.device);
    batch_run(b, mode, flags);
  });
}

int xpcs_batch_stats(xpcs_batch *h, float *ms, int64_t *kernels, int32_t *lanes) {
  return guarded([&] {
    need(h, "null batch");
    Batch &b = *(Batch *)h;
    if (ms) *ms = b.last_ms;
    if (kernels) *kernels = b.kernels;
    if (lanes) *lanes = b.lanes;
  });
}

int xpcs_batch_set_form(xpcs_batch *h, int32_t work_queue) {
  return guarded([&] {
    need(h, "null batch");
    need(work_queue == 0 || work_queue == 1, "work_queue must be 0 or 1");
    Batch &b = *(Batch *)h;
    DeviceGuard g(b.device);
    XG_CUDA(cudaStreamSynchronize(b.origin));
    b.queue = work_queue != 0;
    b.form_tuned = true;
    b.lanes_tuned = false;
    if (b.exec) {
      cudaGraphExecDestroy(b.exec);
      b.exec = nullptr;
    }
  });
}

int xpcs_batch_get_form(xpcs_batch *h, int32_t *work_queue, int32_t *chains) {
  return guarded([&] {
    need(h, "null batch");
    Batch &b = *(Batch *)h;
    if (work_queue) *work_queue = b.queue ? 1 : 0;
    if (chains) *chains = b.lanes;
  });
}

int xpcs_batch_timeline(xpcs_batch *h, float *start_ms, float *end_ms) {
  return guarded([&] {
    need(h, "null batch");
    Batch &b = *(Batch *)h;
    if (b.start_ms.size() != b.ss.size()) throw Error(XPCS_ERR_STATE, "the batch has not run");
    for (size_t i = 0; i < b.ss.size(); i++) {
      if (start_ms) start_ms[i] = b.start_ms[i];
      if (end_ms) end_ms[i] = b.end_ms[i];
    }
  });
}

void xpcs_batch_destroy(xpcs_batch *h) {
  if (!h) return;
  Batch *b = (Batch *)h;
  DeviceGuard g(b->device);
  cudaStreamSynchronize(b->origin);
  delete b;
}

int xpcs_server_create(int32_t device, uint64_t memory_budget, xpcs_server **out) {
  return guarded([&] {
    need(out, "null argument");
    *out = nullptr;
    *out = (xpcs_server *)server_create(device, memory_budget);
  });
}

void xpcs_server_destroy(xpcs_server *h) {
  if (h) server_destroy(h);
}

int xpcs_server_submit(xpcs_server *h, const xpcs_series_desc *desc, int64_t expected_events,
                       int64_t *id) {
  return guarded([&] {
    need(h && desc && id, "null argument");
    *id = server_submit(h, *desc, expected_events);
  });
}

int xpcs_server_push_sparse(xpcs_server *h, int64_t id, const int32_t *idx, const int16_t *val,
                            const uint32_t *nnz, int32_t nframes) {
  return guarded([&] {
    need(h && (nframes == 0 || nnz), "null argument");
    need(nframes >= 0, "negative frame count");
    server_push(h, id, idx, val, nnz, nframes);
  });
}

int xpcs_server_finish(xpcs_server *h, int64_t id, int32_t mode) {
  return guarded([&] {
    need(h, "null server");
    need(mode == XPCS_MODE_REFERENCE || mode == XPCS_MODE_EXACT, "unknown mode");
    server_finish(h, id, mode);
  });
}

int xpcs_server_state(xpcs_server *h, int64_t id, int32_t *state) {
  return guarded([&] {
    need(h && state, "null argument");
    *state = server_state(h, id);
  });
}

int xpcs_server_result(xpcs_server *h, int64_t id, double *g2, double *se, float *G2, float *IP,
                       float *IF) {
  return guarded([&] {
    need(h, "null server");
    server_result(h, id, g2, se, G2, IP, IF);
  });
}

int xpcs_server_release(xpcs_server *h, int64_t id) {
  return guarded([&] {
    need(h, "null server");
    server_release(h, id);
  });
}

int xpcs_server_get_stats(xpcs_server *h, xpcs_server_stats *st) {
  return guarded([&] {
    need(h && st, "null argument");
    server_stats(h, st);
  });
}

int xpcs_synchronize(xpcs_series *h) {
  return guarded([&] {
    need(h, "null handle");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    sync_and_check(s);
  });
}

int xpcs_get_stage_times(xpcs_series *h, xpcs_stage_times *t) {
  return guarded([&] {
    need(h && t, "null argument");
    Series &s = *(Series *)h;
    DeviceGuard g(s.device);
    XG_CUDA(cudaStreamSynchronize(s.stream));
    auto el = [&](int a, int b) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, s.ev[a], s.ev[b]) != cudaSuccess) {
        cudaGetLastError();
        return 0.f;
      }
      return ms;
    };
    std::memset(t, 0, sizeof(*t));
    t->h2d_ms = el(0, 1);
    t->filter_ms = el(2, 3);
    t->multitau_ms = el(3, 6);
    t->multitau_int_ms = el(4, 5);
    t->multitau_float_ms = el(5, 6);
    t->normalize_ms = el(7, 8);
    t->d2h_ms = el(8, 11);
    t->step_ms = el(2, 11);
    t->launches = s.launches;
  });
}

int xpcs_device_properties(int32_t device, int32_t *sm_count, int32_t *cc_major,
                           int32_t *cc_minor) {
  return guarded([&] {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      throw Error(XPCS_ERR_NO_DEVICE, "no CUDA device");
    need(device >= 0 && device < ndev, "device ordinal out of range");
    int v = 0;
    if (sm_count) {
      XG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device));
      *sm_count = v;
    }
    if (cc_major) {
      XG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMajor, device));
      *cc_major = v;
    }
    if (cc_minor) {
      XG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMinor, device));
      *cc_minor = v;
    }
  });
}

int xpcs_set_device_memory_limit(int32_t device, uint64_t bytes) {
  return guarded([&] {
    need(device >= 0 && device < ACCT_DEVICES, "device ordinal out of range");
    g_dev_limit[device].store(bytes);
  });
}

int xpcs_get_device_memory(int32_t device, uint64_t *used, uint64_t *limit) {
  return guarded([&] {
    need(device >= 0 && device < ACCT_DEVICES, "device ordinal out of range");
    if (used) *used = g_dev_used[device].load();
    if (limit) *limit = g_dev_limit[device].load();
  });
}

int xpcs_pin_host(void *ptr, uint64_t bytes) {
  return guarded([&] {
    need(ptr && bytes > 0, "null or empty buffer");
    XG_CUDA(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
  });
}

int xpcs_unpin_host(void *ptr) {
  return guarded([&] {
    need(ptr, "null buffer");
    XG_CUDA(cudaHostUnregister(ptr));
  });
}

int xpcs_multitau2(const int64_t *row_ptr, const int32_t *frame, const float *value,
                   int32_t pixels, int32_t frames, int32_t dpl, int32_t mode, int32_t device,
                   float *G2, float *IP, float *IF) {
  Series *s = nullptr;
  int rc = guarded([&] {
    need(row_ptr && pixels > 0 && frames >= 0 && dpl >= 0, "bad argument");
    need(mode == XPCS_MODE_REFERENCE || mode == XPCS_MODE_EXACT, "unknown mode");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      throw Error(XPCS_ERR_NO_DEVICE, "no CUDA device");
    need(device >= 0 && device < ndev, "device ordinal out of range");
    const int64_t E = row_ptr[pixels];
    need(E >= 0 && row_ptr[0] == 0, "row_ptr must start at 0");
    need(E == 0 || (frame && value), "null event arrays");
    for (int32_t p = 0; p < pixels; p++)
      need(row_ptr[p + 1] >= row_ptr[p], "row_ptr must be non-decreasing");
    s = new Series();
    s->device = device;
    DeviceGuard g(device);
    s->P = pixels;
    s->F = frames;
    s->desc.delays_per_level = dpl;
    s->delays = delay_schedule(frames, dpl);
    s->D = (int32_t)s->delays.level.size();
    init_series(*s);
    multitau_rows_upload(*s, row_ptr, frame, value, E);
    run_multitau(*s, mode);
    const size_t n = (size_t)s->D * pixels;
    if (n) {
      if (G2) XG_CUDA(cudaMemcpyAsync(G2, s->G2.p, 4 * n, cudaMemcpyDeviceToHost, s->stream));
      if (IP) XG_CUDA(cudaMemcpyAsync(IP, s->IP.p, 4 * n, cudaMemcpyDeviceToHost, s->stream));
      if (IF) XG_CUDA(cudaMemcpyAsync(IF, s->IF.p, 4 * n, cudaMemcpyDeviceToHost, s->stream));
    }
    XG_CUDA(cudaStreamSynchronize(s->stream));
  });
  free_series(s);
  return rc;
}

}  // extern "C"
