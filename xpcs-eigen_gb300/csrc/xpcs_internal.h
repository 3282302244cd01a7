// Internal declarations of libxpcs_gpu (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "xpcs_gpu.h"

namespace xg {

// ---------------------------------------------------------------- errors

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define XG_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      throw ::xg::Error(e_ == cudaErrorMemoryAllocation ? XPCS_ERR_OUT_OF_MEMORY      \
                                                        : XPCS_ERR_CUDA,              \
                        std::string(#call) + ": " + cudaGetErrorString(e_));          \
  } while (0)

// Kernels launched by this thread (the stage tracer reports per-call deltas).
extern thread_local int64_t tl_launches;
#define XG_CHECK_LAUNCH()          \
  do {                             \
    ::xg::tl_launches++;           \
    XG_CUDA(cudaGetLastError());   \
  } while (0)

// Device error word bits (set by kernels, read at synchronisation points).
enum : int32_t {
  DEVERR_PIXEL_INDEX = 1,
  DEVERR_WAIT = 2,  // a bounded wait for an asynchronous copy expired
};

// ------------------------------------------------------------ device buffers

// Stream-ordered device allocation through the library's accounting: every
// byte the library holds on a device is counted, and an allocation that would
// take the device past its limit (xpcs_set_device_memory_limit) fails with
// XPCS_ERR_OUT_OF_MEMORY before CUDA is asked (abi.cu).
void *dev_alloc(size_t bytes, cudaStream_t st);
void dev_free(void *p, size_t bytes, cudaStream_t st);

// A stream-ordered device allocation that grows on demand.
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t cap = 0;
  void reserve(size_t n, cudaStream_t st) {
    if (n <= cap) return;
    T *q = (T *)dev_alloc(sizeof(T) * n, st);
    if (p) dev_free(p, sizeof(T) * cap, st);
    p = q;
    cap = n;
  }
  // grow keeping the first `keep` elements
  void grow(size_t n, size_t keep, cudaStream_t st) {
    if (n <= cap) return;
    size_t c = cap ? cap : 1;
    while (c < n) c *= 2;
    T *q = (T *)dev_alloc(sizeof(T) * c, st);
    if (p && keep) {
      const cudaError_t e =
          cudaMemcpyAsync(q, p, sizeof(T) * keep, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) {
        dev_free(q, sizeof(T) * c, st);
        XG_CUDA(e);
      }
    }
    if (p) dev_free(p, sizeof(T) * cap, st);
    p = q;
    cap = c;
  }
  void release(cudaStream_t st) {
    if (p) dev_free(p, sizeof(T) * cap, st);
    p = nullptr;
    cap = 0;
  }
};

// ------------------------------------------------------- delays and q-maps

struct DelaySchedule {
  std::vector<int32_t> level, tau;  // Corr::delaysPerLevel order
};
DelaySchedule delay_schedule(int frames, int dpl);

// Configuration::BuildQMap result, flattened in the reference's iteration
// order (q ascending, sbin ascending, pixels in raster order).
struct QMap {
  int32_t pixels = 0, total_static = 0, total_dynamic = 0;
  std::vector<uint8_t> valid;       // m_validPixelMask
  std::vector<int32_t> sbin;        // m_sbin (1-based, 0 none)
  std::vector<int32_t> pixels_per_bin;
  std::vector<int32_t> q_ids;       // mapping keys
  std::vector<int32_t> q_entry_ptr; // [nq+1] into entry_*
  std::vector<int32_t> entry_sbin;  // 1-based sbin of each (q, sbin) entry
  std::vector<int32_t> entry_pix_ptr;  // [nentries+1]
  std::vector<int32_t> pix;
  std::string error;                // non-empty: reference would index out of bounds
  int32_t nq() const { return (int32_t)q_ids.size(); }
  int32_t nentries() const { return (int32_t)entry_sbin.size(); }
};
QMap build_qmap(const int32_t *dq, const int32_t *sq, int32_t pixels);

// ---------------------------------------------------------- multi-tau plan

constexpr int MAX_LEVELS = 48;

struct McLevel {
  int32_t level;      // multi-tau level L
  int32_t first;      // index of its first delay
  int32_t count;      // delays at this level
  int32_t lastframe;  // lastframe while this level's delays are evaluated
  int32_t tau_lo;     // first delay in level units (delays are consecutive)
  int32_t compact;    // 1: the reference compacts the rows before this level
  int32_t t_end;      // lastframe << level: frames >= t_end are dropped by this level
};

// Kernel-side description of a multi-tau run; lives in device memory.
struct McPlan {
  int32_t P, D, F, nlev, mode, acc;
  int32_t scr;  // scratch words per lane of the thread-per-pixel kernel (>= acc, nlev): levels of
                // at most 32 * scr bins take the bitmask pair search (the level-fold schedule)
  McLevel lv[MAX_LEVELS];
  // followed in device memory by the per-delay arrays (McArrays)
};

// Per-delay arrays stored after McPlan.
struct McArrays {
  const int32_t *tau_lvl;  // delay in level units
  const float *denom;      // (float)(lastframe - tau), 0 = no division
  const int32_t *tau_abs;  // delay in frames = first frame counted by IF
  const int32_t *t_ip;     // (lastframe - tau) << level: IP counts frames below it
  const int32_t *gi;       // level group of the delay
  const float *rcp;        // correctly rounded 1 / denom (0 when denom is 0)
};
__host__ __device__ inline size_t mc_align16(size_t x) { return (x + 15) & ~(size_t)15; }
__host__ __device__ inline size_t mc_plan_bytes(int D) {
  return mc_align16(sizeof(McPlan) + (size_t)D * 6 * sizeof(int32_t));
}
__host__ __device__ inline McArrays mc_arrays(const void *plan, int D) {
  const int32_t *b = (const int32_t *)((const uint8_t *)plan + sizeof(McPlan));
  return McArrays{b, (const float *)(b + D), b + 2 * D, b + 3 * D, b + 4 * D,
                  (const float *)(b + 5 * D)};
}

// Pixel classes assigned by the filter's merge pass.  The integer kernels
// need integer values with sum |v| < 4096 (every float partial sum of the
// reference is then exact) and frames below 65536 (packed with the value in
// one 32-bit word); by row length they go to the thread-per-pixel kernel, the
// warp-per-pixel kernel or its long-row launch.
// Row capacities of the thread-per-pixel kernel (one instantiation each); a
// series uses one of them (Series::thread_cap, default MT_THREAD_CAP_DEFAULT,
// chosen per series by xpcs_autotune).  Rows longer than the series' capacity
// go to the warp-per-pixel kernel.
constexpr int MT_THREAD_CAPS[] = {32, 48, 64, 80, 112};
constexpr int MT_THREAD_NCAPS = 5;
constexpr int MT_THREAD_CAP_DEFAULT = 80;
constexpr int MT_WARP_CAP = 256;
constexpr int MT_LONG_CAP = 4096;  // an integer row with sum |v| < 4096 has fewer non-zero events
enum : uint8_t { PCLASS_EMPTY = 0, PCLASS_THREAD = 1, PCLASS_WARP = 2, PCLASS_FLOAT = 3,
                 PCLASS_LONG = 4 };

__host__ __device__ inline uint8_t pixel_class(int n, bool integral, long long total, int F,
                                               int thread_cap) {
  if (n == 0) return PCLASS_EMPTY;
  if (!integral || total >= 4096) return PCLASS_FLOAT;
  if (F > 65536) return PCLASS_FLOAT;  // the integer kernels pack frames in 16 bits
  if (n <= thread_cap) return PCLASS_THREAD;
  if (n <= MT_WARP_CAP) return PCLASS_WARP;
  if (n <= MT_LONG_CAP) return PCLASS_LONG;
  return PCLASS_FLOAT;
}

// Counters written by device passes.
struct DevStats {
  int32_t error;
  int32_t nfloat;
  int32_t nvalid;
  int32_t nwarp;
  int32_t nlong;
  int32_t fnext;  // next float-path pixel to hand out (k_mt_fwarp)
  unsigned long long events;
  unsigned long long dropped;  // K-a items sorted last (unused frames, bad pixel indices)
};

// -------------------------------------------------------------- two-time

struct TwoTimeReq {
  std::vector<int32_t> qbins;  // q bins to process
  int32_t static_map = 0, average = 0, window = 1, frame_threading = 0;
};
// Rows of the processed q bins in mapping order and their grouping.
struct TwoTimeLayout {
  std::vector<int32_t> row_pix, row_grp;  // per row: its pixel, its smoothing group
  std::vector<int32_t> grp_ptr{0};        // rows of each smoothing group (contiguous)
  std::vector<int32_t> q_ptr{0};          // rows of each processed q bin (contiguous)
  std::vector<int32_t> q_grp_end;         // static map: end group index of each q bin
};
struct TwoTimeOut {
  bool ready = false;
  std::vector<int32_t> qbins;  // processed q bins present in the mapping, in mapping order
  int32_t frames = 0, window = 1, partials = 0, sg_rows = 0, sg_cols = 0;
  float gram_ms = 0.f;      // EXACT: tensor-core Gram kernel time
  double gram_flop = 0.0;      // multiply-adds of the tiles computed (2 x M x N x K each)
  double gram_flop_alg = 0.0;  // of the upper triangle alone (2 x rows x F(F+1)/2)
};

// --------------------------------------------------------------- a series

struct Series {
  xpcs_series_desc desc{};
  int device = 0;
  cudaStream_t stream = nullptr;
  int32_t P = 0, F = 0, D = 0, R_in = 1;
  DelaySchedule delays;
  QMap qmap;

  // ingested raw frames
  std::vector<int64_t> frame_off{0};  // host copy, [raw_frames+1]
  std::vector<int32_t> frame_map;     // per raw frame: its filter frame, -1 if not used
  DBuf<int32_t> d_frame_map;
  DBuf<int32_t> d_chunk_frame;  // raw frame of every 512th raw event
  DBuf<int32_t> raw_idx;
  DBuf<int16_t> raw_val;    // sparse series: raw int16 values
  DBuf<float> raw_valf;     // dense series: filtered float values
  DBuf<int64_t> d_frame_off;
  int64_t raw_events = 0;
  int32_t raw_frames = 0;
  bool frame_off_dirty = true;

  // per-pixel constant data
  DBuf<uint8_t> d_mask;
  DBuf<double> d_flat;
  bool has_flat = false;

  // dense frames: dark statistics and the per-pixel keep threshold
  DBuf<double> dark_avg, dark_std;
  DBuf<int32_t> rmin;
  bool has_dark = false, rmin_ready = false;
  DBuf<int32_t> dn_counts;
  DBuf<int64_t> dn_offsets;
  DBuf<int64_t> dn_frame_end;
  DBuf<uint8_t> dn_prep;  // per pixel: EmuSubPrep of the dark level, EmuMulPrep of the gain
  // dense series without stride or averaging: the filter writes pixel-major
  // blocks of the block store directly; the frames of small ingests wait in
  // dn_pend (raw frames dn_pend_r0 .. +dn_pend_n) until a block's worth is there
  bool dense_px = false;
  DBuf<int16_t> dn_pend;
  int32_t dn_pend_n = 0, dn_pend_r0 = 0;
  DBuf<int32_t> dn_tot;  // per-pixel padded row lengths of the block being written
  DBuf<unsigned long long> dn_sum;  // kept events of the block being written
  DBuf<uint32_t> blk_pk;  // their block store: (frame - block start) << 16 | raw value
  std::vector<int32_t> blk_r0;  // first raw frame of every block
  DBuf<int32_t> d_blk_r0;

  // transpose / event lists
  DBuf<uint32_t> keyA, keyB;
  DBuf<int32_t> frA, frB;
  DBuf<float> vA, vB;
  DBuf<uint32_t> hist, hist_scan;
  // incremental transposes (block_frames > 0): block-local pixel-major rows
  int32_t block_frames = 0;   // filter frames per block; 0: one transpose at xpcs_multitau
  int32_t blk_raw_done = 0;   // raw frames already transposed into blocks
  int64_t blk_events = 0;     // events in the block store
  std::vector<int64_t> blk_base;  // first event of every block in the store
  DBuf<int64_t> d_blk_base;
  DBuf<int32_t> blk_fr;       // block store: filter frames
  DBuf<float> blk_val;        // block store: values
  DBuf<int32_t> blk_off, blk_len;  // [block][P]: row start in its block, merged length
  DBuf<int64_t> blk_rp;       // row pointers of the block being transposed
  DBuf<int32_t> blk_tot;      // merged events per pixel over every block
  DBuf<int64_t> row_ptr;    // [P+1]
  DBuf<int32_t> row_len;    // events per pixel after merging duplicates
  DBuf<uint8_t> pclass;
  DBuf<int32_t> flist;      // pixels of the float path
  DBuf<int32_t> wlist;      // pixels of the warp-per-pixel integer path
  DBuf<int32_t> llist;      // pixels of the long-row warp-per-pixel integer path
  DBuf<int32_t> ev_frame;   // final pixel-major lists
  DBuf<float> ev_val;
  DBuf<float> pixels_sum;
  DBuf<int32_t> d_sbin;     // per pixel: static bin - 1 (-1 none)
  DBuf<int32_t> d_ppb;      // pixels per static bin
  DBuf<int64_t> side_pos;
  DBuf<float> side_out;
  DBuf<float> d_fscale;     // normalize_by_framesum: per-frame divisor frameSum/mean
  DBuf<int32_t> sc_frame;   // float-path scratch rows
  DBuf<float> sc_val;
  DBuf<uint8_t> scan_tmp;
  DBuf<DevStats> stats;

  // multi-tau
  DBuf<uint8_t> plan;       // McPlan + tau_lvl[D] + denom[D]
  int32_t plan_mode = -1;   // mode of the plan in `plan` (-1: none uploaded)
  int32_t thread_cap = MT_THREAD_CAP_DEFAULT;  // rows up to this length: thread per pixel
  int32_t scr_extra = 0;    // scratch words beyond max(delays of a level, levels)
  int32_t radix_ipt = 0;    // transpose items per lane (event tile / 256); 0: by series size
  int32_t plan_scr = -1;    // scratch words of the uploaded plan
  bool tuned = false;       // thread_cap, scr_extra, radix_ipt chosen by xpcs_autotune
  bool knobs_set = false;   // chosen by the caller or the autotuner (else: default_knobs)
  int64_t valid_pixels = -1;  // pixels of the q-map mask (counted once)
  DBuf<float> G2, IP, IF;
  bool have_multitau = false;
  bool have_norm64 = false, have_norm32 = false;
  int64_t generation = 0;   // bumped by every change of the ingested frames

  // normalisation
  DBuf<int32_t> n_q_entry_ptr, n_entry_sbin, n_entry_pix_ptr, n_pix, n_q_row;
  DBuf<float> n_ratio32;
  DBuf<int32_t> n_unsafe;  // float32 replay: a ratio outside the branch-free range
  DBuf<float> n_tg, n_ti, n_tf, n_tx;  // float32 replay: G2/IP/IF and x, [mapped pixel][D]
  DBuf<int32_t> n_ch_k0, n_ch_k1, n_e_chunk_ptr;  // pixel chunks of every entry
  int32_t n_chunks = 0;
  DBuf<double> n_part;                            // [chunk][tau][5] partial sums
  DBuf<double> n_g2, n_se;
  DBuf<float> n_g2f, n_sef;

  // two-time
  TwoTimeOut tt;
  DBuf<int32_t> tt_row_pix, tt_row_grp, tt_grp_ptr, tt_order;
  DBuf<float> tt_V, tt_sg, tt_sga, tt_C, tt_full, tt_part;
  DBuf<int32_t> tt_err, tt_flags;       // tensor-core path: wait timeouts, range flags
  DBuf<uint16_t> tt_XT;                 // fp16 counts X^T [Fp][Kp] of one group
  DBuf<long long> tt_S;                 // per-frame count sums of one group
  DBuf<unsigned long long> tt_bound, tt_Gi;
  DBuf<double> tt_sgd, tt_Cacc, tt_Cq;
  DBuf<float> tt_Gf;

  // tracer
  cudaEvent_t ev[12] = {};
  int32_t launches = 0;     // kernels launched since the last xpcs_multitau began
  bool timed_h2d = false;
  float h2d_ms_acc = 0.f;

  // host staging for pageable ingests
  void *pinned = nullptr;
  size_t pinned_cap = 0;
};

// ------------------------------------------------- batch multi-tau queue

// A batch member as the work-queue multi-tau kernels see it (device memory).
struct MtQueueMember {
  const uint8_t *plan;
  const int64_t *row_ptr;
  const int32_t *row_len;
  const uint8_t *pclass;
  const int32_t *ev_frame;
  const float *ev_val;
  float *G2, *IP, *IF;
  const int32_t *wlist, *llist;
  const DevStats *stats;
  int32_t first;   // the member's first 32-pixel group in its capacity's queue
  int32_t groups;  // its 32-pixel groups
};

// The members of a batch in one table, grouped by thread-kernel row capacity.
struct MtQueue {
  DBuf<MtQueueMember> tab;
  DBuf<int32_t> next;                   // one queue counter per launch
  std::vector<int32_t> cap_first, cap_count, cap_groups;  // per MT_THREAD_CAPS entry
  int32_t scr_max = 0, acc_max = 0;
};
// Builds the table (after an eager pass has sized every buffer and uploaded
// every plan); enqueues the multi-tau of every member as work-queue launches
// (k_multitau.cu).
void mt_queue_build(const std::vector<Series *> &ss, MtQueue &q, cudaStream_t st);
void mt_queue_run(const std::vector<Series *> &ss, MtQueue &q, cudaStream_t st);

// --------------------------------------------------------------- a batch

struct Batch {
  std::vector<Series *> ss;
  int device = 0;
  cudaStream_t origin = nullptr;   // the graph is captured from and launched on it
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
  std::vector<cudaEvent_t> join;
  DBuf<unsigned long long> stamps; // %globaltimer at each member's start and end, then the fork
  std::vector<float> start_ms, end_ms;  // of the last run, from the graph's fork
  std::vector<int64_t> gens;       // member generations at capture
  int mode = -1;
  uint32_t flags = 0;
  int64_t kernels = 0;             // kernel nodes in the graph
  float last_ms = 0.f;
  int32_t lanes = 0;               // concurrent chains of series in the graph (0: one per series)
  bool lanes_tuned = false;
  bool queue = true;               // multi-tau as one work-queue launch over all members
  MtQueue mtq;
  std::vector<cudaEvent_t> join2;  // work-queue form: ends of each member's second phase
  cudaEvent_t fork2 = nullptr;     // work-queue form: the multi-tau launches are done
  bool form_tuned = false;
  ~Batch();
};
Batch *batch_create(Series *const *ss, int32_t n);   // batch.cu
int32_t autotune(Series &s, int mode);               // batch.cu
void batch_run(Batch &b, int mode, uint32_t flags);

// Serving front end (server.cpp); the handle is an opaque Server.
void *server_create(int device, uint64_t budget);
void server_destroy(void *srv);
int64_t server_submit(void *srv, const xpcs_series_desc &desc, int64_t expected_events);
void server_push(void *srv, int64_t id, const int32_t *idx, const int16_t *val,
                 const uint32_t *nnz, int32_t nframes);
void server_finish(void *srv, int64_t id, int mode);
int server_state(void *srv, int64_t id);
void server_result(void *srv, int64_t id, double *g2, double *se, float *G2, float *IP, float *IF);
void server_release(void *srv, int64_t id);
void server_stats(void *srv, xpcs_server_stats *out);

// Sets the message xpcs_last_error() returns on this thread (abi.cu).
void xpcs_set_last_error(const char *msg);

// Scans (scan.cu)
size_t scan_workspace_bytes(int64_t n);
void exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, void *ws, cudaStream_t st);
void exclusive_scan_i32_i64(const int32_t *in, int64_t *out, int64_t n, void *ws,
                            cudaStream_t st);

// Kernel launchers
void run_filter_transpose(Series &s);                       // k_transpose.cu
// Knobs for a series the caller has not tuned, from its mean row length.
void default_knobs(Series &s);
// Incremental transposes: every complete block of ingested frames (k_transpose.cu)
void transpose_ready_blocks(Series &s);
void reset_blocks(Series &s);
void run_multitau(Series &s, int mode);                      // k_multitau.cu
void run_normalize(Series &s, bool want64, bool want32);     // k_normalize.cu
void build_norm_chunks(Series &s);                           // k_normalize.cu
// The float nearest to 1/b (ties to even) for an integer b in [1, 2^24].
float recip_rn(int32_t b);                                   // k_multitau.cu

// Stable radix sort of (key, a, b) by the low key_bits of key (k_transpose.cu);
// returns true when the result is in the second set of arrays.
bool radix_sort_triples(Series &s, uint32_t *key, int32_t *a, float *b, uint32_t *key2,
                        int32_t *a2, float *b2, int64_t n, int key_bits);

// Side statistics (k_side.cu)
struct SideOut {
  float *pixel_sum;       // [P]
  float *frame_sum;       // [2][F]
  float *part_total;      // [S]
  float *part_partial;    // [floor(F / static_window)][S]
};
void run_side_stats(Series &s, const SideOut &out);
void prepare_framesum_scale(Series &s);  // k_side.cu

// Two-time (k_twotime.cu): needs the event lists of run_filter_transpose
void run_twotime(Series &s, const TwoTimeReq &req, int mode, bool force_i64);
void run_twotime_exact(Series &s, const TwoTimeReq &req, const TwoTimeLayout &lay,
                       bool force_i64);  // k_twotime_tc.cu
void get_twotime(Series &s, int32_t *qbins, float *sg, float *c2t, float *g2full, float *g2part);

// Dense frames (k_dense.cu)
void dense_set_dark(Series &s, const int16_t *dark_host, int32_t ndark);
void dense_ingest(Series &s, const int16_t *frames, int32_t nframes, bool on_device);
void dense_px_flush(Series &s);  // pending frames of a pixel-major dense series -> a block
void dense_px_gather(Series &s);  // its blocks -> the event lists and row_ptr
void dense_get_dark(Series &s, double *avg, double *sd);

// Upload caller-held pixel-major rows and classify their pixels (xpcs_multitau2)
void multitau_rows_upload(Series &s, const int64_t *row_ptr, const int32_t *frame,
                          const float *value, int64_t events);

}  // namespace xg
