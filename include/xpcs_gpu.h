/*
 * xpcs_gpu.h — C ABI of the GB300 (sm_103a) multi-tau XPCS correlator.
 *
 * Drop-in boundary for xpcs-eigen's `corr` multi-tau path.  The reference has
 * no plugin or FFI layer: its path is a set of static C++ calls that read their
 * parameters from the Configuration singleton.  Each entry point below names
 * the reference interface it replaces (file:line in xpcs-eigen).
 *
 * Conventions
 *  - Every function returns an xpcs_status (XPCS_OK = 0); no C++ exception
 *    crosses this boundary.  xpcs_last_error() gives a message for the last
 *    failure on the calling thread.
 *  - All array arguments are HOST pointers unless the function name ends in
 *    _device.  Inputs are copied; output buffers are caller-owned.
 *  - A series handle owns one CUDA stream; calls on one handle are ordered.
 *    Distinct handles may be used from distinct threads.
 *  - Work is enqueued asynchronously; functions that return data to the host
 *    (xpcs_get_*, xpcs_normalize, xpcs_synchronize) wait for it and report any
 *    error raised by earlier device work of that handle.
 *  - Layouts follow the reference: G2/IP/IF are float32 [D][P] (tau-major, as
 *    Corr::multiTau2 fills G2s[tauIndex*pixels + pixel], corr.cpp:392), and
 *    g2/stderr are [D][Q] (the on-disk layout of norm-0-g2, h5_result.cpp:76-78).
 */
#ifndef XPCS_GPU_H
#define XPCS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XPCS_GPU_ABI_VERSION 1

typedef enum {
  XPCS_OK = 0,
  XPCS_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or parameter */
  XPCS_ERR_CUDA = 2,             /* a CUDA runtime call failed, or an asynchronous
                                    copy inside a kernel did not complete within its
                                    bounded wait */
  XPCS_ERR_OUT_OF_MEMORY = 3,    /* device or pinned host allocation failed */
  XPCS_ERR_STATE = 4,            /* call out of order (e.g. results before compute) */
  XPCS_ERR_QMAP = 5,             /* partition maps the reference would index out of
                                    bounds (quirks Q5/Q7 of BuildQMap/normalizeG2s) */
  XPCS_ERR_INPUT = 6,            /* frame data out of range (pixel index >= W*H) */
  XPCS_ERR_NO_DEVICE = 7         /* no usable CUDA device */
} xpcs_status;

/* Multi-tau search semantics.
 * REFERENCE: the partner of an event is looked up with std::lower_bound over
 *   the whole row buffer including the stale tail left by in-place level
 *   compaction (corr.cpp:406), so a few G2 products are missed exactly as the
 *   reference misses them.  Bit-identical to Corr::multiTau2.
 * EXACT: the lookup covers only the live prefix (the intended semantics). */
typedef enum { XPCS_MODE_REFERENCE = 0, XPCS_MODE_EXACT = 1 } xpcs_mode;

typedef struct xpcs_series xpcs_series;

/* Series description: the Configuration fields the path reads
 * (Configuration::init, configuration.cpp:80-242). */
typedef struct {
  int32_t width;            /* /measurement/instrument/detector/x_dimension */
  int32_t height;           /* /measurement/instrument/detector/y_dimension */
  int32_t frames;           /* getFrameTodoCount(): (end-begin+1)/(stride*avg) */
  int32_t delays_per_level; /* /xpcs/delays_per_level */
  int32_t stride_frames;    /* /xpcs/stride_frames (>= 1) */
  int32_t avg_frames;       /* /xpcs/avg_frames (>= 1) */
  int32_t static_window;    /* /xpcs/static_mean_window_size (>= 1) */
  const int32_t *dqmap;     /* [height*width] /xpcs/dqmap (final orientation) */
  const int32_t *sqmap;     /* [height*width] /xpcs/sqmap */
  const double *flatfield;  /* [height*width] or NULL when flatfield is disabled */
  int32_t dense;            /* 0: sparse (compressed) IMM frames, 1: dense frames */
  float lld;                /* dense with darks: /xpcs/lld */
  float sigma;              /* dense with darks: /xpcs/sigma */
  int32_t device;           /* CUDA device ordinal */
  int32_t normalize_by_framesum; /* /xpcs/normalize_by_framesum: 1 divides every value by
                                    (frame sum / mean frame sum) before multi-tau
                                    (main.cpp:314-337); such series take the float path
                                    and cannot join a batch */
} xpcs_series_desc;

typedef struct {
  int32_t pixels;             /* width*height */
  int32_t delays;             /* D = number of (level, tau) pairs */
  int32_t total_static;       /* getTotalStaticPartitions() */
  int32_t total_dynamic;      /* getTotalDynamicPartitions() */
  int32_t qbins;              /* rows of g2/stderr = q bins in the mapping */
  int32_t raw_frames;         /* raw frames ingested so far */
  int64_t raw_events;         /* raw events ingested so far */
  int64_t events;             /* pixel events after the filter (valid after multitau) */
  int32_t valid_pixels;       /* pixels with >= 1 event (valid after multitau) */
  int32_t float_path_pixels;  /* pixels on the order-preserving float path */
} xpcs_series_info;

/* Device times of the last xpcs_multitau / xpcs_normalize of a handle, from
 * CUDA events recorded on the handle's stream (milliseconds). */
typedef struct {
  float h2d_ms;        /* host-to-device copies of ingested frames */
  float filter_ms;     /* K-a: mask/flat filter + pixel-major radix transpose */
  float multitau_ms;   /* K-c: integer path + float path */
  float normalize_ms;  /* K-d: g2/stderr (float64 and float32) */
  float d2h_ms;        /* device-to-host copies of results */
  float multitau_int_ms;
  float multitau_float_ms;
  float step_ms;       /* start of xpcs_multitau to the end of xpcs_normalize's copies */
  int32_t launches;    /* kernels launched by the last xpcs_multitau + xpcs_normalize */
} xpcs_stage_times;

/* Library version of this header. */
int xpcs_abi_version(void);

/* Message of the last failure on this thread ("" if none). */
const char *xpcs_last_error(void);

/* Corr::calculateLevelMax + Corr::delaysPerLevel (corr.cpp:1133-1160).
 * Writes min(D, capacity) pairs; *count = D. */
int xpcs_delay_schedule(int32_t frames, int32_t delays_per_level, int32_t *level, int32_t *tau,
                        int32_t capacity, int32_t *count);

/* Configuration::init + BuildQMap (configuration.cpp:80-381) for one series:
 * builds the valid-pixel mask, static/dynamic partitions and the delay
 * schedule, and allocates device state on desc->device. */
int xpcs_series_create(const xpcs_series_desc *desc, xpcs_series **out);

void xpcs_series_destroy(xpcs_series *s);

/* Forget ingested frames and results; keep maps and device buffers. */
int xpcs_series_reset(xpcs_series *s);

int xpcs_series_get_info(xpcs_series *s, xpcs_series_info *info);

/* Incremental transposes (no reference counterpart: SparseFilter::Apply pushes
 * each frame onto per-pixel rows as it is read, sparse_filter.cpp:115-193, and
 * this keeps that property on the GPU).  With block_frames > 0, every time
 * block_frames complete filter frames (block_frames * stride * avg raw frames)
 * have been ingested, they are filtered and transposed on the handle's stream
 * into pixel-major rows that stay on the device; xpcs_multitau then
 * transposes only the last, partial block and joins the blocks' rows in frame
 * order.  The event lists, and every result, are bit-identical to those of one
 * transpose of all frames.  0 (the default) transposes everything at
 * xpcs_multitau.  Set it before ingesting frames (XPCS_ERR_STATE otherwise).
 * Such a handle cannot join a batch. */
int xpcs_series_set_block_frames(xpcs_series *s, int32_t block_frames);

/* Imm::NextFrames + SparseFilter::Apply input (imm.cpp:70-118,
 * sparse_filter.cpp:115-193): append `nframes` raw sparse frames.  Frame r has
 * nnz[r] events idx[..] (int32 pixel index) and val[..] (int16 value, read as
 * signed like the reference); the arrays hold the frames back to back.  Frames
 * are grouped stride*avg per filter frame in arrival order. */
int xpcs_ingest_sparse(xpcs_series *s, const int32_t *idx, const int16_t *val,
                       const uint32_t *nnz, int32_t nframes);

/* As xpcs_ingest_sparse with idx/val already in device memory of the
 * handle's device (nnz stays a host array). */
int xpcs_ingest_sparse_device(xpcs_series *s, const int32_t *idx_device,
                              const int16_t *val_device, const uint32_t *nnz, int32_t nframes);

/* DarkImage::Compute (dark_image.cpp:81-106) for a dense series: `ndark` raw
 * int16 frames [ndark][width*height] (the first frames of the file, main.cpp:
 * 227-239).  Sets the per-pixel dark mean and standard deviation used by
 * xpcs_ingest_dense.  Call before ingesting frames; without it dense frames are
 * kept when their value is > 0 (DenseFilter without a dark image). */
int xpcs_set_dark(xpcs_series *s, const int16_t *dark, int32_t ndark);

/* Imm::NextFrames + DenseFilter::Apply input (imm.cpp:70-118,
 * dense_filter.cpp:121-210): append `nframes` dense int16 frames
 * [nframes][width*height] (values read as signed, like the reference).
 * Dark subtraction, threshold lld + sigma*std and flatfield are applied on the
 * GPU as frames arrive; only kept pixels are stored. */
int xpcs_ingest_dense(xpcs_series *s, const int16_t *frames, int32_t nframes);

/* As xpcs_ingest_dense with the frames already in device memory.  They are
 * read on the series' stream: keep them unchanged until the series has
 * synchronised (xpcs_synchronize or any call that returns results). */
int xpcs_ingest_dense_device(xpcs_series *s, const int16_t *frames_device, int32_t nframes);

/* The --darkout datasets DarkAvg / DarkStd (main.cpp:459-478): float64
 * [height*width] each; either may be NULL. */
int xpcs_get_dark(xpcs_series *s, double *avg, double *std_);

/* Corr::multiTau2 (corr.cpp:315-431), preceded by the filter's transpose of
 * the ingested frames into pixel-major event lists.  Enqueues the work. */
int xpcs_multitau(xpcs_series *s, int32_t mode);

/* The G2/IP/IF arrays of Corr::multiTau2, float32 [D][P] each; any may be NULL. */
int xpcs_get_g2ipif(xpcs_series *s, float *G2, float *IP, float *IF);

/* Corr::normalizeG2s (corr.cpp:927-1091): per-partition g2 and standard error,
 * [D][Q] each.  g2/stderr_: float64 evaluation; g2_f32/stderr_f32: float32
 * evaluation in the reference's operation order (bit-identical to the
 * reference's norm-0-g2 / norm-0-stderr).  Any pointer may be NULL. */
int xpcs_normalize(xpcs_series *s, double *g2, double *stderr_, float *g2_f32,
                   float *stderr_f32);

/* The filters' side statistics after main.cpp's post-processing, bit-identical
 * to the reference's datasets (sparse_filter.cpp:133-190, dense_filter.cpp:
 * 176-208, main.cpp:321-411):
 *   pixel_sum              pixelSum, float32 [height*width]
 *   frame_sum              frameSum, float32 [2][frames]
 *   partition_mean_total   partition-mean-total, float32 [total_static]
 *   partition_mean_partial partition-mean-partial, float32
 *                          [frames / static_window][total_static]
 * Any pointer may be NULL.  Needs xpcs_multitau or xpcs_twotime to have run. */
int xpcs_side_stats(xpcs_series *s, float *pixel_sum, float *frame_sum,
                    float *partition_mean_total, float *partition_mean_partial);

/* The results of the handle's last normalisation (xpcs_normalize or a batch
 * run), without computing again: [D][Q] each, any pointer may be NULL.  A
 * float64 / float32 output that the last normalisation did not compute is
 * an XPCS_ERR_STATE. */
int xpcs_get_normalized(xpcs_series *s, double *g2, double *stderr_, float *g2_f32,
                        float *stderr_f32);

/* Kernel knobs of a series (no reference counterpart).  Results do not
 * depend on them; only the time does.
 *  thread_cap            warps per pixel: rows of up to this many events run
 *                        one thread per pixel (32, 48, 64, 80 or 112), longer
 *                        rows one warp per pixel;
 *  scratch_extra         the level-fold schedule: extra scratch words per
 *                        thread (0 or 8 beyond the delays of a level and the
 *                        levels); levels of at most 32 x words bins take the
 *                        bitmask pair search;
 *  radix_items_per_lane  the transpose's event tile: 8 or 16 items per lane
 *                        (tiles of 2,048 or 4,096 events; 0 chooses by series
 *                        size).
 * Until xpcs_series_set_tuning or xpcs_autotune sets them, each multi-tau
 * derives the first two from the series: thread_cap the smallest capacity of
 * at least 1.5 mean rows (events per mapped pixel), scratch_extra 8 from
 * 16,384 frames on (before the first multi-tau: 80 and 0). */
typedef struct {
  int32_t thread_cap;
  int32_t scratch_extra;
  int32_t radix_items_per_lane;
} xpcs_tuning;
int xpcs_series_get_tuning(xpcs_series *s, xpcs_tuning *t);
int xpcs_series_set_tuning(xpcs_series *s, const xpcs_tuning *t);

/* Autotuner (no reference counterpart).  Times the filter and multi-tau
 * passes of the ingested frames over the knobs above, one knob at a time
 * (thread_cap, then scratch_extra, then radix_items_per_lane), keeping the
 * fastest value of each, and sets them on the series.  *thread_cap (may be
 * NULL) receives the chosen row capacity; xpcs_series_get_tuning gives all
 * three. */
int xpcs_autotune(xpcs_series *s, int32_t mode, int32_t *thread_cap);

/* Waits for the handle's stream; reports deferred device errors. */
int xpcs_synchronize(xpcs_series *s);

int xpcs_get_stage_times(xpcs_series *s, xpcs_stage_times *t);

/* Device-memory limit (no reference counterpart; the reference holds its rows
 * in host memory).  Every device allocation the library makes on `device` is
 * counted; with a non-zero limit, a call whose allocations would take the
 * library's total on that device past `bytes` fails with
 * XPCS_ERR_OUT_OF_MEMORY (message naming the limit) before CUDA is asked, and
 * the handle stays usable: destroy or reset it, or raise the limit and call
 * again.  0 = no limit (the default).  xpcs_get_device_memory reports the
 * bytes the library holds on the device and the limit. */
int xpcs_set_device_memory_limit(int32_t device, uint64_t bytes);
/* Streaming multiprocessors and compute capability of a device (no reference
 * counterpart; for rooflines and launch sizing by callers).  Any pointer may
 * be NULL. */
int xpcs_device_properties(int32_t device, int32_t *sm_count, int32_t *cc_major,
                           int32_t *cc_minor);
int xpcs_get_device_memory(int32_t device, uint64_t *used, uint64_t *limit);

/* Page-lock (cudaHostRegister) / release a caller buffer so that ingest copies
 * from it run at full host-to-device bandwidth.  No reference counterpart: the
 * reference reads frames from disk into pageable memory (imm.cpp:70-118). */
int xpcs_pin_host(void *ptr, uint64_t bytes);
int xpcs_unpin_host(void *ptr);

/* Direct counterpart of Corr::multiTau2(SparseData*, G2, IP, IF)
 * (corr.h:98, corr.cpp:315-431) for callers that already hold pixel-major
 * event lists: row_ptr [pixels+1] (int64), frame/value [row_ptr[pixels]]
 * (Row::indxPtr / Row::valPtr, frames ascending within a row).  Outputs
 * G2/IP/IF float32 [D][pixels] on the host.  Unlike the reference, the input
 * rows are not modified.  Runs on `device`, synchronously. */
int xpcs_multitau2(const int64_t *row_ptr, const int32_t *frame, const float *value,
                   int32_t pixels, int32_t frames, int32_t delays_per_level, int32_t mode,
                   int32_t device, float *G2, float *IP, float *IF);

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- code that runs inside another framework's memory pool, a process
 * whose GPU memory budget is fixed up front, or an acquisition loop that must
 * never call cudaMalloc/cudaFree because they synchronise the device.  It
 * computes the same G2/IP/IF as xpcs_multitau2 (Corr::multiTau2 semantics,
 * bit-identical for any rows) but every array argument is a DEVICE pointer the
 * caller owns: row_ptr [pixels+1] (int64, row_ptr[pixels] == events),
 * frame/value [events], G2/IP/IF [D][pixels].  It allocates nothing: its
 * scratch (the working copy of the rows, the level plan and a status word) is
 * one fixed static device array of 16 KiB + 8 bytes x XPCS_NOALLOC_MAX_EVENTS
 * (about 32 MiB), which every GPU that loads this library holds until the
 * process exits.
 *  - events > XPCS_NOALLOC_MAX_EVENTS, or a delay schedule (frames,
 *    delays_per_level) of more than XPCS_NOALLOC_MAX_DELAYS delays, is
 *    rejected with XPCS_ERR_INVALID_ARGUMENT.
 *  - Runs on the calling thread's current device, on `stream` (a cudaStream_t;
 *    NULL = the default stream), and waits for its own work to finish.
 *  - The first call on a device is the set-up: it looks up the scratch's
 *    device address (cudaGetSymbolAddress).  With CUDA's lazy module loading
 *    (the default) that lookup is also when the driver loads this library's
 *    device code and reserves the array on that device, so make the first
 *    call at initialisation, with device memory to spare and before any
 *    stream capture, or run with CUDA_MODULE_LOADING=EAGER.  A failed set-up
 *    returns XPCS_ERR_OUT_OF_MEMORY or XPCS_ERR_CUDA with a message saying so.
 *  - The address is kept per device for the life of the process; after a
 *    cudaDeviceReset of that device it is stale, so do not call this entry
 *    point on a device after resetting it.
 *  - All calls on a device share the one scratch array, so calls that overlap
 *    on the GPU (other host threads, other streams) race: serialise them.
 *  - Rows whose row_ptr lies outside [0, events] get zero outputs and the call
 *    returns XPCS_ERR_INPUT.  A decreasing row_ptr entry makes the rows around
 *    it overlap; the outputs of overlapping rows are then unspecified (every
 *    access still stays inside [0, events)). */
#define XPCS_NOALLOC_MAX_EVENTS 4194304
#define XPCS_NOALLOC_MAX_DELAYS 512
int xpcs_multitau2_noalloc(const int64_t *row_ptr, const int32_t *frame, const float *value,
                           int32_t pixels, int64_t events, int32_t frames,
                           int32_t delays_per_level, int32_t mode, float *G2, float *IP,
                           float *IF, void *stream);

/* Two-time correlation (Corr::twotime, corr.cpp:560-924, with the smoothing of
 * corr.cpp:433-547 and 1166-1305) of the ingested frames, per processed q bin:
 * C2T [F][F] (upper triangle, zeros below, as the reference writes
 * C2T_all/g2_<q>), g2full [F][Q'] and g2partials [window][P'][Q'] with
 * P' = (F - window) / window, and the smoothing array sg [G][F] (static-map
 * smoothing: G = static bins of the processed q bins; symmetric: G = Q') or
 * [G][1] with the average filter.  Q' = processed q bins present in the
 * partition map, in mapping order.
 * mode REFERENCE: float32 in the reference's operation order (bit-identical to
 * its outputs); the pixel order of the sums is the mapping order
 * (twotimeQBinThreading) or ascending pixel index with frame_threading
 * (twotimeFrameThreading).
 * mode EXACT: needs integer counts; the Gram products of the raw counts of
 * every smoothing group are exact integers, computed on the tensor cores
 * (fp16 operands, fp32 accumulation: exact while the counts are <= 2048 and
 * sum over pixels of (max count)^2 < 2^24; other groups use an int64 CUDA-core
 * Gram), and the smoothing and reductions are applied in float64 (rounded to
 * float32 on output).  XPCS_TWOTIME_EXACT_CUDA_CORES computes the same with
 * the int64 CUDA-core Gram for every group.
 * Runs the filter/transpose itself. */
#define XPCS_TWOTIME_EXACT_CUDA_CORES 2
typedef struct {
  const int32_t *qbins;     /* /xpcs/qphi_bin_to_process */
  int32_t nqbins;
  int32_t static_map;       /* 1: smoothing_method StaticMap, 0: symmetric */
  int32_t average;          /* 1: smoothing_filter Average */
  int32_t window;           /* /xpcs/twotime2onetime_window_size (>= 1) */
  int32_t frame_threading;  /* --frame_threading */
} xpcs_twotime_desc;
typedef struct {
  int32_t qbins;            /* Q' */
  int32_t frames;           /* F */
  int32_t window;
  int32_t partials;         /* (F - window) / window */
  int32_t sg_rows, sg_cols;
  float gram_ms;            /* EXACT mode: device time of the tensor-core Gram kernels */
  double gram_flop;         /* EXACT mode: their multiply-add work, 2 x M x N x K per tile */
  double gram_flop_algorithmic; /* EXACT mode: the upper triangle's own work,
                                   2 x rows x F (F + 1) / 2 per smoothing group */
} xpcs_twotime_info;
int xpcs_twotime(xpcs_series *s, const xpcs_twotime_desc *d, int32_t mode,
                 xpcs_twotime_info *info);
/* Copies the last two-time results; any pointer may be NULL.  qbins [Q'],
 * sg [sg_rows][sg_cols], c2t [Q'][F][F], g2full [F][Q'], g2partials
 * [window][partials][Q']. */
int xpcs_get_twotime(xpcs_series *s, int32_t *qbins, float *sg, float *c2t, float *g2full,
                     float *g2partials);

/* Batches: no counterpart in the reference, which runs one series per
 * process.  A batch holds several series handles of one device (uneven frame
 * counts, detector sizes and occupancies) and runs the whole path for all of
 * them -- filter/transpose, multi-tau and normalisation -- as one CUDA graph,
 * captured on the first run and replayed until a member's frames, the mode or
 * the flags change (then it is captured again).  Members are dealt, largest
 * first, onto a number of concurrent chains.  Two forms:
 *  - work queue (the default): the chains run every member's transpose, then
 *    the multi-tau of all members runs as persistent launches over a device
 *    work queue -- one per thread-kernel row capacity, pulling 32-pixel groups
 *    of every member, and one per warp-per-pixel row tier, pulling rows of
 *    every member -- then the chains run every member's normalisation;
 *  - chains: each member's whole path runs on its chain.
 * XPCS_BATCH_AUTOTUNE times both forms with 1 .. all chains on the first run
 * (and tunes each member's knobs, xpcs_autotune) and keeps the fastest.  The
 * work of each series is the same as xpcs_multitau + xpcs_normalize on its
 * own, so results are bit-identical to running the series alone.  Member
 * handles must outlive the batch and must not be used by other threads while
 * xpcs_batch_run runs.
 *  flags: XPCS_BATCH_F64 (float64 normalisation), XPCS_BATCH_F32 (float32
 *  normalisation in the reference's operation order), XPCS_BATCH_AUTOTUNE
 *  (tune each member's kernel choice first); read the results with
 *  xpcs_get_g2ipif / xpcs_get_normalized on each member. */
typedef struct xpcs_batch xpcs_batch;
#define XPCS_BATCH_F64 1u
#define XPCS_BATCH_F32 2u
#define XPCS_BATCH_AUTOTUNE 4u /* run xpcs_autotune on members not yet tuned before capture */
int xpcs_batch_create(xpcs_series *const *series, int32_t count, xpcs_batch **out);
/* Runs the batch and waits for it. */
int xpcs_batch_run(xpcs_batch *b, int32_t mode, uint32_t flags);
/* Device time of the last run (graph launch to completion, CUDA events), the
 * number of kernels in the graph and the number of concurrent chains of
 * series in it (any pointer may be NULL). */
int xpcs_batch_stats(xpcs_batch *b, float *ms, int64_t *kernels, int32_t *lanes);
/* Occupancy timeline of the last run: for each member (in creation order),
 * when its work started and ended, in ms from the start of the graph (the
 * device's global timer, stamped by one-thread kernels in the graph around
 * each member's work).  Either pointer may be NULL. */
int xpcs_batch_timeline(xpcs_batch *b, float *start_ms, float *end_ms);
/* Chooses the form of the next runs (1: work queue, 0: chains); autotuning
 * then keeps this form and tunes only the chain count.  get_form reports the
 * form and chain count in use (either pointer may be NULL). */
int xpcs_batch_set_form(xpcs_batch *b, int32_t work_queue);
int xpcs_batch_get_form(xpcs_batch *b, int32_t *work_queue, int32_t *chains);
void xpcs_batch_destroy(xpcs_batch *b);

/* Serving (no reference counterpart): several acquisitions streamed at once.
 * An acquisition is submitted with its series description and expected event
 * count; it is admitted -- its series created on the GPU -- as soon as its
 * estimated device footprint (raw events, resident rows and work buffers,
 * ~54 B per event, plus 12 B per pixel and delay for G2/IP/IF) fits
 * `memory_budget`, in submission order (an acquisition larger than the budget
 * is admitted when nothing else is active).  Frames pushed before admission
 * wait in host memory.  push copies frames into the acquisition's resident
 * buffers on its own stream and returns; every 512 frames the acquisition's
 * new frames are transposed on its stream into pixel-major rows that stay
 * resident (xpcs_series_set_block_frames); finish enqueues the last block's
 * transpose, the join of the rows, multi-tau and the float64 normalisation
 * and returns; result waits and reads g2/stderr [D][Q]
 * (and G2/IP/IF [D][P]; any pointer may be NULL); release frees the series and
 * admits waiting acquisitions.  Results equal those of the series run alone.
 * Different acquisitions may be driven from different threads; calls for one
 * acquisition must be ordered by the caller.
 * Statistics: ingest latency per frame = arrival in push to the end of its
 * device copy; time to final g2 per acquisition = arrival of its last frame
 * (or the finish call) to the end of its normalisation. */
typedef struct xpcs_server xpcs_server;
typedef struct {
  int64_t frames_ingested;
  int64_t series_finished;
  double ingest_p50_ms, ingest_p99_ms, ingest_max_ms;
  double final_p50_ms, final_p99_ms;
  int32_t active, pending, peak_active, reserved;
  uint64_t used_bytes, peak_used_bytes;
} xpcs_server_stats;
/* xpcs_server_state values */
#define XPCS_ACQ_PENDING 0
#define XPCS_ACQ_ACTIVE 1
#define XPCS_ACQ_FINISHING 2
#define XPCS_ACQ_DONE 3
#define XPCS_ACQ_FAILED 4
int xpcs_server_create(int32_t device, uint64_t memory_budget, xpcs_server **out);
void xpcs_server_destroy(xpcs_server *srv);
int xpcs_server_submit(xpcs_server *srv, const xpcs_series_desc *desc, int64_t expected_events,
                       int64_t *id);
int xpcs_server_push_sparse(xpcs_server *srv, int64_t id, const int32_t *idx, const int16_t *val,
                            const uint32_t *nnz, int32_t nframes);
int xpcs_server_finish(xpcs_server *srv, int64_t id, int32_t mode);
int xpcs_server_state(xpcs_server *srv, int64_t id, int32_t *state);
int xpcs_server_result(xpcs_server *srv, int64_t id, double *g2, double *stderr_, float *G2,
                       float *IP, float *IF);
int xpcs_server_release(xpcs_server *srv, int64_t id);
int xpcs_server_get_stats(xpcs_server *srv, xpcs_server_stats *stats);

#ifdef __cplusplus
}
#endif

#endif
