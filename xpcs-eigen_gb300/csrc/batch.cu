// Batches of series run as one CUDA graph.
//
// The reference processes one series per `corr` process (main.cpp:86-479).
// A batch runs the path of several series -- filter/transpose (K-a),
// multi-tau (K-c) and normalisation (K-d) -- as one graph in which every
// series is an independent branch: the kernels of small series run side by
// side instead of one after another, and the whole batch costs one launch
// from the host.  The graph is captured from the series' own streams (fork
// from the batch's origin stream, join back), after one eager pass that
// sizes every buffer and uploads every per-series table, so that the
// captured work is kernels and device-side copies only.  It is replayed
// until a member's frames (its generation counter), the mode or the flags
// change.
//
// Schedule: the series are dealt, largest first, onto `lanes` chains (each
// chain runs its series one after another; the chains run side by side), so
// that a few large series do not all compete for the GPU at once while the
// small ones fill the gaps.  With XPCS_BATCH_AUTOTUNE the lane count is chosen
// by timing the candidates on the first run.
#include <algorithm>
#include <numeric>

#include <initializer_list>

#include "xpcs_internal.h"

namespace xg {

Batch::~Batch() {
  if (exec) cudaGraphExecDestroy(exec);
  for (cudaEvent_t e : join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : join2)
    if (e) cudaEventDestroy(e);
  if (fork2) cudaEventDestroy(fork2);
  if (origin) {
    mtq.tab.release(origin);
    mtq.next.release(origin);
  }
  if (origin) {
    stamps.release(origin);
    cudaStreamSynchronize(origin);
  }
  if (fork) cudaEventDestroy(fork);
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  if (origin) cudaStreamDestroy(origin);
}

Batch *batch_create(Series *const *ss, int32_t n) {
  if (n <= 0) throw Error(XPCS_ERR_INVALID_ARGUMENT, "empty batch");
  for (int32_t i = 0; i < n; i++) {
    if (!ss[i]) throw Error(XPCS_ERR_INVALID_ARGUMENT, "null series in batch");
    if (ss[i]->device != ss[0]->device)
      throw Error(XPCS_ERR_INVALID_ARGUMENT, "batch members must use one device");
    for (int32_t j = 0; j < i; j++)
      if (ss[j] == ss[i]) throw Error(XPCS_ERR_INVALID_ARGUMENT, "series twice in one batch");
    if (ss[i]->desc.normalize_by_framesum)
      throw Error(XPCS_ERR_INVALID_ARGUMENT,
                  "normalize_by_framesum reads frame sums back to the host: not in a batch");
    if (ss[i]->block_frames > 0)
      throw Error(XPCS_ERR_INVALID_ARGUMENT,
                  "series with incremental transposes finish from host-held block tables: "
                  "not in a batch");
  }
  Batch *b = new Batch();
  try {
    b->ss.assign(ss, ss + n);
    b->device = ss[0]->device;
    XG_CUDA(cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
    XG_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    XG_CUDA(cudaEventCreate(&b->t0));
    XG_CUDA(cudaEventCreate(&b->t1));
    b->join.assign(n, nullptr);
    for (auto &e : b->join) XG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->join2.assign(n, nullptr);
    for (auto &e : b->join2) XG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    XG_CUDA(cudaEventCreateWithFlags(&b->fork2, cudaEventDisableTiming));
    b->stamps.reserve(2 * (size_t)n + 1, b->origin);
  } catch (...) {
    delete b;
    throw;
  }
  return b;
}

// Autotuner: times filter + multi-tau of the series' frames (one untimed pass
// sizes the buffers, the second pass of each candidate is timed) over the
// kernel knobs, one knob at a time, keeping the fastest value of each before
// moving to the next:
//   1. warps per pixel: the row capacity of the thread-per-pixel kernel (a
//      thread per pixel up to CAP events, a warp per pixel above it);
//   2. the level-fold schedule: scratch words per lane of the thread kernel,
//      which decide up to which level (32 x words bins) the pair search runs
//      on the occupancy bitmask instead of the sparse two-candidate checks;
//   3. the event tile of the transpose: 8 or 16 items per lane (tiles of
//      2,048 or 4,096 events).
// A change of any knob changes the work (pixel classes, kernel launch), so it
// counts as a change of the series for captured batch graphs.  Results do not
// depend on the knobs.
int32_t autotune(Series &s, int mode) {
  cudaStream_t st = s.stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  XG_CUDA(cudaEventCreate(&e0));
  XG_CUDA(cudaEventCreate(&e1));
  const int32_t cap0 = s.thread_cap, scr0 = s.scr_extra, ipt0 = s.radix_ipt;
  const bool set0 = s.knobs_set;
  s.knobs_set = true;  // the candidates below are not replaced by the defaults
  auto time_pass = [&]() {
    float ms = 0.f;
    for (int rep = 0; rep < 2; rep++) {  // the second pass is timed
      XG_CUDA(cudaEventRecord(e0, st));
      run_filter_transpose(s);
      run_multitau(s, mode);
      XG_CUDA(cudaEventRecord(e1, st));
      XG_CUDA(cudaEventSynchronize(e1));
      XG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    }
    return ms;
  };
  // one knob: try each value, keep the fastest
  auto search = [&](int32_t &knob, std::initializer_list<int32_t> values) {
    int32_t best = knob;
    float best_ms = 0.f;
    bool first = true;
    for (int32_t v : values) {
      knob = v;
      const float ms = time_pass();
      if (first || ms < best_ms) {
        best_ms = ms;
        best = v;
        first = false;
      }
    }
    knob = best;
  };
  try {
    s.scr_extra = 0;
    s.radix_ipt = 0;
    search(s.thread_cap, {32, 48, 64, 80, 112});
    search(s.scr_extra, {0, 8});
    search(s.radix_ipt, {8, 16});
  } catch (...) {
    s.thread_cap = cap0;
    s.scr_extra = scr0;
    s.radix_ipt = ipt0;
    s.knobs_set = set0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s.tuned = true;
  s.knobs_set = true;
  s.have_multitau = false;
  s.have_norm64 = s.have_norm32 = false;
  s.generation++;
  return s.thread_cap;
}

namespace {

// The device's global nanosecond timer, for the batch's occupancy timeline.
__global__ void k_stamp(unsigned long long *dst) {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  *dst = t;
}

void series_pass(Series &s, int mode, uint32_t flags) {
  run_filter_transpose(s);
  run_multitau(s, mode);
  run_normalize(s, (flags & XPCS_BATCH_F64) != 0, (flags & XPCS_BATCH_F32) != 0);
}

bool stale(const Batch &b, int mode, uint32_t flags) {
  if (!b.exec || b.mode != mode || b.flags != flags || b.gens.size() != b.ss.size()) return true;
  for (size_t i = 0; i < b.ss.size(); i++) {
    if (b.ss[i]->generation != b.gens[i]) return true;
    if ((flags & XPCS_BATCH_AUTOTUNE) && !b.ss[i]->tuned) return true;
  }
  return false;
}

// The batch as one CUDA graph.  Members are dealt, largest first, onto
// `lanes` chains that run side by side.
//   chains form: each member's whole path (transpose, multi-tau,
//     normalisation) runs on its chain;
//   work-queue form: the chains run every member's transpose; then the
//     multi-tau of all members runs as persistent work-queue launches (one per
//     thread-kernel row capacity, one per warp-per-pixel row tier) that pull
//     32-pixel groups and rows of every member from device counters; then the
//     chains run every member's normalisation.
void build_graph(Batch &b, int mode, uint32_t flags, int lanes, bool queue) {
  if (b.exec) {
    cudaGraphExecDestroy(b.exec);
    b.exec = nullptr;
  }
  const int n = (int)b.ss.size();
  if (lanes <= 0 || lanes > n) lanes = n;
  // largest first, each onto the least loaded chain
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return b.ss[x]->raw_events > b.ss[y]->raw_events;
  });
  std::vector<int64_t> load(lanes, 0);
  std::vector<int> last(lanes, -1);  // last series of each chain
  std::vector<int> chain(n, 0);
  XG_CUDA(cudaStreamBeginCapture(b.origin, cudaStreamCaptureModeRelaxed));
  cudaGraph_t g = nullptr;
  const int64_t l0 = tl_launches;
  try {
    k_stamp<<<1, 1, 0, b.origin>>>(b.stamps.p + 2 * n);
    XG_CHECK_LAUNCH();
    XG_CUDA(cudaEventRecord(b.fork, b.origin));
    for (int i : order) {
      const int c = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      Series &s = *b.ss[i];
      XG_CUDA(cudaStreamWaitEvent(s.stream, last[c] < 0 ? b.fork : b.join[last[c]], 0));
      k_stamp<<<1, 1, 0, s.stream>>>(b.stamps.p + 2 * i);
      XG_CHECK_LAUNCH();
      if (queue) {
        run_filter_transpose(s);
      } else {
        series_pass(s, mode, flags);
        k_stamp<<<1, 1, 0, s.stream>>>(b.stamps.p + 2 * i + 1);
        XG_CHECK_LAUNCH();
      }
      XG_CUDA(cudaEventRecord(b.join[i], s.stream));
      load[c] += s.raw_events + s.P;
      last[c] = i;
      chain[i] = c;
    }
    for (int c = 0; c < lanes; c++)
      if (last[c] >= 0) XG_CUDA(cudaStreamWaitEvent(b.origin, b.join[last[c]], 0));
    if (queue) {
      mt_queue_run(b.ss, b.mtq, b.origin);
      XG_CUDA(cudaEventRecord(b.fork2, b.origin));
      std::vector<int> last2(lanes, -1);
      for (int i : order) {
        const int c = chain[i];
        Series &s = *b.ss[i];
        XG_CUDA(cudaStreamWaitEvent(s.stream, last2[c] < 0 ? b.fork2 : b.join2[last2[c]], 0));
        run_normalize(s, (flags & XPCS_BATCH_F64) != 0, (flags & XPCS_BATCH_F32) != 0);
        k_stamp<<<1, 1, 0, s.stream>>>(b.stamps.p + 2 * i + 1);
        XG_CHECK_LAUNCH();
        XG_CUDA(cudaEventRecord(b.join2[i], s.stream));
        last2[c] = i;
      }
      for (int c = 0; c < lanes; c++)
        if (last2[c] >= 0) XG_CUDA(cudaStreamWaitEvent(b.origin, b.join2[last2[c]], 0));
    }
  } catch (...) {
    cudaStreamEndCapture(b.origin, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    throw;
  }
  XG_CUDA(cudaStreamEndCapture(b.origin, &g));
  b.kernels = tl_launches - l0;
  const cudaError_t e = cudaGraphInstantiate(&b.exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    b.exec = nullptr;
    throw Error(XPCS_ERR_CUDA, cudaGetErrorString(e));
  }
  b.lanes = lanes;
  b.queue = queue;
}

float launch(Batch &b) {
  XG_CUDA(cudaEventRecord(b.t0, b.origin));
  XG_CUDA(cudaGraphLaunch(b.exec, b.origin));
  XG_CUDA(cudaEventRecord(b.t1, b.origin));
  XG_CUDA(cudaStreamSynchronize(b.origin));
  float ms = 0.f;
  XG_CUDA(cudaEventElapsedTime(&ms, b.t0, b.t1));
  // each member's work in this run, from the fork (the occupancy timeline)
  const size_t n = b.ss.size();
  std::vector<unsigned long long> t(2 * n + 1);
  XG_CUDA(cudaMemcpy(t.data(), b.stamps.p, sizeof(unsigned long long) * t.size(),
                     cudaMemcpyDeviceToHost));
  b.start_ms.assign(n, 0.f);
  b.end_ms.assign(n, 0.f);
  for (size_t i = 0; i < n; i++) {
    b.start_ms[i] = (float)((double)(long long)(t[2 * i] - t[2 * n]) * 1e-6);
    b.end_ms[i] = (float)((double)(long long)(t[2 * i + 1] - t[2 * n]) * 1e-6);
  }
  return ms;
}

void capture(Batch &b, int mode, uint32_t flags) {
  if (flags & XPCS_BATCH_AUTOTUNE)
    for (Series *s : b.ss)
      if (!s->tuned) autotune(*s, mode);
  // eager pass: buffers reach their sizes, frame tables and plans are uploaded
  for (Series *s : b.ss) series_pass(*s, mode, flags);
  for (Series *s : b.ss) XG_CUDA(cudaStreamSynchronize(s->stream));
  mt_queue_build(b.ss, b.mtq, b.origin);
  const int n = (int)b.ss.size();
  if ((flags & XPCS_BATCH_AUTOTUNE) && !b.lanes_tuned) {
    // both forms, each with 1 .. n chains; the fastest graph is kept
    int best = n;
    bool best_queue = b.queue;
    float best_ms = 0.f;
    bool first = true;
    for (bool queue : {true, false}) {
      if (b.form_tuned && queue != b.queue) continue;  // a form the caller chose
      for (int lanes : {1, 2, 4, 8, 16, n}) {
        if (lanes > n) continue;
        build_graph(b, mode, flags, lanes, queue);
        launch(b);
        const float ms = launch(b);
        if (first || ms < best_ms) {
          best_ms = ms;
          best = lanes;
          best_queue = queue;
          first = false;
        }
      }
    }
    b.lanes = best;
    b.queue = best_queue;
    b.lanes_tuned = true;
  }
  build_graph(b, mode, flags, b.lanes, b.queue);
  b.mode = mode;
  b.flags = flags;
  b.gens.resize(b.ss.size());
  for (size_t i = 0; i < b.ss.size(); i++) b.gens[i] = b.ss[i]->generation;
}

}  // namespace

void batch_run(Batch &b, int mode, uint32_t flags) {
  if (stale(b, mode, flags)) capture(b, mode, flags);
  b.last_ms = launch(b);
  for (Series *s : b.ss) {
    s->have_multitau = true;
    s->have_norm64 = (flags & XPCS_BATCH_F64) != 0;
    s->have_norm32 = (flags & XPCS_BATCH_F32) != 0;
  }
}

}  // namespace xg
