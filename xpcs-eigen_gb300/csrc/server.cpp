// Serving: a streaming front end over series handles.
//
// The reference analyses one finished acquisition per process.  The server
// takes several acquisitions at once, as their frames arrive:
//  - submit() registers an acquisition with its expected event count; it is
//    admitted (its series created on the GPU) as soon as its estimated device
//    footprint fits the memory budget, in submission order.  Frames pushed
//    before admission wait in host memory.
//  - push() copies a frame into the acquisition's resident raw buffers on its
//    own stream and returns; the copies of different acquisitions overlap
//    with each other and with the compute of acquisitions that finished.
//    Every SERVER_BLOCK_FRAMES frames, the block is filtered and transposed
//    on that stream into pixel-major rows that stay resident in HBM
//    (xpcs_series_set_block_frames), so the event lists are built while the
//    acquisition runs.
//  - finish() enqueues the transpose of the last, partial block, the join of
//    the blocks' rows, multi-tau and the float64 normalisation on the
//    acquisition's stream; it returns at once.
//  - result() waits for that work and reads g2/stderr; release() frees the
//    series, which admits waiting acquisitions.
// Every push records its ingest latency (arrival in push() to the end of the
// device copy, taken by a host callback on the stream); every finish records
// the time to the final g2 (last frame's arrival to the end of the
// normalisation).  The results are those of the same series run alone: each
// acquisition owns its series and its work is the same kernel sequence.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>

#include "xpcs_internal.h"

namespace xg {
namespace {

using Clock = std::chrono::steady_clock;

double now_ms() {
  return std::chrono::duration<double, std::milli>(Clock::now().time_since_epoch()).count();
}

struct Server;

struct Slot {
  int64_t id = 0;
  xpcs_series_desc desc{};
  std::vector<int32_t> dq, sq;
  std::vector<double> flat;
  uint64_t footprint = 0;
  xpcs_series *s = nullptr;
  enum State { PENDING, ACTIVE, FINISHING, DONE, FAILED } state = PENDING;
  int mode = XPCS_MODE_REFERENCE;
  bool finish_requested = false;
  // frames pushed while pending
  std::vector<uint32_t> pnnz;
  std::vector<int32_t> pidx;
  std::vector<int16_t> pval;
  std::vector<double> parrival;
  double last_arrival = 0.0;
  int status = XPCS_OK;
  std::string error;
  std::mutex mu;
  std::condition_variable cv;
};

struct Server {
  int device = 0;
  uint64_t budget = 0, used = 0, peak_used = 0;
  int32_t active = 0, peak_active = 0;
  int64_t next_id = 1;
  std::mutex mu;  // slots, pending, accounting
  std::map<int64_t, std::shared_ptr<Slot>> slots;
  std::deque<int64_t> pending;
  std::mutex stat_mu;  // latency records (also written by stream callbacks)
  std::vector<double> ingest_ms, final_ms;
  int64_t frames = 0;
};

struct IngestRec {
  Server *srv;
  double arrival;
  int32_t frames;
};

void CUDART_CB on_ingested(void *p) {
  IngestRec *r = (IngestRec *)p;
  const double t = now_ms();
  {
    std::lock_guard<std::mutex> g(r->srv->stat_mu);
    for (int32_t k = 0; k < r->frames; k++) r->srv->ingest_ms.push_back(t - r->arrival);
    r->srv->frames += r->frames;
  }
  delete r;
}

struct FinalRec {
  Server *srv;
  std::shared_ptr<Slot> slot;
};

void CUDART_CB on_final(void *p) {
  FinalRec *r = (FinalRec *)p;
  const double t = now_ms();
  {
    std::lock_guard<std::mutex> g(r->srv->stat_mu);
    r->srv->final_ms.push_back(t - r->slot->last_arrival);
  }
  {
    std::lock_guard<std::mutex> g(r->slot->mu);
    r->slot->state = Slot::DONE;
  }
  r->slot->cv.notify_all();
  delete r;
}

// Filter frames per incremental transpose block (2.56 s at 200 Hz).
constexpr int32_t SERVER_BLOCK_FRAMES = 512;

// Device footprint of an acquisition: raw events, the resident block rows and
// the transpose/list buffers (~54 B per event), per-pixel tables and G2/IP/IF
// (12 B per delay), and every block's row offsets and lengths (8 B per pixel).
uint64_t estimate_footprint(const xpcs_series_desc &d, int64_t events) {
  const uint64_t P = (uint64_t)d.width * d.height;
  const DelaySchedule ds = delay_schedule(d.frames, d.delays_per_level);
  const uint64_t blocks = (uint64_t)std::max(d.frames, 0) / SERVER_BLOCK_FRAMES + 1;
  return P * (12ull * ds.level.size() + 64 + 8 * blocks) +
         (uint64_t)std::max<int64_t>(events, 0) * 54 + (64ull << 20);
}

void check_rc(int rc) {
  if (rc != XPCS_OK) throw Error(rc, xpcs_last_error());
}

// slot.mu held.  Enqueues the ingest of frames (host arrays) and its latency record.
void ingest_locked(Server &srv, Slot &sl, const int32_t *idx, const int16_t *val,
                   const uint32_t *nnz, int32_t nframes, double arrival) {
  check_rc(xpcs_ingest_sparse(sl.s, idx, val, nnz, nframes));
  IngestRec *r = new IngestRec{&srv, arrival, nframes};
  Series &s = *(Series *)sl.s;
  const cudaError_t e = cudaLaunchHostFunc(s.stream, on_ingested, r);
  if (e != cudaSuccess) {
    delete r;
    throw Error(XPCS_ERR_CUDA, cudaGetErrorString(e));
  }
}

// slot.mu held, slot ACTIVE: the whole path on the slot's stream.
void finalize_locked(Server &srv, const std::shared_ptr<Slot> &sl) {
  Series &s = *(Series *)sl->s;
  check_rc(xpcs_multitau(sl->s, sl->mode));
  run_normalize(s, true, false);
  s.have_norm64 = true;
  s.have_norm32 = false;
  sl->state = Slot::FINISHING;
  FinalRec *r = new FinalRec{&srv, sl};
  const cudaError_t e = cudaLaunchHostFunc(s.stream, on_final, r);
  if (e != cudaSuccess) {
    delete r;
    throw Error(XPCS_ERR_CUDA, cudaGetErrorString(e));
  }
}

// Creates the series of a pending slot and replays its buffered frames.
void activate(Server &srv, const std::shared_ptr<Slot> &sl) {
  std::lock_guard<std::mutex> g(sl->mu);
  try {
    xpcs_series_desc d = sl->desc;
    d.dqmap = sl->dq.data();
    d.sqmap = sl->sq.data();
    d.flatfield = sl->flat.empty() ? nullptr : sl->flat.data();
    d.device = srv.device;
    check_rc(xpcs_series_create(&d, &sl->s));
    check_rc(xpcs_series_set_block_frames(sl->s, SERVER_BLOCK_FRAMES));
    sl->state = Slot::ACTIVE;
    size_t e0 = 0;
    for (size_t f = 0; f < sl->pnnz.size(); f++) {
      ingest_locked(srv, *sl, sl->pidx.data() + e0, sl->pval.data() + e0, &sl->pnnz[f], 1,
                    sl->parrival[f]);
      e0 += sl->pnnz[f];
    }
    sl->pnnz.clear();
    sl->pidx.clear();
    sl->pval.clear();
    sl->parrival.clear();
    if (sl->finish_requested) finalize_locked(srv, sl);
  } catch (const Error &e) {
    sl->state = Slot::FAILED;
    sl->status = e.code;
    sl->error = e.what();
  }
  sl->cv.notify_all();
}

// srv.mu held: pops the pending slots that fit, in order.
std::vector<std::shared_ptr<Slot>> admit_locked(Server &srv) {
  std::vector<std::shared_ptr<Slot>> out;
  while (!srv.pending.empty()) {
    auto it = srv.slots.find(srv.pending.front());
    if (it == srv.slots.end()) {
      srv.pending.pop_front();
      continue;
    }
    const std::shared_ptr<Slot> &sl = it->second;
    if (srv.active > 0 && srv.used + sl->footprint > srv.budget) break;
    srv.used += sl->footprint;
    srv.peak_used = std::max(srv.peak_used, srv.used);
    srv.active++;
    srv.peak_active = std::max(srv.peak_active, srv.active);
    out.push_back(sl);
    srv.pending.pop_front();
  }
  return out;
}

std::shared_ptr<Slot> find(Server &srv, int64_t id) {
  std::lock_guard<std::mutex> g(srv.mu);
  auto it = srv.slots.find(id);
  if (it == srv.slots.end()) throw Error(XPCS_ERR_INVALID_ARGUMENT, "unknown acquisition id");
  return it->second;
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

void *server_create(int device, uint64_t budget) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    throw Error(XPCS_ERR_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= ndev) throw Error(XPCS_ERR_INVALID_ARGUMENT, "device out of range");
  Server *s = new Server();
  s->device = device;
  s->budget = budget;
  return s;
}

void server_destroy(void *h) {
  Server *srv = (Server *)h;
  std::vector<std::shared_ptr<Slot>> all;
  {
    std::lock_guard<std::mutex> g(srv->mu);
    for (auto &kv : srv->slots) all.push_back(kv.second);
  }
  for (auto &sl : all) {
    // A finishing slot still has on_final queued on its stream, and on_final
    // takes sl->mu: wait for it (as server_release does) and take the series
    // out under the lock, then synchronise and destroy it without the lock.
    xpcs_series *s = nullptr;
    {
      std::unique_lock<std::mutex> g(sl->mu);
      if (sl->state == Slot::FINISHING)
        sl->cv.wait(g, [&] { return sl->state == Slot::DONE || sl->state == Slot::FAILED; });
      s = sl->s;
      sl->s = nullptr;
    }
    if (s) {
      xpcs_synchronize(s);
      xpcs_series_destroy(s);
    }
  }
  delete srv;
}

int64_t server_submit(void *h, const xpcs_series_desc &desc, int64_t expected_events) {
  Server &srv = *(Server *)h;
  if (!desc.dqmap || !desc.sqmap || desc.width <= 0 || desc.height <= 0)
    throw Error(XPCS_ERR_INVALID_ARGUMENT, "bad series description");
  if (desc.dense) throw Error(XPCS_ERR_INVALID_ARGUMENT, "the server streams sparse frames");
  auto sl = std::make_shared<Slot>();
  const size_t P = (size_t)desc.width * desc.height;
  sl->desc = desc;
  sl->dq.assign(desc.dqmap, desc.dqmap + P);
  sl->sq.assign(desc.sqmap, desc.sqmap + P);
  if (desc.flatfield) sl->flat.assign(desc.flatfield, desc.flatfield + P);
  sl->footprint = estimate_footprint(desc, expected_events);
  std::vector<std::shared_ptr<Slot>> go;
  {
    std::lock_guard<std::mutex> g(srv.mu);
    sl->id = srv.next_id++;
    srv.slots[sl->id] = sl;
    srv.pending.push_back(sl->id);
    go = admit_locked(srv);
  }
  for (auto &a : go) activate(srv, a);
  return sl->id;
}

void server_push(void *h, int64_t id, const int32_t *idx, const int16_t *val,
                 const uint32_t *nnz, int32_t nframes) {
  const double arrival = now_ms();
  Server &srv = *(Server *)h;
  std::shared_ptr<Slot> sl = find(srv, id);
  if (nframes <= 0) return;
  int64_t n = 0;
  for (int32_t f = 0; f < nframes; f++) n += nnz[f];
  std::lock_guard<std::mutex> g(sl->mu);
  if (sl->finish_requested) throw Error(XPCS_ERR_STATE, "frames pushed after finish");
  if (sl->state == Slot::FAILED) throw Error(sl->status, sl->error.c_str());
  sl->last_arrival = arrival;
  if (sl->state == Slot::PENDING) {
    sl->pnnz.insert(sl->pnnz.end(), nnz, nnz + nframes);
    sl->pidx.insert(sl->pidx.end(), idx, idx + n);
    sl->pval.insert(sl->pval.end(), val, val + n);
    sl->parrival.insert(sl->parrival.end(), (size_t)nframes, arrival);
    return;
  }
  ingest_locked(srv, *sl, idx, val, nnz, nframes, arrival);
}

void server_finish(void *h, int64_t id, int mode) {
  Server &srv = *(Server *)h;
  std::shared_ptr<Slot> sl = find(srv, id);
  std::lock_guard<std::mutex> g(sl->mu);
  if (sl->finish_requested) throw Error(XPCS_ERR_STATE, "finish called twice");
  if (sl->state == Slot::FAILED) throw Error(sl->status, sl->error.c_str());
  sl->finish_requested = true;
  sl->mode = mode;
  if (sl->last_arrival == 0.0) sl->last_arrival = now_ms();
  if (sl->state == Slot::ACTIVE) finalize_locked(srv, sl);
}

int server_state(void *h, int64_t id) {
  std::shared_ptr<Slot> sl = find(*(Server *)h, id);
  std::lock_guard<std::mutex> g(sl->mu);
  return (int)sl->state;
}

void server_result(void *h, int64_t id, double *g2, double *se, float *G2, float *IP, float *IF) {
  std::shared_ptr<Slot> sl = find(*(Server *)h, id);
  std::unique_lock<std::mutex> g(sl->mu);
  if (!sl->finish_requested) throw Error(XPCS_ERR_STATE, "finish has not been called");
  sl->cv.wait(g, [&] { return sl->state == Slot::DONE || sl->state == Slot::FAILED; });
  if (sl->state == Slot::FAILED) throw Error(sl->status, sl->error.c_str());
  if (g2 || se) check_rc(xpcs_get_normalized(sl->s, g2, se, nullptr, nullptr));
  if (G2 || IP || IF) check_rc(xpcs_get_g2ipif(sl->s, G2, IP, IF));
}

void server_release(void *h, int64_t id) {
  Server &srv = *(Server *)h;
  std::shared_ptr<Slot> sl = find(srv, id);
  bool was_active = false;
  {
    std::unique_lock<std::mutex> g(sl->mu);
    if (sl->state == Slot::FINISHING)
      sl->cv.wait(g, [&] { return sl->state == Slot::DONE || sl->state == Slot::FAILED; });
    if (sl->s) {
      xpcs_synchronize(sl->s);
      xpcs_series_destroy(sl->s);
      sl->s = nullptr;
    }
    was_active = sl->state != Slot::PENDING;
  }
  std::vector<std::shared_ptr<Slot>> go;
  {
    std::lock_guard<std::mutex> g(srv.mu);
    if (was_active) {
      srv.used -= sl->footprint;
      srv.active--;
    } else {
      srv.pending.erase(std::remove(srv.pending.begin(), srv.pending.end(), id), srv.pending.end());
    }
    srv.slots.erase(id);
    go = admit_locked(srv);
  }
  for (auto &a : go) activate(srv, a);
}

void server_stats(void *h, xpcs_server_stats *out) {
  Server &srv = *(Server *)h;
  std::vector<double> ing, fin;
  int64_t frames = 0;
  {
    std::lock_guard<std::mutex> g(srv.stat_mu);
    ing = srv.ingest_ms;
    fin = srv.final_ms;
    frames = srv.frames;
  }
  std::memset(out, 0, sizeof(*out));
  out->frames_ingested = frames;
  out->series_finished = (int64_t)fin.size();
  out->ingest_p50_ms = percentile(ing, 0.50);
  out->ingest_p99_ms = percentile(ing, 0.99);
  out->ingest_max_ms = ing.empty() ? 0.0 : *std::max_element(ing.begin(), ing.end());
  out->final_p50_ms = percentile(fin, 0.50);
  out->final_p99_ms = percentile(fin, 0.99);
  std::lock_guard<std::mutex> g(srv.mu);
  out->active = srv.active;
  out->pending = (int32_t)srv.pending.size();
  out->peak_active = srv.peak_active;
  out->used_bytes = srv.used;
  out->peak_used_bytes = srv.peak_used;
}

}  // namespace xg
