// Serving loop: many render sessions, each a device-resident cache plus frame
// slots, whose frame requests a worker thread batches continuously into
// nrc_infer_many / nrc_train_many launches. Host code only.
//
// The reference serves a single renderer whose frame is one query pass and four
// chained training passes (src/rg/NRCRenderGraph.cpp:46-80, driven once per
// frame from src/main.cpp:84-91); a request here is that frame for one session.
//
// Scheduling:
//   - requests queue in submission order; a session has at most one request in
//     flight (its training must see the previous frame's weights), so later
//     requests of a busy session wait while other sessions' requests pass them;
//   - the worker forms a batch from the eligible requests as long as the batch
//     has fewer than max_batch_sessions requests and their training groups fit
//     in the SMs, launches it (query launch, then training launch, then an
//     event) on the next of max_inflight_batches streams and goes on forming the
//     next batch while this one runs: batches hold disjoint sessions, so they
//     are independent, and their kernels share the SMs (a batch's small
//     training groups run beside the next batch's queries); training launches
//     of different batches run one after another (an event chain across the
//     streams), so two cooperative training grids never wait for each other's
//     SMs;
//   - finished batches are retired by polling their events; a request's latency
//     runs from its submission to the moment the worker sees its batch's event
//     complete.
//   - sessions are admitted against a device-memory budget (cache state + frame
//     slots), so the set of resident sessions never exceeds it.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <set>
#include <thread>
#include <unordered_map>
#include <vector>

#include "nrc_common.cuh"
#include "nrc_kernels.h"
#include "nrc_server_loop.h"

namespace {

constexpr uint32_t kMaxBatch = 32;
constexpr uint32_t kMaxSlots = 16;

using Clock = std::chrono::steady_clock;

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now().time_since_epoch()).count();
}

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

struct Session {
  bool open = false;
  nrc_session_desc desc{};
  nrc_context* ctx = nullptr;
  void* block = nullptr;  // all frame slots, one allocation
  size_t bytes = 0;       // cache state + slots, charged to the budget
  std::vector<nrc_frame_buffers> slots;
  uint32_t train_ctas = 0;
  bool in_flight = false;
  uint32_t pending = 0;   // queued or in flight
};

struct Request {
  uint64_t ticket;
  uint32_t session, slot;
  cudaEvent_t ready;
  int64_t t_submit;
};

// What a launch needs of a request's session, copied under the lock (the
// session table may grow while the launch is issued).
struct LaunchItem {
  nrc_context* ctx;
  nrc_frame_buffers f;
  uint32_t max_queries, train_records, train_ctas;
  cudaEvent_t ready;
};

struct Batch {
  cudaEvent_t done;
  std::vector<Request> reqs;
};

// Training group of a session: one CTA per four tiles of a training batch, a
// fixed function of the session alone (its results must not depend on the mix).
uint32_t default_train_ctas(uint32_t train_records, int sms) {
  const uint32_t tiles = (train_records + nrc::kTile - 1) / nrc::kTile;
  return std::max(1u, std::min<uint32_t>((tiles + 3) / 4, static_cast<uint32_t>(std::min(sms, 152))));
}

size_t slot_bytes(const nrc_session_desc& d) {
  return up256(size_t(d.max_queries) * sizeof(nrc_input)) + 256 + up256(size_t(d.max_queries) * 3 * sizeof(float)) +
         NRC_TRAIN_BATCH_COUNT * up256(size_t(d.train_records) * sizeof(nrc_train_record)) + 256;
}

double quantile(std::vector<int64_t> v, double q) {
  if (v.empty()) return 0.0;
  const size_t k = std::min(v.size() - 1, static_cast<size_t>(q * double(v.size() - 1) + 0.5));
  std::nth_element(v.begin(), v.begin() + k, v.end());
  return double(v[k]) * 1e-6;
}

}  // namespace

struct nrc_server {
  nrc_server_config cfg{};
  int device = 0;
  int sms = 0;
  std::vector<cudaStream_t> streams;  // one per in-flight batch
  // Recorded after each batch's training launch; the next batch's training
  // waits for it, so training grids of batches on different streams never
  // compete for SMs while their grid barriers wait (used by the worker only).
  cudaEvent_t train_tail = nullptr;
  uint64_t launched = 0;
  std::mutex m;
  std::condition_variable cv_work;  // new requests, or stop
  std::condition_variable cv_done;  // requests completed
  std::deque<Request> queue;
  std::deque<Batch> inflight;
  std::vector<cudaEvent_t> free_events;
  std::vector<Session> sessions;
  std::unordered_map<uint64_t, int64_t> done;  // ticket -> latency (ns), until waited on
  std::vector<int64_t> latencies;
  uint64_t next_ticket = 1;
  uint64_t submitted = 0, completed = 0, batches = 0, batched_requests = 0;
  uint64_t bytes_in_use = 0;
  bool stop = false;
  int worker_status = NRC_OK;
  std::thread worker;
  // the device-resident loop (cfg.device_loop): no worker thread
  bool device_loop = false;
  nrc::LoopShared* shared = nullptr;      // pinned, host-mapped: the host's view
  nrc::LoopShared* shared_dev = nullptr;  // the device's view
  nrc::LoopDevice* ldev = nullptr;
  nrc::LoopSlot* lslots = nullptr;        // kLoopMaxSessions x kLoopMaxSlots
  nrc::LoopGraph lgraph;
  cudaStream_t loop_stream = nullptr;
  int64_t clock_offset = 0;  // device clock minus host clock, ns
  std::unordered_map<uint64_t, std::pair<int64_t, uint32_t>> submitted_at;  // ticket -> (submit ns, session)
  std::set<uint64_t> outstanding;  // submitted, completion not yet seen
  uint64_t base_batches = 0, base_batched = 0;  // the loop's counters at the last stats reset
};

namespace {

cudaEvent_t take_event(nrc_server* S) {
  if (!S->free_events.empty()) {
    cudaEvent_t e = S->free_events.back();
    S->free_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  return e;
}

// Retires finished batches (in any order: they run on different streams).
// Caller holds the lock.
bool retire(nrc_server* S) {
  bool any = false;
  for (auto bi = S->inflight.begin(); bi != S->inflight.end();) {
    Batch& b = *bi;
    const cudaError_t q = cudaEventQuery(b.done);
    if (q == cudaErrorNotReady) {
      ++bi;
      continue;
    }
    if (q != cudaSuccess) S->worker_status = NRC_ERROR_CUDA;
    const int64_t t = now_ns();
    for (const Request& r : b.reqs) {
      Session& s = S->sessions[r.session];
      s.in_flight = false;
      --s.pending;
      S->done[r.ticket] = t - r.t_submit;
      S->latencies.push_back(t - r.t_submit);
      ++S->completed;
    }
    S->free_events.push_back(b.done);
    bi = S->inflight.erase(bi);
    any = true;
  }
  return any;
}

// Takes the eligible requests for the next batch out of the queue and fills
// `items` with what their launch needs. Caller holds the lock.
std::vector<Request> pick(nrc_server* S, std::vector<LaunchItem>& items) {
  std::vector<Request> out;
  items.clear();
  uint32_t ctas = 0;
  std::vector<uint32_t> chosen;
  for (auto it = S->queue.begin(); it != S->queue.end() && out.size() < S->cfg.max_batch_sessions;) {
    Session& s = S->sessions[it->session];
    const bool busy = s.in_flight || std::find(chosen.begin(), chosen.end(), it->session) != chosen.end();
    if (busy) {  // keeps this session's later requests behind it too
      chosen.push_back(it->session);
      ++it;
      continue;
    }
    if (ctas + s.train_ctas > static_cast<uint32_t>(S->sms)) break;  // the batch is full: first come, first served
    ctas += s.train_ctas;
    chosen.push_back(it->session);
    s.in_flight = true;
    items.push_back(LaunchItem{s.ctx, s.slots[it->slot], s.desc.max_queries, s.desc.train_records, s.train_ctas,
                               it->ready});
    out.push_back(*it);
    it = S->queue.erase(it);
  }
  return out;
}

int launch_batch(nrc_server* S, const std::vector<LaunchItem>& items, cudaStream_t stream, cudaEvent_t done) {
  nrc_query_job q[kMaxBatch];
  nrc_train_job t[kMaxBatch];
  uint32_t ctas[kMaxBatch];
  const uint32_t n = static_cast<uint32_t>(items.size());
  for (uint32_t j = 0; j < n; ++j) {
    const LaunchItem& it = items[j];
    const nrc_frame_buffers& f = it.f;
    if (it.ready != nullptr && cudaStreamWaitEvent(stream, it.ready, 0) != cudaSuccess) return NRC_ERROR_CUDA;
    q[j] = nrc_query_job{it.ctx, f.queries, f.query_count, it.max_queries, f.out_rgb, NRC_WEIGHTS_USE};
    t[j] = nrc_train_job{};
    t[j].ctx = it.ctx;
    for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) {
      t[j].records[b] = f.train[b];
      t[j].d_counts[b] = f.train_count[b];
    }
    t[j].capacity = it.train_records;
    t[j].nbatches = NRC_TRAIN_BATCH_COUNT;
    t[j].write_use_last = 1;
    ctas[j] = it.train_ctas;
  }
  int st = nrc_infer_many(q, n, nullptr, stream);
  // One training grid at a time across the streams: a cooperative grid whose
  // CTAs wait at its grid barrier for SMs that another batch's training grid
  // holds (and the other way round) would stall both until their bounded
  // waits give up. Queries of other batches still overlap the training.
  if (st == NRC_OK && cudaStreamWaitEvent(stream, S->train_tail, 0) != cudaSuccess) st = NRC_ERROR_CUDA;
  if (st == NRC_OK) st = nrc_train_many(t, n, ctas, stream);
  if (st == NRC_OK && cudaEventRecord(S->train_tail, stream) != cudaSuccess) st = NRC_ERROR_CUDA;
  if (st == NRC_OK && cudaEventRecord(done, stream) != cudaSuccess) st = NRC_ERROR_CUDA;
  return st;
}

void worker_main(nrc_server* S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->m);
  std::vector<LaunchItem> items;
  for (;;) {
    if (retire(S)) S->cv_done.notify_all();
    if (S->stop && S->queue.empty() && S->inflight.empty()) break;
    bool launched = false;
    if (S->inflight.size() < S->cfg.max_inflight_batches && !S->queue.empty()) {
      std::vector<Request> reqs = pick(S, items);
      if (!reqs.empty()) {
        cudaEvent_t ev = take_event(S);
        cudaStream_t stream = S->streams[S->launched++ % S->streams.size()];
        lk.unlock();  // launches are asynchronous; submitters need not wait for them
        const int st = ev ? launch_batch(S, items, stream, ev) : NRC_ERROR_CUDA;
        lk.lock();
        if (st != NRC_OK) {
          // the requests complete as failed: unblock their sessions and waiters
          S->worker_status = st;
          for (const Request& r : reqs) {
            Session& s = S->sessions[r.session];
            s.in_flight = false;
            --s.pending;
            S->done[r.ticket] = -1;
            ++S->completed;
          }
          if (ev) S->free_events.push_back(ev);
          S->cv_done.notify_all();
        } else {
          S->inflight.push_back(Batch{ev, std::move(reqs)});
          ++S->batches;
          S->batched_requests += S->inflight.back().reqs.size();
          launched = true;
        }
      }
    }
    if (launched) continue;
    if (S->inflight.empty()) {
      S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty(); });
    } else {
      // a batch is running: poll its event closely (latency) without holding the lock
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(5));
      lk.lock();
    }
  }
}

bool valid_session(nrc_server* S, uint32_t id) { return id < S->sessions.size() && S->sessions[id].open; }

// A session's cache and frame slots (one allocation, `slots` bytes).
int make_session(nrc_server* S, const nrc_session_desc* d, size_t slots, size_t bytes, Session* out) {
  Session& s = *out;
  s.desc = *d;
  s.bytes = bytes;
  s.train_ctas = d->train_ctas ? d->train_ctas : default_train_ctas(d->train_records, S->sms);
  int st = nrc_create(&d->cache, &s.ctx);
  if (st == NRC_OK && cudaMalloc(&s.block, slots) != cudaSuccess) st = NRC_ERROR_OUT_OF_MEMORY;
  if (st == NRC_OK && cudaMemset(s.block, 0, slots) != cudaSuccess) st = NRC_ERROR_CUDA;
  if (st != NRC_OK) return st;
  uint8_t* p = static_cast<uint8_t*>(s.block);
  for (uint32_t k = 0; k < d->frame_slots; ++k) {
    nrc_frame_buffers f{};
    f.queries = reinterpret_cast<nrc_input*>(p);
    p += up256(size_t(d->max_queries) * sizeof(nrc_input));
    f.query_count = reinterpret_cast<uint32_t*>(p);
    for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) f.train_count[b] = reinterpret_cast<uint32_t*>(p) + 4 + b;
    p += 256;
    f.out_rgb = reinterpret_cast<float*>(p);
    p += up256(size_t(d->max_queries) * 3 * sizeof(float));
    for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) {
      f.train[b] = reinterpret_cast<nrc_train_record*>(p);
      p += up256(size_t(d->train_records) * sizeof(nrc_train_record));
    }
    p += 256;
    s.slots.push_back(f);
  }
  s.open = true;
  return NRC_OK;
}

// ------------------------------------------------------ device-resident loop --
// Caller holds the lock for all of these.

// Launches the loop unless a launch of it runs (called after a request was
// published). A launch that is ending sees the request itself; launching once
// more then only queues an idle pass behind it on the loop's stream.
int loop_kick(nrc_server* S) {
  std::atomic_thread_fence(std::memory_order_seq_cst);  // the published head before the read of `active`
  if (S->shared->active != 0u) return NRC_OK;
  S->shared->active = 1u;
  return cudaGraphLaunch(S->lgraph.exec, S->loop_stream) == cudaSuccess ? NRC_OK : NRC_ERROR_CUDA;
}

// Every request written to the ring completes and the loop's launches end (so
// that device memory can be allocated or freed: both may wait for the device).
// A request still in the ring once the launches have ended (a launch that
// failed, or the two sides' flags crossed) gets a launch of its own first.
int loop_pause(nrc_server* S) {
  S->shared->stop = 1u;
  std::atomic_thread_fence(std::memory_order_seq_cst);
  // bounded: the loop ends once the requests written have run (each kernel's
  // own waits are bounded too)
  const int64_t t0 = now_ns();
  for (;;) {
    const cudaError_t e = cudaStreamQuery(S->loop_stream);
    if (e == cudaSuccess) {
      std::atomic_thread_fence(std::memory_order_seq_cst);
      // no launch runs: every request the loop took from the ring has run
      if (S->shared->tail == S->shared->head) break;
      S->shared->active = 0u;
      if (loop_kick(S) != NRC_OK) return NRC_ERROR_CUDA;  // the requests stay in the ring
    } else if (e != cudaErrorNotReady) {
      return NRC_ERROR_CUDA;
    }
    if (now_ns() - t0 > 60000000000ll) return NRC_ERROR_DEVICE_TIMEOUT;  // still running: left as it is
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  S->shared->stop = 0u;
  return NRC_OK;
}

// Collects the completions the loop has published.
void loop_poll(nrc_server* S) {
  // requests the scheduler completed without running them (no valid slot): never
  // expected, since submit checks the session first
  if (S->shared->dropped != 0ull) S->worker_status = NRC_ERROR_INVALID_ARGUMENT;
  for (auto it = S->outstanding.begin(); it != S->outstanding.end();) {
    const uint64_t t = *it;
    const uint32_t k = static_cast<uint32_t>(t & (nrc::kLoopRing - 1));
    if (S->shared->done_ticket[k] != t) {
      ++it;
      continue;
    }
    std::atomic_thread_fence(std::memory_order_acquire);  // the completion time was written first
    const auto sub = S->submitted_at[t];
    int64_t lat = static_cast<int64_t>(S->shared->done_ns[k]) - S->clock_offset - sub.first;
    if (lat < 0) lat = 0;  // within the clock calibration's error
    S->done[t] = lat;
    S->latencies.push_back(lat);
    S->submitted_at.erase(t);
    if (sub.second < S->sessions.size()) --S->sessions[sub.second].pending;
    ++S->completed;
    it = S->outstanding.erase(it);
  }
}

int loop_create(nrc_server* S) {
  void* h = nullptr;
  if (cudaHostAlloc(&h, sizeof(nrc::LoopShared), cudaHostAllocMapped) != cudaSuccess) return NRC_ERROR_OUT_OF_MEMORY;
  std::memset(h, 0, sizeof(nrc::LoopShared));
  S->shared = static_cast<nrc::LoopShared*>(h);
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess) return NRC_ERROR_CUDA;
  S->shared_dev = static_cast<nrc::LoopShared*>(d);
  const size_t slot_table = size_t(nrc::kLoopMaxSessions) * nrc::kLoopMaxSlots * sizeof(nrc::LoopSlot);
  if (cudaMalloc(&S->ldev, sizeof(nrc::LoopDevice)) != cudaSuccess) return NRC_ERROR_OUT_OF_MEMORY;
  if (cudaMalloc(&S->lslots, slot_table) != cudaSuccess) return NRC_ERROR_OUT_OF_MEMORY;
  if (cudaMemset(S->ldev, 0, sizeof(nrc::LoopDevice)) != cudaSuccess ||
      cudaMemset(S->lslots, 0, slot_table) != cudaSuccess)
    return NRC_ERROR_CUDA;
  if (cudaStreamCreateWithFlags(&S->loop_stream, cudaStreamNonBlocking) != cudaSuccess) return NRC_ERROR_CUDA;
  if (nrc::loop_calibrate(S->shared, S->shared_dev, S->loop_stream, now_ns, &S->clock_offset) != cudaSuccess)
    return NRC_ERROR_CUDA;
  const uint32_t sms = static_cast<uint32_t>(std::min(S->sms, 152));
  const uint32_t kIdlePollNs = 200000;  // a launch of the loop ends after 200 us without requests
  // the training launch node with the cooperative attribute; without it if the
  // graph cannot hold one (its groups still fit on the SMs at once)
  cudaError_t e = nrc::loop_build(S->shared_dev, S->ldev, S->lslots, S->cfg.max_batch_sessions, sms, kIdlePollNs,
                                  true, &S->lgraph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = nrc::loop_build(S->shared_dev, S->ldev, S->lslots, S->cfg.max_batch_sessions, sms, kIdlePollNs, false,
                        &S->lgraph);
  }
  return e == cudaSuccess ? NRC_OK : NRC_ERROR_CUDA;  // the first request launches the loop
}

void loop_free(nrc_server* S) {
  nrc::loop_destroy(&S->lgraph);
  if (S->loop_stream) cudaStreamDestroy(S->loop_stream);
  if (S->lslots) cudaFree(S->lslots);
  if (S->ldev) cudaFree(S->ldev);
  if (S->shared) cudaFreeHost(S->shared);
  S->loop_stream = nullptr;
  S->lslots = nullptr;
  S->ldev = nullptr;
  S->shared = nullptr;
}

// The session's slots as the loop reads them (or zeros: no longer valid).
int loop_write_slots(nrc_server* S, uint32_t id, const Session* s) {
  std::vector<nrc::LoopSlot> rows(nrc::kLoopMaxSlots);
  std::memset(static_cast<void*>(rows.data()), 0, rows.size() * sizeof(nrc::LoopSlot));
  if (s != nullptr) {
    for (uint32_t k = 0; k < s->slots.size(); ++k) {
      nrc::LoopSlot& r = rows[k];
      const int st = nrc::loop_slot_jobs(s->ctx, s->slots[k], s->desc.max_queries, s->desc.train_records, &r.infer,
                                         &r.train);
      if (st != NRC_OK) return st;
      r.train_ctas = s->train_ctas;
      r.query_tiles = (s->desc.max_queries + nrc::kTile - 1) / nrc::kTile;
      r.query_cap = std::max(1u, nrc::infer_grid(s->desc.max_queries, std::min(S->sms, 152)));
      r.valid = 1u;
    }
  }
  return cudaMemcpy(S->lslots + size_t(id) * nrc::kLoopMaxSlots, rows.data(), rows.size() * sizeof(nrc::LoopSlot),
                    cudaMemcpyHostToDevice) == cudaSuccess
             ? NRC_OK
             : NRC_ERROR_CUDA;
}

}  // namespace

extern "C" {

int nrc_server_create(const nrc_server_config* cfg, nrc_server** out) {
  if (cfg == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  if (cfg->max_batch_sessions < 1 || cfg->max_batch_sessions > kMaxBatch || cfg->max_inflight_batches < 1 ||
      cfg->max_inflight_batches > 8 || cfg->hbm_budget_bytes == 0)
    return NRC_ERROR_INVALID_ARGUMENT;
  int dev = 0, count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return NRC_ERROR_NO_DEVICE;
  if (cudaGetDevice(&dev) != cudaSuccess) return NRC_ERROR_CUDA;
  int major = 0, minor = 0, sms = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (!(major == 10 && minor == 3)) return NRC_ERROR_UNSUPPORTED_DEVICE;
  nrc_server* S = new (std::nothrow) nrc_server();
  if (S == nullptr) return NRC_ERROR_OUT_OF_MEMORY;
  S->cfg = *cfg;
  S->device = dev;
  S->sms = sms;
  for (uint32_t k = 0; k < cfg->max_inflight_batches; ++k) {
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      for (cudaStream_t x : S->streams) cudaStreamDestroy(x);
      delete S;
      return NRC_ERROR_CUDA;
    }
    S->streams.push_back(st);
  }
  if (cudaEventCreateWithFlags(&S->train_tail, cudaEventDisableTiming) != cudaSuccess) {
    for (cudaStream_t x : S->streams) cudaStreamDestroy(x);
    delete S;
    return NRC_ERROR_CUDA;
  }
  if (cfg->device_loop != 0) {
    S->device_loop = true;
    const int st = loop_create(S);
    if (st != NRC_OK) {
      loop_free(S);
      cudaEventDestroy(S->train_tail);
      for (cudaStream_t x : S->streams) cudaStreamDestroy(x);
      delete S;
      return st;
    }
    *out = S;
    return NRC_OK;
  }
  S->worker = std::thread(worker_main, S);
  *out = S;
  return NRC_OK;
}

int nrc_server_destroy(nrc_server* S) {
  if (S == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lk(S->m);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  if (S->device_loop) {
    std::lock_guard<std::mutex> lk(S->m);
    if (loop_pause(S) != NRC_OK) S->worker_status = NRC_ERROR_CUDA;  // every written request completes first
    loop_poll(S);
  }
  for (cudaStream_t x : S->streams) cudaStreamSynchronize(x);
  for (Session& s : S->sessions) {
    if (!s.open) continue;
    nrc_destroy(s.ctx);
    cudaFree(s.block);
  }
  for (cudaEvent_t e : S->free_events) cudaEventDestroy(e);
  cudaEventDestroy(S->train_tail);
  if (S->device_loop) loop_free(S);
  for (cudaStream_t x : S->streams) cudaStreamDestroy(x);
  const int st = S->worker_status;
  delete S;
  return st;
}

int nrc_server_open_session(nrc_server* S, const nrc_session_desc* d, uint32_t* id) {
  if (S == nullptr || d == nullptr || id == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (d->max_queries == 0 || d->train_records == 0 || d->frame_slots < 1 || d->frame_slots > kMaxSlots ||
      d->train_ctas > static_cast<uint32_t>(S->sms))
    return NRC_ERROR_INVALID_ARGUMENT;
  const size_t slots = size_t(d->frame_slots) * slot_bytes(*d);
  const size_t bytes = slots + nrc::context_device_bytes_for(S->sms);
  if (S->device_loop) {
    // the loop pauses while the session's memory is allocated and its slots
    // are written; submitters wait on the lock meanwhile
    std::lock_guard<std::mutex> lk(S->m);
    if (S->bytes_in_use + bytes > S->cfg.hbm_budget_bytes) return NRC_ERROR_OUT_OF_MEMORY;
    uint32_t sid = 0;
    while (sid < S->sessions.size() && S->sessions[sid].open) ++sid;
    if (sid >= nrc::kLoopMaxSessions) return NRC_ERROR_INVALID_ARGUMENT;
    int st = loop_pause(S);
    Session s;
    if (st == NRC_OK) st = make_session(S, d, slots, bytes, &s);
    if (st == NRC_OK) st = loop_write_slots(S, sid, &s);
    if (st == NRC_OK) {
      if (sid == S->sessions.size()) S->sessions.emplace_back();
      S->sessions[sid] = std::move(s);
      S->bytes_in_use += bytes;
      *id = sid;
    } else {
      if (s.ctx) nrc_destroy(s.ctx);
      if (s.block) cudaFree(s.block);
    }
    return st;
  }
  {
    std::lock_guard<std::mutex> lk(S->m);
    if (S->bytes_in_use + bytes > S->cfg.hbm_budget_bytes) return NRC_ERROR_OUT_OF_MEMORY;
    S->bytes_in_use += bytes;  // reserved while the session is built
  }
  Session s;
  const int st = make_session(S, d, slots, bytes, &s);
  if (st != NRC_OK) {
    if (s.ctx) nrc_destroy(s.ctx);
    if (s.block) cudaFree(s.block);
    std::lock_guard<std::mutex> lk(S->m);
    S->bytes_in_use -= bytes;
    return st;
  }
  std::lock_guard<std::mutex> lk(S->m);
  for (uint32_t k = 0; k < S->sessions.size(); ++k)
    if (!S->sessions[k].open) {
      S->sessions[k] = std::move(s);
      *id = k;
      return NRC_OK;
    }
  S->sessions.push_back(std::move(s));
  *id = static_cast<uint32_t>(S->sessions.size() - 1);
  return NRC_OK;
}

int nrc_server_close_session(nrc_server* S, uint32_t id) {
  if (S == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  Session s;
  if (S->device_loop) {
    std::lock_guard<std::mutex> lk(S->m);
    if (!valid_session(S, id)) return NRC_ERROR_INVALID_ARGUMENT;
    // every request written, this session's included, completes; if the loop
    // could not be paused its kernels may still read the session: it stays open
    const int paused = loop_pause(S);
    if (paused != NRC_OK) return paused;
    loop_poll(S);
    const int st = loop_write_slots(S, id, nullptr);
    s = std::move(S->sessions[id]);
    S->sessions[id] = Session{};
    S->bytes_in_use -= s.bytes;
    nrc_destroy(s.ctx);
    cudaFree(s.block);
    return st;
  }
  {
    std::unique_lock<std::mutex> lk(S->m);
    if (!valid_session(S, id)) return NRC_ERROR_INVALID_ARGUMENT;
    S->cv_done.wait(lk, [&] { return S->sessions[id].pending == 0; });
    s = std::move(S->sessions[id]);
    S->sessions[id] = Session{};
    S->bytes_in_use -= s.bytes;
  }
  nrc_destroy(s.ctx);
  cudaFree(s.block);
  return NRC_OK;
}

int nrc_server_frame_buffers(nrc_server* S, uint32_t id, uint32_t slot, nrc_frame_buffers* out) {
  if (S == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->m);
  if (!valid_session(S, id) || slot >= S->sessions[id].slots.size()) return NRC_ERROR_INVALID_ARGUMENT;
  *out = S->sessions[id].slots[slot];
  return NRC_OK;
}

int nrc_server_session_cache(nrc_server* S, uint32_t id, nrc_context** ctx) {
  if (S == nullptr || ctx == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->m);
  if (!valid_session(S, id)) return NRC_ERROR_INVALID_ARGUMENT;
  *ctx = S->sessions[id].ctx;
  return NRC_OK;
}

int nrc_server_submit(nrc_server* S, uint32_t id, uint32_t slot, void* ready, uint64_t* ticket) {
  if (S == nullptr || ticket == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (S->device_loop) {
    // the device cannot wait on a host-recorded event: the submitter does
    if (ready != nullptr && cudaEventSynchronize(static_cast<cudaEvent_t>(ready)) != cudaSuccess)
      return NRC_ERROR_CUDA;
    std::unique_lock<std::mutex> lk(S->m);
    if (S->stop || !valid_session(S, id) || slot >= S->sessions[id].slots.size()) return NRC_ERROR_INVALID_ARGUMENT;
    // room in the ring, and no completion record reused before it is read
    const int64_t t0 = now_ns();
    for (;;) {
      loop_poll(S);
      const bool ring_full = S->shared->head - S->shared->tail >= nrc::kLoopRing;
      const bool window_full = !S->outstanding.empty() && S->next_ticket - *S->outstanding.begin() >= nrc::kLoopRing;
      if (!ring_full && !window_full) break;
      if (now_ns() - t0 > 10000000000ll) return NRC_ERROR_DEVICE_TIMEOUT;
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      lk.lock();
    }
    const uint64_t t = S->next_ticket++;
    const unsigned long long h = S->shared->head;
    nrc::LoopEntry& e = S->shared->ring[h & (nrc::kLoopRing - 1)];
    e.session = id;
    e.slot = slot;
    e.ticket = t;
    std::atomic_thread_fence(std::memory_order_seq_cst);  // the entry before the head that publishes it
    S->shared->head = h + 1;
    S->submitted_at[t] = {now_ns(), id};
    S->outstanding.insert(t);
    ++S->sessions[id].pending;
    ++S->submitted;
    *ticket = t;
    return loop_kick(S);  // on failure the request stays in the ring for the next launch
  }
  {
    std::lock_guard<std::mutex> lk(S->m);
    if (S->stop || !valid_session(S, id) || slot >= S->sessions[id].slots.size()) return NRC_ERROR_INVALID_ARGUMENT;
    const uint64_t t = S->next_ticket++;
    S->queue.push_back(Request{t, id, slot, static_cast<cudaEvent_t>(ready), now_ns()});
    ++S->sessions[id].pending;
    ++S->submitted;
    *ticket = t;
  }
  S->cv_work.notify_one();
  return NRC_OK;
}

int nrc_server_wait(nrc_server* S, uint64_t ticket, double timeout_ms, double* latency_ms) {
  if (S == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (S->device_loop) {
    const int64_t t0 = now_ns();
    std::unique_lock<std::mutex> lk(S->m);
    if (ticket == 0 || ticket >= S->next_ticket) return NRC_ERROR_INVALID_ARGUMENT;
    for (;;) {
      if (S->done.count(ticket) == 0) loop_poll(S);
      if (S->done.count(ticket) != 0) break;
      if (S->outstanding.count(ticket) == 0) return NRC_ERROR_INVALID_ARGUMENT;  // already waited for
      if (timeout_ms >= 0 && double(now_ns() - t0) * 1e-6 > timeout_ms) return NRC_ERROR_DEVICE_TIMEOUT;
      // a request left in the ring with no launch of the loop running (should
      // the two sides' flags have crossed): launch it again
      if (now_ns() - t0 > 2000000 && cudaStreamQuery(S->loop_stream) == cudaSuccess &&
          S->shared->tail != S->shared->head) {
        S->shared->active = 0u;
        const int st = loop_kick(S);
        if (st != NRC_OK) return st;
      }
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(5));
      lk.lock();
    }
    const int64_t ns = S->done[ticket];
    S->done.erase(ticket);
    if (latency_ms) *latency_ms = double(ns) * 1e-6;
    return S->worker_status;
  }
  std::unique_lock<std::mutex> lk(S->m);
  if (ticket == 0 || ticket >= S->next_ticket) return NRC_ERROR_INVALID_ARGUMENT;
  auto ready = [&] { return S->done.count(ticket) != 0; };
  if (timeout_ms < 0) {
    S->cv_done.wait(lk, ready);
  } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
    return NRC_ERROR_DEVICE_TIMEOUT;
  }
  const int64_t ns = S->done[ticket];
  S->done.erase(ticket);
  if (latency_ms) *latency_ms = double(ns) * 1e-6;
  return ns < 0 ? (S->worker_status != NRC_OK ? S->worker_status : NRC_ERROR_CUDA) : NRC_OK;
}

int nrc_server_get_stats(nrc_server* S, nrc_server_stats* st, int reset) {
  if (S == nullptr || st == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->m);
  if (S->device_loop) {
    loop_poll(S);
    S->batches = S->shared->batches - S->base_batches;
    S->batched_requests = S->shared->batched_requests - S->base_batched;
  }
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->batches = S->batches;
  st->bytes_in_use = S->bytes_in_use;
  st->latency_p50_ms = quantile(S->latencies, 0.5);
  st->latency_p99_ms = quantile(S->latencies, 0.99);
  st->latency_max_ms = S->latencies.empty() ? 0.0 : double(*std::max_element(S->latencies.begin(),
                                                                               S->latencies.end())) * 1e-6;
  st->mean_batch_sessions = S->batches ? double(S->batched_requests) / double(S->batches) : 0.0;
  if (reset) {
    S->latencies.clear();
    S->batches = 0;
    S->batched_requests = 0;
    if (S->device_loop) {
      S->base_batches = S->shared->batches;
      S->base_batched = S->shared->batched_requests;
    }
  }
  return S->worker_status;
}

}  // extern "C"
