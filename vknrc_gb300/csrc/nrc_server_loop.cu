// The serving loop on the device (nrc_server_config.device_loop): a CUDA graph
// with a while node whose body is
//   scheduler kernel -> batched query (table) -> batched training (table) -> completion kernel
// and which runs while requests keep coming. The scheduler takes the requests the
// host wrote into a ring in host-mapped memory, forms a batch first come, first
// served (one request per session per batch, training groups within the SMs)
// and writes the two launch tables; the completion kernel publishes each
// request's completion time. Batches run one after another; requests that
// arrive while one runs join the next.
#include "nrc_common.cuh"
#include "nrc_server_loop.h"

namespace nrc {

namespace {

__device__ __forceinline__ unsigned long long ld_acquire_sys(const volatile unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.sys.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void tensormap_release() {
  asm volatile("fence.proxy.tensormap::generic.release.gpu;" ::: "memory");
}

// 16-byte words of a job copied by the warp, read from L2 (the host wrote them).
template <typename T>
__device__ __forceinline__ void warp_copy(T* dst, const T* src) {
  static_assert(sizeof(T) % 16 == 0, "whole 16-byte words");
  const uint4* s = reinterpret_cast<const uint4*>(src);
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (uint32_t i = threadIdx.x; i < sizeof(T) / 16; i += 32) d[i] = __ldcg(s + i);
}

// The query CTAs of a batch: in proportion to each request's tiles (largest
// remainder), at least one and at most its useful grid each, within the SMs.
// Which CTAs answer a query does not change its result.
__device__ void split_query(const uint32_t* tiles, const uint32_t* cap, uint32_t n, uint32_t sms, uint32_t* out) {
  uint64_t wsum = 0, want = 0;
  for (uint32_t j = 0; j < n; ++j) {
    wsum += tiles[j];
    want += cap[j];
  }
  const uint32_t total = static_cast<uint32_t>(want < sms ? want : sms);
  double rem[kLoopMaxBatch];
  uint32_t used = 0;
  for (uint32_t j = 0; j < n; ++j) {
    const double share = wsum > 0 ? double(total) * double(tiles[j]) / double(wsum) : double(total) / n;
    uint32_t g = static_cast<uint32_t>(share);
    g = g < 1 ? 1 : (g > cap[j] ? cap[j] : g);
    out[j] = g;
    rem[j] = share - double(g);
    used += g;
  }
  while (used < total) {
    int best = -1;
    for (uint32_t j = 0; j < n; ++j)
      if (out[j] < cap[j] && (best < 0 || rem[j] > rem[best])) best = static_cast<int>(j);
    if (best < 0) break;
    ++out[best];
    rem[best] -= 1.0;
    ++used;
  }
  while (used > total) {
    int best = -1;
    for (uint32_t j = 0; j < n; ++j)
      if (out[j] > 1 && (best < 0 || rem[j] < rem[best])) best = static_cast<int>(j);
    if (best < 0) break;
    --out[best];
    rem[best] += 1.0;
    --used;
  }
}

__global__ void __launch_bounds__(32) loop_schedule_kernel(LoopShared* S, LoopDevice* D, const LoopSlot* slots,
                                                           uint32_t max_batch, uint32_t sms, uint32_t idle_poll_ns,
                                                           cudaGraphConditionalHandle cond) {
  __shared__ uint32_t pick[kLoopMaxBatch];
  __shared__ uint32_t n_sh;
  if (threadIdx.x == 0) {
    unsigned long long tail = D->tail;
    unsigned long long head = ld_acquire_sys(&S->head);
    uint32_t npend = D->npend;
    if (head == tail && npend == 0) {  // idle: wait (bounded) for a request
      const uint64_t t0 = globaltimer_ns();
      while (head == tail && S->stop == 0u && globaltimer_ns() - t0 < idle_poll_ns) {
        __nanosleep(256);
        head = ld_acquire_sys(&S->head);
      }
    }
    // requests move from the ring to the pending list in ring order
    while (tail < head && npend < kLoopPending) {
      const volatile LoopEntry& r = S->ring[tail & (kLoopRing - 1)];
      LoopEntry e;
      e.session = r.session;
      e.slot = r.slot;
      e.ticket = r.ticket;
      D->pend[npend++] = e;
      ++tail;
    }
    D->tail = tail;
    S->tail = tail;
    // the batch: first come, first served; a session's later requests stay
    // behind its first, and the first request that does not fit ends the batch
    uint32_t busy[kLoopMaxSessions / 32] = {};
    uint32_t n = 0, ctas = 0, kept = 0;
    uint32_t tiles[kLoopMaxBatch], cap[kLoopMaxBatch], tctas[kLoopMaxBatch];
    bool full = false;
    for (uint32_t i = 0; i < npend; ++i) {
      const LoopEntry e = D->pend[i];
      const bool in_range = e.session < kLoopMaxSessions && e.slot < kLoopMaxSlots;
      const uint32_t k = in_range ? e.session * kLoopMaxSlots + e.slot : 0u;
      if (!in_range || __ldcg(&slots[k].valid) == 0u) {
        // a request for no open session's slot (the host submits none): its
        // jobs are never launched; it completes at once and is counted
        S->done_ns[e.ticket & (kLoopRing - 1)] = globaltimer_ns();
        __threadfence_system();
        S->done_ticket[e.ticket & (kLoopRing - 1)] = e.ticket;
        S->dropped = S->dropped + 1ull;
        continue;
      }
      const uint32_t s = e.session;
      const bool seen = (busy[s >> 5] >> (s & 31u)) & 1u;
      busy[s >> 5] |= 1u << (s & 31u);
      bool take = false;
      if (!seen && !full) {
        const uint32_t tc = __ldcg(&slots[k].train_ctas);
        if (n < max_batch && ctas + tc <= sms) {
          take = true;
          ctas += tc;
          pick[n] = k;
          tiles[n] = __ldcg(&slots[k].query_tiles);
          cap[n] = __ldcg(&slots[k].query_cap);
          tctas[n] = tc;
          D->batch_ticket[n] = e.ticket;
          ++n;
        } else {
          full = true;
        }
      }
      if (!take) D->pend[kept++] = e;
    }
    D->npend = kept;
    D->batch_n = n;
    uint32_t qctas[kLoopMaxBatch];
    if (n > 0) split_query(tiles, cap, n, sms, qctas);
    uint32_t qg = 0, tg = 0;
    for (uint32_t j = 0; j < n; ++j) {
      D->infer.group_start[j] = qg;
      D->train.group_start[j] = tg;
      qg += qctas[j];
      tg += tctas[j];
    }
    D->infer.group_start[n] = qg;
    D->train.group_start[n] = tg;
    D->infer.njobs = static_cast<int>(n);
    D->train.njobs = static_cast<int>(n);
    if (n == 0 && kept == 0) {
      // nothing to run after the idle window: end this launch of the loop,
      // unless a request came meanwhile. The host publishes a request's head,
      // then reads `active` (launching the loop again if it is 0); here the
      // store of 0 comes before the read of head, so one side sees the other.
      S->idle_polls = S->idle_polls + 1ull;
      S->active = 0u;
      asm volatile("fence.sc.sys;" ::: "memory");
      if (ld_acquire_sys(&S->head) == tail)
        cudaGraphSetConditional(cond, 0u);
      else
        S->active = 1u;
    }
    n_sh = n;
  }
  __syncwarp();
  const uint32_t n = n_sh;
  for (uint32_t j = 0; j < n; ++j) {
    warp_copy(&D->infer.job[j], &slots[pick[j]].infer);
    warp_copy(&D->train.job[j], &slots[pick[j]].train);
  }
  __threadfence();
  tensormap_release();  // the copied jobs hold the tensor maps the next kernels use
}

__global__ void __launch_bounds__(32) loop_complete_kernel(LoopShared* S, const LoopDevice* D) {
  const uint32_t n = D->batch_n;
  if (n == 0) return;
  const unsigned long long t = globaltimer_ns();
  for (uint32_t j = threadIdx.x; j < n; j += 32) S->done_ns[D->batch_ticket[j] & (kLoopRing - 1)] = t;
  __threadfence_system();
  __syncwarp();
  for (uint32_t j = threadIdx.x; j < n; j += 32) {
    const unsigned long long tk = D->batch_ticket[j];
    S->done_ticket[tk & (kLoopRing - 1)] = tk;
  }
  __threadfence_system();
  if (threadIdx.x == 0) {
    S->batches = S->batches + 1ull;
    S->batched_requests = S->batched_requests + n;
  }
}

__global__ void loop_calibrate_kernel(LoopShared* S) {
  S->started = 1u;
  __threadfence_system();
  const uint64_t t0 = globaltimer_ns();
  while (S->go == 0u && globaltimer_ns() - t0 < kWaitLimitNs) {
  }
  S->calib_ns = globaltimer_ns();
  __threadfence_system();
}

}  // namespace

cudaError_t loop_build(LoopShared* shared, LoopDevice* dev, const LoopSlot* slots, uint32_t max_batch, uint32_t sms,
                       uint32_t idle_poll_ns, bool cooperative, LoopGraph* out) {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  cudaError_t e = cudaGraphCreate(&graph, 0);
  cudaGraphConditionalHandle cond = 0;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, graph, 1u, cudaGraphCondAssignDefault);
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = cond;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &p);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    cudaGraph_t body = p.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
      loop_schedule_kernel<<<1, 32, 0, cap>>>(shared, dev, slots, max_batch, sms, idle_poll_ns, cond);
      cudaError_t k = cudaGetLastError();
      if (k == cudaSuccess) k = launch_infer_table(&dev->infer, sms, cap);
      if (k == cudaSuccess) k = launch_train_table(&dev->train, sms, cooperative, cap);
      if (k == cudaSuccess) {
        loop_complete_kernel<<<1, 32, 0, cap>>>(shared, dev);
        k = cudaGetLastError();
      }
      cudaGraph_t captured = nullptr;
      e = cudaStreamEndCapture(cap, &captured);
      if (e == cudaSuccess) e = k;
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (cap != nullptr) cudaStreamDestroy(cap);
  if (e != cudaSuccess) {
    if (exec != nullptr) cudaGraphExecDestroy(exec);
    if (graph != nullptr) cudaGraphDestroy(graph);
    return e;
  }
  out->graph = graph;
  out->exec = exec;
  return cudaSuccess;
}

void loop_destroy(LoopGraph* g) {
  if (g->exec != nullptr) cudaGraphExecDestroy(g->exec);
  if (g->graph != nullptr) cudaGraphDestroy(g->graph);
  g->exec = nullptr;
  g->graph = nullptr;
}

cudaError_t loop_calibrate(LoopShared* host, LoopShared* dev, cudaStream_t stream, int64_t (*host_now_ns)(),
                           int64_t* offset_ns) {
  host->started = 0u;
  host->go = 0u;
  loop_calibrate_kernel<<<1, 1, 0, stream>>>(dev);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int64_t t0 = host_now_ns();
  while (host->started == 0u && host_now_ns() - t0 < 2000000000ll) {
  }
  const int64_t th = host_now_ns();
  host->go = 1u;
  e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return e;
  *offset_ns = static_cast<int64_t>(host->calib_ns) - th;
  return cudaSuccess;
}

}  // namespace nrc
