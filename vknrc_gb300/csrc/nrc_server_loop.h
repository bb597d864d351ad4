// The serving loop's device-resident form: a CUDA graph whose while-loop body
// (scheduler kernel -> batched query -> batched training -> completion kernel)
// runs on the GPU as long as requests keep coming, taking them from a ring in
// host-mapped memory. No host thread takes part in forming or launching a
// batch: the host writes requests into the ring and reads completions back. A
// launch of the loop ends once it finds no request within its idle window (so
// a device-wide synchronisation waits for the requests in flight, not
// forever); the host launches it again with the next request.
#pragma once
#include <cstdint>

#include "nrc_kernels.h"

namespace nrc {

constexpr uint32_t kLoopRing = 1u << 14;   // request ring and completion records (power of two)
constexpr uint32_t kLoopPending = 1024;    // requests taken from the ring, not yet in a batch
constexpr uint32_t kLoopMaxSessions = 256;
constexpr uint32_t kLoopMaxSlots = 16;
constexpr uint32_t kLoopMaxBatch = 32;
static_assert(kLoopMaxBatch <= kMaxInferJobs && kLoopMaxBatch <= kMaxTrainJobs, "batch fits one launch");

struct LoopEntry {
  uint32_t session, slot;
  unsigned long long ticket;
};

// Pinned, host-mapped block that the host and the loop's kernels share.
struct LoopShared {
  volatile unsigned long long head;  // host: requests written to the ring
  unsigned long long pad0[7];
  volatile unsigned long long tail;  // device: requests taken from the ring (their entries may be reused)
  unsigned long long pad1[7];
  volatile uint32_t stop;            // host: finish every request written, then end the loop
  volatile uint32_t started, go;     // clock calibration handshake
  volatile uint32_t active;          // 1 while a launch of the loop runs; the loop sets 0 as it ends
  uint32_t pad2[12];
  volatile unsigned long long batches, batched_requests;  // device: launched batches and their requests
  volatile unsigned long long calib_ns;                   // device clock at the calibration's go
  volatile unsigned long long idle_polls;                 // device: scheduler passes that found no request
  volatile unsigned long long dropped;                    // device: requests for no valid slot, completed unrun
  unsigned long long pad3[3];
  LoopEntry ring[kLoopRing];
  volatile unsigned long long done_ticket[kLoopRing];  // device: completed ticket t at t % kLoopRing
  volatile unsigned long long done_ns[kLoopRing];      // device: its completion time (%globaltimer)
};

// One frame slot of one session, as the loop's launches need it (written by
// the host when the session opens; `valid` last).
struct LoopSlot {
  InferJob infer;
  TrainJob train;
  uint32_t train_ctas, query_tiles, query_cap, valid;
};

// The loop's state in device memory.
struct LoopDevice {
  InferLaunch<kMaxInferJobs> infer;
  TrainLaunch<kMaxTrainJobs> train;
  unsigned long long batch_ticket[kLoopMaxBatch];
  uint32_t batch_n, npend;
  unsigned long long tail;
  LoopEntry pend[kLoopPending];
};

struct LoopGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

// Builds and instantiates the loop graph over `shared` (its device view),
// `dev` and the slot table `slots` (kLoopMaxSessions x kLoopMaxSlots): at most
// `max_batch` requests and `sms` training CTAs per batch; a scheduler pass
// without requests waits up to idle_poll_ns for one, and ends the loop when
// none came. `cooperative`: the training launch node carries the cooperative
// attribute.
cudaError_t loop_build(LoopShared* shared, LoopDevice* dev, const LoopSlot* slots, uint32_t max_batch, uint32_t sms,
                       uint32_t idle_poll_ns, bool cooperative, LoopGraph* out);
void loop_destroy(LoopGraph* g);
// Device clock minus host clock (ns), measured once: a kernel stamps
// %globaltimer when it sees the host's go flag. host_now_ns: the host clock.
cudaError_t loop_calibrate(LoopShared* shared_host, LoopShared* shared_dev, cudaStream_t stream,
                           int64_t (*host_now_ns)(), int64_t* offset_ns);

}  // namespace nrc
