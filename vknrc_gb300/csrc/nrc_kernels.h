// Kernel launchers shared between the kernel translation units and the C ABI.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/nrc.h"

namespace nrc {

// FP8 (E4M3) copy of a cache's rendering weights and its per-layer scales
// (device memory, one per context with fp8 inference on). Layer l's weights are
// stored as e4m3(w * 448 / absmax_w[l]); its input activations as
// e4m3(x * 448 / absmax_x[l]); the query multiplies each layer's fp32 sum by
// c[l] = s_w[l] s_x[l] / s_x[l+1] (the output layer by s_w[5] s_x[5]) with
// s = absmax / 448.
struct Fp8State {
  float scale_w[6];
  float scale_x[6];
  float c[6];
  float inv_sx0;       // 448 / absmax_x[0]: features -> e4m3
  float inv_w[6];      // 448 / absmax_w[l]
  uint32_t amax_x[6];  // activation absmax (fp32 bits) seen by training forwards since the last scale update
  uint32_t epoch;      // t / 16 + 1 at the last scale update (0: never)
  uint32_t pad[4];
};
static_assert(sizeof(Fp8State) == 144, "Fp8State layout");

// Tensor map over an fp16 parameter vector (323 rows x 64, 128-byte swizzle,
// 64 x 16 boxes) for stage_weights_tma(). Host only; allocates nothing.
cudaError_t make_weight_map(CUtensorMap* map, const void* w16);

cudaError_t configure_infer_kernels();
cudaError_t configure_train_kernels();
uint32_t infer_smem_bytes();
int infer_threads();
int infer_tiles_per_cta();
// Where the query kernel puts its results: a dense rgb array (optional,
// clamped or not) and/or the reference's destination epilogue (dst != null).
struct QueryOut {
  float* out;
  int clamp;
  const uint32_t* dst;
  float* bias_factor_r;
  const float* factor_gb;
  uint32_t width, height;
  float* train[NRC_TRAIN_BATCH_COUNT];  // train records whose targets the queries complete
  uint32_t train_cap[NRC_TRAIN_BATCH_COUNT];
  uint32_t train_stride;  // floats per train record: 20 (nrc_train_record) or 10 (nrc_packed_train_record)
};

// bf16: the weights and the operands are bf16 (the bf16 precision form); the
// pre-encoded input path is fp16 only.
cudaError_t launch_infer(const void* input, bool encoded, const uint32_t* d_count, uint32_t capacity,
                         const CUtensorMap* wmap, const QueryOut& q, uint32_t* err, int num_sms,
                         cudaStream_t stream, bool bf16 = false);

// The overlapped frame's copy of the staged rendering weights src -> dst
// (kParams 16-bit words: 2,584 x 16 bytes), made once the training grid has
// completed and no query CTA reads dst any more: by the query CTA that is the
// last to have its weights in shared memory (after its wait for the training
// grid), or, when the frame has no query, by the training's last CTA. src
// null: no copy.
struct FrameJoin {
  const uint4* src;
  uint4* dst;
};

constexpr uint32_t kJoinChunks = 2584;  // 16-byte chunks of the 20,672 16-bit weights

#ifdef __CUDACC__
// The copy by `nthreads` threads of the calling CTA (t: this thread's index
// among them); each thread's loads (from L2: other CTAs wrote the source) are
// in flight before its stores.
__device__ __forceinline__ void join_copy(const FrameJoin& j, uint32_t t, uint32_t nthreads) {
  constexpr uint32_t kUnroll = 8;
  for (uint32_t base = 0; base < kJoinChunks; base += kUnroll * nthreads) {
    uint4 v[kUnroll];
#pragma unroll
    for (uint32_t u = 0; u < kUnroll; ++u) {
      const uint32_t i = base + u * nthreads + t;
      if (i < kJoinChunks) v[u] = __ldcg(j.src + i);
    }
#pragma unroll
    for (uint32_t u = 0; u < kUnroll; ++u) {
      const uint32_t i = base + u * nthreads + t;
      if (i < kJoinChunks) j.dst[i] = v[u];
    }
  }
}
#endif

// One cache's share of a query launch.
struct InferJob {
  CUtensorMap wmap;
  const void* input;  // nrc_input records
  const uint32_t* d_count;
  uint32_t capacity;
  uint32_t* err;
  QueryOut q;
  const Fp8State* fp8;  // the FP8 query's scales (fp8 launches only)
  // Dynamic tiles (single-cache record queries): tiles[0] hands out the next
  // tile, tiles[1] counts exiting CTAs, tiles[2] (with a join) CTAs whose
  // weights have landed (all zero between launches; the last CTA of each
  // count resets it). Null: each CTA takes a fixed share of the tiles.
  uint32_t* tiles;
  // 1: start without waiting for the preceding grid in the stream (the
  // overlapped frame's query, launched behind the training it runs beside,
  // reads nothing that training writes).
  uint32_t no_wait;
  FrameJoin join;  // dynamic tiles only: the staged weights copied by the CTA that loads its weights last
};

// Kernel parameters of a query launch over up to N caches; CTAs
// [group_start[j], group_start[j + 1]) answer job j.
template <int N>
struct InferLaunch {
  InferJob job[N];
  uint32_t group_start[N + 1];
  int njobs;
};

constexpr int kMaxInferJobs = 32;  // caches per batched query launch

// The FP8 query (E4M3 weights and activations, per-layer scales) of one cache.
cudaError_t launch_infer_fp8(const nrc_input* input, const uint32_t* d_count, uint32_t capacity,
                             const CUtensorMap* w8map, const Fp8State* fp8, float* out, uint32_t* err, int num_sms,
                             cudaStream_t stream);
// Re-quantizes the fp8 weights from the 16-bit rendering weights; first
// recomputes the scales when `force` or when the step state has entered a new
// 16-step epoch since the last update. w8: 323 rows x 128 bytes (bytes 64..127
// of each row stay zero).
cudaError_t launch_fp8_refresh(const uint16_t* use16, bool bf16, const nrc_optimizer_state* st, Fp8State* fp8,
                               uint8_t* w8, int force, cudaStream_t stream);

// CTAs the query kernel uses for `capacity` records on `num_sms` SMs.
uint32_t infer_grid(uint32_t capacity, int num_sms);
// The overlapped frame's query: `grid` CTAs taking tiles from the counter
// pair `tiles` (zero between launches), started without waiting for the
// preceding grid (the training launched just before it on `stream`, which
// signals its dependents once all of its CTAs run): the CTAs that find no free
// SM start on the training's SMs as it finishes.
cudaError_t launch_infer_frame(const nrc_input* input, const uint32_t* d_count, uint32_t capacity,
                               const CUtensorMap* wmap, const QueryOut& q, uint32_t* err, uint32_t* tiles,
                               const FrameJoin& join, uint32_t grid, cudaStream_t stream, bool bf16);
// One launch answering njobs caches' record queries (dense rgb output, no
// destination words), group_size[j] >= 1 CTAs for job j, sum <= SMs.
cudaError_t launch_infer_many(const InferJob* jobs, int njobs, const uint32_t* group_size, cudaStream_t stream,
                              bool bf16 = false);

// One launch of the persistent trainer: up to NRC_TRAIN_BATCH_COUNT chained
// batches, each a fused gradient pass followed by the optimizer step (mode
// kTrainStep), or one gradient pass whose fixed-order sum is written to
// grad_out (kGradientOnly).
constexpr int kTrainStep = 0;
constexpr int kGradientOnly = 1;

struct TrainBatch {
  const nrc_train_record* records;
  uint32_t* d_count;
  uint32_t capacity;
  int write_use;  // the optimizer step also writes use_weights
};

struct TrainParams {
  TrainBatch batch[NRC_TRAIN_BATCH_COUNT];
  int steps;
  int mode;
  uint32_t batch_cap;
  float lr, beta1, beta2, eps, ema_alpha, loss_scale;
  int use_ema;
  nrc_optimizer_entry* entries;
  nrc_optimizer_state* state;
  __half* w16;
  __half* use16;
  float* partials;   // one gradient vector per CTA (grid <= the slots given)
  float* grad_out;   // kGradientOnly
  uint32_t* sync;    // grid-barrier counter (zeroed by launch_train)
  double* loss_acc;  // optional check-path loss sum
  unsigned long long* loss_count;
  uint32_t* err;
  int bf16;          // weights and operands in bf16 (host side: selects the kernel)
  uint32_t* amax;    // Fp8State::amax_x of a cache with fp8 inference, or null
  FrameJoin join;    // the staged weights copied by the last CTA out (a frame without a query)
};

// One cache's share of a training launch: its weight tensor map and parameters.
struct TrainJob {
  CUtensorMap wmap;
  TrainParams p;
};

// Kernel parameters of a launch over up to N caches; CTAs
// [group_start[j], group_start[j + 1]) train cache j.
template <int N>
struct TrainLaunch {
  TrainJob job[N];
  uint32_t group_start[N + 1];
  int njobs;
};

constexpr int kMaxTrainJobs = 32;  // caches per batched training launch

// The batched query and training over launch tables in global memory (the
// serving loop's batches, written on the device): CTAs past the table's groups
// return at once; fp16 caches only.
cudaError_t launch_infer_table(const InferLaunch<kMaxInferJobs>* table, uint32_t grid, cudaStream_t stream);
cudaError_t launch_train_table(const TrainLaunch<kMaxTrainJobs>* table, uint32_t grid, bool cooperative,
                               cudaStream_t stream);

// The reference's prepare + optimizer passes over a given gradient sum
// (p supplies the hyper-parameters and the cache's buffers), and the relative-L2
// gradient rows of given predictions (nrc_optimize.cu).
cudaError_t launch_optimize(const TrainParams& p, const float* grad_sum, uint32_t* d_count, bool write_use,
                            cudaStream_t stream);
cudaError_t launch_loss_rows(const float* pred, const float* target, const uint32_t* d_count, uint32_t capacity,
                             float loss_scale, bool bf16, uint32_t* rows, int num_sms, cudaStream_t stream);

uint32_t train_smem_bytes();
uint32_t train_grid(const TrainParams& p, int max_ctas);
// The grid barrier counter p.sync[0] and exit counter p.sync[1] must be zero
// before the first launch on them; every launch leaves them at zero.
cudaError_t launch_train(const TrainParams& p, const CUtensorMap* wmap, int max_ctas, cudaStream_t stream);
// One cooperative launch training njobs caches, group_size[j] CTAs for job j
// (1 .. 160 each, sum <= CTAs resident at one per SM). Jobs must not share a
// context (parameter buffers, partials or barrier counters).
cudaError_t launch_train_many(const TrainJob* jobs, int njobs, const uint32_t* group_size, cudaStream_t stream);

// Device bytes one context holds (its single allocation), and the same for a
// context about to be created on a device with num_sms SMs.
size_t context_device_bytes(const nrc_context* c);
size_t context_device_bytes_for(int num_sms);
// The serving loop's jobs for one frame slot of a session's cache: the query of
// the slot's records with the rendering weights, and the four chained training
// steps on its train records (the last writing use_weights), as
// nrc_infer_many / nrc_train_many build them. NRC_ERROR_INVALID_ARGUMENT for a
// bf16 or fp8 cache (the loop's kernels are the fp16 forms).
int loop_slot_jobs(nrc_context* ctx, const nrc_frame_buffers& f, uint32_t max_queries, uint32_t train_records,
                   InferJob* infer, TrainJob* train);

cudaError_t launch_encode(const nrc_input* in, const uint32_t* d_count, uint32_t capacity, uint16_t* out,
                          int num_sms, cudaStream_t stream);
cudaError_t launch_sph_encode(const float* dirs, const uint32_t* d_count, uint32_t capacity, float* out,
                              int num_sms, cudaStream_t stream);
// The gather tables of nrc_scene_prepare: 64-byte rows, primitive_count of
// them at prim_rows and material_count at mat_rows (16-byte aligned);
// footprints: device array of texture_count descriptors of the textures'
// footprint arrays (launch_texture_footprints), which the material rows point at.
cudaError_t launch_scene_prepare(const nrc_scene& scene, const nrc_texture* footprints, void* prim_rows,
                                 void* mat_rows, cudaStream_t stream);
// One texture's footprint array (16 bytes per texel, 16-byte aligned `out`).
cudaError_t launch_texture_footprints(const nrc_texture& tex, void* out, int num_sms, cudaStream_t stream);
// The train records of nbatches batches (min(*counts[b], capacity) each) in one
// launch, into unpacked arrays out[b]. prim_rows / mat_rows: the scene's
// prepared tables, or both null to gather from the scene buffers.
cudaError_t launch_unpack_train_batches(const nrc_scene& scene, const void* prim_rows, const void* mat_rows,
                                       const nrc_packed_train_record* const* in, uint32_t* const* counts,
                                       uint32_t capacity, nrc_train_record* const* out, int nbatches, int num_sms,
                                       cudaStream_t stream);
cudaError_t launch_unpack(const nrc_scene& scene, const void* prim_rows, const void* mat_rows, bool train,
                          const void* in, const uint32_t* d_count, uint32_t capacity, void* out, uint32_t* out_dst,
                          int num_sms, cudaStream_t stream);
cudaError_t launch_screen(const float* color, float* accum, uint32_t width, uint32_t height, int acc_on,
                          uint32_t acc_count, uint8_t* out8, float* outf, int num_sms, cudaStream_t stream);
cudaError_t launch_fill_f32(float* p, float v, size_t n, cudaStream_t stream);

}  // namespace nrc
