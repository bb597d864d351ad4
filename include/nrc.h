/*
 * nrc.h — C ABI of the GB300 neural-radiance-cache hot path (libnrc.so).
 *
 * Drop-in replacement for the compute side of the reference renderer's cache
 * passes: record encoding, the fused 64-wide MLP query, the fused relative-L2
 * gradient pass and the Adam update. Every entry point below names the
 * reference interface it replaces (paths relative to the reference project).
 *
 * Conventions
 *  - Plain device pointers and sizes; no framework types. `stream` is a
 *    cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Counts live in device memory (`d_count`), as the reference's count buffers
 *    do, so no call needs a host synchronisation. `capacity` is the host-side
 *    bound on the count (the number of records the buffer holds); the device
 *    count is clamped to it, so a bad count can never read past the buffer.
 *  - All compute calls are stream-ordered and asynchronous and return an
 *    nrc_status. Argument errors are reported at the call; device-side errors
 *    (a bounded wait that ran out) are latched in the context and read with
 *    nrc_get_error().
 *  - One context = one cache (weights + Adam state). Contexts are independent;
 *    calls on one context must be ordered by the caller (one stream, or events).
 *  - Device buffers must be 16-byte aligned (cudaMalloc gives 256).
 */
#ifndef NRC_H
#define NRC_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define NRC_API __attribute__((visibility("default")))
#else
#define NRC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Network shape: 64 encoded inputs -> 5 x 64 ReLU -> 3 outputs
 * (src/VkNRCState.hpp:23-25, shader/src/Constant.glsl:6). */
#define NRC_WIDTH 64
#define NRC_HIDDEN_LAYERS 5
#define NRC_OUTPUTS 3
#define NRC_PARAM_COUNT 20672 /* 5*64*64 + 3*64 */
#define NRC_TRAIN_BATCH_SIZE 16384 /* shader/src/Constant.glsl:10 */
#define NRC_TRAIN_BATCH_COUNT 4    /* shader/src/Constant.glsl:9 */

/* Unpacked path-vertex input, field for field UnpackedNRCInput
 * (shader/src/NRCRecord.glsl:40-45); scattered_dir and normal are already
 * sphere-encoded (NRCSphEncode, NRCRecord.glsl:47-49). 56 bytes. */
typedef struct nrc_input {
  float position[3];
  float scattered_dir[2];
  float normal[2];
  float roughness;
  float diffuse[3];
  float specular[3];
} nrc_input;

/* Training record: NRCTrainRecord (shader/src/NRCRecord.glsl:35-38) with its
 * packed input replaced by the unpacked one. The training target is `bias`
 * (shader/src/nrc_gradient.comp:35). 80 bytes. */
typedef struct nrc_train_record {
  float bias[3];
  float factor[3];
  nrc_input input;
} nrc_train_record;

/* Optimizer step state and per-parameter entry (src/VkNRCState.cpp:25-31). */
typedef struct nrc_optimizer_state {
  uint32_t t;
  float beta1_t, beta2_t, alpha_t, alpha_t_1;
} nrc_optimizer_state;

typedef struct nrc_optimizer_entry {
  float m, v, weight, ema_weight;
} nrc_optimizer_entry;

/* Hyper-parameters. nrc_default_config() fills the reference's values:
 * lr 0.002, eps 1e-8 (shader/src/nrc_optimize.comp:10-11), beta 0.9/0.999,
 * EMA 0.99, loss scale 1 (shader/src/Constant.glsl:8-13), batch cap 16384. */
typedef struct nrc_config {
  uint32_t train_batch_size; /* count cap of one nrc_train call */
  float learning_rate;
  float beta1, beta2;
  float epsilon;
  float ema_alpha;
  float loss_scale;
  uint32_t use_ema_weights; /* use_weights receives the EMA instead of the weights */
  uint32_t deterministic;   /* kept for layout; weight gradients are always summed in a fixed
                               order, so results are run-to-run identical either way */
  uint32_t track_loss;      /* 1: accumulate the relative-L2 loss (check path, FP64 sum) */
  uint64_t seed;            /* He initialisation seed */
  uint32_t precision;       /* nrc_precision: the 16-bit format of weights and operands */
  uint32_t fp8_inference;   /* 1: keep an FP8 (E4M3) copy of use_weights for nrc_infer_fp8 */
} nrc_config;

/* Precision forms. FP16 is the reference's (fp16 weights, features and
 * activations, fp32 accumulation). BF16 keeps the same fp32 master weights and
 * Adam moments but stores the weight vectors and runs every operand (features,
 * activations, gradients) in bf16: a wider range (no fp16 overflow of the
 * relative-L2 gradient) for 3 fewer mantissa bits. For a BF16 context the
 * 16-bit vectors of nrc_get_weights / nrc_set_weights / nrc_get_device_buffers
 * hold bf16 bit patterns, and the fp16-feature calls (nrc_encode,
 * nrc_infer_encoded) return NRC_ERROR_INVALID_ARGUMENT. */
typedef enum nrc_precision { NRC_PRECISION_FP16 = 0, NRC_PRECISION_BF16 = 1 } nrc_precision;

typedef enum nrc_status {
  NRC_OK = 0,
  NRC_ERROR_INVALID_ARGUMENT = 1,
  NRC_ERROR_CUDA = 2,
  NRC_ERROR_NO_DEVICE = 3,
  NRC_ERROR_UNSUPPORTED_DEVICE = 4, /* not an sm_103 (GB300) device */
  NRC_ERROR_OUT_OF_MEMORY = 5,
  NRC_ERROR_DEVICE_TIMEOUT = 6, /* a kernel's bounded wait ran out (latched) */
  NRC_ERROR_MISALIGNED = 7,
  NRC_ERROR_TOO_LARGE = 8, /* more records than nrc_train_noalloc's fixed scratch holds */
  NRC_ERROR_BAD_CHECKPOINT = 9 /* checkpoint blob of the wrong size, version or checksum */
} nrc_status;

/* Which fp16 weight vector a query uses. The reference renders with
 * use_weights (last frame's result) and trains on weights
 * (src/rg/NRCRenderGraph.cpp:52, :58-68). */
typedef enum nrc_weight_set { NRC_WEIGHTS_USE = 0, NRC_WEIGHTS_TRAIN = 1 } nrc_weight_set;

typedef struct nrc_context nrc_context;

NRC_API const char* nrc_status_string(int status);

/* Fills the reference's defaults. */
NRC_API int nrc_default_config(nrc_config* cfg);

/* Creates a cache on the current CUDA device and initialises it as
 * VkNRCState::ResetMLPBuffers does (src/VkNRCState.cpp:46-88): He-normal
 * weights N(0, sqrt(2/64)) from std::mt19937(seed) and
 * std::normal_distribution<float>, fp16 copies in weights and use_weights, zero
 * moments, state {0, 1, 1, 1, 0}. Synchronous. */
NRC_API int nrc_create(const nrc_config* cfg, nrc_context** out);
NRC_API int nrc_destroy(nrc_context* ctx);

/* Re-initialises weights and optimizer ("Re-Train", src/main.cpp:144-147). Synchronous. */
NRC_API int nrc_reset(nrc_context* ctx, uint64_t seed);

/* The He initialisation of nrc_create on the host, without a device:
 * out_weights receives NRC_PARAM_COUNT fp32 values (src/VkNRCState.cpp:39-44). */
NRC_API int nrc_he_init_host(uint64_t seed, float* out_weights);

/* Input encoding alone: NRCInputEncode (shader/src/NRCRecord.glsl:78-95) of
 * min(*d_count, capacity) records into 64 fp16 features each (d_encoded,
 * n x 64 halves, feature order of the reference). */
NRC_API int nrc_encode(nrc_context* ctx, const nrc_input* d_inputs, const uint32_t* d_count, uint32_t capacity,
               uint16_t* d_encoded, void* stream);

/* Sphere encoding of unit vectors (NRCSphEncode, NRCRecord.glsl:47-49):
 * d_dirs n x 3 floats -> d_out n x 2 floats. */
NRC_API int nrc_sph_encode(const float* d_dirs, const uint32_t* d_count, uint32_t capacity, float* d_out, void* stream);

/* Cache query: encode + 6-layer fused MLP + clamp to >= 0, one rgb (3 floats)
 * per input. Replaces the compute of NNDispatch<NNInference>
 * (src/rg/NNDispatch.hpp:51-54, src/rg/NNInference.cpp:67-71,
 * shader/src/nrc_inference.comp:30-48). */
NRC_API int nrc_infer(nrc_context* ctx, const nrc_input* d_inputs, const uint32_t* d_count, uint32_t capacity,
              float* d_out_rgb, int weight_set, void* stream);

/* The same query from pre-encoded inputs (n x 64 fp16), as the reference's
 * test kernel test/evaluate_NV.comp takes them. Output unclamped, as there. */
NRC_API int nrc_infer_encoded(nrc_context* ctx, const uint16_t* d_encoded, const uint32_t* d_count, uint32_t capacity,
                      float* d_out_rgb, int weight_set, void* stream);

/* Where query results go when a query carries a destination word
 * (nrc_inference.comp:50-73; the word's encoding is NRCRecord.glsl:19-33):
 *  - 0xFFFFFFFF: nowhere;
 *  - bit 0 = 0, screen: x = (dst >> 1) & 0x7FFF, y = dst >> 16. Pixel (x, y) of
 *    bias_factor_r (rgba32f, row-major [height][width][4]: rgb = bias, a =
 *    factor.r) and factor_gb (rg32f, [height][width][2]) becomes
 *    (bias + (factor.r, factor.g, factor.b) * pred, 0);
 *  - bit 0 = 1, train: batch b = (dst >> 1) & 3, records l = (dst >> 3) & 0x3FFF
 *    to r = dst >> 17 inclusive: bias_rgb += factor_rgb * pred (self-training
 *    target completion).
 * pred = max(query output, 0); each update is one fused multiply-add per
 * channel. Pixels outside width x height, records at or beyond a batch's
 * capacity and batches whose pointer is null are skipped (the reference relies
 * on robust image access and on well-formed ranges). The updates are plain
 * read-modify-writes, as in the reference: destinations of one call must not
 * repeat. */
typedef struct nrc_scatter_targets {
  float* bias_factor_r;
  const float* factor_gb;
  uint32_t width, height;
  nrc_train_record* train_records[NRC_TRAIN_BATCH_COUNT];
  uint32_t train_capacity[NRC_TRAIN_BATCH_COUNT];
} nrc_scatter_targets;

/* Cache query with the reference's destination epilogue fused in: as nrc_infer
 * on d_inputs, then each query's prediction is written where d_dst[i] says
 * (nrc_scatter_targets). d_out_rgb may be null; if given it also receives the
 * clamped predictions. Replaces the whole of nrc_inference.comp:30-73 for
 * unpacked records. */
NRC_API int nrc_infer_scatter(nrc_context* ctx, const nrc_input* d_inputs, const uint32_t* d_dst,
                              const uint32_t* d_count, uint32_t capacity, const nrc_scatter_targets* targets,
                              float* d_out_rgb, int weight_set, void* stream);

/* One training step on min(*d_count, train_batch_size, capacity) records:
 * nrc_train_prepare.comp (count clamp, written back to *d_count; step state
 * advanced only if n > 0) + nrc_gradient.comp (fused encode, forward,
 * relative-L2 loss gradient, backward, weight gradients) + nrc_optimize.comp
 * (Adam + EMA, fp16 weights; use_weights too when write_use_weights != 0).
 * Replaces rg::NNTrain (src/rg/NNTrain.hpp:95-118, src/rg/NNTrain.cpp:29-33,
 * 83-87, 124-133). */
NRC_API int nrc_train(nrc_context* ctx, const nrc_train_record* d_records, uint32_t* d_count, uint32_t capacity,
              int write_use_weights, void* stream);

/* The reference's chained train passes of one frame
 * (src/rg/NRCRenderGraph.cpp:57-80) in one call: nbatches (1..4) training steps
 * as nrc_train does them, batch b on d_records[b] / d_counts[b], each using the
 * weights the previous one produced; the last also writes use_weights when
 * write_use_last != 0. One persistent launch runs all of them. */
NRC_API int nrc_train_batches(nrc_context* ctx, const nrc_train_record* const* d_records, uint32_t* const* d_counts,
                              uint32_t capacity, int nbatches, int write_use_last, void* stream);

/* Weight-gradient pass alone (no optimizer step): d_grad receives the
 * NRC_PARAM_COUNT fp32 gradient sums over min(*d_count, capacity) records
 * (the reference's gradients buffer, src/rg/NNTrain.hpp:96-98), computed with
 * the training weights. */
NRC_API int nrc_gradient(nrc_context* ctx, const nrc_train_record* d_records, const uint32_t* d_count, uint32_t capacity,
                 float* d_grad, void* stream);

/* One frame of the reference schedule (src/rg/NRCRenderGraph.cpp:46-80):
 * query all eval inputs with use_weights, then NRC_TRAIN_BATCH_COUNT chained
 * training steps, the last one writing use_weights. */
NRC_API int nrc_frame(nrc_context* ctx, const nrc_input* d_eval_inputs, const uint32_t* d_eval_count, uint32_t eval_capacity,
              float* d_out_rgb, const nrc_train_record* const* d_train_records, uint32_t* const* d_train_counts,
              uint32_t train_capacity, void* stream);

/* Split of the SMs for nrc_frame_overlapped: train_ctas for the training,
 * query_ctas (query_ctas + train_ctas <= SMs) for the query CTAs that run
 * beside it from the start; the query's other CTAs start on the training's SMs
 * as it finishes. train_ctas = 0 runs the frame sequentially (both on every
 * SM). */
typedef struct nrc_frame_plan {
  uint32_t query_ctas, train_ctas;
} nrc_frame_plan;

/* nrc_frame with the query and the training run at the same time. The
 * reference's frame reads use_weights in its query and writes them in its last
 * training step (src/rg/NRCRenderGraph.cpp:52, :77); here the training writes
 * them into a second buffer of the context, copied into use_weights (41 KB)
 * once the training has completed and every query CTA has loaded the previous
 * ones. The query therefore reads exactly the weights it reads in nrc_frame,
 * and work that follows the call in the stream sees the new ones, as there
 * (no other work may read use_weights while the call runs). The training runs
 * with plan->train_ctas CTAs, so its gradient sums are grouped as
 * nrc_train_many with that count groups them. It is launched first on
 * `stream`; the query follows as a dependent launch that starts once every
 * training CTA runs, takes its record tiles from a counter of the context, and
 * so also fills the training's SMs when the training ends (one frame at a time
 * per context).
 * plan NULL: the context's tuned plan (nrc_autotune_frame), else a quarter of
 * the SMs for the training. query_event (a cudaEvent_t, may be NULL) is recorded
 * on `stream` after the query: it completes with the frame's two kernels. Both
 * kernels run on `stream`, so the call can be captured in a CUDA graph like the
 * others. */
NRC_API int nrc_frame_overlapped(nrc_context* ctx, const nrc_input* d_eval_inputs, const uint32_t* d_eval_count,
                                 uint32_t eval_capacity, float* d_out_rgb, const nrc_train_record* const* d_train_records,
                                 uint32_t* const* d_train_counts, uint32_t train_capacity, const nrc_frame_plan* plan,
                                 void* query_event, void* stream);

/* Autotuner of the overlapped frame: times the sequential frame and training
 * groups of 8, 16, ..., 72 CTAs, and the smallest group for each count of
 * record tiles per CTA, beside the query on this workload (on a scratch
 * copy of the cache, which it then frees; `d_out_rgb` and the counts are written
 * as a frame writes them), keeps the fastest split as the context's plan and
 * returns it with its time per frame. Synchronous. */
NRC_API int nrc_autotune_frame(nrc_context* ctx, const nrc_input* d_eval_inputs, const uint32_t* d_eval_count,
                               uint32_t eval_capacity, float* d_out_rgb, const nrc_train_record* const* d_train_records,
                               uint32_t* const* d_train_counts, uint32_t train_capacity, nrc_frame_plan* best,
                               float* best_ms);

/* One frame of the reference schedule with the destination epilogue
 * (src/rg/NRCRenderGraph.cpp:46-80, nrc_inference.comp:50-73): the queries
 * update the screen images and complete the train records' targets in
 * targets->train_records, then NRC_TRAIN_BATCH_COUNT chained training steps
 * run on those records (targets->train_capacity[b] each, counts in
 * d_train_counts[b]), the last one writing use_weights. */
NRC_API int nrc_frame_scatter(nrc_context* ctx, const nrc_input* d_eval_inputs, const uint32_t* d_eval_dst,
                              const uint32_t* d_eval_count, uint32_t eval_capacity,
                              const nrc_scatter_targets* targets, uint32_t* const* d_train_counts, void* stream);

/* The reference's prepare and optimizer passes on a weight-gradient sum the
 * caller computed (NNTrain's prepare_pass and optimizer_pass,
 * src/rg/NNTrain.hpp:95-118; nrc_train_prepare.comp:16-29 then
 * nrc_optimize.comp:32-54): *d_count is clamped to cfg.train_batch_size and
 * written back; if it is non-zero the step state advances and every parameter i
 * is updated from d_grad_sum[i] / count / loss_scale (NaN and Inf scrubbed to
 * 0), writing the fp32 entries, the 16-bit weights and, with
 * write_use_weights, use_weights. d_grad_sum: NRC_PARAM_COUNT fp32, 16-byte
 * aligned (nrc_gradient's output, undivided). The arithmetic is the fused
 * trainer's optimizer phase. Stream-ordered, two launches. */
NRC_API int nrc_optimize(nrc_context* ctx, const float* d_grad_sum, uint32_t* d_count, int write_use_weights,
                         void* stream);

/* The relative-L2 luminance loss gradient rows of min(*d_count, capacity)
 * (prediction, target) pairs (NNLoadDA3_RelativeL2LuminanceLoss,
 * shader/src/NN_nv.glsl:178-196): d_pred and d_target n x 3 fp32 (predictions
 * unclamped, as nrc_gradient.comp:45-46 passes them); d_rows receives per pair
 * the two 32-bit words (d0 | d1 << 16, d2 | 0 << 16) of the 16-bit row in the
 * given precision (NRC_PRECISION_FP16: values past 65504 become inf, as the
 * reference's packHalf2x16 makes them). The fused trainer computes its rows with
 * the same code; this is its check path. */
NRC_API int nrc_loss_gradient(const float* d_pred, const float* d_target, const uint32_t* d_count, uint32_t capacity,
                              float loss_scale, uint32_t precision, uint32_t* d_rows, void* stream);

/* One training step with nrc_train's semantics that allocates no device memory.
 * No counterpart in the reference: it serves callers that cannot call cudaMalloc,
 * such as a renderer that sub-allocates every device buffer from its own heaps or
 * a process held to a fixed device-memory budget. The caller owns the parameter
 * buffers in the layouts above (fp16 weights, optional fp16 use_weights, Adam
 * entries, step state) as well as the records and the count; `cfg` supplies the
 * hyper-parameters (seed, deterministic, track_loss and fp8_inference are
 * ignored: no FP8 copy of the weights is kept or refreshed).
 * Scratch: the per-CTA weight-gradient partials live in a fixed array compiled
 * into the library, 5,292,288 bytes held by every GPU that loads it until the
 * process exits; it bounds one call to 16,384 records: if min(capacity,
 * cfg->train_batch_size) is larger the call returns NRC_ERROR_TOO_LARGE and does
 * nothing. The gradient is summed in a fixed order.
 * The first call on a device performs a one-time set-up (it resolves the
 * scratch's device address); make that first call before any stream capture.
 * Every call uses the same scratch: calls that may overlap on the GPU (other
 * streams, no ordering) race; order them. d_error (may be NULL) receives the
 * device-timeout flag; when NULL a word in the scratch is used, cleared on each
 * call, which the caller cannot read: a step that hit a bounded-wait timeout
 * then still returns NRC_OK, so pass d_error to observe timeouts. Pointers that
 * are not aligned to their types (16 bytes for weights, entries and records;
 * 4 for the state, count and error words) return NRC_ERROR_MISALIGNED. */
NRC_API int nrc_train_noalloc(uint16_t* d_weights, uint16_t* d_use_weights, nrc_optimizer_entry* d_entries,
                              nrc_optimizer_state* d_state, const nrc_train_record* d_records, uint32_t* d_count,
                              uint32_t capacity, const nrc_config* cfg, uint32_t* d_error, void* stream);

/* ---------------------------------------------------------------------------
 * Batched caches: many independent caches (separate weights and Adam state,
 * uneven record counts) served by one persistent launch per phase. The
 * reference runs one cache per renderer (VkNRCState, src/VkNRCState.hpp:27-52);
 * these calls do, for n caches at once, what nrc_infer / nrc_train_batches do
 * for one, and give each cache exactly the results it gets alone (every
 * reduction runs in a fixed order within the cache's own CTA group).
 * The SMs are split between the caches in proportion to their tiles
 * (capacity / 128 records), at least one CTA each, unless `ctas` gives the split
 * (one entry per job; a job's CTAs beyond its tiles idle). A context may appear
 * at most once per call; all contexts must live on the current device. More
 * than 32 jobs run as successive launches of up to 32.
 * ------------------------------------------------------------------------- */
typedef struct nrc_query_job {
  nrc_context* ctx;
  const nrc_input* inputs;  /* capacity records */
  const uint32_t* d_count;  /* queries = min(*d_count, capacity) */
  uint32_t capacity;
  float* out_rgb;           /* capacity x 3, clamped to >= 0 as nrc_infer */
  int weight_set;           /* NRC_WEIGHTS_USE or NRC_WEIGHTS_TRAIN */
} nrc_query_job;

typedef struct nrc_train_job {
  nrc_context* ctx;
  const nrc_train_record* records[NRC_TRAIN_BATCH_COUNT]; /* first nbatches used */
  uint32_t* d_counts[NRC_TRAIN_BATCH_COUNT];               /* clamped and written back as nrc_train */
  uint32_t capacity;
  int nbatches;       /* 1..4 chained steps, as nrc_train_batches */
  int write_use_last; /* the last step also writes use_weights */
} nrc_train_job;

/* nrc_infer for every job, one launch per 32 jobs. `ctas` may be NULL. */
NRC_API int nrc_infer_many(const nrc_query_job* jobs, uint32_t njobs, const uint32_t* ctas, void* stream);

/* nrc_train_batches for every job, one cooperative launch per 32 jobs. `ctas`
 * may be NULL. Training launches (this, nrc_train*, nrc_frame*) that run at
 * the same time on different streams should be ordered with events: each grid
 * waits at its grid barrier until all of its CTAs run, and two grids that each
 * hold SMs the other needs end in NRC_ERROR_DEVICE_TIMEOUT after the 2 s bound. */
NRC_API int nrc_train_many(const nrc_train_job* jobs, uint32_t njobs, const uint32_t* ctas, void* stream);

/* CTA split that nrc_infer_many / nrc_train_many use when `ctas` is NULL, for
 * one launch of at most 32 jobs of one precision: writes njobs entries to
 * out_ctas. (A batched call runs FP16 and BF16 contexts in separate launches.) */
NRC_API int nrc_plan_query_ctas(const nrc_query_job* jobs, uint32_t njobs, uint32_t* out_ctas);
NRC_API int nrc_plan_train_ctas(const nrc_train_job* jobs, uint32_t njobs, uint32_t* out_ctas);

/* The batched launches' autotuner (no counterpart in the reference, which runs
 * one cache): times candidate CTA splits of one nrc_infer_many launch (nq <= 32
 * jobs, one precision, capacities > 0) and of one nrc_train_many launch
 * (nt <= 32 jobs, one precision) and writes the fastest to q_ctas / t_ctas (nq /
 * nt entries), their mean launch times to q_ms / t_ms (may be NULL). The
 * candidates are the proportional default and, for each number of tiles per
 * CTA, the split that gives every job just the CTAs that number needs. Query
 * candidates run on the jobs themselves (they write the jobs' outputs);
 * training candidates run on scratch copies of the caches, so the caller's
 * caches are not trained (their count buffers are clamped as by a call).
 * Synchronous; allocates the scratch caches for its duration. */
NRC_API int nrc_autotune_many(const nrc_query_job* qjobs, uint32_t nq, const nrc_train_job* tjobs, uint32_t nt,
                              uint32_t* q_ctas, uint32_t* t_ctas, float* q_ms, float* t_ms);

/* ---------------------------------------------------------------------------
 * Serving: a device-resident loop over many render sessions. No counterpart in
 * the reference, which serves one renderer (src/main.cpp:84-91); each session
 * here is one cache (weights and Adam state stay on the GPU) plus frame slots in
 * device memory, and one frame request runs the reference's frame schedule
 * (src/rg/NRCRenderGraph.cpp:46-80) on a slot: the cache query of its records
 * with use_weights, then NRC_TRAIN_BATCH_COUNT chained training steps, the last
 * writing use_weights.
 *  - Sessions are admitted by the server's device-memory budget: opening one
 *    that does not fit returns NRC_ERROR_OUT_OF_MEMORY; closing one frees its
 *    share.
 *  - Requests are batched continuously: a worker thread takes queued requests
 *    (first come, first served; one in flight per session, in submission order)
 *    into the next batched launch, up to max_batch_sessions per launch, while
 *    earlier batches still run; each in-flight batch has its own stream, so the
 *    batches' kernels overlap on the device.
 *  - Every session trains with a fixed CTA group (train_ctas), so its results
 *    are the same whatever it is batched with.
 * ------------------------------------------------------------------------- */
typedef struct nrc_server nrc_server;

typedef struct nrc_server_config {
  uint64_t hbm_budget_bytes;    /* device memory for session state and frame slots */
  uint32_t max_batch_sessions;  /* requests per batched launch, 1..32 */
  uint32_t max_inflight_batches;/* launched, unfinished batches, 1..8 (host worker only) */
  /* 0: a host worker thread forms the batches and launches them on
   * max_inflight_batches streams. 1: the loop runs on the device: a CUDA graph
   * whose while node repeats scheduler kernel -> batched query -> batched
   * training -> completion kernel while requests keep coming (a launch ends
   * after 200 us without one; the next submit launches it again), taking the
   * requests that nrc_server_submit writes into a ring in host-mapped memory
   * (batches then run one after another; requests that arrive during one join
   * the next). Sessions must be fp16 caches without fp8_inference; opening or
   * closing a session pauses the loop (its requests complete first) while
   * device memory is allocated or freed; a submit's ready_event is waited on
   * by the submitting thread. */
  uint32_t device_loop;
} nrc_server_config;

typedef struct nrc_session_desc {
  nrc_config cache;        /* the session cache's hyper-parameters and seed */
  uint32_t max_queries;    /* query records per frame */
  uint32_t train_records;  /* records per training batch (NRC_TRAIN_BATCH_COUNT per frame) */
  uint32_t frame_slots;    /* frame buffers in device memory, 1..16 */
  uint32_t train_ctas;     /* CTAs of the session's training group, 1..152; 0 = one per 4 tiles of 128 records */
} nrc_session_desc;

/* Device buffers of one frame slot. The caller writes the records and counts,
 * then submits the slot; after the request completes the slot's out_rgb holds
 * the clamped query results, the train records hold what the caller wrote
 * (counts are clamped as nrc_train does). */
typedef struct nrc_frame_buffers {
  nrc_input* queries;                             /* max_queries records */
  uint32_t* query_count;
  float* out_rgb;                                 /* max_queries x 3 */
  nrc_train_record* train[NRC_TRAIN_BATCH_COUNT]; /* train_records each */
  uint32_t* train_count[NRC_TRAIN_BATCH_COUNT];
} nrc_frame_buffers;

typedef struct nrc_server_stats {
  uint64_t submitted, completed, batches;
  uint64_t bytes_in_use;
  double latency_p50_ms, latency_p99_ms, latency_max_ms; /* submit -> completion, since the last reset */
  double mean_batch_sessions;
} nrc_server_stats;

/* Creates the server and its worker thread on the current device. */
NRC_API int nrc_server_create(const nrc_server_config* cfg, nrc_server** out);
/* Finishes every submitted request, stops the worker, closes all sessions. */
NRC_API int nrc_server_destroy(nrc_server* srv);
NRC_API int nrc_server_open_session(nrc_server* srv, const nrc_session_desc* desc, uint32_t* session);
/* Waits for the session's requests to finish, then frees its memory. With
 * the device loop every request written so far completes first; if the loop
 * cannot be paused (NRC_ERROR_DEVICE_TIMEOUT after 60 s, or a CUDA error) the
 * session stays open and the status is returned. */
NRC_API int nrc_server_close_session(nrc_server* srv, uint32_t session);
NRC_API int nrc_server_frame_buffers(nrc_server* srv, uint32_t session, uint32_t slot, nrc_frame_buffers* out);
/* The session's cache, for nrc_get_weights / nrc_get_optimizer and the like
 * (only while none of its requests is pending). */
NRC_API int nrc_server_session_cache(nrc_server* srv, uint32_t session, nrc_context** ctx);
/* Queues frame slot `slot` of `session`. `ready_event` (a cudaEvent_t, may be
 * NULL) is waited on by the server's stream before the request runs: record it
 * after writing the slot. Returns a ticket. */
NRC_API int nrc_server_submit(nrc_server* srv, uint32_t session, uint32_t slot, void* ready_event, uint64_t* ticket);
/* Waits until the ticket's request has completed on the GPU (timeout_ms < 0:
 * no limit; NRC_ERROR_DEVICE_TIMEOUT when it runs out). latency_ms (may be
 * NULL) receives its submit-to-completion time. */
NRC_API int nrc_server_wait(nrc_server* srv, uint64_t ticket, double timeout_ms, double* latency_ms);
NRC_API int nrc_server_get_stats(nrc_server* srv, nrc_server_stats* stats, int reset_latencies);

/* ---------------------------------------------------------------------------
 * Scene unpack: the reference's packed path-vertex records are expanded to
 * nrc_input from the scene buffers (UnpackNRCInput, shader/src/NRCRecord.glsl:
 * 97-125, over shader/src/Scene.glsl:8-71), as nrc_inference.comp:33-36 and
 * nrc_gradient.comp:29-33 do before the encode.
 * ------------------------------------------------------------------------- */

/* std430 Material (shader/src/Scene.glsl:12-19), 64 bytes. A texture id of
 * 0xFFFFFFFF selects the constant colour. */
typedef struct nrc_material {
  float diffuse[3];
  uint32_t diffuse_texture_id;
  float specular[3];
  uint32_t specular_texture_id;
  float emission[3];
  uint32_t emission_texture_id;
  float metallic, roughness, ior;
  uint32_t pad_;
} nrc_material;

/* One scene texture: R8G8B8A8_SRGB texels, row-major [height][width][4]
 * (src/VkScene.cpp:190-195). Sampled as the reference's sampler does
 * (src/rg/NRCRenderGraph.cpp:132): bilinear, REPEAT addressing, one mip level,
 * sRGB decoded per texel before filtering. */
typedef struct nrc_texture {
  const uint8_t* texels;
  uint32_t width, height;
} nrc_texture;

/* Scene buffers (device pointers; Scene.glsl:30-48). Counts bound every index a
 * record or an index buffer holds: a record whose primitive, instance, vertex,
 * texcoord or material index is out of range unpacks to zeros, and a texture
 * id at or beyond texture_count reads as the constant colour (the reference
 * trusts its buffers). */
typedef struct nrc_scene_tables nrc_scene_tables;

typedef struct nrc_scene {
  const float* vertices;            /* Vertex {x, y, z}, vertex_count */
  const uint32_t* vertex_indices;   /* 3 per primitive */
  const float* texcoords;           /* vec2, texcoord_count */
  const uint32_t* texcoord_indices; /* 3 per primitive */
  const nrc_material* materials;    /* material_count */
  const uint32_t* material_ids;     /* per primitive */
  const float* transforms;          /* per instance: mat3x4, 3 columns of 4 floats (p' = vec4(p, 1) * T) */
  const nrc_texture* textures;      /* device array, texture_count entries */
  uint32_t vertex_count, texcoord_count, material_count, primitive_count, instance_count, texture_count;
  /* Optional (NULL: the unpack reads the buffers above): gather tables of this
   * scene made by nrc_scene_prepare. With them the unpack reads one 64-byte row
   * per record's primitive and one per material instead of the index, vertex,
   * texcoord, material and texture-table gathers; results are the same bit for
   * bit. The transforms are still read from `transforms`. */
  const nrc_scene_tables* tables;
} nrc_scene;

/* Builds the unpack's gather tables of `scene` on `stream` and returns them in
 * *out (no counterpart in the reference, whose shaders gather from the scene
 * buffers of Scene.glsl:30-48 directly). Per primitive one 64-byte row: its
 * three object-space vertices and texcoords and its material id (marked invalid
 * when one of its indices is out of range); per material one 64-byte row: the
 * constant colours, roughness and the two texture descriptors inline; per
 * texture a footprint array: for each texel, it and its right, lower and
 * lower-right neighbours (wrapped) in one 16-byte word, so a bilinear sample is
 * one load. The tables are a snapshot of the buffers at that point of the
 * stream: after changing the scene's buffers, prepare again. Allocates device
 * memory (64 bytes per primitive and per material, 16 per texel) and waits for
 * the stream, so call it outside stream capture. Texels must be 4-byte aligned
 * (NRC_ERROR_MISALIGNED). Set scene->tables to the result to use them;
 * nrc_scene_tables_destroy frees them (after the work that reads them has
 * finished). */
NRC_API int nrc_scene_prepare(const nrc_scene* scene, void* stream, nrc_scene_tables** out);
NRC_API int nrc_scene_tables_destroy(nrc_scene_tables* tables);

/* PackedNRCInput, NRCEvalRecord, NRCTrainRecord (NRCRecord.glsl:6-38). */
typedef struct nrc_packed_input {
  uint32_t primitive_id;
  uint32_t flip_bit_instance_id; /* bit 31: flip the normal; bits 0..30: instance */
  uint32_t barycentric_2x16u;    /* unorm16 pair: barycentrics 1 and 2 */
  uint32_t scattered_dir_2x16u;  /* unorm16 pair: sphere-encoded direction */
} nrc_packed_input;

typedef struct nrc_eval_record {
  uint32_t dst; /* destination word, as nrc_infer_scatter takes it */
  nrc_packed_input input;
} nrc_eval_record;

typedef struct nrc_packed_train_record {
  float bias[3];
  float factor[3];
  nrc_packed_input input;
} nrc_packed_train_record;

/* The reference's inference pass on its own record format: queries over
 * min(*d_count, capacity) packed eval records (nrc_eval_record, 20 bytes,
 * d_records 4-byte aligned) of `scene`, unpacked (UnpackNRCInput,
 * NRCRecord.glsl:97-125, as nrc_inference.comp:33-36 does) by one launch into a
 * workspace the context keeps, then queried. The first call with a larger
 * capacity allocates the workspace (56 + 4 bytes per record), so make it before
 * any stream capture. nrc_infer_packed writes the clamped
 * predictions to d_out_rgb (3 floats per record; the destination words are not
 * used). nrc_infer_scatter_packed runs the destination epilogue
 * (nrc_inference.comp:50-73) with each record's own destination word: screen
 * pixels as nrc_infer_scatter, and train-target completion in packed train
 * records (nrc_packed_train_record, targets->train_records); d_out_rgb may be
 * NULL. Replaces rg::NNInference (src/rg/NNInference.hpp:18-37) with the
 * scene's buffers as device pointers. */
typedef struct nrc_packed_scatter_targets {
  float* bias_factor_r;
  const float* factor_gb;
  uint32_t width, height;
  nrc_packed_train_record* train_records[NRC_TRAIN_BATCH_COUNT];
  uint32_t train_capacity[NRC_TRAIN_BATCH_COUNT];
} nrc_packed_scatter_targets;

NRC_API int nrc_infer_packed(nrc_context* ctx, const nrc_scene* scene, const nrc_eval_record* d_records,
                             const uint32_t* d_count, uint32_t capacity, float* d_out_rgb, int weight_set,
                             void* stream);
NRC_API int nrc_infer_scatter_packed(nrc_context* ctx, const nrc_scene* scene, const nrc_eval_record* d_records,
                                     const uint32_t* d_count, uint32_t capacity,
                                     const nrc_packed_scatter_targets* targets, float* d_out_rgb, int weight_set,
                                     void* stream);

/* One frame on the reference's record formats: the packed train batches and
 * the packed eval records are unpacked (two launches, into workspaces the
 * context keeps: the first call with a larger capacity allocates them, so make
 * that call before any stream capture), then the frame runs as
 * nrc_frame_overlapped (results to d_out_rgb as nrc_infer_packed). */
NRC_API int nrc_frame_packed(nrc_context* ctx, const nrc_scene* scene, const nrc_eval_record* d_eval_records,
                             const uint32_t* d_eval_count, uint32_t eval_capacity, float* d_out_rgb,
                             const nrc_packed_train_record* const* d_train_records, uint32_t* const* d_train_counts,
                             uint32_t train_capacity, void* stream);

/* The reference's frame schedule on its record formats
 * (src/rg/NRCRenderGraph.cpp:46-80): nrc_infer_scatter_packed with the
 * rendering weights (screen pixels, and the self-training targets completed in
 * targets->train_records), then those packed train batches unpacked (workspace
 * as nrc_frame_packed) and trained in NRC_TRAIN_BATCH_COUNT chained steps, the
 * last writing use_weights. */
NRC_API int nrc_frame_scatter_packed(nrc_context* ctx, const nrc_scene* scene, const nrc_eval_record* d_eval_records,
                                     const uint32_t* d_eval_count, uint32_t eval_capacity,
                                     const nrc_packed_scatter_targets* targets, uint32_t* const* d_train_counts,
                                     void* stream);

/* Unpacks min(*d_count, capacity) eval records into d_inputs (and their
 * destination words into d_dst, may be NULL), ready for nrc_infer_scatter. */
NRC_API int nrc_unpack_eval(const nrc_scene* scene, const nrc_eval_record* d_records, const uint32_t* d_count,
                            uint32_t capacity, nrc_input* d_inputs, uint32_t* d_dst, void* stream);

/* Unpacks min(*d_count, capacity) train records (bias and factor copied) into
 * d_out, ready for nrc_train / nrc_train_batches. */
NRC_API int nrc_unpack_train(const nrc_scene* scene, const nrc_packed_train_record* d_records,
                             const uint32_t* d_count, uint32_t capacity, nrc_train_record* d_out, void* stream);

/* FP8 precision form of the cache query (no counterpart in the reference, whose
 * query runs in fp16). A context created with fp8_inference = 1 keeps an E4M3
 * copy of use_weights with per-layer absmax scales: s_w = max|W_l| / 448 for
 * the weights, s_x = max|x_l| / 448 for each layer's inputs, where max|x_l| is
 * the largest input the training forward passes met since the scales were last
 * set (bounded from the weights for a layer not yet observed). The scales are
 * recomputed once per 16 optimizer steps; the E4M3 weights are re-quantized
 * with the current scales after every training call (a small launch on the
 * same stream), so the FP8 query always uses the latest rendering weights.
 * Accumulation is fp32; each layer's sum is rescaled before the ReLU. */
/* Cache query as nrc_infer with the E4M3 weights and activations. */
NRC_API int nrc_infer_fp8(nrc_context* ctx, const nrc_input* d_inputs, const uint32_t* d_count, uint32_t capacity,
                          float* d_out_rgb, void* stream);
/* Recomputes the scales and re-quantizes now (stream-ordered). */
NRC_API int nrc_fp8_refresh(nrc_context* ctx, void* stream);
/* Host copies (synchronous): host_w8 receives NRC_PARAM_COUNT E4M3 bytes in the
 * parameter layout, host_scales 25 floats: s_w[6], s_x[6], the per-layer
 * epilogue factors c[6] (s_w s_x / s_x of the next layer; s_w s_x for the
 * output layer), 1 / s_x[0], 1 / s_w[6] (as 448 / max|W_l|). Either may be NULL. */
NRC_API int nrc_get_fp8(nrc_context* ctx, uint8_t* host_w8, float* host_scales);

/* ---------------------------------------------------------------------------
 * Record producer: the reference's path tracer (shader/src/path_tracer.comp)
 * as a CUDA kernel over a BVH built on the GPU, emitting the eval and train
 * records the cache consumes. The reference finds primary hits with a
 * rasterised V-buffer and later hits with Vulkan ray queries against its
 * BLAS/TLAS; here both are ray casts through one BVH over the instanced
 * triangles (the primary cast without the secondary rays' 4.0 range).
 * ------------------------------------------------------------------------- */

/* Primitives of one instance: the instance's triangles are scene primitives
 * first .. first + count - 1 (the reference's instance custom index plus the
 * BLAS primitive index, path_tracer.comp:104-106). */
typedef struct nrc_instance_range {
  uint32_t first_primitive, primitive_count;
} nrc_instance_range;

typedef struct nrc_bvh nrc_bvh;

/* Builds a BVH over every instance's transformed triangles on the current
 * device (Morton codes, a radix sort, a binary radix tree, bounds refitted
 * bottom-up). d_ranges: instance_count entries in device memory. Synchronous. */
NRC_API int nrc_bvh_build(const nrc_scene* scene, const nrc_instance_range* d_ranges, nrc_bvh** out);
NRC_API int nrc_bvh_destroy(nrc_bvh* bvh);
NRC_API int nrc_bvh_info(const nrc_bvh* bvh, uint32_t* triangles, uint32_t* nodes);

/* Path tracer methods (path_tracer.comp:26-28). */
enum { NRC_METHOD_NONE = 0, NRC_METHOD_NRC = 1, NRC_METHOD_CACHE = 2 };

/* Camera and frame (the reference's push constants, src/rg/PathTracerPass.cpp:12-21):
 * the primary ray of pixel (x, y) has direction normalize(look + cx side + cy up),
 * c = ((x, y) + 0.5) / extent * 2 - 1. Pixels with x <= width / 2 use
 * left_method, the others right_method (decided per warp, as per subgroup). */
typedef struct nrc_trace_params {
  float origin[3], look[3], side[3], up[3];
  uint32_t width, height;
  uint32_t seed;
  uint32_t left_method, right_method;
  float train_probability;
} nrc_trace_params;

/* Where the tracer writes: eval records (appended at *eval_count, a device
 * counter the caller zeroes first; records past eval_capacity are dropped, the
 * reference sizes its buffer width * height + 65536, src/VkNRCState.cpp:34-36),
 * train records of NRC_TRAIN_BATCH_COUNT batches of NRC_TRAIN_BATCH_SIZE
 * (appended at *train_counts[b], zeroed by the caller; counts may end above the
 * batch size, as the reference's do, and training clamps them), and the
 * bias_factor_r (rgba32f) / factor_gb (rg32f) images of width x height. */
typedef struct nrc_trace_targets {
  nrc_eval_record* eval_records;
  uint32_t* eval_count;
  uint32_t eval_capacity;
  nrc_packed_train_record* train_records[NRC_TRAIN_BATCH_COUNT];
  uint32_t* train_counts[NRC_TRAIN_BATCH_COUNT];
  float* bias_factor_r;
  float* factor_gb;
} nrc_trace_targets;

/* One frame of the path tracer (path_tracer.comp:377-420): per pixel a primary
 * hit, then PathTrace or, for warps chosen for training, ExtendedPathTrace
 * (Cook-Torrance sampling, up to 8 bounces, the reference's path-length
 * heuristic), eval records for the cache queries and train records with their
 * self-training ranges, and the screen's bias / factor. Stream-ordered. */
NRC_API int nrc_path_trace(const nrc_scene* scene, const nrc_bvh* bvh, const nrc_trace_params* params,
                           const nrc_trace_targets* targets, void* stream);

/* Screen pass (shader/src/screen.frag:10-31) on a headless image: `d_color` is
 * the composited rgba32f image ([height][width][4], rgb used; the bias_factor_r
 * image after nrc_infer_scatter). With accumulate != 0 the color becomes the
 * running average (color + acc * accumulate_count) / (accumulate_count + 1)
 * (none when the count is 0) and is stored to d_accumulate (rgba32f, alpha 0),
 * as the reference's accumulation image. Then the Hejl 2015 filmic tone map
 * (white point 3.2) and gamma 1/2.2; results to d_out_rgba8 (UNORM8, alpha 255)
 * and/or d_out_rgba (float, alpha 1), either may be NULL. The tone curve's small
 * negative values near black take pow() of 0. Replaces rg::ScreenPass
 * (src/rg/ScreenPass.cpp:60-68) minus the swapchain. */
NRC_API int nrc_screen(const float* d_color, float* d_accumulate, uint32_t width, uint32_t height, int accumulate,
                       uint32_t accumulate_count, uint8_t* d_out_rgba8, float* d_out_rgba, void* stream);

/* Checkpoints of one cache (no counterpart in the reference, which keeps its
 * cache for the process's lifetime): a self-describing host blob of
 * nrc_checkpoint_bytes() bytes holding the hyper-parameters, the optimizer step
 * state, the Adam entries {m, v, w, ema} and both fp16 weight vectors, with a
 * checksum. nrc_load_checkpoint restores all of them into an existing context
 * (any seed), so training continues exactly as it would have in the saved one;
 * a blob of the wrong size, version or checksum returns
 * NRC_ERROR_BAD_CHECKPOINT and changes nothing. Both are synchronous. */
NRC_API size_t nrc_checkpoint_bytes(void);
NRC_API int nrc_save_checkpoint(nrc_context* ctx, void* host_blob, size_t bytes);
NRC_API int nrc_load_checkpoint(nrc_context* ctx, const void* host_blob, size_t bytes);

/* Host copies of the parameter state (synchronous). `which` selects
 * NRC_WEIGHTS_USE or NRC_WEIGHTS_TRAIN for the fp16 vectors. */
NRC_API int nrc_get_weights(nrc_context* ctx, int which, uint16_t* host_w16);
/* Sets both fp16 vectors and the fp32 master/EMA copies from host fp16
 * weights; moments and step state are left as they are. */
NRC_API int nrc_set_weights(nrc_context* ctx, const uint16_t* host_w16);
NRC_API int nrc_get_optimizer(nrc_context* ctx, nrc_optimizer_state* host_state, nrc_optimizer_entry* host_entries);
NRC_API int nrc_set_optimizer(nrc_context* ctx, const nrc_optimizer_state* host_state,
                      const nrc_optimizer_entry* host_entries);

/* Check path (config track_loss): sum of the per-record relative-L2 loss and
 * the number of records since the last call; resets both. Synchronous. */
NRC_API int nrc_get_loss(nrc_context* ctx, double* loss_sum, uint64_t* records);

/* Reads and clears the context's latched device error word; returns
 * NRC_ERROR_DEVICE_TIMEOUT if a kernel reported a timed-out wait. Synchronous. */
NRC_API int nrc_get_error(nrc_context* ctx);

/* Device pointers of the context's parameter buffers, for callers that bind
 * them directly (e.g. through external-memory interop). Any may be NULL. */
NRC_API int nrc_get_device_buffers(nrc_context* ctx, uint16_t** weights, uint16_t** use_weights,
                           nrc_optimizer_entry** entries, nrc_optimizer_state** state);

#ifdef __cplusplus
}
#endif
#endif /* NRC_H */
