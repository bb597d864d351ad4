// C ABI of libnrc.so (include/nrc.h): context ownership, argument checks and
// kernel launches. Host code only; kernels live in nrc_infer.cu, nrc_train.cu
// and nrc_encode.cu.
#include <algorithm>
#include <cmath>
#include <cudaTypedefs.h>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "nrc_common.cuh"
#include "nrc_kernels.h"

struct nrc_context {
  nrc_config cfg;
  bool bf16 = false;  // precision form: 16-bit vectors and operands in bf16
  int device = 0;
  int num_sms = 0;
  void* block = nullptr;  // one device allocation, carved below
  size_t block_bytes = 0;
  __half* w16 = nullptr;  // training weights (reference: weights)
  __half* use16 = nullptr;  // rendering weights (reference: use_weights)
  nrc_optimizer_entry* entries = nullptr;
  nrc_optimizer_state* state = nullptr;
  float* partials = nullptr;  // one weight-gradient vector per training CTA
  uint32_t* sync = nullptr;   // grid-barrier counter of the trainer
  uint32_t* tiles = nullptr;  // tile and exit counters of the overlapped frame's query
  uint32_t* err = nullptr;
  double* loss_acc = nullptr;
  unsigned long long* loss_count = nullptr;
  CUtensorMap map_w16;    // TMA views of the two fp16 weight vectors
  CUtensorMap map_use16;
  bool fp8 = false;       // FP8 query form on: activation absmax gathered, E4M3 copy refreshed
  uint8_t* w8 = nullptr;  // E4M3 rendering weights, 323 rows x 128 bytes (bytes 64..127 zero)
  nrc::Fp8State* fp8s = nullptr;
  CUtensorMap map_w8;
  __half* use_next = nullptr;   // the overlapped frame's training writes use_weights here first
  nrc_frame_plan plan = {0u, 0u};  // the overlapped frame's split, once tuned
  bool plan_tuned = false;         // nrc_autotune_frame has set `plan` (which may be sequential)
  // packed-record calls: the unpacked eval records and their destination words
  // (eval_ws_cap each), and the unpacked train records of a frame's batches
  // (NRC_TRAIN_BATCH_COUNT x train_ws_cap), allocated by the first call that needs them
  nrc_input* eval_ws = nullptr;
  uint32_t* eval_dst_ws = nullptr;
  uint32_t eval_ws_cap = 0;
  nrc_train_record* train_ws = nullptr;
  uint32_t train_ws_cap = 0;
};

namespace nrc {

cudaError_t make_weight_map(CUtensorMap* map, const void* w16) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (encode == nullptr) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || fn == nullptr || q != cudaDriverEntryPointSuccess) return cudaErrorNotSupported;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  // 323 rows of 64 fp16 (128-byte rows); boxes of 64 x 16, 128-byte swizzle;
  // rows past 322 read as zero.
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(kWidth), static_cast<cuuint64_t>(kWeightRows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(kWidth) * 2};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(kWidth), 16};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(w16), dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

size_t context_device_bytes(const nrc_context* c) { return c->block_bytes; }

constexpr size_t kW8Bytes = size_t(kWeightRows) * 128;

size_t context_device_bytes_for(int num_sms) {
  auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
  return 3 * up(kParams * 2) + up(kParams * sizeof(nrc_optimizer_entry)) + up(sizeof(nrc_optimizer_state)) + 512 +
         up(kW8Bytes) + up(sizeof(Fp8State)) + up(size_t(num_sms) * kParams * sizeof(float));
}

}  // namespace nrc

namespace {

using nrc::kParams;

int from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return NRC_OK;
  if (e == cudaErrorMemoryAllocation) return NRC_ERROR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return NRC_ERROR_NO_DEVICE;
  return NRC_ERROR_CUDA;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

int configure_kernels() {
  // Dynamic shared-memory limits on the current device; idempotent.
  cudaError_t e = nrc::configure_infer_kernels();
  if (e == cudaSuccess) e = nrc::configure_train_kernels();
  return from_cuda(e);
}

void he_init(uint64_t seed, float* w) {
  // src/VkNRCState.cpp:39-44: std::normal_distribution<float>{0, sqrt(2/64)}
  // over std::mt19937, one draw per parameter in index order.
  std::mt19937 rng(static_cast<std::mt19937::result_type>(seed));
  std::normal_distribution<float> norm{0.0f, std::sqrt(2.0f / float(NRC_WIDTH))};
  for (int i = 0; i < kParams; ++i) w[i] = norm(rng);
}

uint16_t f32_to_16_bits(float x, bool bf16) {
  uint16_t b;
  if (bf16) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    std::memcpy(&b, &h, 2);
  } else {
    const __half h = __float2half_rn(x);
    std::memcpy(&b, &h, 2);
  }
  return b;
}

float bits16_to_f32(uint16_t b, bool bf16) {
  if (bf16) {
    __nv_bfloat16 h;
    std::memcpy(&h, &b, 2);
    return __bfloat162float(h);
  }
  __half h;
  std::memcpy(&h, &b, 2);
  return __half2float(h);
}

int upload_init(nrc_context* c, uint64_t seed) {
  std::vector<float> w(kParams);
  he_init(seed, w.data());
  std::vector<uint16_t> w16(kParams);
  std::vector<nrc_optimizer_entry> ent(kParams);
  for (int i = 0; i < kParams; ++i) {
    w16[i] = f32_to_16_bits(w[i], c->bf16);
    ent[i] = nrc_optimizer_entry{0.0f, 0.0f, w[i], w[i]};
  }
  const nrc_optimizer_state st{0u, 1.0f, 1.0f, 1.0f, 0.0f};
  cudaError_t e;
  if ((e = cudaMemcpy(c->w16, w16.data(), kParams * 2, cudaMemcpyHostToDevice)) != cudaSuccess) return from_cuda(e);
  if ((e = cudaMemcpy(c->use16, w16.data(), kParams * 2, cudaMemcpyHostToDevice)) != cudaSuccess) return from_cuda(e);
  if ((e = cudaMemcpy(c->entries, ent.data(), kParams * sizeof(nrc_optimizer_entry), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return from_cuda(e);
  if ((e = cudaMemcpy(c->state, &st, sizeof(st), cudaMemcpyHostToDevice)) != cudaSuccess) return from_cuda(e);
  return NRC_OK;
}

// The FP8 query form's refresh after the rendering weights changed: re-quantize
// (and recompute the scales when forced or in a new 16-step epoch).
int fp8_refresh(nrc_context* c, int force, cudaStream_t stream) {
  if (!c->fp8) return NRC_OK;
  return from_cuda(nrc::launch_fp8_refresh(reinterpret_cast<const uint16_t*>(c->use16), c->bf16, c->state, c->fp8s,
                                           c->w8, force, stream));
}

int check_ctx(nrc_context* c) {
  if (c == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return NRC_ERROR_CUDA;
  if (dev != c->device) return NRC_ERROR_INVALID_ARGUMENT;  // calls must run on the context's device
  return NRC_OK;
}

}  // namespace

extern "C" {

const char* nrc_status_string(int s) {
  switch (s) {
    case NRC_OK: return "ok";
    case NRC_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case NRC_ERROR_CUDA: return "CUDA error";
    case NRC_ERROR_NO_DEVICE: return "no CUDA device";
    case NRC_ERROR_UNSUPPORTED_DEVICE: return "unsupported device (requires sm_103, GB300)";
    case NRC_ERROR_OUT_OF_MEMORY: return "out of device memory";
    case NRC_ERROR_DEVICE_TIMEOUT: return "a kernel's bounded wait timed out";
    case NRC_ERROR_MISALIGNED: return "device buffer not 16-byte aligned";
    case NRC_ERROR_TOO_LARGE: return "more records than the fixed no-allocation scratch holds (16,384)";
    case NRC_ERROR_BAD_CHECKPOINT: return "checkpoint blob of the wrong size, version or checksum";
    default: return "unknown status";
  }
}

int nrc_default_config(nrc_config* cfg) {
  if (cfg == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  *cfg = nrc_config{};
  cfg->train_batch_size = NRC_TRAIN_BATCH_SIZE;
  cfg->learning_rate = 0.002f;  // shader/src/nrc_optimize.comp:10
  cfg->beta1 = 0.9f;            // shader/src/Constant.glsl:11-12
  cfg->beta2 = 0.999f;
  cfg->epsilon = 1e-8f;         // shader/src/nrc_optimize.comp:11
  cfg->ema_alpha = 0.99f;       // shader/src/Constant.glsl:13
  cfg->loss_scale = 1.0f;       // shader/src/Constant.glsl:8
  cfg->use_ema_weights = 0;     // src/VkNRCState.hpp:36
  cfg->deterministic = 1;       // the only reduction there is
  cfg->track_loss = 0;
  cfg->seed = 0;
  return NRC_OK;
}

int nrc_he_init_host(uint64_t seed, float* out) {
  if (out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  he_init(seed, out);
  return NRC_OK;
}

int nrc_create(const nrc_config* cfg_in, nrc_context** out) {
  if (out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  nrc_config cfg;
  if (cfg_in) cfg = *cfg_in;
  else nrc_default_config(&cfg);
  if (cfg.train_batch_size == 0 || !(cfg.learning_rate >= 0.0f) || !(cfg.loss_scale != 0.0f) ||
      (cfg.precision != NRC_PRECISION_FP16 && cfg.precision != NRC_PRECISION_BF16))
    return NRC_ERROR_INVALID_ARGUMENT;
  int dev = 0, count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return NRC_ERROR_NO_DEVICE;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return from_cuda(e);
  cudaDeviceProp prop;
  if ((e = cudaGetDeviceProperties(&prop, dev)) != cudaSuccess) return from_cuda(e);
  if (!(prop.major == 10 && prop.minor == 3)) return NRC_ERROR_UNSUPPORTED_DEVICE;
  int s = configure_kernels();
  if (s != NRC_OK) return s;

  nrc_context* c = new (std::nothrow) nrc_context();
  if (c == nullptr) return NRC_ERROR_OUT_OF_MEMORY;
  c->cfg = cfg;
  c->bf16 = cfg.precision == NRC_PRECISION_BF16;
  c->device = dev;
  c->num_sms = prop.multiProcessorCount;
  const size_t o_w16 = 0;
  const size_t o_use = o_w16 + up256(kParams * 2);
  const size_t o_use2 = o_use + up256(kParams * 2);
  const size_t o_ent = o_use2 + up256(kParams * 2);
  const size_t o_st = o_ent + up256(kParams * sizeof(nrc_optimizer_entry));
  const size_t o_err = o_st + up256(sizeof(nrc_optimizer_state));
  const size_t o_loss = o_err + 256;
  const size_t o_w8 = o_loss + 256;
  const size_t o_fp8 = o_w8 + up256(nrc::kW8Bytes);
  const size_t o_part = o_fp8 + up256(sizeof(nrc::Fp8State));
  const size_t part_bytes = up256(size_t(c->num_sms) * kParams * sizeof(float));
  const size_t total = o_part + part_bytes;
  if ((e = cudaMalloc(&c->block, total)) != cudaSuccess) {
    delete c;
    return from_cuda(e);
  }
  c->block_bytes = total;
  uint8_t* b = static_cast<uint8_t*>(c->block);
  c->w16 = reinterpret_cast<__half*>(b + o_w16);
  c->use16 = reinterpret_cast<__half*>(b + o_use);
  c->use_next = reinterpret_cast<__half*>(b + o_use2);
  c->entries = reinterpret_cast<nrc_optimizer_entry*>(b + o_ent);
  c->state = reinterpret_cast<nrc_optimizer_state*>(b + o_st);
  c->err = reinterpret_cast<uint32_t*>(b + o_err);
  c->loss_acc = reinterpret_cast<double*>(b + o_loss);
  c->loss_count = reinterpret_cast<unsigned long long*>(b + o_loss + 8);
  c->sync = reinterpret_cast<uint32_t*>(b + o_err + 64);
  c->tiles = reinterpret_cast<uint32_t*>(b + o_err + 128);
  c->partials = reinterpret_cast<float*>(b + o_part);
  c->w8 = b + o_w8;
  c->fp8s = reinterpret_cast<nrc::Fp8State*>(b + o_fp8);
  c->fp8 = cfg.fp8_inference != 0;
  if ((e = nrc::make_weight_map(&c->map_w16, c->w16)) != cudaSuccess ||
      (e = nrc::make_weight_map(&c->map_use16, c->use16)) != cudaSuccess ||
      (e = nrc::make_weight_map(&c->map_w8, c->w8)) != cudaSuccess ||  // same geometry: 128-byte rows
      (e = cudaMemset(c->err, 0, 256 + 256)) != cudaSuccess ||
      (e = cudaMemset(c->w8, 0, o_part - o_w8)) != cudaSuccess) {
    cudaFree(c->block);
    delete c;
    return from_cuda(e);
  }
  s = upload_init(c, cfg.seed);
  if (s == NRC_OK) s = fp8_refresh(c, 1, nullptr);
  if (s == NRC_OK) s = from_cuda(cudaDeviceSynchronize());
  if (s != NRC_OK) {
    cudaFree(c->block);
    delete c;
    return s;
  }
  *out = c;
  return NRC_OK;
}

int nrc_destroy(nrc_context* c) {
  if (c == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != c->device) cudaSetDevice(c->device);
  cudaDeviceSynchronize();
  cudaFree(c->block);
  if (c->train_ws != nullptr) cudaFree(c->train_ws);
  if (c->eval_ws != nullptr) cudaFree(c->eval_ws);
  if (dev >= 0 && dev != c->device) cudaSetDevice(dev);
  delete c;
  return NRC_OK;
}

int nrc_reset(nrc_context* c, uint64_t seed) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  cudaDeviceSynchronize();
  c->cfg.seed = seed;
  s = upload_init(c, seed);
  if (s == NRC_OK) s = fp8_refresh(c, 1, nullptr);
  if (s == NRC_OK) s = from_cuda(cudaDeviceSynchronize());
  return s;
}

int nrc_encode(nrc_context* c, const nrc_input* in, const uint32_t* d_count, uint32_t capacity, uint16_t* out,
               void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (capacity == 0) return NRC_OK;
  if (in == nullptr || d_count == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(in) || !aligned16(out)) return NRC_ERROR_MISALIGNED;
  if (c->bf16) return NRC_ERROR_INVALID_ARGUMENT;  // the stand-alone encoding writes fp16 features
  return from_cuda(nrc::launch_encode(in, d_count, capacity, out, c->num_sms, static_cast<cudaStream_t>(stream)));
}

int nrc_sph_encode(const float* dirs, const uint32_t* d_count, uint32_t capacity, float* out, void* stream) {
  if (capacity == 0) return NRC_OK;
  if (dirs == nullptr || d_count == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(out) & 7u) != 0 || (reinterpret_cast<uintptr_t>(dirs) & 3u) != 0)
    return NRC_ERROR_MISALIGNED;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return from_cuda(nrc::launch_sph_encode(dirs, d_count, capacity, out, sms, static_cast<cudaStream_t>(stream)));
}

static const __half* weights_of(nrc_context* c, int which) {
  return which == NRC_WEIGHTS_TRAIN ? c->w16 : c->use16;
}

static const CUtensorMap* weight_map_of(nrc_context* c, int which) {
  return which == NRC_WEIGHTS_TRAIN ? &c->map_w16 : &c->map_use16;
}

int nrc_infer(nrc_context* c, const nrc_input* in, const uint32_t* d_count, uint32_t capacity, float* out,
              int weight_set, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (weight_set != NRC_WEIGHTS_USE && weight_set != NRC_WEIGHTS_TRAIN) return NRC_ERROR_INVALID_ARGUMENT;
  if (capacity == 0) return NRC_OK;
  if (in == nullptr || d_count == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(in) || (reinterpret_cast<uintptr_t>(out) & 3u)) return NRC_ERROR_MISALIGNED;
  nrc::QueryOut q = {};
  q.out = out;
  q.clamp = 1;
  return from_cuda(nrc::launch_infer(in, false, d_count, capacity, weight_map_of(c, weight_set), q, c->err,
                                     c->num_sms, static_cast<cudaStream_t>(stream), c->bf16));
}

// Checks a destination set and copies it into the kernel's output description.
static int scatter_out(const nrc_scatter_targets* t, nrc::QueryOut* q) {
  if (t == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (t->width > 0x8000u || t->height > 0x10000u) return NRC_ERROR_INVALID_ARGUMENT;  // 15 / 16 coordinate bits
  if (t->width > 0 && t->height > 0) {
    if (t->bias_factor_r == nullptr || t->factor_gb == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
    if (!aligned16(t->bias_factor_r) || (reinterpret_cast<uintptr_t>(t->factor_gb) & 7u)) return NRC_ERROR_MISALIGNED;
    q->width = t->width;
    q->height = t->height;
    q->bias_factor_r = t->bias_factor_r;
    q->factor_gb = t->factor_gb;
  }
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) {
    if (t->train_records[b] != nullptr && (reinterpret_cast<uintptr_t>(t->train_records[b]) & 3u))
      return NRC_ERROR_MISALIGNED;
    q->train[b] = reinterpret_cast<float*>(t->train_records[b]);
    q->train_cap[b] = t->train_records[b] != nullptr ? t->train_capacity[b] : 0u;
  }
  q->train_stride = sizeof(nrc_train_record) / 4;
  return NRC_OK;
}

int nrc_infer_scatter(nrc_context* c, const nrc_input* in, const uint32_t* d_dst, const uint32_t* d_count,
                      uint32_t capacity, const nrc_scatter_targets* targets, float* out, int weight_set,
                      void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (weight_set != NRC_WEIGHTS_USE && weight_set != NRC_WEIGHTS_TRAIN) return NRC_ERROR_INVALID_ARGUMENT;
  nrc::QueryOut q = {};
  if ((s = scatter_out(targets, &q)) != NRC_OK) return s;
  if (capacity == 0) return NRC_OK;
  if (in == nullptr || d_dst == nullptr || d_count == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(in) || (reinterpret_cast<uintptr_t>(d_dst) & 3u) || (reinterpret_cast<uintptr_t>(out) & 3u))
    return NRC_ERROR_MISALIGNED;
  q.out = out;
  q.clamp = 1;
  q.dst = d_dst;
  return from_cuda(nrc::launch_infer(in, false, d_count, capacity, weight_map_of(c, weight_set), q, c->err,
                                     c->num_sms, static_cast<cudaStream_t>(stream), c->bf16));
}

int nrc_infer_encoded(nrc_context* c, const uint16_t* enc, const uint32_t* d_count, uint32_t capacity, float* out,
                      int weight_set, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (weight_set != NRC_WEIGHTS_USE && weight_set != NRC_WEIGHTS_TRAIN) return NRC_ERROR_INVALID_ARGUMENT;
  if (capacity == 0) return NRC_OK;
  if (enc == nullptr || d_count == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(enc) || (reinterpret_cast<uintptr_t>(out) & 3u)) return NRC_ERROR_MISALIGNED;
  nrc::QueryOut q = {};
  q.out = out;
  q.clamp = 0;
  if (c->bf16) return NRC_ERROR_INVALID_ARGUMENT;  // pre-encoded inputs are fp16 features
  return from_cuda(nrc::launch_infer(enc, true, d_count, capacity, weight_map_of(c, weight_set), q, c->err,
                                     c->num_sms, static_cast<cudaStream_t>(stream)));
}

static nrc::TrainParams train_params(nrc_context* c, int steps, int mode) {
  const nrc_config& g = c->cfg;
  nrc::TrainParams p = {};
  p.steps = steps;
  p.mode = mode;
  p.batch_cap = mode == nrc::kTrainStep ? g.train_batch_size : 0xFFFFFFFFu;
  p.lr = g.learning_rate;
  p.beta1 = g.beta1;
  p.beta2 = g.beta2;
  p.eps = g.epsilon;
  p.ema_alpha = g.ema_alpha;
  p.loss_scale = g.loss_scale;
  p.use_ema = g.use_ema_weights != 0;
  p.entries = c->entries;
  p.state = c->state;
  p.w16 = c->w16;
  p.use16 = c->use16;
  p.partials = c->partials;
  p.sync = c->sync;
  p.loss_acc = (g.track_loss && mode == nrc::kTrainStep) ? c->loss_acc : nullptr;
  p.loss_count = (g.track_loss && mode == nrc::kTrainStep) ? c->loss_count : nullptr;
  p.err = c->err;
  p.bf16 = c->bf16 ? 1 : 0;
  p.amax = (c->fp8 && mode == nrc::kTrainStep) ? c->fp8s->amax_x : nullptr;
  return p;
}

int nrc_train(nrc_context* c, const nrc_train_record* rec, uint32_t* d_count, uint32_t capacity,
              int write_use_weights, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (d_count == nullptr || (capacity > 0 && rec == nullptr)) return NRC_ERROR_INVALID_ARGUMENT;
  if (rec != nullptr && !aligned16(rec)) return NRC_ERROR_MISALIGNED;
  nrc::TrainParams p = train_params(c, 1, nrc::kTrainStep);
  p.batch[0] = nrc::TrainBatch{rec, d_count, capacity, write_use_weights != 0};
  s = from_cuda(nrc::launch_train(p, &c->map_w16, c->num_sms, static_cast<cudaStream_t>(stream)));
  return s == NRC_OK ? fp8_refresh(c, 0, static_cast<cudaStream_t>(stream)) : s;
}

int nrc_gradient(nrc_context* c, const nrc_train_record* rec, const uint32_t* d_count, uint32_t capacity,
                 float* d_grad, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (d_count == nullptr || d_grad == nullptr || (capacity > 0 && rec == nullptr)) return NRC_ERROR_INVALID_ARGUMENT;
  if ((rec != nullptr && !aligned16(rec)) || !aligned16(d_grad)) return NRC_ERROR_MISALIGNED;
  // The whole gradient vector is written (zero for an empty batch), as the
  // reference's cleared gradient buffer would read (src/rg/NNTrain.hpp:96-98).
  nrc::TrainParams p = train_params(c, 1, nrc::kGradientOnly);
  p.batch[0] = nrc::TrainBatch{rec, const_cast<uint32_t*>(d_count), capacity, 0};
  p.grad_out = d_grad;
  return from_cuda(nrc::launch_train(p, &c->map_w16, c->num_sms, static_cast<cudaStream_t>(stream)));
}

int nrc_optimize(nrc_context* c, const float* d_grad_sum, uint32_t* d_count, int write_use_weights, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (d_grad_sum == nullptr || d_count == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(d_grad_sum) || (reinterpret_cast<uintptr_t>(d_count) & 3u)) return NRC_ERROR_MISALIGNED;
  const nrc::TrainParams p = train_params(c, 1, nrc::kTrainStep);
  s = from_cuda(nrc::launch_optimize(p, d_grad_sum, d_count, write_use_weights != 0, static_cast<cudaStream_t>(stream)));
  return s == NRC_OK ? fp8_refresh(c, 0, static_cast<cudaStream_t>(stream)) : s;
}

int nrc_loss_gradient(const float* d_pred, const float* d_target, const uint32_t* d_count, uint32_t capacity,
                      float loss_scale, uint32_t precision, uint32_t* d_rows, void* stream) {
  if (d_count == nullptr || (capacity > 0 && (d_pred == nullptr || d_target == nullptr || d_rows == nullptr)) ||
      (precision != NRC_PRECISION_FP16 && precision != NRC_PRECISION_BF16))
    return NRC_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(d_pred) | reinterpret_cast<uintptr_t>(d_target) |
       reinterpret_cast<uintptr_t>(d_rows) | reinterpret_cast<uintptr_t>(d_count)) & 3u)
    return NRC_ERROR_MISALIGNED;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return NRC_ERROR_NO_DEVICE;
  return from_cuda(nrc::launch_loss_rows(d_pred, d_target, d_count, capacity, loss_scale,
                                         precision == NRC_PRECISION_BF16, d_rows, sms,
                                         static_cast<cudaStream_t>(stream)));
}

int nrc_train_batches(nrc_context* c, const nrc_train_record* const* recs, uint32_t* const* counts, uint32_t capacity,
                      int nbatches, int write_use_last, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (recs == nullptr || counts == nullptr || nbatches < 1 || nbatches > NRC_TRAIN_BATCH_COUNT)
    return NRC_ERROR_INVALID_ARGUMENT;
  for (int b = 0; b < nbatches; ++b) {
    if (counts[b] == nullptr || (capacity > 0 && recs[b] == nullptr)) return NRC_ERROR_INVALID_ARGUMENT;
    if (recs[b] != nullptr && !aligned16(recs[b])) return NRC_ERROR_MISALIGNED;
  }
  nrc::TrainParams p = train_params(c, nbatches, nrc::kTrainStep);
  for (int b = 0; b < nbatches; ++b)
    p.batch[b] = nrc::TrainBatch{recs[b], counts[b], capacity, (write_use_last != 0 && b == nbatches - 1) ? 1 : 0};
  s = from_cuda(nrc::launch_train(p, &c->map_w16, c->num_sms, static_cast<cudaStream_t>(stream)));
  return s == NRC_OK ? fp8_refresh(c, 0, static_cast<cudaStream_t>(stream)) : s;
}

int nrc_frame(nrc_context* c, const nrc_input* eval_in, const uint32_t* d_eval_count, uint32_t eval_capacity,
              float* out, const nrc_train_record* const* train_rec, uint32_t* const* train_counts,
              uint32_t train_capacity, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (train_rec == nullptr || train_counts == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  s = nrc_infer(c, eval_in, d_eval_count, eval_capacity, out, NRC_WEIGHTS_USE, stream);
  if (s != NRC_OK) return s;
  return nrc_train_batches(c, train_rec, train_counts, train_capacity, NRC_TRAIN_BATCH_COUNT, 1, stream);
}

}  // extern "C"

namespace nrc {
int loop_slot_jobs(nrc_context* c, const nrc_frame_buffers& f, uint32_t max_queries, uint32_t train_records,
                   InferJob* ij, TrainJob* tj) {
  const int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (c->bf16 || c->fp8) return NRC_ERROR_INVALID_ARGUMENT;
  *ij = InferJob{};
  ij->wmap = *weight_map_of(c, NRC_WEIGHTS_USE);
  ij->input = f.queries;
  ij->d_count = f.query_count;
  ij->capacity = max_queries;
  ij->err = c->err;
  ij->q.out = f.out_rgb;
  ij->q.clamp = 1;
  TrainParams p = train_params(c, NRC_TRAIN_BATCH_COUNT, kTrainStep);
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b)
    p.batch[b] = TrainBatch{f.train[b], f.train_count[b], train_records, b == NRC_TRAIN_BATCH_COUNT - 1 ? 1 : 0};
  *tj = TrainJob{};
  tj->wmap = c->map_w16;
  tj->p = p;
  return NRC_OK;
}
}  // namespace nrc


// Gather tables of one scene (nrc_scene_prepare): primitive_count 64-byte
// primitive rows, then material_count material rows, in one allocation.
struct nrc_scene_tables {
  void* prims;
  void* mats;
  uint32_t primitive_count, material_count;
};

static int scene_check_impl(const nrc_scene* sc) {
  if (sc == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (sc->tables != nullptr &&
      (sc->tables->primitive_count != sc->primitive_count || sc->tables->material_count != sc->material_count))
    return NRC_ERROR_INVALID_ARGUMENT;  // tables of another scene
  const bool geometry = sc->primitive_count > 0 && sc->instance_count > 0;
  if (geometry && (sc->vertices == nullptr || sc->vertex_indices == nullptr || sc->texcoords == nullptr ||
                   sc->texcoord_indices == nullptr || sc->materials == nullptr || sc->material_ids == nullptr ||
                   sc->transforms == nullptr))
    return NRC_ERROR_INVALID_ARGUMENT;
  if (sc->texture_count > 0 && sc->textures == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(sc->materials) & 15u) || (reinterpret_cast<uintptr_t>(sc->textures) & 7u) ||
      (reinterpret_cast<uintptr_t>(sc->transforms) & 15u) || (reinterpret_cast<uintptr_t>(sc->texcoords) & 7u))
    return NRC_ERROR_MISALIGNED;
  return NRC_OK;
}

static const void* prim_rows(const nrc_scene* sc) { return sc->tables != nullptr ? sc->tables->prims : nullptr; }
static const void* mat_rows(const nrc_scene* sc) { return sc->tables != nullptr ? sc->tables->mats : nullptr; }

namespace {

cudaError_t launch_frame_query(nrc_context* c, const nrc_input* in, const uint32_t* d_count, uint32_t capacity,
                               const nrc::QueryOut& q, bool overlapped, const nrc::FrameJoin& join, cudaStream_t st) {
  if (overlapped)
    return nrc::launch_infer_frame(in, d_count, capacity, &c->map_use16, q, c->err, c->tiles, join,
                                   nrc::infer_grid(capacity, c->num_sms), st, c->bf16);
  return nrc::launch_infer(in, false, d_count, capacity, &c->map_use16, q, c->err, c->num_sms, st, c->bf16);
}

// The body of nrc_frame_overlapped.
int frame_overlapped(nrc_context* c, const nrc_input* eval_in, const uint32_t* d_eval_count, uint32_t eval_capacity,
                     float* out, const nrc_train_record* const* train_rec, uint32_t* const* train_counts,
                     uint32_t train_capacity, const nrc_frame_plan* plan_in, void* query_event, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (train_rec == nullptr || train_counts == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) {
    if (train_counts[b] == nullptr || (train_capacity > 0 && train_rec[b] == nullptr)) return NRC_ERROR_INVALID_ARGUMENT;
    if (train_rec[b] != nullptr && !aligned16(train_rec[b])) return NRC_ERROR_MISALIGNED;
  }
  if (eval_capacity > 0) {
    if (eval_in == nullptr || d_eval_count == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
    if (!aligned16(eval_in) || (reinterpret_cast<uintptr_t>(out) & 3u)) return NRC_ERROR_MISALIGNED;
  }
  nrc_frame_plan plan = plan_in ? *plan_in : c->plan;
  if (plan_in == nullptr && !c->plan_tuned) {
    plan.train_ctas = static_cast<uint32_t>(c->num_sms) / 4;  // default split before any tuning
    plan.query_ctas = static_cast<uint32_t>(c->num_sms) - plan.train_ctas;
  }
  const bool sequential = plan.train_ctas == 0;
  if (!sequential && (plan.query_ctas == 0 || plan.query_ctas + plan.train_ctas > static_cast<uint32_t>(c->num_sms) ||
                      plan.train_ctas > nrc::train_grid(nrc::TrainParams{}, c->num_sms)))
    return NRC_ERROR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  nrc::QueryOut q = {};
  q.out = out;
  q.clamp = 1;
  nrc::TrainParams p = train_params(c, NRC_TRAIN_BATCH_COUNT, nrc::kTrainStep);
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b)
    p.batch[b] = nrc::TrainBatch{train_rec[b], train_counts[b], train_capacity, b == NRC_TRAIN_BATCH_COUNT - 1 ? 1 : 0};
  if (sequential) {
    // the query with the current rendering weights, then the training, which writes them
    if (eval_capacity > 0) {
      e = launch_frame_query(c, eval_in, d_eval_count, eval_capacity, q, false, nrc::FrameJoin{}, st);
      if (e != cudaSuccess) return from_cuda(e);
    }
    if (query_event != nullptr && (e = cudaEventRecord(static_cast<cudaEvent_t>(query_event), st)) != cudaSuccess)
      return from_cuda(e);
    p.use16 = c->use16;
    e = nrc::launch_train(p, &c->map_w16, c->num_sms, st);
    if (e != cudaSuccess) return from_cuda(e);
    return fp8_refresh(c, 0, st);
  }
  // Overlapped: the training first, on plan.train_ctas SMs, writing the new
  // rendering weights to a staging buffer; behind it in the stream the query,
  // a grid over every SM that takes its tiles from a counter and starts as soon
  // as all training CTAs run (programmatic dependence, no wait for the
  // training's end): plan.query_ctas of its CTAs start beside the training and
  // the others on the training's SMs as it finishes.
  // The staged weights are copied into use_weights by the query CTA that is
  // the last to load its weights, after its wait for the training grid (or,
  // without a query, by the training's last CTA), so no copy waits in the
  // stream between frames.
  nrc::FrameJoin join = {};
  join.src = reinterpret_cast<const uint4*>(c->use_next);
  join.dst = reinterpret_cast<uint4*>(c->use16);
  p.use16 = c->use_next;
  if (eval_capacity == 0) p.join = join;
  e = nrc::launch_train(p, &c->map_w16, static_cast<int>(plan.train_ctas), st);
  if (e != cudaSuccess) return from_cuda(e);
  if (eval_capacity > 0) {
    e = launch_frame_query(c, eval_in, d_eval_count, eval_capacity, q, true, join, st);
    if (e != cudaSuccess) return from_cuda(e);
  }
  if (query_event != nullptr && (e = cudaEventRecord(static_cast<cudaEvent_t>(query_event), st)) != cudaSuccess)
    return from_cuda(e);
  return fp8_refresh(c, 0, st);
}

// Grows the context's unpacked-eval-record workspace to `capacity` records
// (an allocation: not inside a stream capture).
int ensure_eval_ws(nrc_context* c, uint32_t capacity) {
  if (capacity <= c->eval_ws_cap) return NRC_OK;
  cudaError_t e = cudaSuccess;
  if (c->eval_ws != nullptr) {
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return from_cuda(e);
    cudaFree(c->eval_ws);
    c->eval_ws = nullptr;
    c->eval_dst_ws = nullptr;
    c->eval_ws_cap = 0;
  }
  const size_t in_bytes = up256(size_t(capacity) * sizeof(nrc_input));
  void* p = nullptr;
  e = cudaMalloc(&p, in_bytes + size_t(capacity) * sizeof(uint32_t));
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? NRC_ERROR_OUT_OF_MEMORY : from_cuda(e);
  c->eval_ws = static_cast<nrc_input*>(p);
  c->eval_dst_ws = reinterpret_cast<uint32_t*>(static_cast<uint8_t*>(p) + in_bytes);
  c->eval_ws_cap = capacity;
  return NRC_OK;
}

// Unpacks min(*d_count, capacity) packed eval records (and, with dst, their
// destination words) into the context's workspace.
int unpack_eval_ws(nrc_context* c, const nrc_scene* scene, const nrc_eval_record* rec, const uint32_t* d_count,
                   uint32_t capacity, bool dst, cudaStream_t st) {
  if (rec == nullptr || d_count == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (reinterpret_cast<uintptr_t>(rec) & 3u) return NRC_ERROR_MISALIGNED;
  int s = ensure_eval_ws(c, capacity);
  if (s != NRC_OK) return s;
  return from_cuda(nrc::launch_unpack(*scene, prim_rows(scene), mat_rows(scene), false, rec, d_count, capacity,
                                      c->eval_ws, dst ? c->eval_dst_ws : nullptr, c->num_sms, st));
}

// Grows the context's unpacked-train-record workspace to `capacity` records
// per batch (an allocation: not inside a stream capture).
int ensure_train_ws(nrc_context* c, uint32_t capacity) {
  if (capacity <= c->train_ws_cap) return NRC_OK;
  cudaError_t e = cudaSuccess;
  if (c->train_ws != nullptr) {
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return from_cuda(e);
    cudaFree(c->train_ws);
    c->train_ws = nullptr;
    c->train_ws_cap = 0;
  }
  void* p = nullptr;
  e = cudaMalloc(&p, size_t(NRC_TRAIN_BATCH_COUNT) * capacity * sizeof(nrc_train_record));
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? NRC_ERROR_OUT_OF_MEMORY : from_cuda(e);
  c->train_ws = static_cast<nrc_train_record*>(p);
  c->train_ws_cap = capacity;
  return NRC_OK;
}

// Unpacks the frame's packed train batches into the workspace; ws[b] receives
// batch b's array.
int unpack_train_ws(nrc_context* c, const nrc_scene* scene, const nrc_packed_train_record* const* rec,
                    uint32_t* const* counts, uint32_t capacity, const nrc_train_record** ws, cudaStream_t st) {
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) {
    if (counts[b] == nullptr || (capacity > 0 && rec[b] == nullptr)) return NRC_ERROR_INVALID_ARGUMENT;
    if (rec[b] != nullptr && (reinterpret_cast<uintptr_t>(rec[b]) & 3u)) return NRC_ERROR_MISALIGNED;
  }
  int s = ensure_train_ws(c, capacity > 0 ? capacity : 1);
  if (s != NRC_OK) return s;
  nrc_train_record* out[NRC_TRAIN_BATCH_COUNT];
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) {
    out[b] = c->train_ws + size_t(b) * c->train_ws_cap;
    ws[b] = out[b];
  }
  if (capacity == 0) return NRC_OK;
  return from_cuda(nrc::launch_unpack_train_batches(*scene, prim_rows(scene), mat_rows(scene), rec, counts, capacity,
                                                    out, NRC_TRAIN_BATCH_COUNT, c->num_sms, st));
}

}  // namespace

extern "C" {

int nrc_frame_overlapped(nrc_context* c, const nrc_input* eval_in, const uint32_t* d_eval_count, uint32_t eval_capacity,
                         float* out, const nrc_train_record* const* train_rec, uint32_t* const* train_counts,
                         uint32_t train_capacity, const nrc_frame_plan* plan_in, void* query_event, void* stream) {
  return frame_overlapped(c, eval_in, d_eval_count, eval_capacity, out, train_rec, train_counts, train_capacity, plan_in,
                          query_event, stream);
}

int nrc_infer_packed(nrc_context* c, const nrc_scene* scene, const nrc_eval_record* rec, const uint32_t* d_count,
                     uint32_t capacity, float* out, int weight_set, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if ((s = scene_check_impl(scene)) != NRC_OK) return s;
  if (weight_set != NRC_WEIGHTS_USE && weight_set != NRC_WEIGHTS_TRAIN) return NRC_ERROR_INVALID_ARGUMENT;
  if (capacity == 0) return NRC_OK;
  if (out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (reinterpret_cast<uintptr_t>(out) & 3u) return NRC_ERROR_MISALIGNED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if ((s = unpack_eval_ws(c, scene, rec, d_count, capacity, false, st)) != NRC_OK) return s;
  nrc::QueryOut q = {};
  q.out = out;
  q.clamp = 1;
  return from_cuda(nrc::launch_infer(c->eval_ws, false, d_count, capacity, weight_map_of(c, weight_set), q, c->err,
                                     c->num_sms, st, c->bf16));
}

int nrc_infer_scatter_packed(nrc_context* c, const nrc_scene* scene, const nrc_eval_record* rec,
                             const uint32_t* d_count, uint32_t capacity, const nrc_packed_scatter_targets* targets,
                             float* out, int weight_set, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if ((s = scene_check_impl(scene)) != NRC_OK) return s;
  if (weight_set != NRC_WEIGHTS_USE && weight_set != NRC_WEIGHTS_TRAIN) return NRC_ERROR_INVALID_ARGUMENT;
  nrc::QueryOut q = {};
  // the packed targets differ from nrc_scatter_targets only in the train records' type
  static_assert(sizeof(nrc_packed_scatter_targets) == sizeof(nrc_scatter_targets), "target layouts");
  if ((s = scatter_out(reinterpret_cast<const nrc_scatter_targets*>(targets), &q)) != NRC_OK) return s;
  q.train_stride = sizeof(nrc_packed_train_record) / 4;
  if (capacity == 0) return NRC_OK;
  if (reinterpret_cast<uintptr_t>(out) & 3u) return NRC_ERROR_MISALIGNED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if ((s = unpack_eval_ws(c, scene, rec, d_count, capacity, true, st)) != NRC_OK) return s;
  q.out = out;
  q.clamp = 1;
  q.dst = c->eval_dst_ws;
  return from_cuda(nrc::launch_infer(c->eval_ws, false, d_count, capacity, weight_map_of(c, weight_set), q, c->err,
                                     c->num_sms, st, c->bf16));
}

int nrc_frame_scatter_packed(nrc_context* c, const nrc_scene* scene, const nrc_eval_record* eval_rec,
                             const uint32_t* d_eval_count, uint32_t eval_capacity,
                             const nrc_packed_scatter_targets* targets, uint32_t* const* train_counts, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (targets == nullptr || train_counts == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  uint32_t cap = 0;
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) {
    if (targets->train_records[b] == nullptr || train_counts[b] == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
    if (b > 0 && targets->train_capacity[b] != cap) return NRC_ERROR_INVALID_ARGUMENT;  // one capacity, as nrc_frame
    cap = targets->train_capacity[b];
  }
  s = nrc_infer_scatter_packed(c, scene, eval_rec, d_eval_count, eval_capacity, targets, nullptr, NRC_WEIGHTS_USE,
                               stream);
  if (s != NRC_OK) return s;
  const nrc_packed_train_record* prec[NRC_TRAIN_BATCH_COUNT];
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) prec[b] = targets->train_records[b];
  const nrc_train_record* ws[NRC_TRAIN_BATCH_COUNT];
  if ((s = unpack_train_ws(c, scene, prec, train_counts, cap, ws, static_cast<cudaStream_t>(stream))) != NRC_OK)
    return s;
  return nrc_train_batches(c, ws, train_counts, cap, NRC_TRAIN_BATCH_COUNT, 1, stream);
}

int nrc_frame_packed(nrc_context* c, const nrc_scene* scene, const nrc_eval_record* eval_rec,
                     const uint32_t* d_eval_count, uint32_t eval_capacity, float* out,
                     const nrc_packed_train_record* const* train_rec, uint32_t* const* train_counts,
                     uint32_t train_capacity, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if ((s = scene_check_impl(scene)) != NRC_OK) return s;
  if (train_rec == nullptr || train_counts == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  const nrc_train_record* ws[NRC_TRAIN_BATCH_COUNT];
  if ((s = unpack_train_ws(c, scene, train_rec, train_counts, train_capacity, ws, static_cast<cudaStream_t>(stream))) !=
      NRC_OK)
    return s;
  if (eval_capacity > 0 &&
      (s = unpack_eval_ws(c, scene, eval_rec, d_eval_count, eval_capacity, false, static_cast<cudaStream_t>(stream))) !=
          NRC_OK)
    return s;
  return frame_overlapped(c, c->eval_ws, d_eval_count, eval_capacity, out, ws, train_counts, train_capacity, nullptr, nullptr,
                          stream);
}

int nrc_autotune_frame(nrc_context* c, const nrc_input* eval_in, const uint32_t* d_eval_count, uint32_t eval_capacity,
                       float* out, const nrc_train_record* const* train_rec, uint32_t* const* train_counts,
                       uint32_t train_capacity, nrc_frame_plan* best_out, float* best_ms) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  // a scratch cache with this one's configuration and state: tuning trains it, not this one
  nrc_context* t = nullptr;
  if ((s = nrc_create(&c->cfg, &t)) != NRC_OK) return s;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(t->w16, c->w16, kParams * 2, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(t->use16, c->use16, kParams * 2, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(t->entries, c->entries, kParams * sizeof(nrc_optimizer_entry), cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(t->state, c->state, sizeof(nrc_optimizer_state), cudaMemcpyDeviceToDevice);
  cudaStream_t st = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  nrc_frame_plan best = {0u, 0u};
  float best_t = 1e30f;
  if (e == cudaSuccess) {
    // candidates: the sequential frame, then training groups of 8 .. 72 CTAs beside the query:
    // multiples of 8, and the smallest group for each count of tiles per CTA (a batch's
    // step takes as long as its busiest CTA, so e.g. 43 CTAs finish 128 tiles as soon as 48)
    std::vector<nrc_frame_plan> cand = {{0u, 0u}};
    const uint32_t sms = static_cast<uint32_t>(c->num_sms);
    std::vector<uint32_t> groups;
    for (uint32_t tc = 8; tc <= 72; tc += 8) groups.push_back(tc);
    const uint32_t tiles = (train_capacity + nrc::kTile - 1) / nrc::kTile;
    for (uint32_t k = 1; k <= 16 && tiles > 0; ++k) groups.push_back((tiles + k - 1) / k);
    std::sort(groups.begin(), groups.end());
    groups.erase(std::unique(groups.begin(), groups.end()), groups.end());
    for (uint32_t tc : groups)
      if (tc >= 8 && tc <= 72 && tc < sms) cand.push_back({sms - tc, tc});
    for (const nrc_frame_plan& pl : cand) {
      for (int k = 0; k < 3 && s == NRC_OK; ++k)
        s = nrc_frame_overlapped(t, eval_in, d_eval_count, eval_capacity, out, train_rec, train_counts,
                                 train_capacity, &pl, nullptr, st);
      if (s != NRC_OK) break;
      const int reps = 10;
      cudaEventRecord(a, st);
      for (int k = 0; k < reps && s == NRC_OK; ++k)
        s = nrc_frame_overlapped(t, eval_in, d_eval_count, eval_capacity, out, train_rec, train_counts,
                                 train_capacity, &pl, nullptr, st);
      cudaEventRecord(b, st);
      if (s != NRC_OK || (e = cudaEventSynchronize(b)) != cudaSuccess) break;
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, a, b);
      ms /= reps;
      if (ms < best_t) {
        best_t = ms;
        best = pl;
      }
    }
  }
  if (s == NRC_OK && e == cudaSuccess && nrc_get_error(t) != NRC_OK) s = NRC_ERROR_DEVICE_TIMEOUT;
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (st) cudaStreamDestroy(st);
  nrc_destroy(t);
  if (s != NRC_OK) return s;
  if (e != cudaSuccess) return from_cuda(e);
  c->plan = best;
  c->plan_tuned = true;
  if (best_out) *best_out = best;
  if (best_ms) *best_ms = best_t;
  return NRC_OK;
}

int nrc_frame_scatter(nrc_context* c, const nrc_input* eval_in, const uint32_t* d_eval_dst,
                      const uint32_t* d_eval_count, uint32_t eval_capacity, const nrc_scatter_targets* targets,
                      uint32_t* const* train_counts, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (targets == nullptr || train_counts == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  uint32_t cap = 0;
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) {
    if (targets->train_records[b] == nullptr || train_counts[b] == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
    if (b > 0 && targets->train_capacity[b] != cap) return NRC_ERROR_INVALID_ARGUMENT;  // one capacity, as nrc_frame
    cap = targets->train_capacity[b];
  }
  s = nrc_infer_scatter(c, eval_in, d_eval_dst, d_eval_count, eval_capacity, targets, nullptr, NRC_WEIGHTS_USE,
                        stream);
  if (s != NRC_OK) return s;
  const nrc_train_record* rec[NRC_TRAIN_BATCH_COUNT];
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b) rec[b] = targets->train_records[b];
  return nrc_train_batches(c, rec, train_counts, cap, NRC_TRAIN_BATCH_COUNT, 1, stream);
}

}  // extern "C"

// ------------------------------------------------------------ batched caches --
namespace {

constexpr uint32_t kMaxJobsPerLaunch = 32;  // nrc::kMaxInferJobs == nrc::kMaxTrainJobs
static_assert(nrc::kMaxInferJobs == kMaxJobsPerLaunch && nrc::kMaxTrainJobs == kMaxJobsPerLaunch, "job caps");

// Split `total` CTAs over n jobs in proportion to weight[j] (largest remainder),
// at least one and at most cap[j] each. Requires n <= total.
void split_ctas(const uint64_t* weight, const uint32_t* cap, uint32_t n, uint32_t total, uint32_t* out) {
  uint64_t wsum = 0;
  for (uint32_t j = 0; j < n; ++j) wsum += weight[j];
  uint32_t used = 0;
  std::vector<double> rem(n, 0.0);
  for (uint32_t j = 0; j < n; ++j) {
    const double share = wsum > 0 ? double(total) * double(weight[j]) / double(wsum) : double(total) / n;
    uint32_t g = static_cast<uint32_t>(share);
    g = std::max(1u, std::min(g, cap[j]));
    out[j] = g;
    rem[j] = share - double(g);
    used += g;
  }
  // hand out what is left (or take back the excess), largest remainder first
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

int query_job_check(const nrc_query_job& q, int dev) {
  if (q.ctx == nullptr || q.ctx->device != dev) return NRC_ERROR_INVALID_ARGUMENT;
  if (q.weight_set != NRC_WEIGHTS_USE && q.weight_set != NRC_WEIGHTS_TRAIN) return NRC_ERROR_INVALID_ARGUMENT;
  if (q.capacity == 0) return NRC_OK;
  if (q.inputs == nullptr || q.d_count == nullptr || q.out_rgb == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(q.inputs) || (reinterpret_cast<uintptr_t>(q.out_rgb) & 3u)) return NRC_ERROR_MISALIGNED;
  return NRC_OK;
}

int train_job_check(const nrc_train_job& t, int dev) {
  if (t.ctx == nullptr || t.ctx->device != dev) return NRC_ERROR_INVALID_ARGUMENT;
  if (t.nbatches < 1 || t.nbatches > NRC_TRAIN_BATCH_COUNT) return NRC_ERROR_INVALID_ARGUMENT;
  for (int b = 0; b < t.nbatches; ++b) {
    if (t.d_counts[b] == nullptr || (t.capacity > 0 && t.records[b] == nullptr)) return NRC_ERROR_INVALID_ARGUMENT;
    if (t.records[b] != nullptr && !aligned16(t.records[b])) return NRC_ERROR_MISALIGNED;
  }
  return NRC_OK;
}

template <typename Job>
int check_jobs(const Job* jobs, uint32_t n, int (*one)(const Job&, int)) {
  if (jobs == nullptr && n > 0) return NRC_ERROR_INVALID_ARGUMENT;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return NRC_ERROR_CUDA;
  for (uint32_t j = 0; j < n; ++j) {
    const int s = one(jobs[j], dev);
    if (s != NRC_OK) return s;
    for (uint32_t k = 0; k < j; ++k)
      if (jobs[k].ctx == jobs[j].ctx) return NRC_ERROR_INVALID_ARGUMENT;  // one group per context
  }
  return NRC_OK;
}

int device_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

// The default split of one launch's CTAs (n <= 32 jobs of non-empty capacity).
void plan_query(const nrc_query_job* jobs, uint32_t n, int sms, uint32_t* out) {
  uint64_t w[kMaxJobsPerLaunch];
  uint32_t cap[kMaxJobsPerLaunch];
  uint32_t want = 0;
  for (uint32_t j = 0; j < n; ++j) {
    w[j] = (uint64_t(jobs[j].capacity) + nrc::kTile - 1) / nrc::kTile;
    cap[j] = std::max(1u, nrc::infer_grid(jobs[j].capacity, sms));
    want += cap[j];
  }
  split_ctas(w, cap, n, std::min<uint32_t>(want, static_cast<uint32_t>(sms)), out);
}

void plan_train(const nrc_train_job* jobs, uint32_t n, int sms, uint32_t* out) {
  uint64_t w[kMaxJobsPerLaunch];
  uint32_t cap[kMaxJobsPerLaunch];
  for (uint32_t j = 0; j < n; ++j) {
    const uint32_t rec = std::min(jobs[j].capacity, jobs[j].ctx->cfg.train_batch_size);
    w[j] = uint64_t(jobs[j].nbatches) * std::max<uint64_t>(1, (uint64_t(rec) + nrc::kTile - 1) / nrc::kTile);
    cap[j] = nrc::train_grid(nrc::TrainParams{}, sms);
  }
  split_ctas(w, cap, n, static_cast<uint32_t>(sms), out);
}

// The launches of a batched call: jobs of one operand format (fp16 first,
// then bf16), at most 32 per launch, in job order; jobs that `skip` rejects are
// left out. With explicit CTA counts each launch must fit in the SMs.
template <typename Job>
int launch_groups(const Job* jobs, uint32_t n, const uint32_t* ctas, int sms, bool (*skip)(const Job&),
                  std::vector<std::vector<uint32_t>>* out) {
  out->clear();
  for (int bf16 = 0; bf16 < 2; ++bf16) {
    std::vector<uint32_t> cur;
    for (uint32_t j = 0; j < n; ++j) {
      if (skip(jobs[j]) || jobs[j].ctx->bf16 != (bf16 != 0)) continue;
      cur.push_back(j);
      if (cur.size() == kMaxJobsPerLaunch) {
        out->push_back(cur);
        cur.clear();
      }
    }
    if (!cur.empty()) out->push_back(cur);
  }
  for (const auto& grp : *out) {
    if (grp.size() > static_cast<size_t>(sms)) return NRC_ERROR_INVALID_ARGUMENT;
    if (ctas == nullptr) continue;
    uint64_t sum = 0;
    for (uint32_t j : grp) sum += ctas[j];
    if (sum > static_cast<uint64_t>(sms)) return NRC_ERROR_INVALID_ARGUMENT;
  }
  return NRC_OK;
}

bool query_skip(const nrc_query_job& q) { return q.capacity == 0; }  // nothing to answer
bool train_skip(const nrc_train_job&) { return false; }

}  // namespace

extern "C" {

int nrc_plan_query_ctas(const nrc_query_job* jobs, uint32_t n, uint32_t* out) {
  if (out == nullptr || n == 0 || n > kMaxJobsPerLaunch) return NRC_ERROR_INVALID_ARGUMENT;
  int s = check_jobs(jobs, n, query_job_check);
  if (s != NRC_OK) return s;
  plan_query(jobs, n, device_sms(), out);
  return NRC_OK;
}

int nrc_plan_train_ctas(const nrc_train_job* jobs, uint32_t n, uint32_t* out) {
  if (out == nullptr || n == 0 || n > kMaxJobsPerLaunch) return NRC_ERROR_INVALID_ARGUMENT;
  int s = check_jobs(jobs, n, train_job_check);
  if (s != NRC_OK) return s;
  plan_train(jobs, n, device_sms(), out);
  return NRC_OK;
}

int nrc_infer_many(const nrc_query_job* jobs, uint32_t n, const uint32_t* ctas, void* stream) {
  int s = check_jobs(jobs, n, query_job_check);
  if (s != NRC_OK) return s;
  const int sms = device_sms();
  if (ctas != nullptr)
    for (uint32_t j = 0; j < n; ++j)
      if (ctas[j] == 0) return NRC_ERROR_INVALID_ARGUMENT;
  std::vector<std::vector<uint32_t>> groups;
  if ((s = launch_groups(jobs, n, ctas, sms, query_skip, &groups)) != NRC_OK) return s;
  nrc::InferJob ij[kMaxJobsPerLaunch];
  uint32_t g[kMaxJobsPerLaunch];
  nrc_query_job kept[kMaxJobsPerLaunch];
  for (const auto& grp : groups) {
    const uint32_t k = static_cast<uint32_t>(grp.size());
    for (uint32_t j = 0; j < k; ++j) {
      kept[j] = jobs[grp[j]];
      if (ctas != nullptr) g[j] = ctas[grp[j]];
    }
    if (ctas == nullptr) plan_query(kept, k, sms, g);
    for (uint32_t j = 0; j < k; ++j) {
      const nrc_query_job& q = kept[j];
      ij[j] = nrc::InferJob{};
      ij[j].wmap = *weight_map_of(q.ctx, q.weight_set);
      ij[j].input = q.inputs;
      ij[j].d_count = q.d_count;
      ij[j].capacity = q.capacity;
      ij[j].err = q.ctx->err;
      ij[j].q.out = q.out_rgb;
      ij[j].q.clamp = 1;
    }
    const cudaError_t e = nrc::launch_infer_many(ij, static_cast<int>(k), g, static_cast<cudaStream_t>(stream),
                                                 kept[0].ctx->bf16);
    if (e != cudaSuccess) return from_cuda(e);
  }
  return NRC_OK;
}

int nrc_train_many(const nrc_train_job* jobs, uint32_t n, const uint32_t* ctas, void* stream) {
  int s = check_jobs(jobs, n, train_job_check);
  if (s != NRC_OK) return s;
  const int sms = device_sms();
  if (ctas != nullptr)
    for (uint32_t j = 0; j < n; ++j)
      if (ctas[j] == 0 || ctas[j] > nrc::train_grid(nrc::TrainParams{}, sms)) return NRC_ERROR_INVALID_ARGUMENT;
  std::vector<std::vector<uint32_t>> groups;
  if ((s = launch_groups(jobs, n, ctas, sms, train_skip, &groups)) != NRC_OK) return s;
  std::vector<nrc::TrainJob> tj(kMaxJobsPerLaunch);
  uint32_t g[kMaxJobsPerLaunch];
  nrc_train_job kept[kMaxJobsPerLaunch];
  for (const auto& grp : groups) {
    const uint32_t m = static_cast<uint32_t>(grp.size());
    for (uint32_t j = 0; j < m; ++j) {
      kept[j] = jobs[grp[j]];
      if (ctas != nullptr) g[j] = ctas[grp[j]];
    }
    if (ctas == nullptr) plan_train(kept, m, sms, g);
    for (uint32_t j = 0; j < m; ++j) {
      const nrc_train_job& t = kept[j];
      nrc::TrainParams p = train_params(t.ctx, t.nbatches, nrc::kTrainStep);
      for (int b = 0; b < t.nbatches; ++b)
        p.batch[b] = nrc::TrainBatch{t.records[b], t.d_counts[b], t.capacity,
                                     (t.write_use_last != 0 && b == t.nbatches - 1) ? 1 : 0};
      tj[j].wmap = t.ctx->map_w16;
      tj[j].p = p;
    }
    const cudaError_t e = nrc::launch_train_many(tj.data(), static_cast<int>(m), g, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return from_cuda(e);
    for (uint32_t j = 0; j < m; ++j)
      if ((s = fp8_refresh(kept[j].ctx, 0, static_cast<cudaStream_t>(stream))) != NRC_OK) return s;
  }
  return NRC_OK;
}

}  // extern "C"

namespace {

// Candidate CTA splits of one batched launch: the proportional default first,
// then for every count k of tiles per CTA (per pass of the query's slots, per
// step of the training) the split that gives each job just enough CTAs to take
// its tiles in k rounds, when those fit on the SMs. A launch lasts as long as
// its busiest group, so a job gains nothing from CTAs beyond those that cut its
// rounds; the largest k that fits wastes the fewest.
std::vector<std::vector<uint32_t>> split_candidates(const std::vector<uint64_t>& tiles, uint32_t per_round,
                                                    uint32_t group_cap, uint32_t sms,
                                                    const std::vector<uint32_t>& proportional) {
  std::vector<std::vector<uint32_t>> cand = {proportional};
  uint64_t most = 1;
  for (uint64_t t : tiles) most = std::max(most, t);
  for (uint64_t k = 1; k <= (most + per_round - 1) / per_round; ++k) {
    std::vector<uint32_t> g(tiles.size());
    uint64_t sum = 0;
    bool ok = true;
    for (size_t j = 0; j < tiles.size(); ++j) {
      const uint64_t want = std::max<uint64_t>(1, (tiles[j] + k * per_round - 1) / (k * per_round));
      if (want > group_cap) ok = false;
      g[j] = static_cast<uint32_t>(std::min<uint64_t>(want, group_cap));
      sum += g[j];
    }
    if (!ok || sum > sms) continue;
    if (std::find(cand.begin(), cand.end(), g) == cand.end()) cand.push_back(g);
    if (cand.size() >= 12) break;
  }
  return cand;
}

// Mean duration in ms of `reps` launches of fn on `st`, after two untimed ones.
template <typename F>
int time_launches(F fn, cudaStream_t st, cudaEvent_t a, cudaEvent_t b, int reps, float* ms) {
  int s = NRC_OK;
  for (int k = 0; k < 2 && s == NRC_OK; ++k) s = fn();
  if (s != NRC_OK) return s;
  cudaEventRecord(a, st);
  for (int k = 0; k < reps && s == NRC_OK; ++k) s = fn();
  cudaEventRecord(b, st);
  if (s != NRC_OK) return s;
  const cudaError_t e = cudaEventSynchronize(b);
  if (e != cudaSuccess) return from_cuda(e);
  cudaEventElapsedTime(ms, a, b);
  *ms /= static_cast<float>(reps);
  return NRC_OK;
}

}  // namespace

extern "C" {

int nrc_autotune_many(const nrc_query_job* qjobs, uint32_t nq, const nrc_train_job* tjobs, uint32_t nt,
                      uint32_t* q_ctas, uint32_t* t_ctas, float* q_ms, float* t_ms) {
  if (nq > kMaxJobsPerLaunch || nt > kMaxJobsPerLaunch || (nq > 0 && q_ctas == nullptr) ||
      (nt > 0 && t_ctas == nullptr))
    return NRC_ERROR_INVALID_ARGUMENT;
  int s = check_jobs(qjobs, nq, query_job_check);
  if (s == NRC_OK) s = check_jobs(tjobs, nt, train_job_check);
  if (s != NRC_OK) return s;
  for (uint32_t j = 0; j < nq; ++j)
    if (qjobs[j].capacity == 0 || qjobs[j].ctx->bf16 != qjobs[0].ctx->bf16) return NRC_ERROR_INVALID_ARGUMENT;
  for (uint32_t j = 0; j < nt; ++j)
    if (tjobs[j].ctx->bf16 != tjobs[0].ctx->bf16) return NRC_ERROR_INVALID_ARGUMENT;
  const uint32_t sms = static_cast<uint32_t>(device_sms());
  cudaStream_t st = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e != cudaSuccess) s = from_cuda(e);
  // queries: timed on the jobs themselves (a query writes only its outputs)
  if (s == NRC_OK && nq > 0) {
    std::vector<uint64_t> tiles(nq);
    for (uint32_t j = 0; j < nq; ++j) tiles[j] = (uint64_t(qjobs[j].capacity) + nrc::kTile - 1) / nrc::kTile;
    std::vector<uint32_t> prop(nq);
    plan_query(qjobs, nq, static_cast<int>(sms), prop.data());
    const auto cand = split_candidates(tiles, static_cast<uint32_t>(nrc::infer_tiles_per_cta()), sms, sms, prop);
    float best = 1e30f;
    for (const auto& g : cand) {
      float ms = 0.0f;
      s = time_launches([&] { return nrc_infer_many(qjobs, nq, g.data(), st); }, st, a, b, 5, &ms);
      if (s != NRC_OK) break;
      if (ms < best) {
        best = ms;
        std::copy(g.begin(), g.end(), q_ctas);
      }
    }
    if (s == NRC_OK && q_ms) *q_ms = best;
  }
  // training: timed on scratch copies of the caches (tuning trains them, not the caller's)
  std::vector<nrc_context*> scratch;
  if (s == NRC_OK && nt > 0) {
    std::vector<nrc_train_job> sj(tjobs, tjobs + nt);
    for (uint32_t j = 0; j < nt && s == NRC_OK; ++j) {
      nrc_context* t = nullptr;
      if ((s = nrc_create(&tjobs[j].ctx->cfg, &t)) != NRC_OK) break;
      scratch.push_back(t);
      const nrc_context* c = tjobs[j].ctx;
      e = cudaMemcpy(t->w16, c->w16, kParams * 2, cudaMemcpyDeviceToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(t->use16, c->use16, kParams * 2, cudaMemcpyDeviceToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(t->entries, c->entries, kParams * sizeof(nrc_optimizer_entry), cudaMemcpyDeviceToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(t->state, c->state, sizeof(nrc_optimizer_state), cudaMemcpyDeviceToDevice);
      if (e != cudaSuccess) s = from_cuda(e);
      sj[j].ctx = t;
    }
    if (s == NRC_OK) {
      std::vector<uint64_t> tiles(nt);
      for (uint32_t j = 0; j < nt; ++j) {
        const uint32_t rec = std::min(sj[j].capacity, sj[j].ctx->cfg.train_batch_size);
        tiles[j] = std::max<uint64_t>(1, (uint64_t(rec) + nrc::kTile - 1) / nrc::kTile);
      }
      std::vector<uint32_t> prop(nt);
      plan_train(sj.data(), nt, static_cast<int>(sms), prop.data());
      const auto cand = split_candidates(tiles, 1u, nrc::train_grid(nrc::TrainParams{}, static_cast<int>(sms)), sms,
                                         prop);
      float best = 1e30f;
      for (const auto& g : cand) {
        float ms = 0.0f;
        s = time_launches([&] { return nrc_train_many(sj.data(), nt, g.data(), st); }, st, a, b, 5, &ms);
        if (s != NRC_OK) break;
        if (ms < best) {
          best = ms;
          std::copy(g.begin(), g.end(), t_ctas);
        }
      }
      if (s == NRC_OK && t_ms) *t_ms = best;
    }
    for (nrc_context* t : scratch)
      if (s == NRC_OK && nrc_get_error(t) != NRC_OK) s = NRC_ERROR_DEVICE_TIMEOUT;
  }
  for (nrc_context* t : scratch) nrc_destroy(t);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (st) cudaStreamDestroy(st);
  return s;
}

// ------------------------------------------------------------------- fp8 --
int nrc_infer_fp8(nrc_context* c, const nrc_input* in, const uint32_t* d_count, uint32_t capacity, float* out,
                  void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (!c->fp8) return NRC_ERROR_INVALID_ARGUMENT;  // created without fp8_inference
  if (capacity == 0) return NRC_OK;
  if (in == nullptr || d_count == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(in) || (reinterpret_cast<uintptr_t>(out) & 3u)) return NRC_ERROR_MISALIGNED;
  return from_cuda(nrc::launch_infer_fp8(in, d_count, capacity, &c->map_w8, c->fp8s, out, c->err, c->num_sms,
                                         static_cast<cudaStream_t>(stream)));
}

int nrc_fp8_refresh(nrc_context* c, void* stream) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (!c->fp8) return NRC_ERROR_INVALID_ARGUMENT;
  return fp8_refresh(c, 1, static_cast<cudaStream_t>(stream));
}

int nrc_get_fp8(nrc_context* c, uint8_t* host_w8, float* host_scales) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (!c->fp8) return NRC_ERROR_INVALID_ARGUMENT;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess && host_w8)
    e = cudaMemcpy2D(host_w8, 64, c->w8, 128, 64, nrc::kWeightRows, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && host_scales) {
    nrc::Fp8State st;
    e = cudaMemcpy(&st, c->fp8s, sizeof(st), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) {
      std::memcpy(host_scales, st.scale_w, 6 * 4);
      std::memcpy(host_scales + 6, st.scale_x, 6 * 4);
      std::memcpy(host_scales + 12, st.c, 6 * 4);
      host_scales[18] = st.inv_sx0;
      std::memcpy(host_scales + 19, st.inv_w, 6 * 4);
    }
  }
  return from_cuda(e);
}

// ---------------------------------------------------------------- unpack --

int nrc_unpack_eval(const nrc_scene* sc, const nrc_eval_record* rec, const uint32_t* d_count, uint32_t capacity,
                    nrc_input* out, uint32_t* out_dst, void* stream) {
  int s = scene_check_impl(sc);
  if (s != NRC_OK) return s;
  if (capacity == 0) return NRC_OK;
  if (rec == nullptr || d_count == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(rec) & 3u) || (reinterpret_cast<uintptr_t>(out) & 7u) ||
      (reinterpret_cast<uintptr_t>(out_dst) & 3u))
    return NRC_ERROR_MISALIGNED;
  return from_cuda(nrc::launch_unpack(*sc, prim_rows(sc), mat_rows(sc), false, rec, d_count, capacity, out, out_dst,
                                      device_sms(),
                                      static_cast<cudaStream_t>(stream)));
}

int nrc_unpack_train(const nrc_scene* sc, const nrc_packed_train_record* rec, const uint32_t* d_count,
                     uint32_t capacity, nrc_train_record* out, void* stream) {
  int s = scene_check_impl(sc);
  if (s != NRC_OK) return s;
  if (capacity == 0) return NRC_OK;
  if (rec == nullptr || d_count == nullptr || out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(rec) & 3u) || !aligned16(out)) return NRC_ERROR_MISALIGNED;
  return from_cuda(nrc::launch_unpack(*sc, prim_rows(sc), mat_rows(sc), true, rec, d_count, capacity, out, nullptr,
                                      device_sms(),
                                      static_cast<cudaStream_t>(stream)));
}

int nrc_scene_prepare(const nrc_scene* sc, void* stream, nrc_scene_tables** out) {
  if (out == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  if (sc == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  nrc_scene plain = *sc;
  plain.tables = nullptr;  // the tables are made from the buffers
  int s = scene_check_impl(&plain);
  if (s != NRC_OK) return s;
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the texture descriptors (device array), to size the footprint arrays
  std::vector<nrc_texture> tex(sc->texture_count);
  cudaError_t e = cudaSuccess;
  if (!tex.empty()) {
    e = cudaMemcpyAsync(tex.data(), sc->textures, tex.size() * sizeof(nrc_texture), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return from_cuda(e);
  }
  const size_t prim_bytes = size_t(sc->primitive_count) * 64, mat_bytes = size_t(sc->material_count) * 64;
  const size_t table_bytes = up256(tex.size() * sizeof(nrc_texture));
  size_t fp_bytes = 0;
  std::vector<size_t> fp_off(tex.size(), 0);
  for (size_t i = 0; i < tex.size(); ++i) {
    if (reinterpret_cast<uintptr_t>(tex[i].texels) & 3u) return NRC_ERROR_MISALIGNED;
    fp_off[i] = fp_bytes;
    if (tex[i].texels != nullptr) fp_bytes += size_t(tex[i].width) * tex[i].height * 16;
  }
  const size_t head = up256(prim_bytes + mat_bytes) + table_bytes;
  void* p = nullptr;
  e = cudaMalloc(&p, head + fp_bytes + 64);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? NRC_ERROR_OUT_OF_MEMORY : from_cuda(e);
  uint8_t* base = static_cast<uint8_t*>(p);
  auto* t = new (std::nothrow) nrc_scene_tables{p, base + prim_bytes, sc->primitive_count, sc->material_count};
  if (t == nullptr) {
    cudaFree(p);
    return NRC_ERROR_OUT_OF_MEMORY;
  }
  // descriptors of the footprint arrays, in texture order
  nrc_texture* d_fp = reinterpret_cast<nrc_texture*>(base + up256(prim_bytes + mat_bytes));
  std::vector<nrc_texture> fp(tex.size());
  for (size_t i = 0; i < tex.size(); ++i) {
    const bool any = tex[i].texels != nullptr && tex[i].width > 0 && tex[i].height > 0;
    fp[i].texels = any ? base + head + fp_off[i] : nullptr;
    fp[i].width = tex[i].width;
    fp[i].height = tex[i].height;
  }
  if (!fp.empty()) e = cudaMemcpyAsync(d_fp, fp.data(), fp.size() * sizeof(nrc_texture), cudaMemcpyHostToDevice, st);
  for (size_t i = 0; i < tex.size() && e == cudaSuccess; ++i)
    if (fp[i].texels != nullptr)
      e = nrc::launch_texture_footprints(tex[i], const_cast<uint8_t*>(fp[i].texels), device_sms(), st);
  if (e == cudaSuccess) e = nrc::launch_scene_prepare(plain, d_fp, t->prims, t->mats, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host descriptor arrays are read by then
  if (e != cudaSuccess) {
    cudaFree(p);
    delete t;
    return from_cuda(e);
  }
  *out = t;
  return NRC_OK;
}

int nrc_scene_tables_destroy(nrc_scene_tables* t) {
  if (t == nullptr) return NRC_OK;
  const cudaError_t e = cudaFree(t->prims);
  delete t;
  return from_cuda(e);
}

// ---------------------------------------------------------------- screen --
int nrc_screen(const float* color, float* accum, uint32_t width, uint32_t height, int accumulate,
               uint32_t accumulate_count, uint8_t* out8, float* outf, void* stream) {
  if (width == 0 || height == 0) return NRC_OK;
  if (uint64_t(width) * height > 0xFFFFFFFFull) return NRC_ERROR_INVALID_ARGUMENT;
  if (color == nullptr || (accumulate && accum == nullptr)) return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(color) || (accumulate && !aligned16(accum)) || (outf && !aligned16(outf)) ||
      (out8 && (reinterpret_cast<uintptr_t>(out8) & 3u)))
    return NRC_ERROR_MISALIGNED;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return from_cuda(nrc::launch_screen(color, accumulate ? accum : nullptr, width, height, accumulate != 0,
                                      accumulate_count, out8, outf, sms, static_cast<cudaStream_t>(stream)));
}

// ------------------------------------------------------------ checkpoints --
// Blob layout (little-endian): a 64-byte header, then the step state padded to
// 32 bytes, the Adam entries, the training weights and the rendering weights.
//   0 magic "NRCCKPT1" | 8 version | 12 parameter count | 16 batch cap |
//   20 lr, beta1, beta2, eps, ema alpha, loss scale (f32) | 44 use_ema (bit 0),
//   precision (bits 8..15) |
//   48 payload bytes (u64) | 56 FNV-1a 64 of the payload
namespace {
constexpr size_t kCkptHeader = 64;
constexpr size_t kCkptPayload = 32 + size_t(kParams) * sizeof(nrc_optimizer_entry) + 2 * size_t(kParams) * 2;
constexpr uint32_t kCkptVersion = 1;

uint64_t fnv1a(const uint8_t* p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}
}  // namespace

size_t nrc_checkpoint_bytes(void) { return kCkptHeader + kCkptPayload; }

int nrc_save_checkpoint(nrc_context* c, void* blob, size_t bytes) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (blob == nullptr || bytes < nrc_checkpoint_bytes()) return NRC_ERROR_INVALID_ARGUMENT;
  uint8_t* b = static_cast<uint8_t*>(blob);
  std::memset(b, 0, nrc_checkpoint_bytes());
  uint8_t* pay = b + kCkptHeader;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(pay, c->state, sizeof(nrc_optimizer_state), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(pay + 32, c->entries, size_t(kParams) * sizeof(nrc_optimizer_entry), cudaMemcpyDeviceToHost);
  uint8_t* w = pay + 32 + size_t(kParams) * sizeof(nrc_optimizer_entry);
  if (e == cudaSuccess) e = cudaMemcpy(w, c->w16, size_t(kParams) * 2, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(w + size_t(kParams) * 2, c->use16, size_t(kParams) * 2, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return from_cuda(e);
  const nrc_config& g = c->cfg;
  std::memcpy(b, "NRCCKPT1", 8);
  const uint32_t u[3] = {kCkptVersion, static_cast<uint32_t>(kParams), g.train_batch_size};
  std::memcpy(b + 8, u, 12);
  const float f[6] = {g.learning_rate, g.beta1, g.beta2, g.epsilon, g.ema_alpha, g.loss_scale};
  std::memcpy(b + 20, f, 24);
  const uint32_t flags = (g.use_ema_weights ? 1u : 0u) | (g.precision << 8);  // use_ema bit 0, precision bits 8..15
  std::memcpy(b + 44, &flags, 4);
  const uint64_t pb = kCkptPayload, h = fnv1a(pay, kCkptPayload);
  std::memcpy(b + 48, &pb, 8);
  std::memcpy(b + 56, &h, 8);
  return NRC_OK;
}

int nrc_load_checkpoint(nrc_context* c, const void* blob, size_t bytes) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (blob == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (bytes != nrc_checkpoint_bytes()) return NRC_ERROR_BAD_CHECKPOINT;
  const uint8_t* b = static_cast<const uint8_t*>(blob);
  uint32_t u[3];
  uint64_t pb = 0, h = 0;
  std::memcpy(u, b + 8, 12);
  std::memcpy(&pb, b + 48, 8);
  std::memcpy(&h, b + 56, 8);
  const uint8_t* pay = b + kCkptHeader;
  if (std::memcmp(b, "NRCCKPT1", 8) != 0 || u[0] != kCkptVersion || u[1] != static_cast<uint32_t>(kParams) ||
      pb != kCkptPayload || fnv1a(pay, kCkptPayload) != h)
    return NRC_ERROR_BAD_CHECKPOINT;
  float f[6];
  uint32_t flags = 0;
  std::memcpy(f, b + 20, 24);
  std::memcpy(&flags, b + 44, 4);
  if (u[2] == 0 || !(f[5] != 0.0f) || (flags & ~0xFF01u) != 0) return NRC_ERROR_BAD_CHECKPOINT;
  // the blob's 16-bit vectors must be in this context's format
  if ((flags >> 8) != c->cfg.precision) return NRC_ERROR_INVALID_ARGUMENT;
  const uint32_t use_ema = flags & 1u;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(c->state, pay, sizeof(nrc_optimizer_state), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->entries, pay + 32, size_t(kParams) * sizeof(nrc_optimizer_entry), cudaMemcpyHostToDevice);
  const uint8_t* w = pay + 32 + size_t(kParams) * sizeof(nrc_optimizer_entry);
  if (e == cudaSuccess) e = cudaMemcpy(c->w16, w, size_t(kParams) * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c->use16, w + size_t(kParams) * 2, size_t(kParams) * 2, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return from_cuda(e);
  c->cfg.train_batch_size = u[2];
  c->cfg.learning_rate = f[0];
  c->cfg.beta1 = f[1];
  c->cfg.beta2 = f[2];
  c->cfg.epsilon = f[3];
  c->cfg.ema_alpha = f[4];
  c->cfg.loss_scale = f[5];
  c->cfg.use_ema_weights = use_ema;
  s = fp8_refresh(c, 1, nullptr);
  return s == NRC_OK ? from_cuda(cudaDeviceSynchronize()) : s;
}

int nrc_get_weights(nrc_context* c, int which, uint16_t* host) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (host == nullptr || (which != NRC_WEIGHTS_USE && which != NRC_WEIGHTS_TRAIN)) return NRC_ERROR_INVALID_ARGUMENT;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(host, weights_of(c, which), kParams * 2, cudaMemcpyDeviceToHost);
  return from_cuda(e);
}

int nrc_set_weights(nrc_context* c, const uint16_t* host) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (host == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  std::vector<nrc_optimizer_entry> ent(kParams);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess)
    e = cudaMemcpy(ent.data(), c->entries, kParams * sizeof(nrc_optimizer_entry), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return from_cuda(e);
  for (int i = 0; i < kParams; ++i) {
    const float w = bits16_to_f32(host[i], c->bf16);
    ent[i].weight = w;
    ent[i].ema_weight = w;
  }
  if ((e = cudaMemcpy(c->entries, ent.data(), kParams * sizeof(nrc_optimizer_entry), cudaMemcpyHostToDevice)) ==
          cudaSuccess &&
      (e = cudaMemcpy(c->w16, host, kParams * 2, cudaMemcpyHostToDevice)) == cudaSuccess)
    e = cudaMemcpy(c->use16, host, kParams * 2, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return from_cuda(e);
  s = fp8_refresh(c, 1, nullptr);
  return s == NRC_OK ? from_cuda(cudaDeviceSynchronize()) : s;
}

int nrc_get_optimizer(nrc_context* c, nrc_optimizer_state* st, nrc_optimizer_entry* ent) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess && st) e = cudaMemcpy(st, c->state, sizeof(*st), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && ent) e = cudaMemcpy(ent, c->entries, kParams * sizeof(*ent), cudaMemcpyDeviceToHost);
  return from_cuda(e);
}

int nrc_set_optimizer(nrc_context* c, const nrc_optimizer_state* st, const nrc_optimizer_entry* ent) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess && st) e = cudaMemcpy(c->state, st, sizeof(*st), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ent) e = cudaMemcpy(c->entries, ent, kParams * sizeof(*ent), cudaMemcpyHostToDevice);
  return from_cuda(e);
}

int nrc_get_loss(nrc_context* c, double* loss_sum, uint64_t* records) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  if (loss_sum == nullptr || records == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  struct {
    double sum;
    unsigned long long n;
  } h;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&h, c->loss_acc, 16, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(c->loss_acc, 0, 16);
  if (e != cudaSuccess) return from_cuda(e);
  *loss_sum = h.sum;
  *records = h.n;
  return NRC_OK;
}

int nrc_get_error(nrc_context* c) {
  int s = check_ctx(c);
  if (s != NRC_OK) return s;
  uint32_t h = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&h, c->err, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(c->err, 0, 4);
  if (e != cudaSuccess) return from_cuda(e);
  return h ? NRC_ERROR_DEVICE_TIMEOUT : NRC_OK;
}

int nrc_get_device_buffers(nrc_context* c, uint16_t** w, uint16_t** use, nrc_optimizer_entry** ent,
                           nrc_optimizer_state** st) {
  if (c == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (w) *w = reinterpret_cast<uint16_t*>(c->w16);
  if (use) *use = reinterpret_cast<uint16_t*>(c->use16);
  if (ent) *ent = c->entries;
  if (st) *st = c->state;
  return NRC_OK;
}

}  // extern "C"
