// nrc_train_noalloc: one training step that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a renderer that sub-allocates every
// device buffer from its own heaps (as the reference's Vulkan side does through
// its allocator), or a process that runs under a fixed device-memory budget
// imposed before this library is loaded. nrc_create allocates the cache's
// buffers, so those callers pass their own parameter buffers to this entry
// point instead, and the one piece of scratch the step needs, the per-CTA
// weight-gradient partials, lives in a fixed array compiled into the library.
#include <mutex>

#include "nrc_common.cuh"
#include "nrc_kernels.h"

namespace {

// One gradient partial per CTA, for at most kNoAllocSlots CTAs; a CTA sums any
// number of record tiles into its partial, so the slots do not bound the record
// count. The 16,384-record limit is this entry point's documented policy: one
// call is one training batch of the reference's size (NRC_TRAIN_BATCH_SIZE),
// which keeps a call's duration, and so the window in which a second call on
// another stream would race on the shared array, within one step's length.
constexpr int kNoAllocSlots = 64;
constexpr uint32_t kNoAllocMaxRecords = 16384;
constexpr size_t kScratchFloats = size_t(kNoAllocSlots) * nrc::kParams + 64;  // + error word, barrier counter

// Held by every GPU that loads the library until the process exits:
// 64 x 20,672 x 4 B + 256 B = 5,292,288 bytes.
static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

struct DeviceSetup {
  bool ready = false;
  int status = NRC_OK;
  float* scratch = nullptr;  // device address of g_noalloc_scratch on that device
  int num_sms = 0;
};

std::mutex g_setup_mutex;
DeviceSetup g_setup[64];

// Once per device, with that device current: check the architecture, raise the
// kernels' shared-memory limit and resolve the scratch array's device address.
// In host code the array's name only stands for the symbol; a kernel must be
// given the address that cudaGetSymbolAddress returns.
int setup_current_device(DeviceSetup** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return NRC_ERROR_NO_DEVICE;
  if (dev >= 64) return NRC_ERROR_UNSUPPORTED_DEVICE;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup& s = g_setup[dev];
  if (!s.ready) {
    int major = 0, minor = 0, sms = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      s.status = NRC_ERROR_CUDA;
    } else if (!(major == 10 && minor == 3)) {
      s.status = NRC_ERROR_UNSUPPORTED_DEVICE;
    } else if (nrc::configure_train_kernels() != cudaSuccess) {
      s.status = NRC_ERROR_CUDA;
    } else {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || p == nullptr) {
        s.status = NRC_ERROR_CUDA;
      } else {
        s.scratch = static_cast<float*>(p);
        s.num_sms = sms;
        s.status = NRC_OK;
      }
    }
    s.ready = true;
  }
  *out = &s;
  return s.status;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
bool aligned4(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) == 0; }

}  // namespace

extern "C" NRC_API int nrc_train_noalloc(uint16_t* d_weights, uint16_t* d_use_weights,
                                         nrc_optimizer_entry* d_entries, nrc_optimizer_state* d_state,
                                         const nrc_train_record* d_records, uint32_t* d_count, uint32_t capacity,
                                         const nrc_config* cfg, uint32_t* d_error, void* stream) {
  if (cfg == nullptr || d_weights == nullptr || d_entries == nullptr || d_state == nullptr || d_count == nullptr ||
      (capacity > 0 && d_records == nullptr) || cfg->train_batch_size == 0 || !(cfg->loss_scale != 0.0f) ||
      (cfg->precision != NRC_PRECISION_FP16 && cfg->precision != NRC_PRECISION_BF16))
    return NRC_ERROR_INVALID_ARGUMENT;
  if (!aligned16(d_weights) || !aligned16(d_entries) || (d_records && !aligned16(d_records)) ||
      (d_use_weights && (reinterpret_cast<uintptr_t>(d_use_weights) & 1u)) || !aligned4(d_state) ||
      !aligned4(d_count) || (d_error && !aligned4(d_error)))
    return NRC_ERROR_MISALIGNED;
  const uint32_t records = capacity < cfg->train_batch_size ? capacity : cfg->train_batch_size;
  if (records > kNoAllocMaxRecords) return NRC_ERROR_TOO_LARGE;
  DeviceSetup* s = nullptr;
  const int st = setup_current_device(&s);
  if (st != NRC_OK) return st;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  uint32_t* err = d_error;
  if (err == nullptr) {
    err = reinterpret_cast<uint32_t*>(s->scratch + size_t(kNoAllocSlots) * nrc::kParams);
    if (cudaMemsetAsync(err, 0, sizeof(uint32_t), cs) != cudaSuccess) return NRC_ERROR_CUDA;
  }
  // At most kNoAllocSlots CTAs, one gradient partial each, summed in CTA order.
  const int max_ctas = s->num_sms < kNoAllocSlots ? s->num_sms : kNoAllocSlots;
  CUtensorMap wmap;  // host-side descriptor of the caller's weights; no device memory
  if (nrc::make_weight_map(&wmap, d_weights) != cudaSuccess) return NRC_ERROR_CUDA;
  nrc::TrainParams p = {};
  p.steps = 1;
  p.mode = nrc::kTrainStep;
  p.batch[0] = nrc::TrainBatch{d_records, d_count, capacity, d_use_weights != nullptr};
  p.batch_cap = cfg->train_batch_size;
  p.lr = cfg->learning_rate;
  p.beta1 = cfg->beta1;
  p.beta2 = cfg->beta2;
  p.eps = cfg->epsilon;
  p.ema_alpha = cfg->ema_alpha;
  p.loss_scale = cfg->loss_scale;
  p.use_ema = cfg->use_ema_weights != 0;
  p.bf16 = cfg->precision == NRC_PRECISION_BF16 ? 1 : 0;
  p.entries = d_entries;
  p.state = d_state;
  p.w16 = reinterpret_cast<__half*>(d_weights);
  p.use16 = reinterpret_cast<__half*>(d_use_weights);
  p.partials = s->scratch;
  p.sync = reinterpret_cast<uint32_t*>(s->scratch + size_t(kNoAllocSlots) * nrc::kParams) + 16;
  p.err = err;
  const cudaError_t e = nrc::launch_train(p, &wmap, max_ctas, cs);
  return e == cudaSuccess ? NRC_OK : NRC_ERROR_CUDA;
}
