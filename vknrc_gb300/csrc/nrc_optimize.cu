// The reference's prepare and optimizer passes as separate launches over a
// gradient sum the caller supplies, and the relative-L2 loss gradient rows on
// their own. The fused trainer runs the same device functions
// (nrc_train_math.cuh) inside its launch; these entry points let a caller that
// computes gradients elsewhere keep the reference's pass structure
// (src/rg/NNTrain.hpp:95-118: prepare -> gradient -> optimizer), and let the
// update and the loss rows be checked against the reference's compiled shaders.
#include "nrc_common.cuh"
#include "nrc_kernels.h"
#include "nrc_train_math.cuh"

namespace nrc {

namespace {

// nrc_train_prepare.comp:16-29 in one thread: clamp the count (written back),
// advance the step state only when records remain.
__global__ void prepare_kernel(uint32_t* __restrict__ d_count, uint32_t batch_cap, nrc_optimizer_state* state,
                               float beta1, float beta2, float ema_alpha) {
  const uint32_t n = min(*d_count, batch_cap);
  *d_count = n;
  if (n > 0) {
    nrc_optimizer_state st = *state;
    st.t += 1;
    st.beta1_t *= beta1;
    st.beta2_t *= beta2;
    st.alpha_t_1 = st.alpha_t;
    st.alpha_t *= ema_alpha;
    *state = st;
  }
}

// nrc_optimize.comp:32-54, one thread per parameter, reading the prepared state
// and count; nothing is written when the count is zero (the shader returns).
template <bool kBF16>
__global__ void __launch_bounds__(256) optimize_kernel(const float* __restrict__ grad, const uint32_t* __restrict__ d_count,
                                                       const nrc_optimizer_state* __restrict__ state, AdamHyper hp,
                                                       nrc_optimizer_entry* __restrict__ entries,
                                                       uint16_t* __restrict__ w16, uint16_t* __restrict__ use16) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const uint32_t n = *d_count;
  if (n == 0) return;
  const nrc_optimizer_state st = *state;
  nrc_optimizer_entry e = entries[i];
  adam_one<kBF16>(i, grad[i], n, st, hp, e, entries, w16, use16);
}

template <bool kBF16>
__global__ void loss_rows_kernel(const float* __restrict__ pred, const float* __restrict__ target,
                                 const uint32_t* __restrict__ d_count, uint32_t capacity, float loss_scale,
                                 uint32_t* __restrict__ rows) {
  const uint32_t n = min(*d_count, capacity);
  for (size_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const float t[3] = {target[3 * k], target[3 * k + 1], target[3 * k + 2]};
    float d[3];
    rel_l2_grad(pred[3 * k], pred[3 * k + 1], pred[3 * k + 2], t, loss_scale, d);
    uint32_t w[2];
    loss_row<kBF16>(d, w);
    rows[2 * k] = w[0];
    rows[2 * k + 1] = w[1];
  }
}

}  // namespace

cudaError_t launch_optimize(const TrainParams& p, const float* grad_sum, uint32_t* d_count, bool write_use,
                            cudaStream_t stream) {
  prepare_kernel<<<1, 1, 0, stream>>>(d_count, p.batch_cap, p.state, p.beta1, p.beta2, p.ema_alpha);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const AdamHyper hp{p.lr, p.beta1, p.beta2, p.eps, p.ema_alpha, p.loss_scale, p.use_ema};
  uint16_t* w16 = reinterpret_cast<uint16_t*>(p.w16);
  uint16_t* use16 = write_use ? reinterpret_cast<uint16_t*>(p.use16) : nullptr;
  const int blocks = (kParams + 255) / 256;
  if (p.bf16)
    optimize_kernel<true><<<blocks, 256, 0, stream>>>(grad_sum, d_count, p.state, hp, p.entries, w16, use16);
  else
    optimize_kernel<false><<<blocks, 256, 0, stream>>>(grad_sum, d_count, p.state, hp, p.entries, w16, use16);
  return cudaGetLastError();
}

cudaError_t launch_loss_rows(const float* pred, const float* target, const uint32_t* d_count, uint32_t capacity,
                             float loss_scale, bool bf16, uint32_t* rows, int num_sms, cudaStream_t stream) {
  if (capacity == 0) return cudaSuccess;
  const uint32_t want = (capacity + 255) / 256, cap = static_cast<uint32_t>(num_sms) * 8;
  const uint32_t blocks = want < cap ? want : cap;
  if (bf16)
    loss_rows_kernel<true><<<blocks, 256, 0, stream>>>(pred, target, d_count, capacity, loss_scale, rows);
  else
    loss_rows_kernel<false><<<blocks, 256, 0, stream>>>(pred, target, d_count, capacity, loss_scale, rows);
  return cudaGetLastError();
}

}  // namespace nrc
