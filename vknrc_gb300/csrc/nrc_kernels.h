// Kernel launchers shared between the kernel translation units and the C ABI.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/nrc.h"

namespace nrc {

cudaError_t configure_infer_kernels();
cudaError_t configure_train_kernels();
uint32_t infer_smem_bytes();
int infer_threads();
int infer_tiles_per_cta();
cudaError_t launch_infer(const void* input, bool encoded, const uint32_t* d_count, uint32_t capacity,
                         const __half* w16, float* out, bool clamp_out, uint32_t* err, int num_sms,
                         cudaStream_t stream);

uint32_t train_smem_bytes();
uint32_t train_grid(uint32_t capacity, uint32_t batch_cap, int num_sms);
cudaError_t launch_train_grad(const nrc_train_record* records, uint32_t* d_count, uint32_t capacity,
                              uint32_t batch_cap, const __half* w16, float* grad, float* partials,
                              nrc_optimizer_state* state, float loss_scale, float beta1, float beta2,
                              float ema_alpha, bool do_prepare, double* loss_acc, unsigned long long* loss_count,
                              uint32_t* err, int num_sms, cudaStream_t stream);
cudaError_t launch_adam(const uint32_t* d_count, uint32_t capacity, uint32_t batch_cap, float* grad,
                        const float* partials, uint32_t grad_ctas, nrc_optimizer_entry* entries,
                        const nrc_optimizer_state* state, __half* w16, __half* use16, float lr, float beta1,
                        float beta2, float eps, float ema_alpha, float loss_scale, bool use_ema,
                        cudaStream_t stream);

cudaError_t launch_encode(const nrc_input* in, const uint32_t* d_count, uint32_t capacity, uint16_t* out,
                          int num_sms, cudaStream_t stream);
cudaError_t launch_sph_encode(const float* dirs, const uint32_t* d_count, uint32_t capacity, float* out,
                              int num_sms, cudaStream_t stream);
cudaError_t launch_fill_f32(float* p, float v, size_t n, cudaStream_t stream);

}  // namespace nrc
