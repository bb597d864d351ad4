// FP8 (E4M3) precision form of the cache query: the refresh kernel that keeps
// an E4M3 copy of the rendering weights and the per-layer scales.
//
// Scales are per layer and absmax-based: s_w[l] = max|W_l| / 448 for the
// weights, s_x[l] = max|x_l| / 448 for layer l's input activations, where
// max|x_l| is the largest value the training forward passes produced for that
// layer since the last update (the training kernel gathers it), or, for a
// layer never observed, the bound max|x_{l-1}| * max_o sum_i |W_{l-1}[o][i]|
// (max|x_0| = 1: the encoded features lie in [-1, 1] apart from the albedos).
// The scales are recomputed once per 16 optimizer steps (when the step state
// enters a new 16-step epoch) or on request; the weights are re-quantized with
// the current scales after every training launch, so the FP8 query always uses
// the latest rendering weights.
//
// Op sequence (the CPU oracle repeats it): row sums of |w| are a 32-lane
// butterfly over pairs (|w_k| + |w_{k+32}|); scales are divisions by 448; the
// quantized weight is e4m3(w * (448 / max|W_l|)), rounded to nearest even and
// saturated at 448.
#include "nrc_common.cuh"
#include "nrc_kernels.h"

namespace nrc {

namespace {

constexpr int kRefreshThreads = 1024;

__device__ __forceinline__ float dec16(uint16_t b, bool bf16) {
  return bf16 ? __bfloat162float(__ushort_as_bfloat16(b)) : __half2float(__ushort_as_half(b));
}

__global__ void __launch_bounds__(kRefreshThreads) fp8_refresh_kernel(const uint16_t* __restrict__ use16, int bf16,
                                                                      const nrc_optimizer_state* __restrict__ st,
                                                                      Fp8State* S, uint8_t* __restrict__ w8,
                                                                      int force) {
  __shared__ uint32_t amax_w[6], rowsum[6];
  __shared__ float inv_w[6];
  __shared__ int update;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  griddep_wait();  // the rendering weights of the preceding training launch
  const uint32_t epoch = st->t / 16 + 1;
  if (tid < 6) {
    amax_w[tid] = 0u;
    rowsum[tid] = 0u;
  }
  if (tid == 0) update = force || S->epoch != epoch;
  __syncthreads();
  if (update) {
    for (int row = warp; row < kWeightRows; row += kRefreshThreads / 32) {
      const int l = row < kHidden * kWidth ? row / kWidth : kHidden;
      const float a = fabsf(dec16(use16[row * kWidth + lane], bf16));
      const float b = fabsf(dec16(use16[row * kWidth + 32 + lane], bf16));
      float m = fmaxf(a, b), s = __fadd_rn(a, b);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
        s = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, off));
      }
      if (lane == 0) {  // non-negative floats order as their bit patterns
        atomicMax(&amax_w[l], __float_as_uint(m));
        atomicMax(&rowsum[l], __float_as_uint(s));
      }
    }
    __syncthreads();
    if (tid == 0) {
      float ax[6];
      for (int l = 0; l < 6; ++l) {
        const float seen = __uint_as_float(S->amax_x[l]);
        const float bound = l == 0 ? 1.0f : __fmul_rn(ax[l - 1], __uint_as_float(rowsum[l - 1]));
        ax[l] = seen > 0.0f ? seen : bound;
        if (!(ax[l] > 0.0f)) ax[l] = 1.0f;
        float aw = __uint_as_float(amax_w[l]);
        if (!(aw > 0.0f)) aw = 1.0f;  // an all-zero layer
        S->scale_w[l] = __fdiv_rn(aw, 448.0f);
        S->inv_w[l] = __fdiv_rn(448.0f, aw);
        S->scale_x[l] = __fdiv_rn(ax[l], 448.0f);
      }
      for (int l = 0; l < 5; ++l) S->c[l] = __fdiv_rn(__fmul_rn(S->scale_w[l], S->scale_x[l]), S->scale_x[l + 1]);
      S->c[5] = __fmul_rn(S->scale_w[5], S->scale_x[5]);
      S->inv_sx0 = __fdiv_rn(1.0f, S->scale_x[0]);
      for (int l = 0; l < 6; ++l) S->amax_x[l] = 0u;
      S->epoch = epoch;
    }
  }
  __syncthreads();
  if (tid < 6) inv_w[tid] = S->inv_w[tid];
  __syncthreads();
  // four weights of one row per thread and step; bytes 64..127 of a row stay zero
  for (int q = tid; q < kWeightRows * 16; q += kRefreshThreads) {
    const int row = q >> 4, k = (q & 15) * 4;
    const int l = row < kHidden * kWidth ? row / kWidth : kHidden;
    const uint16_t* src = use16 + row * kWidth + k;
    const float iw = inv_w[l];
    const uint32_t v = pack4_e4m3(__fmul_rn(dec16(src[0], bf16), iw), __fmul_rn(dec16(src[1], bf16), iw),
                                  __fmul_rn(dec16(src[2], bf16), iw), __fmul_rn(dec16(src[3], bf16), iw));
    *reinterpret_cast<uint32_t*>(w8 + row * 128 + k) = v;
  }
}

}  // namespace

cudaError_t launch_fp8_refresh(const uint16_t* use16, bool bf16, const nrc_optimizer_state* st, Fp8State* fp8,
                               uint8_t* w8, int force, cudaStream_t stream) {
  fp8_refresh_kernel<<<1, kRefreshThreads, 0, stream>>>(use16, bf16 ? 1 : 0, st, fp8, w8, force);
  return cudaGetLastError();
}

}  // namespace nrc
