// Screen pass: shader/src/screen.frag:10-31 as a CUDA kernel over a headless
// image. The reference draws a full-screen triangle whose fragment shader reads
// the composited color (the rgba32f image the query epilogue wrote,
// nrc_inference.comp:52-58), optionally keeps a running average in the
// accumulation image, tone-maps it (ToneMapFilmic_Hejl2015, white point 3.2),
// applies gamma 1/2.2 and writes the swapchain. Here the result goes to device
// buffers: UNORM8 rgba and/or float rgba.
//
// Op sequence (the CPU oracle repeats it): each `a * b + c` of the shader is one
// fused multiply-add, `color += acc * count` too; pow() of the tone curve's
// small negative values near black (undefined in GLSL) takes a base clamped to
// zero; UNORM8 = round-to-nearest-even of clamp(x, 0, 1) * 255.
#include "nrc_common.cuh"
#include "nrc_kernels.h"

namespace nrc {

namespace {

__device__ __forceinline__ float hejl_curve(float x) {
  const float va = __fmaf_rn(1.425f, x, 0.05f);
  return __fsub_rn(__fdiv_rn(__fmaf_rn(x, va, 0.004f), __fmaf_rn(x, __fadd_rn(va, 0.55f), 0.0491f)), 0.0821f);
}

__global__ void screen_kernel(const float4* __restrict__ color, float4* __restrict__ accum, uint32_t n, int acc_on,
                              uint32_t acc_count, uchar4* __restrict__ out8, float4* __restrict__ outf) {
  const float wf = hejl_curve(3.2f);
  const float k = static_cast<float>(acc_count), k1 = static_cast<float>(acc_count + 1u);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 c4 = color[i];
    float c[3] = {c4.x, c4.y, c4.z};
    if (acc_on) {
      if (acc_count != 0) {
        const float4 a = accum[i];
        c[0] = __fdiv_rn(__fmaf_rn(a.x, k, c[0]), k1);
        c[1] = __fdiv_rn(__fmaf_rn(a.y, k, c[1]), k1);
        c[2] = __fdiv_rn(__fmaf_rn(a.z, k, c[2]), k1);
      }
      accum[i] = make_float4(c[0], c[1], c[2], 0.0f);
    }
    float s[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) s[j] = powf(fmaxf(__fdiv_rn(hejl_curve(c[j]), wf), 0.0f), 1.0f / 2.2f);
    if (outf != nullptr) outf[i] = make_float4(s[0], s[1], s[2], 1.0f);
    if (out8 != nullptr)
      out8[i] = make_uchar4(static_cast<unsigned char>(__float2uint_rn(__saturatef(s[0]) * 255.0f)),
                            static_cast<unsigned char>(__float2uint_rn(__saturatef(s[1]) * 255.0f)),
                            static_cast<unsigned char>(__float2uint_rn(__saturatef(s[2]) * 255.0f)), 255);
  }
}

}  // namespace

cudaError_t launch_screen(const float* color, float* accum, uint32_t width, uint32_t height, int acc_on,
                          uint32_t acc_count, uint8_t* out8, float* outf, int num_sms, cudaStream_t stream) {
  const uint32_t n = width * height;
  if (n == 0) return cudaSuccess;
  const uint32_t want = (n + 255) / 256;
  const uint32_t grid = want < static_cast<uint32_t>(num_sms) * 8 ? want : static_cast<uint32_t>(num_sms) * 8;
  screen_kernel<<<grid, 256, 0, stream>>>(reinterpret_cast<const float4*>(color), reinterpret_cast<float4*>(accum), n,
                                          acc_on, acc_count, reinterpret_cast<uchar4*>(out8),
                                          reinterpret_cast<float4*>(outf));
  return cudaGetLastError();
}

}  // namespace nrc
