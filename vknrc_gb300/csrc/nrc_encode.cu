// Stand-alone encoding kernels: NRCInputEncode (shader/src/NRCRecord.glsl:78-95)
// to 64 fp16 features per record, and NRCSphEncode (NRCRecord.glsl:47-49).
#include "nrc_common.cuh"
#include "nrc_kernels.h"

namespace nrc {

namespace {

__global__ void __launch_bounds__(256) encode_kernel(const nrc_input* __restrict__ in, const uint32_t* __restrict__ d_count,
                                                     uint32_t capacity, uint4* __restrict__ out) {
  const uint32_t n = min(*d_count, capacity);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2* src = reinterpret_cast<const float2*>(in + i);
    float r[kInFloats];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const float2 v = src[k];
      r[2 * k] = v.x;
      r[2 * k + 1] = v.y;
    }
    uint32_t e[32];
    encode_input(r, e);
    uint4* dst = out + static_cast<size_t>(i) * 8;
#pragma unroll
    for (int c = 0; c < 8; ++c) dst[c] = make_uint4(e[4 * c], e[4 * c + 1], e[4 * c + 2], e[4 * c + 3]);
  }
}

__global__ void __launch_bounds__(256) sph_kernel(const float* __restrict__ dirs, const uint32_t* __restrict__ d_count,
                                                  uint32_t capacity, float2* __restrict__ out) {
  const uint32_t n = min(*d_count, capacity);
  const float pi = 3.14159265358979323846f;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float x = dirs[3 * i], y = dirs[3 * i + 1], z = dirs[3 * i + 2];
    const float u = (x == 0.0f && y == 0.0f) ? 0.5f : 0.5f + atan2f(y, x) / (2.0f * pi);
    const float v = acosf(fminf(fmaxf(z, -1.0f), 1.0f)) / pi;
    out[i] = make_float2(u, v);
  }
}

__global__ void fill_kernel(float* __restrict__ p, float v, size_t n) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    p[i] = v;
}

uint32_t grid_for(uint32_t capacity, int num_sms) {
  const uint32_t want = (capacity + 255) / 256;
  const uint32_t cap = static_cast<uint32_t>(num_sms) * 8;
  return want < cap ? want : cap;
}

}  // namespace

cudaError_t launch_encode(const nrc_input* in, const uint32_t* d_count, uint32_t capacity, uint16_t* out,
                          int num_sms, cudaStream_t stream) {
  const uint32_t grid = grid_for(capacity, num_sms);
  if (grid == 0) return cudaSuccess;
  encode_kernel<<<grid, 256, 0, stream>>>(in, d_count, capacity, reinterpret_cast<uint4*>(out));
  return cudaGetLastError();
}

cudaError_t launch_sph_encode(const float* dirs, const uint32_t* d_count, uint32_t capacity, float* out,
                              int num_sms, cudaStream_t stream) {
  const uint32_t grid = grid_for(capacity, num_sms);
  if (grid == 0) return cudaSuccess;
  sph_kernel<<<grid, 256, 0, stream>>>(dirs, d_count, capacity, reinterpret_cast<float2*>(out));
  return cudaGetLastError();
}

cudaError_t launch_fill_f32(float* p, float v, size_t n, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  size_t blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  fill_kernel<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(p, v, n);
  return cudaGetLastError();
}

}  // namespace nrc
