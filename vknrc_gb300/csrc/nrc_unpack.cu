// Scene unpack kernel: UnpackNRCInput (shader/src/NRCRecord.glsl:97-125) of
// eval records (nrc_inference.comp:33-36) and train records
// (nrc_gradient.comp:29-33) into nrc_input / nrc_train_record arrays; the
// per-record arithmetic is in nrc_unpack.cuh.
#include <cmath>

#include "nrc_common.cuh"
#include "nrc_kernels.h"
#include "nrc_unpack.cuh"

namespace nrc {

namespace {

struct UnpackParams {
  nrc_scene scene;
  SrgbLut lut;
};

// Train records of up to NRC_TRAIN_BATCH_COUNT batches in one launch
// (blockIdx.y = batch).
struct UnpackBatches {
  const nrc_packed_train_record* in[NRC_TRAIN_BATCH_COUNT];
  const uint32_t* count[NRC_TRAIN_BATCH_COUNT];
  nrc_train_record* out[NRC_TRAIN_BATCH_COUNT];
};

__device__ __forceinline__ void write_train(nrc_train_record* dst, const nrc_packed_train_record& rec,
                                            const float (&r)[kInFloats]) {
  float4* o = reinterpret_cast<float4*>(dst);
  o[0] = make_float4(rec.bias[0], rec.bias[1], rec.bias[2], rec.factor[0]);
  o[1] = make_float4(rec.factor[1], rec.factor[2], r[0], r[1]);
  o[2] = make_float4(r[2], r[3], r[4], r[5]);
  o[3] = make_float4(r[6], r[7], r[8], r[9]);
  o[4] = make_float4(r[10], r[11], r[12], r[13]);
}

__global__ void __launch_bounds__(256, 4) unpack_batches_kernel(const __grid_constant__ UnpackParams P,
                                                              const __grid_constant__ UnpackBatches U,
                                                              uint32_t capacity) {
  __shared__ float lut[256];
  lut[threadIdx.x] = P.lut.v[threadIdx.x];
  __syncthreads();
  const uint32_t bt = blockIdx.y;
  const uint32_t n = min(*U.count[bt], capacity);
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += 2 * stride) {
    const size_t j = i + stride;
    const bool two = j < n;
    const nrc_packed_train_record a = U.in[bt][i], b = U.in[bt][two ? j : i];
    float ra[kInFloats], rb[kInFloats];
    unpack_one(P.scene, a.input, lut, ra);
    unpack_one(P.scene, b.input, lut, rb);
    write_train(U.out[bt] + i, a, ra);
    if (two) write_train(U.out[bt] + j, b, rb);
  }
}

// One thread per two records (i and i + stride of the grid-stride loop), so
// that the dependent gathers of two records are in flight at once.
template <bool kTrain>
__global__ void __launch_bounds__(256, 4) unpack_kernel(const __grid_constant__ UnpackParams P, const void* __restrict__ in,
                                                      const uint32_t* __restrict__ d_count, uint32_t capacity,
                                                      void* __restrict__ out, uint32_t* __restrict__ out_dst) {
  __shared__ float lut[256];
  lut[threadIdx.x] = P.lut.v[threadIdx.x];
  __syncthreads();
  const uint32_t n = min(*d_count, capacity);
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += 2 * stride) {
    const size_t j = i + stride;
    const bool two = j < n;
    float ra[kInFloats], rb[kInFloats];
    if (kTrain) {
      const nrc_packed_train_record* rec = static_cast<const nrc_packed_train_record*>(in);
      const nrc_packed_train_record a = rec[i], b = rec[two ? j : i];
      unpack_one(P.scene, a.input, lut, ra);
      unpack_one(P.scene, b.input, lut, rb);
      write_train(static_cast<nrc_train_record*>(out) + i, a, ra);
      if (two) write_train(static_cast<nrc_train_record*>(out) + j, b, rb);
    } else {
      const nrc_eval_record* rec = static_cast<const nrc_eval_record*>(in);
      const nrc_eval_record a = rec[i], b = rec[two ? j : i];
      unpack_one(P.scene, a.input, lut, ra);
      unpack_one(P.scene, b.input, lut, rb);
      float2* oa = reinterpret_cast<float2*>(static_cast<nrc_input*>(out) + i);
#pragma unroll
      for (int k = 0; k < 7; ++k) oa[k] = make_float2(ra[2 * k], ra[2 * k + 1]);
      if (out_dst != nullptr) out_dst[i] = a.dst;
      if (two) {
        float2* ob = reinterpret_cast<float2*>(static_cast<nrc_input*>(out) + j);
#pragma unroll
        for (int k = 0; k < 7; ++k) ob[k] = make_float2(rb[2 * k], rb[2 * k + 1]);
        if (out_dst != nullptr) out_dst[j] = b.dst;
      }
    }
  }
}

}  // namespace

// sRGB -> linear of the 256 byte values, in double, rounded once.
const SrgbLut& srgb_lut() {
  static const SrgbLut lut = [] {
    SrgbLut l;
    for (int i = 0; i < 256; ++i) {
      const double c = i / 255.0;
      l.v[i] = static_cast<float>(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
    return l;
  }();
  return lut;
}


cudaError_t launch_unpack(const nrc_scene& scene, bool train, const void* in, const uint32_t* d_count,
                          uint32_t capacity, void* out, uint32_t* out_dst, int num_sms, cudaStream_t stream) {
  const uint32_t want = (capacity + 255) / 256;
  const uint32_t cap = static_cast<uint32_t>(num_sms) * 4;  // the resident blocks (4 per SM)
  const uint32_t grid = want < cap ? want : cap;
  if (grid == 0) return cudaSuccess;
  UnpackParams p;
  p.scene = scene;
  p.lut = srgb_lut();
  if (train)
    unpack_kernel<true><<<grid, 256, 0, stream>>>(p, in, d_count, capacity, out, nullptr);
  else
    unpack_kernel<false><<<grid, 256, 0, stream>>>(p, in, d_count, capacity, out, out_dst);
  return cudaGetLastError();
}

cudaError_t launch_unpack_train_batches(const nrc_scene& scene, const nrc_packed_train_record* const* in,
                                       uint32_t* const* counts, uint32_t capacity, nrc_train_record* const* out,
                                       int nbatches, int num_sms, cudaStream_t stream) {
  if (nbatches < 1 || nbatches > NRC_TRAIN_BATCH_COUNT) return cudaErrorInvalidValue;
  const uint32_t want = (capacity + 255) / 256;
  const uint32_t cap = static_cast<uint32_t>(num_sms) * 2;
  const uint32_t gx = want < cap ? want : cap;
  if (gx == 0) return cudaSuccess;
  UnpackParams p;
  p.scene = scene;
  p.lut = srgb_lut();
  UnpackBatches u = {};
  for (int b = 0; b < nbatches; ++b) {
    u.in[b] = in[b];
    u.count[b] = counts[b];
    u.out[b] = out[b];
  }
  unpack_batches_kernel<<<dim3(gx, static_cast<uint32_t>(nbatches)), 256, 0, stream>>>(p, u, capacity);
  return cudaGetLastError();
}

}  // namespace nrc
