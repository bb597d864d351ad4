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
  SceneRows rows;  // prepared tables, or {nullptr, nullptr}: gather from the scene buffers
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

template <bool kRows>
__global__ void __launch_bounds__(256, 4) unpack_batches_kernel(const __grid_constant__ UnpackParams P,
                                                              const __grid_constant__ UnpackBatches U,
                                                              uint32_t capacity) {
  __shared__ float lut_smem[256];
  const float* lut = stage_lut(lut_smem, P.lut);
  const uint32_t bt = blockIdx.y;
  const uint32_t n = min(*U.count[bt], capacity);
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += 2 * stride) {
    const size_t j = i + stride;
    const bool two = j < n;
    const nrc_packed_train_record a = U.in[bt][i], b = U.in[bt][two ? j : i];
    float ra[kInFloats], rb[kInFloats];
    unpack_one<kRows>(P.scene, P.rows, a.input, lut, ra);
    unpack_one<kRows>(P.scene, P.rows, b.input, lut, rb);
    write_train(U.out[bt] + i, a, ra);
    if (two) write_train(U.out[bt] + j, b, rb);
  }
}

// One thread per two records (i and i + stride of the grid-stride loop), so
// that the dependent gathers of two records are in flight at once.
template <bool kTrain, bool kRows>
__global__ void __launch_bounds__(256, 4) unpack_kernel(const __grid_constant__ UnpackParams P, const void* __restrict__ in,
                                                      const uint32_t* __restrict__ d_count, uint32_t capacity,
                                                      void* __restrict__ out, uint32_t* __restrict__ out_dst) {
  __shared__ float lut_smem[256];
  const float* lut = stage_lut(lut_smem, P.lut);
  const uint32_t n = min(*d_count, capacity);
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += 2 * stride) {
    const size_t j = i + stride;
    const bool two = j < n;
    float ra[kInFloats], rb[kInFloats];
    if (kTrain) {
      const nrc_packed_train_record* rec = static_cast<const nrc_packed_train_record*>(in);
      const nrc_packed_train_record a = rec[i], b = rec[two ? j : i];
      unpack_one<kRows>(P.scene, P.rows, a.input, lut, ra);
      unpack_one<kRows>(P.scene, P.rows, b.input, lut, rb);
      write_train(static_cast<nrc_train_record*>(out) + i, a, ra);
      if (two) write_train(static_cast<nrc_train_record*>(out) + j, b, rb);
    } else {
      const nrc_eval_record* rec = static_cast<const nrc_eval_record*>(in);
      const nrc_eval_record a = rec[i], b = rec[two ? j : i];
      unpack_one<kRows>(P.scene, P.rows, a.input, lut, ra);
      unpack_one<kRows>(P.scene, P.rows, b.input, lut, rb);
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

// nrc_scene_prepare, primitive rows: the gathers of Scene.glsl:50-58 done once
// per primitive (vertices and texcoords copied bit for bit).
__global__ void __launch_bounds__(256) prepare_prims_kernel(const nrc_scene S, uint4* __restrict__ rows) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= S.primitive_count) return;
  uint32_t vi[3], ti[3];
  bool ok = S.material_ids[p] < S.material_count;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vi[k] = S.vertex_indices[size_t(p) * 3 + k];
    ti[k] = S.texcoord_indices[size_t(p) * 3 + k];
    ok = ok && vi[k] < S.vertex_count && ti[k] < S.texcoord_count;
  }
  uint32_t w[16] = {};
  if (ok) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float* v = S.vertices + size_t(vi[k]) * 3;
      w[4 * k] = __float_as_uint(v[0]);
      w[4 * k + 1] = __float_as_uint(v[1]);
      w[4 * k + 2] = __float_as_uint(v[2]);
    }
    const float2* tc = reinterpret_cast<const float2*>(S.texcoords);
    const float2 t0 = tc[ti[0]], t1 = tc[ti[1]], t2 = tc[ti[2]];
    w[3] = __float_as_uint(t0.x);
    w[7] = __float_as_uint(t0.y);
    w[11] = __float_as_uint(t1.x);
    w[12] = __float_as_uint(t1.y);
    w[13] = __float_as_uint(t2.x);
    w[14] = __float_as_uint(t2.y);
    w[15] = S.material_ids[p];
  } else {
    w[15] = kInvalidRow;
  }
  uint4* o = rows + size_t(p) * 4;
#pragma unroll
  for (int q = 0; q < 4; ++q) o[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
}

// nrc_scene_prepare, material rows: colours, roughness and the texture
// descriptors of GetSceneDiffuse / GetSceneSpecular (Scene.glsl:64-69) inline.
__global__ void __launch_bounds__(256) prepare_mats_kernel(const nrc_scene S, uint4* __restrict__ rows) {
  const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= S.material_count) return;
  const uint4* m4 = reinterpret_cast<const uint4*>(S.materials + m);
  const uint4 md = m4[0], ms = m4[1], mr = m4[3];
  const uint32_t ids[2] = {md.w, ms.w};
  uint4 tex[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
  uint32_t flags = 0;
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    if (ids[c] != 0xFFFFFFFFu && ids[c] < S.texture_count) {
      const nrc_texture t = S.textures[ids[c]];
      const uint64_t a = reinterpret_cast<uint64_t>(t.texels);
      tex[c] = make_uint4(static_cast<uint32_t>(a), static_cast<uint32_t>(a >> 32), t.width, t.height);
      flags |= 1u << c;
    }
  }
  uint4* o = rows + size_t(m) * 4;
  o[0] = make_uint4(md.x, md.y, md.z, mr.y);
  o[1] = make_uint4(ms.x, ms.y, ms.z, flags);
  o[2] = tex[0];
  o[3] = tex[1];
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


cudaError_t launch_scene_prepare(const nrc_scene& scene, void* prim_rows, void* mat_rows, cudaStream_t stream) {
  if (scene.primitive_count > 0)
    prepare_prims_kernel<<<(scene.primitive_count + 255) / 256, 256, 0, stream>>>(scene, static_cast<uint4*>(prim_rows));
  if (scene.material_count > 0)
    prepare_mats_kernel<<<(scene.material_count + 255) / 256, 256, 0, stream>>>(scene, static_cast<uint4*>(mat_rows));
  return cudaGetLastError();
}

cudaError_t launch_unpack(const nrc_scene& scene, const void* prim_rows, const void* mat_rows, bool train,
                          const void* in, const uint32_t* d_count, uint32_t capacity, void* out, uint32_t* out_dst,
                          int num_sms, cudaStream_t stream) {
  const uint32_t want = (capacity + 255) / 256;
  const uint32_t cap = static_cast<uint32_t>(num_sms) * 4;  // the resident blocks (4 per SM)
  const uint32_t grid = want < cap ? want : cap;
  if (grid == 0) return cudaSuccess;
  UnpackParams p;
  p.scene = scene;
  p.rows = SceneRows{static_cast<const uint4*>(prim_rows), static_cast<const uint4*>(mat_rows)};
  p.lut = srgb_lut();
  const bool rows = prim_rows != nullptr;
  if (train && rows)
    unpack_kernel<true, true><<<grid, 256, 0, stream>>>(p, in, d_count, capacity, out, nullptr);
  else if (train)
    unpack_kernel<true, false><<<grid, 256, 0, stream>>>(p, in, d_count, capacity, out, nullptr);
  else if (rows)
    unpack_kernel<false, true><<<grid, 256, 0, stream>>>(p, in, d_count, capacity, out, out_dst);
  else
    unpack_kernel<false, false><<<grid, 256, 0, stream>>>(p, in, d_count, capacity, out, out_dst);
  return cudaGetLastError();
}

cudaError_t launch_unpack_train_batches(const nrc_scene& scene, const void* prim_rows, const void* mat_rows,
                                       const nrc_packed_train_record* const* in,
                                       uint32_t* const* counts, uint32_t capacity, nrc_train_record* const* out,
                                       int nbatches, int num_sms, cudaStream_t stream) {
  if (nbatches < 1 || nbatches > NRC_TRAIN_BATCH_COUNT) return cudaErrorInvalidValue;
  const uint32_t want = (capacity + 255) / 256;
  const uint32_t cap = static_cast<uint32_t>(num_sms) * 2;
  const uint32_t gx = want < cap ? want : cap;
  if (gx == 0) return cudaSuccess;
  UnpackParams p;
  p.scene = scene;
  p.rows = SceneRows{static_cast<const uint4*>(prim_rows), static_cast<const uint4*>(mat_rows)};
  p.lut = srgb_lut();
  UnpackBatches u = {};
  for (int b = 0; b < nbatches; ++b) {
    u.in[b] = in[b];
    u.count[b] = counts[b];
    u.out[b] = out[b];
  }
  const dim3 grid(gx, static_cast<uint32_t>(nbatches));
  if (prim_rows != nullptr)
    unpack_batches_kernel<true><<<grid, 256, 0, stream>>>(p, u, capacity);
  else
    unpack_batches_kernel<false><<<grid, 256, 0, stream>>>(p, u, capacity);
  return cudaGetLastError();
}

}  // namespace nrc
