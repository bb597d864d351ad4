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

constexpr int kUnpackThreads = 256, kUnpackBlocksPerSM = 3;

// Output floats per record: nrc_input, or nrc_train_record (bias, factor, input).
template <bool kTrain>
constexpr int kOutFloats = kTrain ? 20 : kInFloats;

// Stores the records of one warp (lane l's in v, for record out + l) through
// the warp's staging area in shared memory, so that each store instruction
// writes 256 contiguous bytes instead of 32 records' scattered words; `valid`
// of the warp's records are written. Warp-wide.
template <int kF>
__device__ __forceinline__ void warp_store(float2* __restrict__ stage, const float (&v)[kF], float* __restrict__ out,
                                           uint32_t valid) {
  static_assert(kF % 2 == 0, "records of whole float pairs");
  const uint32_t lane = threadIdx.x & 31u;
  __syncwarp();
#pragma unroll
  for (int k = 0; k < kF / 2; ++k) stage[lane * (kF / 2) + k] = make_float2(v[2 * k], v[2 * k + 1]);
  __syncwarp();
  float2* o = reinterpret_cast<float2*>(out);
  const uint32_t words = valid * (kF / 2);
#pragma unroll
  for (uint32_t w = lane; w < 32u * (kF / 2); w += 32u)
    if (w < words) o[w] = stage[w];
}

template <bool kTrain>
__device__ __forceinline__ const nrc_packed_input& packed_input(const void* __restrict__ in, size_t i) {
  if constexpr (kTrain)
    return static_cast<const nrc_packed_train_record*>(in)[i].input;
  else
    return static_cast<const nrc_eval_record*>(in)[i].input;
}

// The unpacked record of `in` entry i as output floats (a train record keeps its bias and factor).
template <bool kTrain>
__device__ __forceinline__ void out_floats(const void* in, size_t i, const float (&r)[kInFloats],
                                           float (&o)[kOutFloats<kTrain>]) {
  int k0 = 0;
  if constexpr (kTrain) {
    const nrc_packed_train_record& t = static_cast<const nrc_packed_train_record*>(in)[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      o[k] = t.bias[k];
      o[3 + k] = t.factor[k];
    }
    k0 = 6;
  }
#pragma unroll
  for (int k = 0; k < kInFloats; ++k) o[k0 + k] = r[k];
}

// Shared memory per warp, in 16-byte words: the primitive rows of 32 records
// (warp_rows_share, 2 KB), reused for the 32 output records (warp_store).
template <bool kTrain>
constexpr int kStageU4 = (32 * kOutFloats<kTrain> / 4) > 128 ? (32 * kOutFloats<kTrain> / 4) : 128;

// Unpacks records [0, n) of `in` into `out` (nrc_input or nrc_train_record
// array; eval destination words into out_dst when given). Each warp takes 32
// consecutive records and the 32 at `stride` past them (two records per
// thread, so the dependent gathers of both are in flight at once); whole warps
// iterate together, lanes past n unpack a duplicate that is not stored.
// kRows: the scene's gather tables, primitive rows loaded by the warp together.
template <bool kTrain, bool kRows>
__device__ __forceinline__ void unpack_range(const UnpackParams& P, const void* __restrict__ in, uint32_t n,
                                             float* __restrict__ out, uint32_t* __restrict__ out_dst,
                                             uint4* __restrict__ stage, const float* lut, size_t first,
                                             size_t stride) {
  constexpr int F = kOutFloats<kTrain>;
  const uint32_t lane = threadIdx.x & 31u;
  const bool empty = scene_empty(P.scene);  // the same for every thread
  for (size_t b0 = first; b0 < n; b0 += 2 * stride) {
    const size_t b1 = b0 + stride;  // warp-uniform
    const size_t i = b0 + lane < n ? b0 + lane : b0, j = b1 + lane < n ? b1 + lane : b0;
    const nrc_packed_input pi = packed_input<kTrain>(in, i), pj = packed_input<kTrain>(in, j);
    float ri[kInFloats], rj[kInFloats];
    if constexpr (kRows) {
      if (empty) {
#pragma unroll
        for (int k = 0; k < kInFloats; ++k) ri[k] = rj[k] = 0.0f;
      } else {
        const RecordRef fi = record_ref(P.scene, pi), fj = record_ref(P.scene, pj);
        uint4 vi[4], vj[4], q[4];
        warp_rows_load(P.rows.prims, fi.prim, vi);
        warp_rows_load(P.rows.prims, fj.prim, vj);
        Gathered g;
        warp_rows_share(vi, stage, q);
        gather_row(q, P.rows.mats, fi.ok, g);
        finish_unpack<true>(P.scene, pi, fi, g, lut, ri);
        warp_rows_share(vj, stage, q);
        gather_row(q, P.rows.mats, fj.ok, g);
        finish_unpack<true>(P.scene, pj, fj, g, lut, rj);
      }
    } else {
      unpack_one(P.scene, pi, lut, ri);
      unpack_one(P.scene, pj, lut, rj);
    }
    float2* st = reinterpret_cast<float2*>(stage);
    float o[F];
    out_floats<kTrain>(in, i, ri, o);
    warp_store<F>(st, o, out + b0 * F, static_cast<uint32_t>(n - b0 < 32 ? n - b0 : 32));
    if (b1 < n) {
      out_floats<kTrain>(in, j, rj, o);
      warp_store<F>(st, o, out + b1 * F, static_cast<uint32_t>(n - b1 < 32 ? n - b1 : 32));
    }
    if constexpr (!kTrain) {
      if (out_dst != nullptr) {
        const nrc_eval_record* rec = static_cast<const nrc_eval_record*>(in);
        if (b0 + lane < n) out_dst[i] = rec[i].dst;
        if (b1 + lane < n) out_dst[j] = rec[j].dst;
      }
    }
  }
}

template <bool kRows>
__global__ void __launch_bounds__(kUnpackThreads, kUnpackBlocksPerSM)
    unpack_batches_kernel(const __grid_constant__ UnpackParams P, const __grid_constant__ UnpackBatches U,
                          uint32_t capacity) {
  __shared__ float lut_smem[256 * kLutCopies];
  __shared__ uint4 stage_smem[kUnpackThreads / 32 * kStageU4<true>];
  const float* lut = stage_lut(lut_smem, P.lut);
  const uint32_t bt = blockIdx.y;
  const uint32_t n = min(*U.count[bt], capacity);
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  unpack_range<true, kRows>(P, U.in[bt], n, reinterpret_cast<float*>(U.out[bt]), nullptr,
                            stage_smem + (threadIdx.x >> 5) * kStageU4<true>, lut,
                            static_cast<size_t>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u), stride);
}

template <bool kTrain, bool kRows>
__global__ void __launch_bounds__(kUnpackThreads, kUnpackBlocksPerSM)
    unpack_kernel(const __grid_constant__ UnpackParams P, const void* __restrict__ in,
                  const uint32_t* __restrict__ d_count, uint32_t capacity, void* __restrict__ out,
                  uint32_t* __restrict__ out_dst) {
  __shared__ float lut_smem[256 * kLutCopies];
  __shared__ uint4 stage_smem[kUnpackThreads / 32 * kStageU4<kTrain>];
  const float* lut = stage_lut(lut_smem, P.lut);
  const uint32_t n = min(*d_count, capacity);
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  unpack_range<kTrain, kRows>(P, in, n, static_cast<float*>(out), out_dst,
                              stage_smem + (threadIdx.x >> 5) * kStageU4<kTrain>, lut,
                              static_cast<size_t>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u), stride);
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
// descriptors of GetSceneDiffuse / GetSceneSpecular (Scene.glsl:64-69) inline,
// pointing at the textures' footprint arrays (`footprints`: one descriptor per
// scene texture, its texels field the footprint array).
__global__ void __launch_bounds__(256) prepare_mats_kernel(const nrc_scene S, const nrc_texture* __restrict__ footprints,
                                                          uint4* __restrict__ rows) {
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
      const nrc_texture t = footprints[ids[c]];
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

// nrc_scene_prepare, one texture's footprint array: entry (j, i) = texels
// (i, j), (i + 1, j), (i, j + 1), (i + 1, j + 1), neighbours wrapped (REPEAT).
__global__ void __launch_bounds__(256) footprints_kernel(const uint32_t* __restrict__ texels, uint32_t w, uint32_t h,
                                                        uint4* __restrict__ out) {
  const size_t n = size_t(w) * h;
  for (size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x) {
    const uint32_t j = static_cast<uint32_t>(k / w), i = static_cast<uint32_t>(k % w);
    const uint32_t i1 = i + 1 == w ? 0 : i + 1, j1 = j + 1 == h ? 0 : j + 1;
    out[k] = make_uint4(texels[size_t(j) * w + i], texels[size_t(j) * w + i1], texels[size_t(j1) * w + i],
                        texels[size_t(j1) * w + i1]);
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


cudaError_t launch_texture_footprints(const nrc_texture& tex, void* out, int num_sms, cudaStream_t stream) {
  const size_t n = size_t(tex.width) * tex.height;
  if (n == 0 || tex.texels == nullptr) return cudaSuccess;
  const size_t want = (n + 255) / 256, cap = size_t(num_sms) * 8;
  footprints_kernel<<<static_cast<uint32_t>(want < cap ? want : cap), 256, 0, stream>>>(
      reinterpret_cast<const uint32_t*>(tex.texels), tex.width, tex.height, static_cast<uint4*>(out));
  return cudaGetLastError();
}

cudaError_t launch_scene_prepare(const nrc_scene& scene, const nrc_texture* footprints, void* prim_rows,
                                 void* mat_rows, cudaStream_t stream) {
  if (scene.primitive_count > 0)
    prepare_prims_kernel<<<(scene.primitive_count + 255) / 256, 256, 0, stream>>>(scene, static_cast<uint4*>(prim_rows));
  if (scene.material_count > 0)
    prepare_mats_kernel<<<(scene.material_count + 255) / 256, 256, 0, stream>>>(scene, footprints,
                                                                               static_cast<uint4*>(mat_rows));
  return cudaGetLastError();
}

cudaError_t launch_unpack(const nrc_scene& scene, const void* prim_rows, const void* mat_rows, bool train,
                          const void* in, const uint32_t* d_count, uint32_t capacity, void* out, uint32_t* out_dst,
                          int num_sms, cudaStream_t stream) {
  const uint32_t want = (capacity + kUnpackThreads - 1) / kUnpackThreads;
  const uint32_t cap = static_cast<uint32_t>(num_sms) * kUnpackBlocksPerSM;  // the resident blocks
  const uint32_t grid = want < cap ? want : cap;
  if (grid == 0) return cudaSuccess;
  UnpackParams p;
  p.scene = scene;
  p.rows = SceneRows{static_cast<const uint4*>(prim_rows), static_cast<const uint4*>(mat_rows)};
  p.lut = srgb_lut();
  const bool rows = prim_rows != nullptr;
  if (train && rows)
    unpack_kernel<true, true><<<grid, kUnpackThreads, 0, stream>>>(p, in, d_count, capacity, out, nullptr);
  else if (train)
    unpack_kernel<true, false><<<grid, kUnpackThreads, 0, stream>>>(p, in, d_count, capacity, out, nullptr);
  else if (rows)
    unpack_kernel<false, true><<<grid, kUnpackThreads, 0, stream>>>(p, in, d_count, capacity, out, out_dst);
  else
    unpack_kernel<false, false><<<grid, kUnpackThreads, 0, stream>>>(p, in, d_count, capacity, out, out_dst);
  return cudaGetLastError();
}

cudaError_t launch_unpack_train_batches(const nrc_scene& scene, const void* prim_rows, const void* mat_rows,
                                       const nrc_packed_train_record* const* in,
                                       uint32_t* const* counts, uint32_t capacity, nrc_train_record* const* out,
                                       int nbatches, int num_sms, cudaStream_t stream) {
  if (nbatches < 1 || nbatches > NRC_TRAIN_BATCH_COUNT) return cudaErrorInvalidValue;
  const uint32_t want = (capacity + kUnpackThreads - 1) / kUnpackThreads;
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
    unpack_batches_kernel<true><<<grid, kUnpackThreads, 0, stream>>>(p, u, capacity);
  else
    unpack_batches_kernel<false><<<grid, kUnpackThreads, 0, stream>>>(p, u, capacity);
  return cudaGetLastError();
}

}  // namespace nrc
