// Fused cache query: record tile (bulk copy) -> encode -> 5 x (64x64 ReLU) ->
// 3 outputs, one persistent CTA per SM.
//
// Follows shader/src/nrc_inference.comp:30-48 with NN_nv.glsl's forward
// (NNLoadInput :84-97, NNForward64_ReLU :99-127, NNForward3/NNOutput3 :129-158),
// re-laid out for tcgen05:
//   - the 42 KB of fp16 weights are staged once per CTA into shared memory as
//     128-byte-swizzled K-major tiles (the MMA's B operand);
//   - activations never leave the SM: each layer's fp16 input sits in tensor
//     memory as the MMA's A operand (the TMEM-A form), its fp32 result lands in
//     TMEM, and the epilogue threads convert it (ReLU + fp16) back into the A
//     operand of the next layer;
//   - kSlots independent 128-record tiles are in flight per CTA (128 TMEM
//     columns each) so the single MMA-issuing thread always has a ready tile
//     while the epilogue warps of the others convert.
// Warp 0: TMEM allocator, lane 0 issues all MMAs. Warps 1..16: four epilogue
// warpgroups, one per slot; thread <-> record row, warp w reads TMEM lanes
// 32*(w%4)..+31.
#include "nrc_common.cuh"
#include "nrc_kernels.h"

namespace nrc {

namespace {

constexpr int kSlots = 4;
constexpr int kInferThreads = 32 + kSlots * 128;
constexpr uint32_t kRecBytes = sizeof(nrc_input);   // 56
constexpr uint32_t kRecTileBytes = kTile * kRecBytes;  // 7168
constexpr uint32_t kRecSmemOff = kWeightSmemBytes;     // 43008, 1024-aligned
constexpr uint32_t kBarOff = kRecSmemOff + kSlots * 2 * kRecTileBytes;
constexpr uint32_t kSmemBytes = kBarOff + 256 + 1024;  // + alignment slack
static_assert(kWeightSmemBytes % 1024 == 0, "weight tiles 1024-aligned");

struct SlotBars {
  uint64_t rec_full[2];   // bulk copy of a record tile landed (tx bytes)
  uint64_t rec_empty[2];  // all 128 threads of the slot finished reading the stage
  uint64_t a_ready;       // 128 arrivals: A operand in TMEM for the next layer
  uint64_t d_ready;       // MMA commit: accumulator ready
};
static_assert(sizeof(SlotBars) * kSlots + 16 <= 256, "barrier area");

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// Issue the bulk copy of record tile `tile` into `dst`. Full tiles move 7168
// bytes; the last, partial tile moves the largest 16-byte multiple of its bytes
// and its trailing record (if cut) is read directly from global memory.
__device__ __forceinline__ void issue_record_tile(const nrc_input* __restrict__ in, uint32_t tile, uint32_t n,
                                                  uint8_t* dst, uint64_t* full) {
  const uint32_t rows = min(static_cast<uint32_t>(kTile), n - tile * kTile);
  const uint32_t bytes = rows == kTile ? kRecTileBytes : ((rows * kRecBytes) & ~15u);
  if (bytes > 0) {
    mbar_arrive_expect_tx(full, bytes);
    bulk_g2s(dst, reinterpret_cast<const uint8_t*>(in) + static_cast<size_t>(tile) * kRecTileBytes, bytes, full);
  } else {
    mbar_arrive(full);
  }
}

__device__ __forceinline__ bool warp_all(bool ok) { return __all_sync(0xffffffffu, ok); }

template <bool kEncoded>
__global__ void __launch_bounds__(kInferThreads, 1)
    infer_kernel(const void* __restrict__ input, const uint32_t* __restrict__ d_count, uint32_t capacity,
                 const __half* __restrict__ w16, float* __restrict__ out, int clamp_out, uint32_t* err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* smem_w = smem;
  uint8_t* smem_rec = smem + kRecSmemOff;
  SlotBars* bars = reinterpret_cast<SlotBars*>(smem + kBarOff);
  uint64_t* drain = reinterpret_cast<uint64_t*>(bars + kSlots);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t n = min(*d_count, capacity);
  const uint32_t num_tiles = (n + kTile - 1) / kTile;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kSlots; ++s) {
      mbar_init(&bars[s].rec_full[0], 1);
      mbar_init(&bars[s].rec_full[1], 1);
      mbar_init(&bars[s].rec_empty[0], 128);
      mbar_init(&bars[s].rec_empty[1], 128);
      mbar_init(&bars[s].a_ready, 128);
      mbar_init(&bars[s].d_ready, 1);
    }
    mbar_init(drain, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, 512);
    tmem_relinquish();
  }
  stage_weights(smem_w, w16);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------ MMA issuer --
    if (lane == 0) {
      bool ok = true;
      uint32_t ph_a[kSlots] = {0, 0, 0, 0};
      const uint32_t id64 = idesc_f16_f32(128, 64, 0, 0);
      const uint32_t id16 = idesc_f16_f32(128, 16, 0, 0);
      const uint32_t sw = smem_u32(smem_w);
      for (uint32_t it = 0; ok; ++it) {
        const uint32_t tile0 = (it * gridDim.x + blockIdx.x) * kSlots;
        if (tile0 >= num_tiles) break;
        for (int l = 0; l < 6 && ok; ++l) {
          for (int s = 0; s < kSlots; ++s) {
            if (tile0 + s >= num_tiles) break;
            if (!mbar_wait(&bars[s].a_ready, ph_a[s], kWaitLimitNs)) {
              ok = false;
              break;
            }
            ph_a[s] ^= 1u;
            tc_fence_after();
            const uint32_t base = tmem + s * 128;
            const uint32_t a = base + ((l & 1) ? 64u : 0u);
            const uint32_t d = base + ((l & 1) ? 0u : 64u);
            const uint32_t wl = sw + l * 8192;
#pragma unroll
            for (int j = 0; j < 4; ++j)
              mma_ts(d, a + 8 * j, sdesc_sw128(wl + 32 * j, 16, 1024), l < 5 ? id64 : id16, j > 0);
            mma_commit(&bars[s].d_ready);
          }
        }
      }
      if (!ok) atomicOr(err, kErrTimeout);
      // all issued MMAs must be complete before TMEM is released
      mma_commit(drain);
      if (!mbar_wait(drain, 0, kWaitLimitNs)) atomicOr(err, kErrTimeout);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------ epilogue warpgroups --
    const int ew = warp - 1;
    const int s = ew >> 2;
    const int q = warp & 3;  // TMEM lane quadrant accessible to this warp
    const int row = q * 32 + lane;
    const bool leader = (ew & 3) == 0 && lane == 0;
    SlotBars& B = bars[s];
    const uint32_t lane_base = tmem + (static_cast<uint32_t>(q * 32) << 16) + s * 128;
    uint8_t* stage[2] = {smem_rec + (s * 2 + 0) * kRecTileBytes, smem_rec + (s * 2 + 1) * kRecTileBytes};
    const nrc_input* rec_in = static_cast<const nrc_input*>(input);
    auto tile_of = [&](uint32_t it) { return (it * gridDim.x + blockIdx.x) * kSlots + s; };

    if (!kEncoded && leader) {
      for (uint32_t b = 0; b < 2; ++b)
        if (tile_of(b) < num_tiles) issue_record_tile(rec_in, tile_of(b), n, stage[b], &B.rec_full[b]);
    }
    bool ok = true;
    uint32_t ph_d = 0;
    for (uint32_t it = 0; ok; ++it) {
      const uint32_t tile = tile_of(it);
      if (tile >= num_tiles) break;
      const uint32_t rows_valid = min(static_cast<uint32_t>(kTile), n - tile * kTile);
      const size_t grow = static_cast<size_t>(tile) * kTile + row;
      uint32_t e[32];
      if (!kEncoded) {
        const uint32_t b = it & 1;
        ok = warp_all(mbar_wait(&B.rec_full[b], (it >> 1) & 1, kWaitLimitNs));
        if (!ok) break;
        const uint32_t bulk = rows_valid == kTile ? kRecTileBytes : ((rows_valid * kRecBytes) & ~15u);
        float r[kInFloats];
        if (row < static_cast<int>(rows_valid)) {
          const float2* src = (static_cast<uint32_t>(row + 1) * kRecBytes <= bulk)
                                  ? reinterpret_cast<const float2*>(stage[b] + row * kRecBytes)
                                  : reinterpret_cast<const float2*>(rec_in + grow);
#pragma unroll
          for (int k = 0; k < 7; ++k) {
            const float2 v = src[k];
            r[2 * k] = v.x;
            r[2 * k + 1] = v.y;
          }
        } else {
#pragma unroll
          for (int k = 0; k < kInFloats; ++k) r[k] = 0.0f;
        }
        // the stage may be refilled once all 128 threads have read it
        mbar_arrive(&B.rec_empty[b]);
        encode_input(r, e);
        if (leader && tile_of(it + 2) < num_tiles) {
          if (!mbar_wait(&B.rec_empty[b], (it >> 1) & 1, kWaitLimitNs)) {
            atomicOr(err, kErrTimeout);
          } else {
            issue_record_tile(rec_in, tile_of(it + 2), n, stage[b], &B.rec_full[b]);
          }
        }
      } else {
        const uint16_t* enc_in = static_cast<const uint16_t*>(input);
        if (row < static_cast<int>(rows_valid)) {
          const uint4* src = reinterpret_cast<const uint4*>(enc_in + grow * 64);
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const uint4 v = __ldg(src + c);
            e[4 * c] = v.x;
            e[4 * c + 1] = v.y;
            e[4 * c + 2] = v.z;
            e[4 * c + 3] = v.w;
          }
        } else {
#pragma unroll
          for (int c = 0; c < 32; ++c) e[c] = 0u;
        }
      }
      __syncwarp();  // reconverge before the warp-collective TMEM store
      // layer-0 A operand: fp16 features, column pair (2j, 2j+1) in word j
      tmem_st32(lane_base, e);
      tc_fence_before();
      mbar_arrive(&B.a_ready);
#pragma unroll 1
      for (int l = 0; l < 5; ++l) {
        ok = warp_all(mbar_wait(&B.d_ready, ph_d, kWaitLimitNs));
        if (!ok) break;
        ph_d ^= 1u;
        tc_fence_after();
        const uint32_t dcol = (l & 1) ? 0u : 64u;
        uint32_t v[32], p[32];
        tmem_ld32(lane_base + dcol, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) p[j] = pack_relu_f16x2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
        tmem_ld32(lane_base + dcol + 32, v);
#pragma unroll
        for (int j = 0; j < 16; ++j)
          p[16 + j] = pack_relu_f16x2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
        tmem_st32(lane_base + dcol, p);
        tc_fence_before();
        mbar_arrive(&B.a_ready);
      }
      if (!ok) break;
      ok = warp_all(mbar_wait(&B.d_ready, ph_d, kWaitLimitNs));
      if (!ok) break;
      ph_d ^= 1u;
      tc_fence_after();
      uint32_t o4[4];
      tmem_ld4(lane_base + 0, o4);  // output layer (odd) accumulates at column 0
      if (row < static_cast<int>(rows_valid)) {
        float* dst = out + grow * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float v = __uint_as_float(o4[c]);
          dst[c] = clamp_out ? fmaxf(v, 0.0f) : v;
        }
      }
    }
    if (!ok && lane == 0) atomicOr(err, kErrTimeout);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

}  // namespace

cudaError_t configure_infer_kernels() {
  cudaError_t e = cudaFuncSetAttribute(infer_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(infer_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  return e;
}

uint32_t infer_smem_bytes() { return kSmemBytes; }
int infer_threads() { return kInferThreads; }
int infer_tiles_per_cta() { return kSlots; }

cudaError_t launch_infer(const void* input, bool encoded, const uint32_t* d_count, uint32_t capacity,
                         const __half* w16, float* out, bool clamp_out, uint32_t* err, int num_sms,
                         cudaStream_t stream) {
  const uint32_t tiles = (capacity + kTile - 1) / kTile;
  const uint32_t want = (tiles + kSlots - 1) / kSlots;
  const uint32_t grid = want < static_cast<uint32_t>(num_sms) ? want : static_cast<uint32_t>(num_sms);
  if (grid == 0) return cudaSuccess;
  if (encoded)
    infer_kernel<true><<<grid, kInferThreads, kSmemBytes, stream>>>(input, d_count, capacity, w16, out, clamp_out,
                                                                     err);
  else
    infer_kernel<false><<<grid, kInferThreads, kSmemBytes, stream>>>(input, d_count, capacity, w16, out, clamp_out,
                                                                      err);
  return cudaGetLastError();
}

}  // namespace nrc
