// Fused cache query: record tile (bulk copy) -> encode -> 5 x (64x64 ReLU) ->
// 3 outputs, one persistent CTA per SM.
//
// Follows shader/src/nrc_inference.comp:30-48 with NN_nv.glsl's forward
// (NNLoadInput :84-97, NNForward64_ReLU :99-127, NNForward3/NNOutput3 :129-158),
// re-laid out for tcgen05:
//   - the 42 KB of fp16 weights are staged once per CTA by TMA (tensor map,
//     128-byte swizzle) into shared memory as K-major tiles (the MMA's B operand);
//   - activations never leave the SM: each layer's fp16 input sits in tensor
//     memory as the MMA's A operand (32 columns), its fp32 result lands in
//     tensor memory (64 columns), and the epilogue threads convert it (ReLU +
//     fp16) back into the A columns for the next layer;
//   - kSlots independent 128-record tiles are in flight per CTA, one warpgroup
//     each (thread <-> record row, warp k of a slot reads TMEM lanes 32k..+31).
//     Every slot issues its own MMAs from its first warp (converged, one lane
//     elected): a single issuing thread is bounded by its issue rate, several
//     issuing warps keep the tensor pipe busy while other slots convert.
#include <mutex>

#include "nrc_common.cuh"
#include "nrc_kernels.h"

namespace nrc {

namespace {

constexpr int kSlots = 5;
constexpr int kInferThreads = kSlots * 128;
constexpr uint32_t kSlotCols = 96;                     // A: cols 0..31, D: cols 32..95
constexpr uint32_t kRecBytes = sizeof(nrc_input);      // 56
constexpr uint32_t kRecTileBytes = kTile * kRecBytes;  // 7168
constexpr uint32_t kRecSmemOff = kWeightSmemBytes;     // 43008, 1024-aligned
constexpr uint32_t kBarOff = kRecSmemOff + kSlots * 2 * kRecTileBytes;
constexpr uint32_t kSmemBytes = kBarOff + 512 + 1024;  // + alignment slack
static_assert(kWeightSmemBytes % 1024 == 0, "weight tiles 1024-aligned");
static_assert(kSlots * kSlotCols <= 512, "TMEM columns");
static_assert(kJoinChunks * 16 == kParams * 2, "join copy covers the weights");


struct SlotBars {
  uint64_t rec_full[2];   // bulk copy of a record tile landed (tx bytes)
  uint64_t rec_empty[2];  // all 128 threads of the slot finished reading the stage
  uint64_t a_ready;       // 4 arrivals (one per warp): A operand in TMEM for the next layer
  uint64_t d_ready;       // MMA commit: accumulator ready
  uint32_t tile[2];       // dynamic tiles: the tile (or end mark) whose records land in stage b
};
static_assert(sizeof(SlotBars) * kSlots + 16 <= 512, "barrier area (+ weight barrier, TMEM slot)");

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// Issue the bulk copy of record tile `tile` (records of rec_bytes each) into
// `dst`. Full tiles move 128 records; the last, partial tile moves the largest
// 16-byte multiple of its bytes and its trailing record (if cut) is read
// directly from global memory.
__device__ __forceinline__ void issue_record_tile(const void* __restrict__ in, uint32_t rec_bytes, uint32_t tile,
                                                  uint32_t n, uint8_t* dst, uint64_t* full) {
  const uint32_t rows = min(static_cast<uint32_t>(kTile), n - tile * kTile);
  const uint32_t bytes = (rows * rec_bytes) & ~15u;  // full tiles: 7168 or 2560, multiples of 16
  if (bytes > 0) {
    mbar_arrive_expect_tx(full, bytes);
    bulk_g2s(dst, static_cast<const uint8_t*>(in) + static_cast<size_t>(tile) * kTile * rec_bytes, bytes, full);
  } else {
    mbar_arrive(full);
  }
}

__device__ __forceinline__ bool warp_all(bool ok) { return __all_sync(0xffffffffu, ok); }

// One arrival for the whole warp once every lane has reached this point (its
// TMEM stores complete and fenced before the warp synchronisation).
__device__ __forceinline__ void arrive_warp(uint64_t* bar) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(bar);
}

// The four K-steps of one layer: D[128 x N] = A[128 x 64] (TMEM) * W^T.
// bdesc0 addresses the layer's weight tile; each K-step advances 32 bytes
// (2 in the descriptor's 16-byte address units).
__device__ __forceinline__ void issue_layer(uint32_t d, uint32_t a, uint64_t bdesc0, uint32_t idesc) {
  mma_ts(d, a + 0, bdesc0 + 0, idesc, 0u);
  mma_ts(d, a + 8, bdesc0 + 2, idesc, 1u);
  mma_ts(d, a + 16, bdesc0 + 4, idesc, 1u);
  mma_ts(d, a + 24, bdesc0 + 6, idesc, 1u);
}

// The destination epilogue of nrc_inference.comp:50-73 for one query (encoding
// of the word: NRCRecord.glsl:19-33). p = max(prediction, 0).
__device__ __forceinline__ void scatter_query(const QueryOut& Q, uint32_t dst, float p0, float p1, float p2) {
  if (dst == 0xFFFFFFFFu) return;
  const uint32_t e = dst >> 1;
  if ((dst & 1u) == 0u) {  // screen pixel: color = bias + (factor_r, factor_gb) * p, alpha 0
    const uint32_t x = e & 0x7FFFu, y = e >> 15;
    if (x >= Q.width || y >= Q.height) return;
    const size_t px = static_cast<size_t>(y) * Q.width + x;
    float4* bf = reinterpret_cast<float4*>(Q.bias_factor_r) + px;
    const float4 v = *bf;
    const float2 gb = reinterpret_cast<const float2*>(Q.factor_gb)[px];
    *bf = make_float4(__fmaf_rn(v.w, p0, v.x), __fmaf_rn(gb.x, p1, v.y), __fmaf_rn(gb.y, p2, v.z), 0.0f);
  } else {  // train records l..r of batch b: bias += factor * p
    const uint32_t b = e & 3u, l = (e >> 2) & 0x3FFFu, r = e >> 16;
    float* rec = Q.train[b];
    if (rec == nullptr) return;
    const uint32_t end = min(r + 1, Q.train_cap[b]);
    for (uint32_t i = l; i < end; ++i) {
      float* t = rec + static_cast<size_t>(i) * Q.train_stride;
      t[0] = __fmaf_rn(t[3], p0, t[0]);
      t[1] = __fmaf_rn(t[4], p1, t[1]);
      t[2] = __fmaf_rn(t[5], p2, t[2]);
    }
  }
}

// kScatter: the query carries a destination word (nrc_infer_scatter); the
// plain query path is compiled without the destination load and epilogue.
// One launch serves up to N caches: CTAs [group_start[j], group_start[j+1])
// answer cache j's queries with its weights; with N = 1 the group is the grid.
// kFmt: operand format of weights, features and activations: 0 fp16 (the
// reference's), 1 bf16, 2 E4M3 (the FP8 query: two K = 32 MMAs per layer, each
// layer's fp32 sum multiplied by its scale constant before the ReLU and the
// conversion; the weights keep the 128-byte rows of the 16-bit layout, K bytes
// 64..127 being zero and never read).
// kTable: the launch's parameters come from a table in global memory (the
// serving loop's batches, written by its scheduler kernel) instead of the
// kernel parameters; CTAs past the table's groups return at once.
template <bool kEncoded, bool kScatter, int N, int kFmt, bool kTable>
__device__ __forceinline__ void infer_body(const InferLaunch<N>& L) {
  constexpr bool kBF16 = kFmt == 1, kF8 = kFmt == 2;
  if (kTable && blockIdx.x >= L.group_start[L.njobs]) return;
  int job = 0;
  while (job + 1 < L.njobs && blockIdx.x >= L.group_start[job + 1]) ++job;
  const InferJob& J = L.job[job];
  const QueryOut& Q = J.q;
  const uint32_t G = L.group_start[job + 1] - L.group_start[job];  // CTAs of this cache
  const uint32_t rank = blockIdx.x - L.group_start[job];           // this CTA within them
  const void* input = J.input;
  uint32_t* err = J.err;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* smem_w = smem;
  uint8_t* smem_rec = smem + kRecSmemOff;
  SlotBars* bars = reinterpret_cast<SlotBars*>(smem + kBarOff);
  uint64_t* w_full = reinterpret_cast<uint64_t*>(bars + kSlots);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(w_full + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr uint32_t rec_bytes = kRecBytes;

  // dynamic tiles (single-cache record queries with a tile counter)
  const bool dyn = N == 1 && !kEncoded && J.tiles != nullptr;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kSlots; ++s) {
      mbar_init(&bars[s].rec_full[0], 1);
      mbar_init(&bars[s].rec_full[1], 1);
      mbar_init(&bars[s].rec_empty[0], 128);
      mbar_init(&bars[s].rec_empty[1], 128);
      mbar_init(&bars[s].a_ready, 4);
      mbar_init(&bars[s].d_ready, 1);
    }
    mbar_init(w_full, 1);
    mbar_fence_init();
  }
  // Everything below may read what the preceding kernel in the stream wrote
  // (unless this launch reads nothing of it: no_wait).
  if (!J.no_wait) griddep_wait();
  griddep_launch_dependents();
  const uint32_t n = min(*J.d_count, J.capacity);
  const float inv_sx0 = kF8 ? J.fp8->inv_sx0 : 1.0f;  // written by the preceding refresh launch
  const uint32_t num_tiles = (n + kTile - 1) / kTile;
  if (warp == 0) {
    tmem_alloc(tmem_slot, 512);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    if (kTable) tensormap_acquire(&J.wmap);
    stage_weights_tma(smem_w, &J.wmap, w_full);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  const int s = warp >> 2;  // slot
  const int q = warp & 3;   // TMEM lane quadrant of this warp
  const int row = q * 32 + lane;
  const bool issuer = q == 0;
  const bool leader = q == 0 && lane == 0;
  SlotBars& B = bars[s];
  const uint32_t tmem = __shfl_sync(0xffffffffu, *tmem_slot, 0);
  const uint32_t a_col = tmem + s * kSlotCols, d_col = a_col + 32;  // lane-0 addresses of the slot
  const uint32_t lane_off = static_cast<uint32_t>(q * 32) << 16;
  const uint64_t wdesc = sdesc_sw128(smem_u32(smem_w), 16, 1024);  // layer l: + l * 512
  const uint32_t id64 = idesc_16_f32(128, 64, 0, 0, kBF16), id16 = idesc_16_f32(128, 16, 0, 0, kBF16);
  uint8_t* stage0 = smem_rec + (s * 2 + 0) * kRecTileBytes;
  const uint8_t* rec_in = static_cast<const uint8_t*>(input);
  auto tile_of = [&](uint32_t it) { return (it * G + rank) * kSlots + s; };

  // The copy of the slot's tile into record stage b; with dynamic tiles the
  // tile comes from the counter and is published with the stage (an end mark,
  // a plain arrival, once the tiles are exhausted).
  auto fill_stage = [&](uint32_t b, uint32_t static_tile) {
    if (dyn) {
      const uint32_t t = atomicAdd(J.tiles, 1u);
      B.tile[b] = t;
      if (t < num_tiles)
        issue_record_tile(rec_in, rec_bytes, t, n, stage0 + b * kRecTileBytes, &B.rec_full[b]);
      else
        mbar_arrive(&B.rec_full[b]);
    } else if (static_tile < num_tiles) {
      issue_record_tile(rec_in, rec_bytes, static_tile, n, stage0 + b * kRecTileBytes, &B.rec_full[b]);
    }
  };
  if (!kEncoded && leader)
    for (uint32_t b = 0; b < 2; ++b) fill_stage(b, tile_of(b));
  bool ok = true;
  uint32_t ph_d = 0, ph_a = 0;
  if (issuer) ok = warp_all(mbar_wait(w_full, 0, kWaitLimitNs));  // before this slot's first MMA
  // The overlapped frame: once every CTA has its weights in shared memory,
  // use_weights is read no more; the CTA that loaded last waits for the
  // training grid and copies the staged weights in (its first slot starts
  // late, off the frame's end).
  if (dyn && J.join.src != nullptr && warp == 0) {
    uint32_t last_load = 0;
    if (lane == 0) {
      __threadfence();
      last_load = atomicAdd(J.tiles + 2, 1u) == gridDim.x - 1 ? 1u : 0u;
      if (last_load != 0u) {
        reinterpret_cast<volatile uint32_t*>(J.tiles)[2] = 0u;  // for the next launch
        __threadfence();
      }
    }
    if (__shfl_sync(0xffffffffu, last_load, 0) != 0u) {
      griddep_wait();  // the training grid has completed: its staged weights are final
      join_copy(J.join, lane, 32);
    }
  }
  for (uint32_t it = 0; ok; ++it) {
    uint32_t tile = tile_of(it);
    if (dyn) {  // the slot's next tile (or the end mark) arrives with its record stage
      ok = warp_all(mbar_wait(&B.rec_full[it & 1], (it >> 1) & 1, kWaitLimitNs));
      if (!ok) break;
      tile = *reinterpret_cast<volatile uint32_t*>(&B.tile[it & 1]);
    }
    if (tile >= num_tiles) break;
    const uint32_t rows_valid = min(static_cast<uint32_t>(kTile), n - tile * kTile);
    const size_t grow = static_cast<size_t>(tile) * kTile + row;
    uint32_t qdst = 0xFFFFFFFFu;  // the query's destination word (scatter epilogue)
    uint32_t e[32];
    if (!kEncoded) {
      const uint32_t b = it & 1;
      uint8_t* stage = stage0 + b * kRecTileBytes;
      if (!dyn) {
        ok = warp_all(mbar_wait(&B.rec_full[b], (it >> 1) & 1, kWaitLimitNs));
        if (!ok) break;
      }
      const uint32_t bulk = (rows_valid * rec_bytes) & ~15u;
      float r[kInFloats];
      if (row < static_cast<int>(rows_valid)) {
        const float2* src = (static_cast<uint32_t>(row + 1) * rec_bytes <= bulk)
                                ? reinterpret_cast<const float2*>(stage + row * rec_bytes)
                                : reinterpret_cast<const float2*>(rec_in + grow * rec_bytes);
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
      if (kF8) {
        encode_input_e4m3(r, inv_sx0, e);
      } else {
        encode_input<kBF16>(r, e);
      }
      if (leader && (dyn || tile_of(it + 2) < num_tiles)) {
        if (!mbar_wait(&B.rec_empty[b], (it >> 1) & 1, kWaitLimitNs))
          atomicOr(err, kErrTimeout);
        else
          fill_stage(b, tile_of(it + 2));
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
    // layer-0 A operand: 16-bit features, column pair (2j, 2j+1) in word j, or
    // E4M3 features 4j..4j+3 in word j
    if (kF8)
      tmem_st16(a_col + lane_off, e);
    else
      tmem_st32(a_col + lane_off, e);
    tc_fence_before();
    arrive_warp(&B.a_ready);
#pragma unroll 1
    for (int l = 0; l < 6; ++l) {
      if (issuer) {
        ok = warp_all(mbar_wait(&B.a_ready, ph_a, kWaitLimitNs));
        if (ok) {
          ph_a ^= 1u;  // counts issued layers; ph_d counts observed completions
          tc_fence_after();
          if (elect_one()) {
            const uint64_t wl = wdesc + static_cast<uint64_t>(l * 512);
            if (kF8) {
              mma_ts_f8(d_col, a_col + 0, wl + 0, l < 5 ? id64 : id16, 0u);
              mma_ts_f8(d_col, a_col + 8, wl + 2, l < 5 ? id64 : id16, 1u);
            } else {
              issue_layer(d_col, a_col, wl, l < 5 ? id64 : id16);
            }
            mma_commit(&B.d_ready);
          }
          __syncwarp();
        }
      }
      // load the destination word while the output layer's MMAs run
      if (kScatter && l == 5 && row < static_cast<int>(rows_valid)) qdst = __ldg(Q.dst + grow);
      const float cl = kF8 ? J.fp8->c[l] : 1.0f;  // the layer's scale constant (FP8 query)
      ok = ok && warp_all(mbar_wait(&B.d_ready, ph_d, kWaitLimitNs));
      if (!ok) break;
      ph_d ^= 1u;
      tc_fence_after();
      if (kF8 && l < 5) {
        // all 64 accumulator columns in one load and one wait, packed in place
        // (word j from values 4j..4j+3, j <= 4j); the scale multiplies two
        // lanes per instruction (IEEE-rounded like __fmul_rn each)
        uint32_t v[64];
        tmem_ld64(d_col + lane_off, v);
        const uint64_t c2 = f32x2(cl, cl);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float a0, a1, a2, a3;
          f32x2_split(mul_x2(f32x2(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1])), c2), a0, a1);
          f32x2_split(mul_x2(f32x2(__uint_as_float(v[4 * j + 2]), __uint_as_float(v[4 * j + 3])), c2), a2, a3);
          v[j] = pack4_relu_e4m3(a0, a1, a2, a3);
        }
        tmem_st16(a_col + lane_off, *reinterpret_cast<uint32_t(*)[16]>(v));
        tc_fence_before();
        arrive_warp(&B.a_ready);
      } else if (l < 5) {
        // all 64 accumulator columns in one load and one wait, converted in place
        uint32_t v[64];
        tmem_ld64(d_col + lane_off, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = pack2_relu<kBF16>(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
        tmem_st32(a_col + lane_off, *reinterpret_cast<uint32_t(*)[32]>(v));
        tc_fence_before();
        arrive_warp(&B.a_ready);
      } else {
        uint32_t o4[4];
        tmem_ld4(d_col + lane_off, o4);
        if (row < static_cast<int>(rows_valid)) {
          if (Q.out != nullptr) {
            float* dst = Q.out + grow * 3;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float v = kF8 ? __fmul_rn(__uint_as_float(o4[c]), cl) : __uint_as_float(o4[c]);
              dst[c] = Q.clamp ? fmaxf(v, 0.0f) : v;
            }
          }
          if (kScatter)
            scatter_query(Q, qdst, fmaxf(__uint_as_float(o4[0]), 0.0f), fmaxf(__uint_as_float(o4[1]), 0.0f),
                          fmaxf(__uint_as_float(o4[2]), 0.0f));
        }
      }
    }
  }
  if (!ok && lane == 0) atomicOr(err, kErrTimeout);
  // A slot that stopped early may still have MMAs in flight (issued, d_ready
  // not yet observed): wait for them, bounded, before TMEM is released.
  if (!ok && issuer && ph_a != ph_d) warp_all(mbar_wait(&B.d_ready, ph_d, kWaitLimitNs));
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
  // dynamic tiles: the last CTA out, when every CTA has taken its last tile,
  // returns the counters to zero for the next launch and joins the frame
  if (dyn) {
    uint32_t* last = tmem_slot;  // free once TMEM is released
    if (threadIdx.x == 0) {
      __threadfence();
      *last = atomicAdd(J.tiles + 1, 1u) == gridDim.x - 1 ? 1u : 0u;
      if (*last != 0u) {  // every CTA has taken its last tile and counted itself out
        reinterpret_cast<volatile uint32_t*>(J.tiles)[0] = 0u;
        reinterpret_cast<volatile uint32_t*>(J.tiles)[1] = 0u;
        __threadfence();
      }
    }
    __syncthreads();
    // A launch that started without waiting for the preceding grid (the
    // overlapped frame's training) completes only after it, so that whatever
    // follows this query in the stream also follows the training: the CTA that
    // copied the staged weights has waited for that grid, else the last CTA
    // out waits here. The training is resident (this grid launched once all of
    // its CTAs ran) and never waits for the query.
    if (*last != 0u && J.no_wait && J.join.src == nullptr) griddep_wait();
  }
}

template <bool kEncoded, bool kScatter, int N, int kFmt>
__global__ void __launch_bounds__(kInferThreads, 1) infer_kernel(const __grid_constant__ InferLaunch<N> L) {
  infer_body<kEncoded, kScatter, N, kFmt, false>(L);
}

// The batched record query over a launch table in global memory.
__global__ void __launch_bounds__(kInferThreads, 1) infer_table_kernel(const InferLaunch<kMaxInferJobs>* __restrict__ L) {
  infer_body<false, false, kMaxInferJobs, 0, true>(*L);
}

template <bool kEncoded, bool kScatter, int N, int kFmt>
cudaError_t launch(const InferLaunch<N>& L, uint32_t grid, cudaStream_t stream) {
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr.val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kInferThreads);
  cfg.dynamicSmemBytes = kSmemBytes;
  cfg.stream = stream;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, infer_kernel<kEncoded, kScatter, N, kFmt>, L);
}

// The shared-memory limit, and the largest carveout: the query and the trainer
// (206 KB) then run in the same SM configuration, so an SM passing from one to
// the other between kernels needs no reconfiguration.
template <bool kEncoded, bool kScatter, int N, int kFmt>
cudaError_t set_smem() {
  cudaError_t e = cudaFuncSetAttribute(infer_kernel<kEncoded, kScatter, N, kFmt>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(infer_kernel<kEncoded, kScatter, N, kFmt>,
                              cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
}

}  // namespace

cudaError_t configure_infer_kernels() {
  cudaError_t e = set_smem<true, false, 1, 0>();
  if (e == cudaSuccess) e = set_smem<false, false, 1, 0>();
  if (e == cudaSuccess) e = set_smem<false, true, 1, 0>();
  if (e == cudaSuccess) e = set_smem<false, false, kMaxInferJobs, 0>();
  if (e == cudaSuccess) e = set_smem<false, false, 1, 1>();
  if (e == cudaSuccess) e = set_smem<false, true, 1, 1>();
  if (e == cudaSuccess) e = set_smem<false, false, kMaxInferJobs, 1>();
  if (e == cudaSuccess) e = set_smem<false, false, 1, 2>();
  if (e == cudaSuccess) e = cudaFuncSetAttribute(infer_table_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(infer_table_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  return e;
}

cudaError_t launch_infer_table(const InferLaunch<kMaxInferJobs>* table, uint32_t grid, cudaStream_t stream) {
  infer_table_kernel<<<grid, kInferThreads, kSmemBytes, stream>>>(table);
  return cudaGetLastError();
}

uint32_t infer_smem_bytes() { return kSmemBytes; }
int infer_threads() { return kInferThreads; }
int infer_tiles_per_cta() { return kSlots; }

uint32_t infer_grid(uint32_t capacity, int num_sms) {
  const uint32_t tiles = (capacity + kTile - 1) / kTile;
  const uint32_t want = (tiles + kSlots - 1) / kSlots;
  return want < static_cast<uint32_t>(num_sms) ? want : static_cast<uint32_t>(num_sms);
}

cudaError_t launch_infer(const void* input, bool encoded, const uint32_t* d_count, uint32_t capacity,
                         const CUtensorMap* wmap, const QueryOut& q, uint32_t* err, int num_sms,
                         cudaStream_t stream, bool bf16) {
  const uint32_t grid = infer_grid(capacity, num_sms);
  if (grid == 0) return cudaSuccess;
  InferLaunch<1> L;
  L.job[0] = InferJob{};
  L.job[0].wmap = *wmap;
  L.job[0].input = input;
  L.job[0].d_count = d_count;
  L.job[0].capacity = capacity;
  L.job[0].err = err;
  L.job[0].q = q;
  L.group_start[0] = 0;
  L.group_start[1] = grid;
  L.njobs = 1;
  if (encoded) return bf16 ? cudaErrorInvalidValue : launch<true, false, 1, 0>(L, grid, stream);
  if (q.dst != nullptr)
    return bf16 ? launch<false, true, 1, 1>(L, grid, stream) : launch<false, true, 1, 0>(L, grid, stream);
  return bf16 ? launch<false, false, 1, 1>(L, grid, stream) : launch<false, false, 1, 0>(L, grid, stream);
}

cudaError_t launch_infer_frame(const nrc_input* input, const uint32_t* d_count, uint32_t capacity,
                               const CUtensorMap* wmap, const QueryOut& q, uint32_t* err, uint32_t* tiles,
                               const FrameJoin& join, uint32_t grid, cudaStream_t stream, bool bf16) {
  if (grid == 0 || tiles == nullptr) return cudaErrorInvalidValue;
  InferLaunch<1> L;
  L.job[0] = InferJob{};
  L.job[0].wmap = *wmap;
  L.job[0].input = input;
  L.job[0].d_count = d_count;
  L.job[0].capacity = capacity;
  L.job[0].err = err;
  L.job[0].q = q;
  L.job[0].tiles = tiles;
  L.job[0].no_wait = 1;
  L.job[0].join = join;
  L.group_start[0] = 0;
  L.group_start[1] = grid;
  L.njobs = 1;
  if (q.dst != nullptr)
    return bf16 ? launch<false, true, 1, 1>(L, grid, stream) : launch<false, true, 1, 0>(L, grid, stream);
  return bf16 ? launch<false, false, 1, 1>(L, grid, stream) : launch<false, false, 1, 0>(L, grid, stream);
}

cudaError_t launch_infer_fp8(const nrc_input* input, const uint32_t* d_count, uint32_t capacity,
                             const CUtensorMap* w8map, const Fp8State* fp8, float* out, uint32_t* err, int num_sms,
                             cudaStream_t stream) {
  const uint32_t grid = infer_grid(capacity, num_sms);
  if (grid == 0) return cudaSuccess;
  InferLaunch<1> L;
  L.job[0] = InferJob{};
  L.job[0].wmap = *w8map;
  L.job[0].input = input;
  L.job[0].d_count = d_count;
  L.job[0].capacity = capacity;
  L.job[0].err = err;
  L.job[0].q.out = out;
  L.job[0].q.clamp = 1;
  L.job[0].fp8 = fp8;
  L.group_start[0] = 0;
  L.group_start[1] = grid;
  L.njobs = 1;
  return launch<false, false, 1, 2>(L, grid, stream);
}

cudaError_t launch_infer_many(const InferJob* jobs, int njobs, const uint32_t* group_size, cudaStream_t stream,
                              bool bf16) {
  if (njobs < 1 || njobs > kMaxInferJobs) return cudaErrorInvalidValue;
  static InferLaunch<kMaxInferJobs> L;  // host staging of the kernel parameters (copied at launch)
  static std::mutex m;
  std::lock_guard<std::mutex> lock(m);
  uint32_t grid = 0;
  for (int j = 0; j < njobs; ++j) {
    if (jobs[j].q.dst != nullptr || group_size[j] < 1) return cudaErrorInvalidValue;
    L.job[j] = jobs[j];
    L.group_start[j] = grid;
    grid += group_size[j];
  }
  L.group_start[njobs] = grid;
  L.njobs = njobs;
  return bf16 ? launch<false, false, kMaxInferJobs, 1>(L, grid, stream)
              : launch<false, false, kMaxInferJobs, 0>(L, grid, stream);
}

}  // namespace nrc
