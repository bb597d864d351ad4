// Fused training: for each of up to four chained batches, record tiles (bulk
// copy) -> encode -> forward keeping all six activations -> relative-L2 loss
// gradient -> backward -> weight gradients, then the Adam/EMA update, all in
// one persistent cooperative kernel.
//
// Follows shader/src/nrc_gradient.comp:26-58 with NN_nv.glsl's backward
// (NNLoadDA3_RelativeL2LuminanceLoss :178-196, NNBackwardDA3/64_ReLU :222-278,
// NNUpdateDW3/64 :280-367), nrc_train_prepare.comp:16-29 and
// nrc_optimize.comp:32-54, and the chaining of the four train passes of one
// frame (src/rg/NRCRenderGraph.cpp:57-80), re-laid out for tcgen05:
//   - the weights arrive by TMA (tensor map, 128-byte swizzle) as the MMA's B
//     operand tiles, again after every optimizer step;
//   - activations act_0..act_5 (fp16, 128 x 64 per tile) stay in shared memory
//     as 128-byte-swizzled rows and serve as the MN-major B operand of each
//     layer's weight gradient; the forward and dA MMAs take their A operand
//     (act_l, or the gradient g_{l+1}) from tensor memory, where the epilogue
//     writes it beside the shared-memory copy (the shared-memory form would be
//     bound by shared-memory bandwidth at this width). The epilogue hands the
//     TMEM copy to the MMA warp first (a_ready) and writes the shared-memory
//     copy after it, off the layer chain; the gradients' shared-memory copies
//     have their own barrier (g_ready), which only the weight-gradient MMAs
//     wait for;
//   - dA = (g W) masked by act > 0 uses the weight tile itself as an MN-major B
//     operand (the reference's NaN-mask trick becomes a bit mask on packed
//     halves); it is issued before the layer's weight-gradient MMAs so the
//     epilogue, which needs only dA, is not held up by them;
//   - dW_l += g^T act_l is an M=64 MMA (K = records) accumulated in TMEM across
//     the CTA's tiles of a batch; on its last tile each layer's dW is written
//     to the CTA's slot of a per-CTA partial-gradient array as soon as it is
//     final, overlapping that write with the rest of the backward chain;
//   - a grid-wide barrier (cooperative launch, bounded waits) then lets every
//     CTA update one slice of the parameters: it sums the partials of its slice
//     in CTA order (run-to-run identical) and applies Adam + EMA; a second
//     barrier publishes the new weights, which the next batch reloads by TMA.
//     The reference's prepare pass (count clamp, step state) runs in CTA 0.
//   - the epilogue runs on eight warps: the two warps that share a TMEM lane
//     quadrant split each 64-wide row between them.
#include <mutex>

#include "nrc_common.cuh"
#include "nrc_kernels.h"
#include "nrc_train_math.cuh"

namespace nrc {

namespace {

constexpr int kEpiWarps = 8;
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kTrainThreads = 32 + kEpiThreads;
constexpr uint32_t kTRecBytes = sizeof(nrc_train_record);  // 80
constexpr uint32_t kTRecTileBytes = kTile * kTRecBytes;     // 10240
constexpr uint32_t kActBytes = kTile * 128;                 // 16384: 128 rows x 64 fp16
constexpr uint32_t kActOff = kWeightSmemBytes;              // 43008
constexpr uint32_t kGOff = kActOff + 6 * kActBytes;         // two gradient buffers
constexpr uint32_t kStageOff = kGOff + 2 * kActBytes;
constexpr uint32_t kTBarOff = kStageOff + 2 * kTRecTileBytes;
constexpr uint32_t kECacheOff = kTBarOff + 256;
static_assert(kActOff % 1024 == 0 && kGOff % 1024 == 0 && kStageOff % 16 == 0, "alignment");

// TMEM columns: dW_l accumulators (M=64 layout) at 64*l, l = 0..5; scratch D at
// 384..447; the A operand of the forward / dA MMAs (fp16 pairs) at 448..479.
constexpr uint32_t kDCol = 384;
constexpr uint32_t kACol = 448;

// Parameter slices of the optimizer phase: float4 columns of the gradient. The
// grid has between kMinTrainCtas and kMaxTrainCtas CTAs: the first bounds a
// CTA's slice (its optimizer entries stay in shared memory for the whole
// launch), the second the staged partials (slice x CTAs <= kCols4 + grid).
constexpr int kCols4 = kParams / 4;  // 5168
constexpr uint32_t kMinTrainCtas = 32;
constexpr uint32_t kMaxTrainCtas = 160;
constexpr uint32_t kMaxSlice4 = (kCols4 + kMinTrainCtas - 1) / kMinTrainCtas;  // 162
constexpr uint32_t kTrainSmemBytes = kECacheOff + kMaxSlice4 * 4 * sizeof(nrc_optimizer_entry) + 1024;
static_assert(kParams % 4 == 0, "parameters in float4 columns");
static_assert(kTrainSmemBytes <= 227 * 1024, "shared memory");
// The partials are staged behind act_0, which the next batch's first tile may
// already be encoded into.
static_assert(5 * kActBytes + 2 * kActBytes >= (kCols4 + kMaxTrainCtas) * 16, "staged slice fits");

struct TrainBars {
  uint64_t rec_full[2];
  uint64_t rec_empty[2];
  uint64_t a_ready;    // 8 arrivals (one per epilogue warp): the next A operand is in TMEM
  uint64_t g_ready;    // 8 arrivals: a gradient's shared-memory rows (weight-gradient operand) are written
  uint64_t d_ready;    // MMA commit: scratch accumulator ready
  uint64_t tile_done;  // MMA commit after the tile's last weight-gradient MMA
  uint64_t drain;
  uint64_t w_full;     // weights landed (TMA)
  uint32_t tmem_base;
  uint32_t sync_ok;
  uint32_t count[NRC_TRAIN_BATCH_COUNT];  // record counts as read at launch
  nrc_optimizer_state st;                 // optimizer step state as read at launch
};
static_assert(sizeof(TrainBars) <= 256, "barrier area");

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

__device__ __forceinline__ bool warp_all(bool ok) { return __all_sync(0xffffffffu, ok); }

__device__ __forceinline__ void issue_train_tile(const nrc_train_record* __restrict__ in, uint32_t tile, uint32_t n,
                                                 uint8_t* dst, uint64_t* full) {
  const uint32_t rows = min(static_cast<uint32_t>(kTile), n - tile * kTile);
  const uint32_t bytes = rows * kTRecBytes;  // multiple of 16
  mbar_arrive_expect_tx(full, bytes);
  bulk_g2s(dst, reinterpret_cast<const uint8_t*>(in) + static_cast<size_t>(tile) * kTRecTileBytes, bytes, full);
}

// Half h (16 words = chunks 4h..4h+3) of one 128-byte row of a swizzled operand tile.
__device__ __forceinline__ void store_half(uint8_t* tile, int row, int h, const uint32_t* w) {
#pragma unroll
  for (int c = 0; c < 4; ++c)
    *reinterpret_cast<uint4*>(tile + sw128_offset(row, 4 * h + c)) =
        make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
}

__device__ __forceinline__ void load_half(const uint8_t* tile, int row, int h, uint32_t* w) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const uint4 v = *reinterpret_cast<const uint4*>(tile + sw128_offset(row, 4 * h + c));
    w[4 * c] = v.x;
    w[4 * c + 1] = v.y;
    w[4 * c + 2] = v.z;
    w[4 * c + 3] = v.w;
  }
}

// ReLU backward on packed halves: keep g where act > 0, and zero NaN sums as
// the reference's NaN-mask trick does (NN_nv.glsl:240-243, 272-277).
__device__ __forceinline__ uint32_t relu_mask_f16x2(uint32_t g, uint32_t a) {
  const __half2 g2 = *reinterpret_cast<const __half2*>(&g);
  const __half2 a2 = *reinterpret_cast<const __half2*>(&a);
  return g & __hgt2_mask(a2, __float2half2_rn(0.0f)) & ~__hneu2_mask(g2, g2);
}

// The same on bf16 pairs: a half is kept where the activation is greater than
// zero (IEEE compare: positive, non-zero, not NaN; subnormals count) and the
// gradient is not NaN, two packed compares as for fp16.
__device__ __forceinline__ uint32_t relu_mask_bf16x2(uint32_t g, uint32_t a) {
  const __nv_bfloat162 g2 = *reinterpret_cast<const __nv_bfloat162*>(&g);
  const __nv_bfloat162 a2 = *reinterpret_cast<const __nv_bfloat162*>(&a);
  return g & __hgt2_mask(a2, __float2bfloat162_rn(0.0f)) & ~__hneu2_mask(g2, g2);
}

template <bool kBF16>
__device__ __forceinline__ uint32_t relu_mask2(uint32_t g, uint32_t a) {
  return kBF16 ? relu_mask_bf16x2(g, a) : relu_mask_f16x2(g, a);
}


// Write half h (32 inputs) of one layer's final weight gradient from TMEM to the
// CTA's partial slot. M=64 accumulator layout: output row 16q+t lives in TMEM
// lane 32q+t (t < 16), so lanes 0..15 of each warp own one output row.
__device__ __forceinline__ void drain_dw(uint32_t lane_base, int layer, int q, int h, int lane, float* dst) {
  const int o = q * 16 + lane;
  const bool keep = lane < 16 && (layer < kHidden || o < kOut);
  uint32_t v[32];
  tmem_ld32(lane_base + 64 * layer + 32 * h, v);
  if (keep) {
    float4* g4 = reinterpret_cast<float4*>(dst + layer * kLayerElems + o * 64 + 32 * h);
#pragma unroll
    for (int j = 0; j < 8; ++j)
      g4[j] = make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]), __uint_as_float(v[4 * j + 2]),
                          __uint_as_float(v[4 * j + 3]));
  }
}

// Warp maximum of a non-negative value, merged into *slot (fp32 bits; non-negative
// floats order as their bit patterns).
__device__ __forceinline__ void amax_record(uint32_t* slot, float m) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) atomicMax(slot, __float_as_uint(m));
}

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Grid-wide barrier of a cooperative launch: every CTA adds one to the counter
// and waits (bounded) until it reaches `target`. Writes before the barrier,
// generic or read later by TMA, are visible after it. Returns false on timeout.
__device__ __forceinline__ bool grid_sync(uint32_t* counter, uint32_t target, uint32_t* sync_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    fence_proxy_async_global();
    // the arrival releases the CTA's writes (ordered before it by the CTA
    // barrier above); the polling load acquires the other CTAs'
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(counter) : "memory");
    bool ok = true;
    if (ld_acquire_gpu(counter) < target) {
      const uint64_t t0 = globaltimer_ns();
      while (ld_acquire_gpu(counter) < target) {
        if (globaltimer_ns() - t0 > kWaitLimitNs) {
          ok = false;
          break;
        }
        __nanosleep(32);
      }
    }
    fence_proxy_async_global();
    *sync_ok = ok ? 1u : 0u;
  }
  __syncthreads();
  return *reinterpret_cast<volatile uint32_t*>(sync_ok) != 0;
}

// One launch trains up to N caches: CTAs [group_start[j], group_start[j+1])
// form cache j's group, which runs the whole schedule below on its own (its own
// grid barrier, partial slots and parameter slices). With N = 1 the group is the
// grid.
// kBF16: weights, activations and gradients in bf16 instead of fp16 (the master
// weights and moments are fp32 either way).
// kTable: the launch's parameters come from a table in global memory (the
// serving loop's batches) instead of the kernel parameters; CTAs past the
// table's groups return at once (they belong to no group's barrier).
template <int N, bool kBF16, bool kTable>
__device__ __forceinline__ void train_body(const TrainLaunch<N>& L) {
  if (kTable && blockIdx.x >= L.group_start[L.njobs]) return;
  int job = 0;
  while (job + 1 < L.njobs && blockIdx.x >= L.group_start[job + 1]) ++job;
  const TrainParams& P = L.job[job].p;
  const CUtensorMap& wmap = L.job[job].wmap;
  if (kTable && threadIdx.x == 0) tensormap_acquire(&wmap);  // thread 0 issues the weight copies
  const uint32_t G = L.group_start[job + 1] - L.group_start[job];  // CTAs of this cache
  const uint32_t rank = blockIdx.x - L.group_start[job];           // this CTA within them
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* smem_w = smem;
  uint8_t* act = smem + kActOff;
  uint8_t* gbuf = smem + kGOff;
  uint8_t* stage = smem + kStageOff;
  TrainBars* B = reinterpret_cast<TrainBars*>(smem + kTBarOff);
  nrc_optimizer_entry* ecache = reinterpret_cast<nrc_optimizer_entry*>(smem + kECacheOff);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    mbar_init(&B->rec_full[0], 1);
    mbar_init(&B->rec_full[1], 1);
    mbar_init(&B->rec_empty[0], kEpiThreads);
    mbar_init(&B->rec_empty[1], kEpiThreads);
    mbar_init(&B->a_ready, kEpiWarps);
    mbar_init(&B->g_ready, kEpiWarps);
    mbar_init(&B->d_ready, 1);
    mbar_init(&B->tile_done, 1);
    mbar_init(&B->drain, 1);
    mbar_init(&B->w_full, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&B->tmem_base, 512);
    tmem_relinquish();
  }
  // Everything below may read what the preceding kernel in the stream wrote.
  griddep_wait();
  // A dependent launch may start once every CTA of this cooperative grid runs
  // (the overlapped frame's query, which reads nothing this launch writes and
  // fills the SMs this grid leaves free); dependents that read this launch's
  // results wait for its completion in their own griddepcontrol.wait.
  griddep_launch_dependents();

  // This CTA's slice [c0, c1) of float4 gradient columns in the optimizer phase;
  // its optimizer entries stay in shared memory for the whole launch (only this
  // CTA updates them).
  const uint32_t per = (kCols4 + G - 1) / G;
  const uint32_t c0 = min(static_cast<uint32_t>(kCols4), rank * per);
  const uint32_t ncols = min(static_cast<uint32_t>(kCols4), c0 + per) - c0;
  // Groups of fewer than kMinTrainCtas CTAs have slices too large to keep in
  // shared memory; their optimizer reads and writes the entries in memory.
  const bool cached = ncols <= kMaxSlice4;
  if (P.mode == kTrainStep && cached) {
    for (uint32_t k = threadIdx.x; k < 4 * ncols; k += blockDim.x) cp_async16(ecache + k, P.entries + 4 * c0 + k);
    cp_async_commit();
  }
  // Every batch's record count and the optimizer step state, read once before
  // CTA 0 writes them back (nrc_train_prepare.comp:16-29).
  if (threadIdx.x == 0) {
    for (int s = 0; s < P.steps; ++s) B->count[s] = *reinterpret_cast<volatile const uint32_t*>(P.batch[s].d_count);
    if (P.mode == kTrainStep) B->st = *P.state;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = __shfl_sync(0xffffffffu, B->tmem_base, 0);
  float* const my_partial = P.partials + static_cast<size_t>(rank) * kParams;
  nrc_optimizer_state st = B->st;  // advanced per batch in every CTA alike
  if (P.mode == kTrainStep && rank == 0 && threadIdx.x == 0) {
    // Other CTAs read either the raw or the clamped count; both clamp to the same n.
    for (int s = 0; s < P.steps; ++s) *P.batch[s].d_count = min(B->count[s], P.batch_cap);
  }
  auto batch_records = [&](int s) { return min(min(B->count[s], P.batch_cap), P.batch[s].capacity); };
  auto tiles_of = [&](uint32_t num_tiles) { return rank < num_tiles ? (num_tiles - rank + G - 1) / G : 0u; };

  // Role state that persists across the batches (mbarrier phases).
  const int ew = warp - 1;   // epilogue warp index (warps 1..8)
  const int h = ew >> 2;     // column half of the epilogue warp
  const int q = warp & 3;    // TMEM lane quadrant
  const int row = q * 32 + lane;
  const bool leader = ew == 0 && lane == 0;
  const uint32_t lane_base = tmem + (static_cast<uint32_t>(q * 32) << 16);
  const uint32_t a_lane = lane_base + kACol + 16 * h;
  const uint32_t d_lane = lane_base + kDCol + 32 * h;
  uint32_t ph_a = 0, ph_d = 0;  // MMA warp / epilogue d_ready phases
  uint32_t ph_g = 0;            // MMA warp: g_ready phase
  uint32_t ct = 0;              // tiles this CTA has processed over all batches
  uint32_t wloads = 0;          // weight loads issued to this CTA
  uint32_t barriers = 0;        // grid barriers passed
  bool ok = true;
  bool prefetched = false;      // the batch's first tile is already encoded and published
  float target[3] = {0.f, 0.f, 0.f};
  double loss_local = 0.0;
  uint32_t loss_n = 0;
  const AdamHyper hp{P.lr, P.beta1, P.beta2, P.eps, P.ema_alpha, P.loss_scale, P.use_ema};

  // Bulk copies of a batch's first two record tiles into the two stages.
  auto issue_first_tiles = [&](const TrainBatch& bt, uint32_t n, uint32_t my_tiles) {
    for (uint32_t k = 0; k < 2 && k < my_tiles; ++k) {
      const uint32_t s = (ct + k) & 1;
      issue_train_tile(bt.records, rank + k * G, n, stage + s * kTRecTileBytes, &B->rec_full[s]);
    }
  };
  // The next MMA's A operand is in TMEM: hand it to the MMA warp, one arrival
  // per warp. Shared-memory rows written after this (the weight-gradient
  // operands) are published by the next release_smem.
  auto release_tmem = [&]() {
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&B->a_ready);
  };
  // Every shared-memory operand row this thread wrote so far (activations, the
  // gradient just stored) is visible to the tensor core: one arrival per warp.
  auto release_smem = [&]() {
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&B->g_ready);
  };
  // Epilogue warps: records of the CTA's tile `it` -> target, and the encoded
  // input act_0 in shared memory and TMEM, published to the MMA warp.
  auto prep_tile = [&](const TrainBatch& bt, uint32_t n, uint32_t it, uint32_t my_tiles) -> bool {
    const uint32_t tile = rank + it * G;
    const bool valid = row < static_cast<int>(min(static_cast<uint32_t>(kTile), n - tile * kTile));
    const uint32_t s = ct & 1, use = ct >> 1;  // stage and its use count
    if (!warp_all(mbar_wait(&B->rec_full[s], use & 1, kWaitLimitNs))) return false;
    float r[kInFloats];
    {
      const float4* src = reinterpret_cast<const float4*>(stage + s * kTRecTileBytes + row * kTRecBytes);
      float f[20];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const float4 v = valid ? src[k] : make_float4(0.f, 0.f, 0.f, 0.f);
        f[4 * k] = v.x;
        f[4 * k + 1] = v.y;
        f[4 * k + 2] = v.z;
        f[4 * k + 3] = v.w;
      }
      target[0] = f[0];
      target[1] = f[1];
      target[2] = f[2];
#pragma unroll
      for (int k = 0; k < kInFloats; ++k) r[k] = f[6 + k];
    }
    mbar_arrive(&B->rec_empty[s]);
    if (leader && it + 2 < my_tiles) {
      if (mbar_wait(&B->rec_empty[s], use & 1, kWaitLimitNs))
        issue_train_tile(bt.records, tile + 2 * G, n, stage + s * kTRecTileBytes, &B->rec_full[s]);
      else
        atomicOr(P.err, kErrTimeout);
    }
    __syncwarp();
    // the previous tile's last MMAs read act_0 and the gradient buffers
    if (it > 0) {
      if (!warp_all(mbar_wait(&B->tile_done, (ct - 1) & 1, kWaitLimitNs))) return false;
      tc_fence_after();
    }
    uint32_t e[16];
    if (h == 0)
      encode_half0<kBF16>(r, e);
    else
      encode_half1<kBF16>(r, e);
    if (!valid) {
#pragma unroll
      for (int k = 0; k < 16; ++k) e[k] = 0u;
    }
    if (P.amax != nullptr && h == 1) {
      // largest encoded feature (FP8 query scales): 1 for the frequency and
      // one-blob features and the constants, else an albedo
      float m = 1.0f;
#pragma unroll
      for (int k = 8; k < 14; ++k) m = fmaxf(m, valid ? fabsf(r[k]) : 0.0f);
      amax_record(P.amax, m);
    }
    tmem_st16(a_lane, e);
    release_tmem();
    store_half(act, row, h, e);  // read by dW_0 at the end of the backward pass
    return true;
  };

  if (leader && P.steps > 0) {
    const uint32_t n0 = batch_records(0);
    issue_first_tiles(P.batch[0], n0, tiles_of((n0 + kTile - 1) / kTile));
  }

  for (int step = 0; step < P.steps && ok; ++step) {
    const TrainBatch bt = P.batch[step];
    const uint32_t n = batch_records(step);
    const uint32_t num_tiles = (n + kTile - 1) / kTile;
    const uint32_t my_tiles = tiles_of(num_tiles);
    if (P.mode == kTrainStep && n > 0) {  // the optimizer phase updates exactly when records were processed
      st.t += 1;
      st.beta1_t *= P.beta1;
      st.beta2_t *= P.beta2;
      st.alpha_t_1 = st.alpha_t;
      st.alpha_t *= P.ema_alpha;
    }
    if (threadIdx.x == 0 && my_tiles > 0) stage_weights_tma(smem_w, &wmap, &B->w_full);

    if (warp == 0) {
      // ---------------------------------------------------- MMA issuer --
      // The whole warp runs the schedule (converged, so descriptors stay
      // warp-uniform); one elected lane issues each group of MMAs.
      const uint32_t id_fwd = idesc_16_f32(128, 64, 0, 0, kBF16);
      const uint32_t id_out = idesc_16_f32(128, 16, 0, 0, kBF16);
      const uint32_t id_dw = idesc_16_f32(64, 64, 1, 1, kBF16);
      const uint32_t id_da = idesc_16_f32(128, 64, 0, 1, kBF16);
      const uint32_t dcol = tmem + kDCol, acol = tmem + kACol;
      // descriptor bases; +1 in the address field = 16 bytes
      const uint64_t dk_w = sdesc_sw128(smem_u32(smem_w), 16, 1024);    // K-major W_l: + l*512 + 2j
      const uint64_t dm_g = sdesc_sw128(smem_u32(gbuf), 8192, 1024);    // MN-major g: + buf*1024 + 128j
      const uint64_t dm_act = sdesc_sw128(smem_u32(act), 8192, 1024);   // MN-major act_l: + l*1024 + 128j
      const uint64_t dm_w = sdesc_sw128(smem_u32(smem_w), 8192, 1024);  // MN-major W_l: + l*512 + 128j
      auto wait_a = [&]() {
        if (!ok) return;
        ok = warp_all(mbar_wait(&B->a_ready, ph_a, kWaitLimitNs));
        if (!ok) return;
        ph_a ^= 1u;
        tc_fence_after();
      };
      if (my_tiles > 0) ok = ok && warp_all(mbar_wait(&B->w_full, wloads & 1, kWaitLimitNs));
      for (uint32_t it = 0; it < my_tiles && ok; ++it) {
        wait_a();  // act_0
        for (int l = 0; l < 6 && ok; ++l) {
          if (elect_one()) {
            const uint64_t w = dk_w + static_cast<uint64_t>(l * 512);
            const uint32_t id = l < 5 ? id_fwd : id_out;
            mma_ts(dcol, acol + 0, w + 0, id, 0u);
            mma_ts(dcol, acol + 8, w + 2, id, 1u);
            mma_ts(dcol, acol + 16, w + 4, id, 1u);
            mma_ts(dcol, acol + 24, w + 6, id, 1u);
            mma_commit(&B->d_ready);
          }
          __syncwarp();
          wait_a();  // act_{l+1}, or g_6 after the output layer
        }
        // backward: g_{l+1} lives in gradient buffer (5 - l) & 1
        for (int l = 5; l >= 0 && ok; --l) {
          const uint64_t gb = static_cast<uint64_t>(((5 - l) & 1) * 1024);
          if (l > 0) {
            if (elect_one()) {
              // dA_l = g W_l  (K = 64 outputs, or 16 for the padded output layer)
              const uint64_t wm = dm_w + static_cast<uint64_t>(l * 512);
              mma_ts(dcol, acol + 0, wm + 0, id_da, 0u);
              if (l < 5) {
                mma_ts(dcol, acol + 8, wm + 128, id_da, 1u);
                mma_ts(dcol, acol + 16, wm + 256, id_da, 1u);
                mma_ts(dcol, acol + 24, wm + 384, id_da, 1u);
              }
              mma_commit(&B->d_ready);
            }
            __syncwarp();
          }
          // the weight gradient reads g_{l+1}'s shared-memory rows (and act_l),
          // written after the TMEM copy that dA_l reads
          ok = warp_all(mbar_wait(&B->g_ready, ph_g, kWaitLimitNs));
          if (!ok) break;
          ph_g ^= 1u;
          tc_fence_after();
          if (elect_one()) {
            // dW_l += g^T act_l   (M = 64 outputs, N = 64 inputs, K = 128 records);
            // complete by the next d_ready (or tile_done for l = 0)
            const uint64_t ga = dm_g + gb, ab = dm_act + static_cast<uint64_t>(l * 1024);
            const uint32_t dw = tmem + 64 * l;
            mma_ss(dw, ga + 0, ab + 0, id_dw, it > 0 ? 1u : 0u);
#pragma unroll
            for (int j = 1; j < 8; ++j) mma_ss(dw, ga + 128 * j, ab + 128 * j, id_dw, 1u);
            if (l == 0) mma_commit(&B->tile_done);
          }
          __syncwarp();
          if (l > 0) wait_a();  // g_l
        }
      }
      ct += my_tiles;
    } else {
      // ------------------------------------------------------ epilogue --
      auto wait_d = [&]() -> bool {
        ok = ok && warp_all(mbar_wait(&B->d_ready, ph_d, kWaitLimitNs));
        ph_d ^= 1u;
        tc_fence_after();
        return ok;
      };
      for (uint32_t it = 0; it < my_tiles && ok; ++it, ++ct) {
        const uint32_t tile = rank + it * G;
        const uint32_t rows_valid = min(static_cast<uint32_t>(kTile), n - tile * kTile);
        const bool valid = row < static_cast<int>(rows_valid);
        const bool last = it + 1 == my_tiles;
        if (!(it == 0 && prefetched)) {
          ok = prep_tile(bt, n, it, my_tiles);
          if (!ok) break;
        }
        prefetched = false;
        // forward: act_{l+1} = fp16(relu(W_l act_l))
        for (int l = 0; l < 5; ++l) {
          if (!wait_d()) break;
          uint32_t v[32], p[16];
          tmem_ld32(d_lane, v);
#pragma unroll
          for (int j = 0; j < 16; ++j)
            p[j] = pack2_relu<kBF16>(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
          tmem_st16(a_lane, p);
          release_tmem();
          store_half(act + (l + 1) * kActBytes, row, h, p);  // read by dW_{l+1}
          if (P.amax != nullptr) {  // largest input of layer l + 1 (FP8 query scales)
            float m = 0.0f;
#pragma unroll
            for (int j = 0; j < 32; ++j) m = fmaxf(m, __uint_as_float(v[j]));
            amax_record(P.amax + l + 1, m);
          }
        }
        if (!ok) break;
        // output + relative-L2 luminance loss gradient (NN_nv.glsl:178-196), fp16;
        // outputs 3..63 of the gradient row are zero (the output layer's padding)
        if (!wait_d()) break;
        {
          uint32_t gw[16];
#pragma unroll
          for (int k = 0; k < 16; ++k) gw[k] = 0u;
          if (h == 0) {
            uint32_t o4[4];
            tmem_ld4(lane_base + kDCol, o4);
            const float p0 = __uint_as_float(o4[0]), p1 = __uint_as_float(o4[1]), p2 = __uint_as_float(o4[2]);
            float d[3];
            const float den = rel_l2_grad(p0, p1, p2, target, P.loss_scale, d);
            if (valid) {
              loss_row<kBF16>(d, gw);
              if (P.loss_acc != nullptr) {
                const double dd = static_cast<double>(den);
                const double e0 = static_cast<double>(p0) - target[0], e1 = static_cast<double>(p1) - target[1],
                             e2 = static_cast<double>(p2) - target[2];
                loss_local += (e0 * e0 + e1 * e1 + e2 * e2) / dd;
                ++loss_n;
              }
            }
            tmem_st16(a_lane, gw);  // dA_5 reads K = 16 (A words 0..7)
          }
          release_tmem();
          store_half(gbuf, row, h, gw);  // read by dW_5
          release_smem();                // (with act_0 .. act_5)
        }
        // backward: g_l = fp16((g_{l+1} W_l) masked by act_l > 0), l = 5..1
        for (int l = 5; l >= 1; --l) {
          uint32_t aw[16], gw[16], v[32];
          load_half(act + l * kActBytes, row, h, aw);  // the mask rows, while dA_l runs
          if (!wait_d()) break;
          tmem_ld32(d_lane, v);
#pragma unroll
          for (int j = 0; j < 16; ++j)
            gw[j] = relu_mask2<kBF16>(pack2<kBF16>(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1])), aw[j]);
          tmem_st16(a_lane, gw);
          release_tmem();
          store_half(gbuf + ((6 - l) & 1) * kActBytes, row, h, gw);  // read by dW_{l-1}
          release_smem();
          // dA_l completing means dW_{l+1} (issued before it) is complete too;
          // on the CTA's last tile it is final: write it out while the chain goes on.
          if (last && l <= 4) drain_dw(lane_base, l + 1, q, h, lane, my_partial);
        }
        if (!ok) break;
        if (last) {
          ok = warp_all(mbar_wait(&B->tile_done, ct & 1, kWaitLimitNs));
          if (!ok) break;
          tc_fence_after();
          drain_dw(lane_base, 1, q, h, lane, my_partial);
          drain_dw(lane_base, 0, q, h, lane, my_partial);
        }
      }
    }
    if (my_tiles > 0) ++wloads;
    if (!ok && lane == 0) atomicOr(P.err, kErrTimeout);
    ok = __syncthreads_and(ok) != 0;  // one decision per CTA from here on

    // The record stages are free again: the next batch's first tiles land
    // during the grid barrier and the optimizer phase.
    const bool has_next = step + 1 < P.steps;
    const uint32_t n_next = has_next ? batch_records(step + 1) : 0u;
    const uint32_t tiles_next = tiles_of((n_next + kTile - 1) / kTile);
    if (ok && leader && tiles_next > 0) issue_first_tiles(P.batch[step + 1], n_next, tiles_next);

    // ------------------------------------------- reduction + optimizer --
    if (!grid_sync(P.sync, ++barriers * G, &B->sync_ok)) {
      ok = false;
      if (threadIdx.x == 0) atomicOr(P.err, kErrTimeout);
      break;
    }
    // Gather this CTA's slice of every partial (one per CTA that had tiles)
    // behind act_0, many 16-byte copies in flight per thread.
    float4* stg = reinterpret_cast<float4*>(act + kActBytes);  // [active][ncols]
    const uint32_t active = min(G, num_tiles);
    const bool reduce = n > 0 && ncols > 0;
    if (reduce) {
      const uint32_t total = active * ncols;
      for (uint32_t i = threadIdx.x; i < total; i += blockDim.x) {
        const uint32_t r = i / ncols, cc = i - r * ncols;
        cp_async16(stg + i, P.partials + static_cast<size_t>(r) * kParams + 4 * (c0 + cc));
      }
      cp_async_commit();
    }
    // Meanwhile the epilogue warps encode the next batch's first tile into act_0.
    if (ok && warp > 0 && tiles_next > 0) {
      prefetched = prep_tile(P.batch[step + 1], n_next, 0, tiles_next);
      if (!prefetched) {
        ok = false;
        if (lane == 0) atomicOr(P.err, kErrTimeout);
      }
    }
    if (reduce) cp_async_wait_all();
    ok = __syncthreads_and(ok) != 0;
    if (ok && reduce) {
      // Four threads per float4 column sum every fourth partial, then combine
      // as (s0 + s1) + (s2 + s3): a fixed order, so runs are identical. Thread
      // `part` then owns parameter 4 * column + part.
      const uint32_t part = threadIdx.x & 3;
      uint16_t* use16 = bt.write_use ? reinterpret_cast<uint16_t*>(P.use16) : nullptr;
      for (uint32_t cb = 0; cb < ncols; cb += kTrainThreads / 4) {
        const uint32_t cc = cb + (threadIdx.x >> 2);
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        if (cc < ncols) {
          for (uint32_t r = part; r < active; r += 4) {
            const float4 v = stg[static_cast<size_t>(r) * ncols + cc];
            acc.x += v.x;
            acc.y += v.y;
            acc.z += v.z;
            acc.w += v.w;
          }
        }
#pragma unroll
        for (int off = 1; off <= 2; off <<= 1) {
          acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
          acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
          acc.z += __shfl_xor_sync(0xffffffffu, acc.z, off);
          acc.w += __shfl_xor_sync(0xffffffffu, acc.w, off);
        }
        if (cc < ncols) {
          const float gsum = part == 0 ? acc.x : part == 1 ? acc.y : part == 2 ? acc.z : acc.w;
          const uint32_t k = 4 * cc + part;  // parameter index within the slice
          if (P.mode == kTrainStep) {
            nrc_optimizer_entry e = cached ? ecache[k] : P.entries[4 * c0 + k];
            adam_one<kBF16>(4 * c0 + k, gsum, n, st, hp, e, P.entries, reinterpret_cast<uint16_t*>(P.w16), use16);
            if (cached) ecache[k] = e;
          } else
            P.grad_out[4 * c0 + k] = gsum;
        }
      }
    } else if (ok && P.mode == kGradientOnly) {
      for (uint32_t k = threadIdx.x; k < 4 * ncols; k += blockDim.x) P.grad_out[4 * c0 + k] = 0.0f;  // no records
    }
    if (has_next) {  // publish the new weights before the next batch loads them
      if (!grid_sync(P.sync, ++barriers * G, &B->sync_ok)) {
        ok = false;
        if (threadIdx.x == 0) atomicOr(P.err, kErrTimeout);
        break;
      }
    }
  }
  cp_async_wait_all();  // entry loads of a launch whose batches were all empty
  // Every CTA has read the step state at launch and passed at least one grid
  // barrier since, so CTA 0 may now write the advanced state.
  if (P.mode == kTrainStep && ok && barriers > 0 && rank == 0 && threadIdx.x == 0) *P.state = st;

  if (P.loss_acc != nullptr && warp > 0) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      loss_local += __shfl_xor_sync(0xffffffffu, loss_local, off);
      loss_n += __shfl_xor_sync(0xffffffffu, loss_n, off);
    }
    if (lane == 0 && loss_n > 0) {
      atomicAdd(P.loss_acc, loss_local);
      atomicAdd(P.loss_count, static_cast<unsigned long long>(loss_n));
    }
  }
  // all issued MMAs must be complete before TMEM is released
  if (warp == 0) {
    if (elect_one()) mma_commit(&B->drain);
    __syncwarp();
    if (!warp_all(mbar_wait(&B->drain, 0, kWaitLimitNs)) && lane == 0) atomicOr(P.err, kErrTimeout);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
  // The group's barrier counter (sync[0]) starts every launch at zero: the last
  // CTA of the group to get here, when every CTA has left its barrier waits,
  // resets it and the exit counter (sync[1]).
  if (threadIdx.x == 0) {
    __threadfence();
    B->sync_ok = atomicAdd(P.sync + 1, 1u) == G - 1 ? 1u : 0u;
    if (B->sync_ok != 0u) {
      atomicExch(P.sync, 0u);
      atomicExch(P.sync + 1, 0u);
      __threadfence();
    }
  }
  // the overlapped frame: the group's last CTA out joins the frame (every CTA's
  // weight writes are complete and fenced by now)
  if (P.join.src != nullptr) {
    __syncthreads();
    if (B->sync_ok != 0u) join_copy(P.join, threadIdx.x, blockDim.x);
  }
}

template <int N, bool kBF16>
__global__ void __launch_bounds__(kTrainThreads, 1) train_steps_kernel(const __grid_constant__ TrainLaunch<N> L) {
  train_body<N, kBF16, false>(L);
}

// The batched training over a launch table in global memory.
__global__ void __launch_bounds__(kTrainThreads, 1)
    train_table_kernel(const TrainLaunch<kMaxTrainJobs>* __restrict__ L) {
  train_body<kMaxTrainJobs, false, true>(*L);
}

template <int N>
cudaError_t launch(const TrainLaunch<N>& L, uint32_t grid, cudaStream_t stream, bool bf16) {
  // Cooperative (the grid barrier needs every CTA resident) and a programmatic
  // dependent of the preceding kernel: the launch is issued before that kernel
  // ends, its CTAs take SMs as the preceding kernel's CTAs leave, and
  // griddepcontrol.wait holds them until it has completed.
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kTrainThreads);
  cfg.dynamicSmemBytes = kTrainSmemBytes;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  return bf16 ? cudaLaunchKernelEx(&cfg, train_steps_kernel<N, true>, L)
              : cudaLaunchKernelEx(&cfg, train_steps_kernel<N, false>, L);
}

}  // namespace

cudaError_t configure_train_kernels() {
  const void* k[5] = {reinterpret_cast<const void*>(train_steps_kernel<1, false>),
                      reinterpret_cast<const void*>(train_steps_kernel<kMaxTrainJobs, false>),
                      reinterpret_cast<const void*>(train_steps_kernel<1, true>),
                      reinterpret_cast<const void*>(train_steps_kernel<kMaxTrainJobs, true>),
                      reinterpret_cast<const void*>(train_table_kernel)};
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 5 && e == cudaSuccess; ++i)
    if ((e = cudaFuncSetAttribute(k[i], cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmemBytes)) == cudaSuccess)
      e = cudaFuncSetAttribute(k[i], cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  return e;
}

uint32_t train_smem_bytes() { return kTrainSmemBytes; }

// One CTA per SM up to kMaxTrainCtas, whatever the batch sizes: CTAs without
// tiles in a batch still own a slice of the parameters in its optimizer phase.
uint32_t train_grid(const TrainParams&, int max_ctas) {
  return static_cast<uint32_t>(max_ctas) < kMaxTrainCtas ? static_cast<uint32_t>(max_ctas) : kMaxTrainCtas;
}

cudaError_t launch_train(const TrainParams& p, const CUtensorMap* wmap, int max_ctas, cudaStream_t stream) {
  if (p.steps < 1 || p.steps > NRC_TRAIN_BATCH_COUNT) return cudaErrorInvalidValue;
  const uint32_t grid = train_grid(p, max_ctas);
  if (grid < 1) return cudaErrorInvalidConfiguration;
  TrainLaunch<1> L;
  L.job[0].wmap = *wmap;
  L.job[0].p = p;
  L.group_start[0] = 0;
  L.group_start[1] = grid;
  L.njobs = 1;
  return launch(L, grid, stream, p.bf16 != 0);
}

cudaError_t launch_train_table(const TrainLaunch<kMaxTrainJobs>* table, uint32_t grid, bool cooperative,
                               cudaStream_t stream) {
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeCooperative;
  attr.val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kTrainThreads);
  cfg.dynamicSmemBytes = kTrainSmemBytes;
  cfg.stream = stream;
  cfg.attrs = &attr;
  cfg.numAttrs = cooperative ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, train_table_kernel, table);
}

cudaError_t launch_train_many(const TrainJob* jobs, int njobs, const uint32_t* group_size, cudaStream_t stream) {
  if (njobs < 1 || njobs > kMaxTrainJobs) return cudaErrorInvalidValue;
  static TrainLaunch<kMaxTrainJobs> L;  // host staging of the kernel parameters (copied at launch)
  static std::mutex m;
  std::lock_guard<std::mutex> lock(m);
  uint32_t grid = 0;
  for (int j = 0; j < njobs; ++j) {
    if (jobs[j].p.steps < 1 || jobs[j].p.steps > NRC_TRAIN_BATCH_COUNT) return cudaErrorInvalidValue;
    if (jobs[j].p.bf16 != jobs[0].p.bf16) return cudaErrorInvalidValue;  // one operand format per launch
    if (group_size[j] < 1 || group_size[j] > kMaxTrainCtas) return cudaErrorInvalidConfiguration;
    L.job[j] = jobs[j];
    L.group_start[j] = grid;
    grid += group_size[j];
  }
  L.group_start[njobs] = grid;
  L.njobs = njobs;
  return launch(L, grid, stream, jobs[0].p.bf16 != 0);
}

}  // namespace nrc
