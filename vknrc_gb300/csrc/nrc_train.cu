// Fused training step: record tile (bulk copy) -> encode -> forward keeping all
// six activations -> relative-L2 loss gradient -> backward -> weight gradients,
// then the Adam/EMA update.
//
// Follows shader/src/nrc_gradient.comp:26-58 with NN_nv.glsl's backward
// (NNLoadDA3_RelativeL2LuminanceLoss :178-196, NNBackwardDA3/64_ReLU :222-278,
// NNUpdateDW3/64 :280-367), nrc_train_prepare.comp:16-29 and
// nrc_optimize.comp:32-54, re-laid out for tcgen05:
//   - activations act_0..act_5 (fp16, 128 x 64 per tile) stay in shared memory
//     as 128-byte-swizzled rows; the same tile is the K-major A operand of the
//     next forward layer and the MN-major B operand of that layer's weight
//     gradient, so nothing is transposed or copied;
//   - dA = (g W) masked by act > 0 uses the weight tile itself as an MN-major B
//     operand (the reference's NaN-mask trick becomes a select in the epilogue);
//   - dW_l += g^T act_l is an M=64 MMA (K = records) accumulated in TMEM across
//     every tile the CTA processes, so the cross-CTA reduction happens once per
//     CTA: fp32 vector atomics, or per-CTA partials summed in a fixed order by
//     the optimizer kernel (deterministic mode);
//   - the count clamp and step-state advance (the reference's prepare pass) run
//     in CTA 0 of the gradient kernel; the optimizer kernel zeroes the gradient
//     accumulator after reading it, replacing the reference's clear pass.
#include "nrc_common.cuh"
#include "nrc_kernels.h"

namespace nrc {

namespace {

constexpr int kTrainThreads = 32 + 128;
constexpr uint32_t kTRecBytes = sizeof(nrc_train_record);  // 80
constexpr uint32_t kTRecTileBytes = kTile * kTRecBytes;     // 10240
constexpr uint32_t kActBytes = kTile * 128;                 // 16384: 128 rows x 64 fp16
constexpr uint32_t kActOff = kWeightSmemBytes;              // 43008
constexpr uint32_t kGOff = kActOff + 6 * kActBytes;         // two gradient buffers
constexpr uint32_t kStageOff = kGOff + 2 * kActBytes;
constexpr uint32_t kTBarOff = kStageOff + 2 * kTRecTileBytes;
constexpr uint32_t kTrainSmemBytes = kTBarOff + 128 + 1024;
static_assert(kActOff % 1024 == 0 && kGOff % 1024 == 0 && kStageOff % 16 == 0, "alignment");
static_assert(kTrainSmemBytes <= 227 * 1024, "shared memory");

// TMEM columns: dW_l accumulators (M=64 layout) at 64*l, l = 0..5; scratch D at 384.
constexpr uint32_t kDCol = 384;

struct TrainBars {
  uint64_t rec_full[2];
  uint64_t rec_empty[2];
  uint64_t a_ready;    // 128 arrivals: the next operand tile is in shared memory
  uint64_t d_ready;    // MMA commit: scratch accumulator ready
  uint64_t tile_done;  // MMA commit after the tile's last weight-gradient MMA
  uint64_t drain;
};

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

// fp16 bit pattern strictly positive (finite or +inf), i.e. act > 0 in the reference.
__device__ __forceinline__ bool h_pos(uint32_t bits16) { return ((bits16 - 1u) & 0xFFFFu) < 0x7C00u; }

// Store one 128-byte row (32 words) of a swizzled operand tile.
__device__ __forceinline__ void store_row(uint8_t* tile, int row, const uint32_t (&w)[32]) {
#pragma unroll
  for (int c = 0; c < 8; ++c)
    *reinterpret_cast<uint4*>(tile + sw128_offset(row, c)) = make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
}

__device__ __forceinline__ void load_row(const uint8_t* tile, int row, uint32_t (&w)[32]) {
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const uint4 v = *reinterpret_cast<const uint4*>(tile + sw128_offset(row, c));
    w[4 * c] = v.x;
    w[4 * c + 1] = v.y;
    w[4 * c + 2] = v.z;
    w[4 * c + 3] = v.w;
  }
}

__global__ void __launch_bounds__(kTrainThreads, 1)
    train_grad_kernel(const nrc_train_record* __restrict__ records, uint32_t* __restrict__ d_count,
                      uint32_t capacity, uint32_t batch_cap, const __half* __restrict__ w16, float* __restrict__ grad,
                      float* __restrict__ partials, nrc_optimizer_state* __restrict__ state, float loss_scale,
                      float beta1, float beta2, float ema_alpha, int do_prepare, double* loss_acc,
                      unsigned long long* loss_count, uint32_t* err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* smem_w = smem;
  uint8_t* act = smem + kActOff;
  uint8_t* gbuf = smem + kGOff;
  uint8_t* stage = smem + kStageOff;
  TrainBars* B = reinterpret_cast<TrainBars*>(smem + kTBarOff);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(B + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t raw = *d_count;
  const uint32_t clamped = min(raw, batch_cap);
  const uint32_t n = min(clamped, capacity);
  const uint32_t num_tiles = (n + kTile - 1) / kTile;

  if (threadIdx.x == 0) {
    mbar_init(&B->rec_full[0], 1);
    mbar_init(&B->rec_full[1], 1);
    mbar_init(&B->rec_empty[0], 128);
    mbar_init(&B->rec_empty[1], 128);
    mbar_init(&B->a_ready, 128);
    mbar_init(&B->d_ready, 1);
    mbar_init(&B->tile_done, 1);
    mbar_init(&B->drain, 1);
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
  // Every CTA has read the count above; CTA 0 now plays nrc_train_prepare.comp.
  // Other CTAs may still read the count concurrently: they see either the raw or
  // the clamped value, and both clamp to the same n.
  if (do_prepare && blockIdx.x == 0 && threadIdx.x == 0) {
    *d_count = clamped;
    if (n > 0) {  // the optimizer kernel updates exactly when records were processed
      nrc_optimizer_state st = *state;
      st.t += 1;
      st.beta1_t *= beta1;
      st.beta2_t *= beta2;
      st.alpha_t_1 = st.alpha_t;
      st.alpha_t *= ema_alpha;
      *state = st;
    }
  }

  if (warp == 0) {
    // ------------------------------------------------------ MMA issuer --
    // The whole warp runs the schedule (converged, so descriptors stay
    // warp-uniform); one elected lane issues each group of MMAs.
    bool ok = true;
    uint32_t ph_a = 0;
    const uint32_t tm = __shfl_sync(0xffffffffu, tmem, 0);
    const uint32_t id_fwd = idesc_f16_f32(128, 64, 0, 0);
    const uint32_t id_out = idesc_f16_f32(128, 16, 0, 0);
    const uint32_t id_dw = idesc_f16_f32(64, 64, 1, 1);
    const uint32_t id_da = idesc_f16_f32(128, 64, 0, 1);
    const uint32_t dcol = tm + kDCol;
    // descriptor bases; +1 in the address field = 16 bytes
    const uint64_t dk_act = sdesc_sw128(smem_u32(act), 16, 1024);   // K-major act_l: + l*1024 + 2j
    const uint64_t dk_w = sdesc_sw128(smem_u32(smem_w), 16, 1024);  // K-major W_l: + l*512 + 2j
    const uint64_t dm_g = sdesc_sw128(smem_u32(gbuf), 8192, 1024);  // MN-major g: + buf*1024 + 128j
    const uint64_t dk_g = sdesc_sw128(smem_u32(gbuf), 16, 1024);    // K-major g: + buf*1024 + 2j
    const uint64_t dm_act = sdesc_sw128(smem_u32(act), 8192, 1024); // MN-major act_l: + l*1024 + 128j
    const uint64_t dm_w = sdesc_sw128(smem_u32(smem_w), 8192, 1024); // MN-major W_l: + l*512 + 128j
    auto wait_a = [&]() {
      if (!ok) return;
      ok = warp_all(mbar_wait(&B->a_ready, ph_a, kWaitLimitNs));
      if (!ok) return;
      ph_a ^= 1u;
      tc_fence_after();
    };
    uint32_t it = 0;
    for (uint32_t tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x, ++it) {
      wait_a();  // act_0
      for (int l = 0; l < 6 && ok; ++l) {
        if (elect_one()) {
          const uint64_t a = dk_act + static_cast<uint64_t>(l * 1024), w = dk_w + static_cast<uint64_t>(l * 512);
          const uint32_t id = l < 5 ? id_fwd : id_out;
          mma_ss(dcol, a + 0, w + 0, id, 0u);
          mma_ss(dcol, a + 2, w + 2, id, 1u);
          mma_ss(dcol, a + 4, w + 4, id, 1u);
          mma_ss(dcol, a + 6, w + 6, id, 1u);
          mma_commit(&B->d_ready);
        }
        __syncwarp();
        wait_a();  // act_{l+1}, or g_6 after the output layer
      }
      // backward: g_{l+1} lives in gradient buffer (5 - l) & 1
      for (int l = 5; l >= 0 && ok; --l) {
        const uint64_t gb = static_cast<uint64_t>(((5 - l) & 1) * 1024);
        if (elect_one()) {
          // dW_l += g^T act_l   (M = 64 outputs, N = 64 inputs, K = 128 records)
          const uint64_t ga = dm_g + gb, ab = dm_act + static_cast<uint64_t>(l * 1024);
          const uint32_t acc0 = it > 0 ? 1u : 0u;
          const uint32_t dw = tm + 64 * l;
          mma_ss(dw, ga + 0, ab + 0, id_dw, acc0);
#pragma unroll
          for (int j = 1; j < 8; ++j) mma_ss(dw, ga + 128 * j, ab + 128 * j, id_dw, 1u);
          if (l > 0) {
            // dA_l = g W_l  (K = 64 outputs, or 16 for the padded output layer)
            const uint64_t gk = dk_g + gb, wm = dm_w + static_cast<uint64_t>(l * 512);
            mma_ss(dcol, gk + 0, wm + 0, id_da, 0u);
            if (l < 5) {
              mma_ss(dcol, gk + 2, wm + 128, id_da, 1u);
              mma_ss(dcol, gk + 4, wm + 256, id_da, 1u);
              mma_ss(dcol, gk + 6, wm + 384, id_da, 1u);
            }
            mma_commit(&B->d_ready);
          } else {
            mma_commit(&B->tile_done);
          }
        }
        __syncwarp();
        if (l > 0) wait_a();  // g_l
      }
    }
    if (!ok && lane == 0) atomicOr(err, kErrTimeout);
    // all issued MMAs must be complete before TMEM is released
    if (elect_one()) mma_commit(&B->drain);
    __syncwarp();
    if (!warp_all(mbar_wait(&B->drain, 0, kWaitLimitNs)) && lane == 0) atomicOr(err, kErrTimeout);
  } else {
    // ------------------------------------------------ epilogue warpgroup --
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const bool leader = warp == 1 && lane == 0;
    const uint32_t lane_base = tmem + (static_cast<uint32_t>(q * 32) << 16);
    bool ok = true;
    uint32_t ph_d = 0;
    double loss_local = 0.0;
    uint32_t loss_n = 0;
    if (leader) {
      for (uint32_t b = 0; b < 2; ++b) {
        const uint32_t t = blockIdx.x + b * gridDim.x;
        if (t < num_tiles) issue_train_tile(records, t, n, stage + b * kTRecTileBytes, &B->rec_full[b]);
      }
    }
    auto wait_d = [&]() -> bool {
      ok = ok && warp_all(mbar_wait(&B->d_ready, ph_d, kWaitLimitNs));
      ph_d ^= 1u;
      tc_fence_after();
      return ok;
    };
    auto publish = [&]() {  // operand tile rows written: hand them to the tensor core
      fence_proxy_async_smem();
      tc_fence_before();
      mbar_arrive(&B->a_ready);
    };
    uint32_t it = 0;
    for (uint32_t tile = blockIdx.x; tile < num_tiles && ok; tile += gridDim.x, ++it) {
      const uint32_t rows_valid = min(static_cast<uint32_t>(kTile), n - tile * kTile);
      const bool valid = row < static_cast<int>(rows_valid);
      const uint32_t b = it & 1;
      ok = warp_all(mbar_wait(&B->rec_full[b], (it >> 1) & 1, kWaitLimitNs));
      if (!ok) break;
      float r[kInFloats], target[3];
      {
        const float4* src = reinterpret_cast<const float4*>(stage + b * kTRecTileBytes + row * kTRecBytes);
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
      mbar_arrive(&B->rec_empty[b]);
      if (leader && blockIdx.x + (it + 2) * gridDim.x < num_tiles) {
        if (mbar_wait(&B->rec_empty[b], (it >> 1) & 1, kWaitLimitNs))
          issue_train_tile(records, blockIdx.x + (it + 2) * gridDim.x, n, stage + b * kTRecTileBytes,
                           &B->rec_full[b]);
        else
          atomicOr(err, kErrTimeout);
      }
      __syncwarp();
      // the previous tile's last MMAs read act_0 and the gradient buffers
      if (it > 0) {
        ok = warp_all(mbar_wait(&B->tile_done, (it - 1) & 1, kWaitLimitNs));
        if (!ok) break;
        tc_fence_after();
      }
      {
        uint32_t e[32];
        encode_input(r, e);
        if (!valid) {
#pragma unroll
          for (int k = 0; k < 32; ++k) e[k] = 0u;
        }
        store_row(act, row, e);
      }
      publish();
      // forward: act_{l+1} = fp16(relu(W_l act_l))
      for (int l = 0; l < 5; ++l) {
        if (!wait_d()) break;
        uint32_t v[32], p[32];
        tmem_ld32(lane_base + kDCol, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) p[j] = pack_relu_f16x2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
        tmem_ld32(lane_base + kDCol + 32, v);
#pragma unroll
        for (int j = 0; j < 16; ++j)
          p[16 + j] = pack_relu_f16x2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
        store_row(act + (l + 1) * kActBytes, row, p);
        publish();
      }
      if (!ok) break;
      // output + relative-L2 luminance loss gradient (NN_nv.glsl:178-196), fp16
      if (!wait_d()) break;
      {
        uint32_t o4[4];
        tmem_ld4(lane_base + kDCol, o4);
        const float p0 = __uint_as_float(o4[0]), p1 = __uint_as_float(o4[1]), p2 = __uint_as_float(o4[2]);
        const float lum = __fmaf_rn(0.114f, fmaxf(p2, 0.0f), __fmaf_rn(0.587f, fmaxf(p1, 0.0f), __fmul_rn(0.299f, fmaxf(p0, 0.0f))));
        const float den = __fmaf_rn(lum, lum, 0.01f);
        const float s2 = __fmul_rn(2.0f, loss_scale);
        const float d0 = __fdiv_rn(__fmul_rn(s2, __fsub_rn(p0, target[0])), den);
        const float d1 = __fdiv_rn(__fmul_rn(s2, __fsub_rn(p1, target[1])), den);
        const float d2 = __fdiv_rn(__fmul_rn(s2, __fsub_rn(p2, target[2])), den);
        uint32_t gw[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) gw[k] = 0u;
        if (valid) {
          gw[0] = pack_f16x2(d0, d1);
          gw[1] = pack_f16x2(d2, 0.0f);
          if (loss_acc != nullptr) {
            const double dd = static_cast<double>(den);
            const double e0 = static_cast<double>(p0) - target[0], e1 = static_cast<double>(p1) - target[1],
                         e2 = static_cast<double>(p2) - target[2];
            loss_local += (e0 * e0 + e1 * e1 + e2 * e2) / dd;
            ++loss_n;
          }
        }
        store_row(gbuf, row, gw);
        publish();
      }
      // backward: g_l = fp16((g_{l+1} W_l) masked by act_l > 0), l = 5..1
      for (int l = 5; l >= 1; --l) {
        if (!wait_d()) break;
        uint32_t aw[32], gw[32], v[32];
        load_row(act + l * kActBytes, row, aw);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          tmem_ld32(lane_base + kDCol + 32 * h, v);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const uint32_t a2 = aw[16 * h + j];
            float x0 = __uint_as_float(v[2 * j]), x1 = __uint_as_float(v[2 * j + 1]);
            x0 = (h_pos(a2 & 0xFFFFu) && !isnan(x0)) ? x0 : 0.0f;
            x1 = (h_pos(a2 >> 16) && !isnan(x1)) ? x1 : 0.0f;
            gw[16 * h + j] = pack_f16x2(x0, x1);
          }
        }
        store_row(gbuf + ((6 - l) & 1) * kActBytes, row, gw);
        publish();
      }
    }
    // cross-CTA reduction of this CTA's weight gradients
    if (ok && it > 0) {
      ok = warp_all(mbar_wait(&B->tile_done, (it - 1) & 1, kWaitLimitNs));
      tc_fence_after();
      if (ok) {
        const bool has_row = lane < 16;  // M=64 layout: rows 16q+t live in lanes 32q+t, t < 16
        const int o = q * 16 + lane;
        float* dst = partials ? partials + static_cast<size_t>(blockIdx.x) * kParams : grad;
        for (int l = 0; l < 6; ++l) {
          uint32_t v[32];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            tmem_ld32(lane_base + 64 * l + 32 * h, v);
            const bool keep = has_row && (l < 5 || o < kOut);
            if (keep) {
              float4* g4 = reinterpret_cast<float4*>(dst + l * kLayerElems + o * 64 + 32 * h);
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const float4 val = make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]),
                                               __uint_as_float(v[4 * j + 2]), __uint_as_float(v[4 * j + 3]));
                if (partials)
                  g4[j] = val;
                else
                  atomicAdd(g4 + j, val);
              }
            }
          }
        }
      }
    }
    if (loss_acc != nullptr) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        loss_local += __shfl_xor_sync(0xffffffffu, loss_local, off);
        loss_n += __shfl_xor_sync(0xffffffffu, loss_n, off);
      }
      if (lane == 0 && loss_n > 0) {
        atomicAdd(loss_acc, loss_local);
        atomicAdd(loss_count, static_cast<unsigned long long>(loss_n));
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

// nrc_optimize.comp:32-54 over all parameters (one thread each). In
// deterministic mode the per-CTA partial gradients are summed in CTA order;
// otherwise the atomic accumulator is read and zeroed for the next step.
__global__ void __launch_bounds__(256) adam_kernel(const uint32_t* __restrict__ d_count, uint32_t capacity,
                                                   uint32_t batch_cap, float* __restrict__ grad,
                                                   const float* __restrict__ partials, uint32_t grad_ctas,
                                                   nrc_optimizer_entry* __restrict__ entries,
                                                   const nrc_optimizer_state* __restrict__ state,
                                                   __half* __restrict__ w16, __half* __restrict__ use16, float lr,
                                                   float beta1, float beta2, float eps, float ema_alpha,
                                                   float loss_scale, int use_ema) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const uint32_t n = min(min(*d_count, batch_cap), capacity);
  if (n == 0) return;
  float gsum;
  if (partials != nullptr) {
    const uint32_t active = min(grad_ctas, (n + kTile - 1) / kTile);
    gsum = 0.0f;
    for (uint32_t b = 0; b < active; ++b) gsum += partials[static_cast<size_t>(b) * kParams + i];
  } else {
    gsum = grad[i];
    grad[i] = 0.0f;
  }
  const nrc_optimizer_state st = *state;
  float g = __fdiv_rn(__fdiv_rn(gsum, static_cast<float>(n)), loss_scale);
  if (isnan(g) || isinf(g)) g = 0.0f;
  nrc_optimizer_entry e = entries[i];
  const float m = __fmaf_rn(beta1, e.m, __fmul_rn(__fsub_rn(1.0f, beta1), g));
  const float v = __fmaf_rn(beta2, e.v, __fmul_rn(__fsub_rn(1.0f, beta2), __fmul_rn(g, g)));
  const float hm = __fdiv_rn(m, __fsub_rn(1.0f, st.beta1_t));
  const float hv = __fdiv_rn(v, __fsub_rn(1.0f, st.beta2_t));
  const float w = __fsub_rn(e.weight, __fdiv_rn(__fmul_rn(lr, hm), __fadd_rn(__fsqrt_rn(hv), eps)));
  const float eta_t = __fsub_rn(1.0f, st.alpha_t), eta_t1 = __fsub_rn(1.0f, st.alpha_t_1);
  const float ea = __fdiv_rn(__fsub_rn(1.0f, ema_alpha), eta_t), eb = __fmul_rn(ema_alpha, eta_t1);
  const float ema = __fmaf_rn(ea, w, __fmul_rn(eb, e.ema_weight));
  e.m = m;
  e.v = v;
  e.weight = w;
  e.ema_weight = ema;
  entries[i] = e;
  w16[i] = __float2half_rn(w);
  if (use16 != nullptr) use16[i] = __float2half_rn(use_ema ? ema : w);
}

}  // namespace

cudaError_t configure_train_kernels() {
  return cudaFuncSetAttribute(train_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmemBytes);
}

uint32_t train_smem_bytes() { return kTrainSmemBytes; }

uint32_t train_grid(uint32_t capacity, uint32_t batch_cap, int num_sms) {
  const uint32_t cap = capacity < batch_cap ? capacity : batch_cap;
  const uint32_t tiles = (cap + kTile - 1) / kTile;
  return tiles < static_cast<uint32_t>(num_sms) ? tiles : static_cast<uint32_t>(num_sms);
}

cudaError_t launch_train_grad(const nrc_train_record* records, uint32_t* d_count, uint32_t capacity,
                              uint32_t batch_cap, const __half* w16, float* grad, float* partials,
                              nrc_optimizer_state* state, float loss_scale, float beta1, float beta2,
                              float ema_alpha, bool do_prepare, double* loss_acc, unsigned long long* loss_count,
                              uint32_t* err, int num_sms, cudaStream_t stream) {
  uint32_t grid = train_grid(capacity, batch_cap, num_sms);
  if (grid == 0) grid = 1;  // the prepare step still runs on an empty batch
  train_grad_kernel<<<grid, kTrainThreads, kTrainSmemBytes, stream>>>(
      records, d_count, capacity, batch_cap, w16, grad, partials, state, loss_scale, beta1, beta2, ema_alpha,
      do_prepare ? 1 : 0, loss_acc, loss_count, err);
  return cudaGetLastError();
}

cudaError_t launch_adam(const uint32_t* d_count, uint32_t capacity, uint32_t batch_cap, float* grad,
                        const float* partials, uint32_t grad_ctas, nrc_optimizer_entry* entries,
                        const nrc_optimizer_state* state, __half* w16, __half* use16, float lr, float beta1,
                        float beta2, float eps, float ema_alpha, float loss_scale, bool use_ema,
                        cudaStream_t stream) {
  const int threads = 256, blocks = (kParams + threads - 1) / threads;
  adam_kernel<<<blocks, threads, 0, stream>>>(d_count, capacity, batch_cap, grad, partials, grad_ctas, entries, state,
                                              w16, use16, lr, beta1, beta2, eps, ema_alpha, loss_scale,
                                              use_ema ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace nrc
