// Training arithmetic shared by the fused trainer (nrc_train.cu), the
// no-allocation step and the standalone optimizer and loss passes
// (nrc_optimize.cu), so every path computes the reference's update and loss
// gradient with the same operations.
#pragma once
#include "nrc_common.cuh"

namespace nrc {

template <bool kBF16>
__device__ __forceinline__ uint16_t to16(float x) {
  return kBF16 ? __bfloat16_as_ushort(__float2bfloat16_rn(x)) : __half_as_ushort(__float2half_rn(x));
}

// Relative-L2 luminance loss gradient of one record (NN_nv.glsl:178-196):
// d_c = 2 s (p_c - t_c) / (lum(max(p, 0))^2 + 0.01), lum = 0.299 r + 0.587 g +
// 0.114 b, the denominator held constant; p is the unclamped output
// (nrc_gradient.comp:45-46). Returns the denominator. The multiply-adds of lum
// and of the denominator are fused (GLSL leaves contraction to the compiler).
__device__ __forceinline__ float rel_l2_grad(float p0, float p1, float p2, const float (&t)[3], float loss_scale,
                                             float (&d)[3]) {
  const float lum =
      __fmaf_rn(0.114f, fmaxf(p2, 0.0f), __fmaf_rn(0.587f, fmaxf(p1, 0.0f), __fmul_rn(0.299f, fmaxf(p0, 0.0f))));
  const float den = __fmaf_rn(lum, lum, 0.01f);
  const float s2 = __fmul_rn(2.0f, loss_scale);
  d[0] = __fdiv_rn(__fmul_rn(s2, __fsub_rn(p0, t[0])), den);
  d[1] = __fdiv_rn(__fmul_rn(s2, __fsub_rn(p1, t[1])), den);
  d[2] = __fdiv_rn(__fmul_rn(s2, __fsub_rn(p2, t[2])), den);
  return den;
}

// The first two words of the 16-bit gradient row (d0 | d1 << 16, d2 | 0 << 16),
// rounded to nearest even as packHalf2x16 does; beyond the format's range a
// value becomes inf (NN_nv.glsl:185-186). The other 14 halves of the row are 0.
template <bool kBF16>
__device__ __forceinline__ void loss_row(const float (&d)[3], uint32_t* w) {
  w[0] = pack2<kBF16>(d[0], d[1]);
  w[1] = pack2<kBF16>(d[2], 0.0f);
}

// One optimizer update (nrc_optimize.comp:32-54) of parameter i from its
// gradient sum; exactly the CPU oracle's operation order. `e` is the CTA's
// shared-memory copy of the entry; the entry is also written back to memory.
struct AdamHyper {
  float lr, beta1, beta2, eps, ema_alpha, loss_scale;
  int use_ema;
};

template <bool kBF16>
__device__ __forceinline__ void adam_one(int i, float gsum, uint32_t n, const nrc_optimizer_state& st,
                                         const AdamHyper& hp, nrc_optimizer_entry& e,
                                         nrc_optimizer_entry* __restrict__ entries, uint16_t* __restrict__ w16,
                                         uint16_t* __restrict__ use16) {
  float g = __fdiv_rn(__fdiv_rn(gsum, static_cast<float>(n)), hp.loss_scale);
  if (isnan(g) || isinf(g)) g = 0.0f;
  const float m = __fmaf_rn(hp.beta1, e.m, __fmul_rn(__fsub_rn(1.0f, hp.beta1), g));
  const float v = __fmaf_rn(hp.beta2, e.v, __fmul_rn(__fsub_rn(1.0f, hp.beta2), __fmul_rn(g, g)));
  const float hm = __fdiv_rn(m, __fsub_rn(1.0f, st.beta1_t));
  const float hv = __fdiv_rn(v, __fsub_rn(1.0f, st.beta2_t));
  const float w = __fsub_rn(e.weight, __fdiv_rn(__fmul_rn(hp.lr, hm), __fadd_rn(__fsqrt_rn(hv), hp.eps)));
  const float eta_t = __fsub_rn(1.0f, st.alpha_t), eta_t1 = __fsub_rn(1.0f, st.alpha_t_1);
  const float ea = __fdiv_rn(__fsub_rn(1.0f, hp.ema_alpha), eta_t), eb = __fmul_rn(hp.ema_alpha, eta_t1);
  const float ema = __fmaf_rn(ea, w, __fmul_rn(eb, e.ema_weight));
  e.m = m;
  e.v = v;
  e.weight = w;
  e.ema_weight = ema;
  entries[i] = e;
  w16[i] = to16<kBF16>(w);
  if (use16 != nullptr) use16[i] = to16<kBF16>(hp.use_ema ? ema : w);
}

}  // namespace nrc
