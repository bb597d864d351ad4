// Shared constants and device code for the neural-radiance-cache kernels:
// record layouts, the fp32 input encoding, and the weight staging (TMA) into
// shared memory in the tensor-core operand layout.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "../../include/nrc.h"
#include "ptx.cuh"

namespace nrc {

constexpr int kWidth = 64;            // hidden width (src/VkNRCState.hpp:23)
constexpr int kHidden = 5;            // hidden layers (Constant.glsl:6)
constexpr int kOut = 3;               // outputs
constexpr int kOutPad = 16;           // output rows padded for the MMA (NN_nv.glsl:77-82)
constexpr int kLayerElems = kWidth * kWidth;
constexpr int kParams = kHidden * kLayerElems + kOut * kWidth;  // 20672
constexpr int kTile = 128;            // records per MMA tile (M)
constexpr int kInFloats = 14;         // nrc_input
constexpr int kTrainFloats = 20;      // nrc_train_record
constexpr uint32_t kWaitLimitNs = 2000000000u;  // bounded waits: 2 s

static_assert(sizeof(nrc_input) == kInFloats * 4, "nrc_input layout");
static_assert(sizeof(nrc_train_record) == kTrainFloats * 4, "nrc_train_record layout");

// Shared-memory bytes of the staged weights: 5 layers x 64 rows x 128 B, then the
// output layer as 16 rows (3 real, 13 zero) x 128 B.
constexpr uint32_t kWeightSmemBytes = kHidden * 8192 + kOutPad * 128;

// Weight staging by TMA. The parameter vector is viewed as a 2-D tensor of
// 323 rows x 64 fp16 (row r = output row r%64 of layer r/64; rows 320..322 are
// the output layer) with the 128-byte swizzle; 21 boxes of 16 rows land as the
// same swizzled K-major tiles as stage_weights() writes. The last box covers
// rows 320..335, and the tensor map zero-fills rows 323..335: the output
// layer's padding to 16 rows (NN_nv.glsl:77-82). One thread issues; `bar`
// completes when all 43,008 bytes have landed.
constexpr int kWeightRows = kHidden * kWidth + kOut;  // 323
constexpr uint32_t kWeightTmaBytes = (kHidden * 4 + 1) * 16 * 128;
static_assert(kWeightTmaBytes == kWeightSmemBytes, "weight staging size");

__device__ __forceinline__ void stage_weights_tma(uint8_t* smem_w, const CUtensorMap* map, uint64_t* bar) {
  mbar_arrive_expect_tx(bar, kWeightTmaBytes);
#pragma unroll
  for (int l = 0; l < kHidden; ++l)
#pragma unroll
    for (int k = 0; k < 4; ++k) tma_load_2d(smem_w + l * 8192 + k * 2048, map, 0, l * kWidth + k * 16, bar);
  tma_load_2d(smem_w + kHidden * 8192, map, 0, kHidden * kWidth, bar);
}

// ------------------------------------------------------------- encoding --
// Restatement of shader/src/NRCRecord.glsl:51-95 in an explicit fp32 op
// sequence (no compiler contraction), identical to the CPU oracle's.

// _nrc_tri (NRCRecord.glsl:65-68) of x = p * 2^k: 2|mod(x - 0.5, 2) - 1| - 1.
// p * 2^k is exact, so the first op fuses it with the -0.5.
__device__ __forceinline__ float enc_tri(float p, float scale) {
  const float y = __fmaf_rn(p, scale, -0.5f);
  const float f = floorf(__fmul_rn(y, 0.5f));
  const float m = __fmaf_rn(-2.0f, f, y);
  const float t = __fadd_rn(m, -1.0f);
  return __fmaf_rn(2.0f, fabsf(t), -1.0f);
}

// The same value from h = p 2^(k-1) - 0.25, one multiply fewer. Scaling by a
// power of two commutes with rounding while nothing overflows or turns
// subnormal, so h = y / 2 and floor(h) = f exactly, d = h - f = m / 2 exactly,
// and t = 2d - 1 rounds as m - 1 does: every rounding is the one enc_tri makes.
// Valid for |p| < 2^100 (p * 2^11 finite); NaN gives NaN in both.
__device__ __forceinline__ float enc_tri_h(float p, float half_scale) {
  const float h = __fmaf_rn(p, half_scale, -0.25f);
  const float d = __fsub_rn(h, floorf(h));
  const float t = __fmaf_rn(2.0f, d, -1.0f);
  return __fmaf_rn(2.0f, fabsf(t), -1.0f);
}

// _quartic_cdf at radius 1/4 (NRCRecord.glsl:51-56), u = 4 (edge - x).
__device__ __forceinline__ float enc_qcdf(float edge4, float x) {
  const float u = __fmaf_rn(x, -4.0f, edge4);
  const float u2 = __fmul_rn(u, u);
  const float s = __fmaf_rn(__fmaf_rn(u2, 0.2f, -0.6666667f), u2, 1.0f);
  const float c = __fmaf_rn(__fmul_rn(0.9375f, u), s, 0.5f);
  return __saturatef(c);
}

// Two fp32 lanes in one 64-bit register: Blackwell's packed fp32 arithmetic
// (fma/mul .f32x2) does both lanes with the scalar instructions' IEEE rounding.
__device__ __forceinline__ uint64_t f32x2(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f32x2_split(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t fma_x2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ uint64_t mul_x2(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

// enc_qcdf at two edges for one x, lane by lane the same operations.
__device__ __forceinline__ void enc_qcdf_x2(float edge4_lo, float edge4_hi, float x, float& c_lo, float& c_hi) {
  const uint64_t u = fma_x2(f32x2(x, x), f32x2(-4.0f, -4.0f), f32x2(edge4_lo, edge4_hi));
  const uint64_t u2 = mul_x2(u, u);
  const uint64_t s =
      fma_x2(fma_x2(u2, f32x2(0.2f, 0.2f), f32x2(-0.6666667f, -0.6666667f)), u2, f32x2(1.0f, 1.0f));
  const uint64_t c = fma_x2(mul_x2(f32x2(0.9375f, 0.9375f), u), s, f32x2(0.5f, 0.5f));
  f32x2_split(c, c_lo, c_hi);
  c_lo = __saturatef(c_lo);
  c_hi = __saturatef(c_hi);
}

// NRCOneBlob4Encode (NRCRecord.glsl:58-63), packed to two 16-bit pair words
// (fp16, or bf16 for the bf16 precision form).
template <bool kBF16>
__device__ __forceinline__ void enc_oneblob4(float x, uint32_t& w0, uint32_t& w1) {
  float f0, f1, f2, f3;
  enc_qcdf_x2(0.0f, 1.0f, x, f0, f1);
  enc_qcdf_x2(2.0f, 3.0f, x, f2, f3);
  const float f4 = enc_qcdf(4.0f, x);
  w0 = pack2<kBF16>(__fsub_rn(f1, f0), __fsub_rn(f2, f1));
  w1 = pack2<kBF16>(__fsub_rn(f3, f2), __fsub_rn(f4, f3));
}

// e^x by Cody-Waite reduction and a degree-7 Taylor polynomial (the same
// sequence as the CPU oracle, so the roughness feature is bit-identical).
__device__ __forceinline__ float enc_expf(float x) {
  x = fminf(fmaxf(x, -87.0f), 88.0f);  // NaN becomes -87 here; inputs are finite
  const float k = rintf(__fmul_rn(x, 1.44269504f));
  float r = __fmaf_rn(k, -0.693145751953125f, x);
  r = __fmaf_rn(k, -1.42860677e-06f, r);
  float p = 1.98412698e-04f;
  p = __fmaf_rn(p, r, 1.38888889e-03f);
  p = __fmaf_rn(p, r, 8.33333333e-03f);
  p = __fmaf_rn(p, r, 4.16666667e-02f);
  p = __fmaf_rn(p, r, 1.66666667e-01f);
  p = __fmaf_rn(p, r, 0.5f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  const float s = __int_as_float((static_cast<int>(k) + 127) << 23);
  return __fmul_rn(p, s);
}

// Frequency features k0 .. k0+2n-1 of one coordinate -> n words.
template <int K0, int N, bool kBF16>
__device__ __forceinline__ void enc_freq(float p, uint32_t* o) {
  if (fabsf(p) < 0x1p100f) {
#pragma unroll
    for (int i = 0; i < N; ++i)
      o[i] = pack2<kBF16>(enc_tri_h(p, 0.5f * static_cast<float>(1 << (K0 + 2 * i))),
                          enc_tri_h(p, 0.5f * static_cast<float>(1 << (K0 + 2 * i + 1))));
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i)
      o[i] = pack2<kBF16>(enc_tri(p, static_cast<float>(1 << (K0 + 2 * i))),
                          enc_tri(p, static_cast<float>(1 << (K0 + 2 * i + 1))));
  }
}

// NRCInputEncode (NRCRecord.glsl:78-95) split at feature 32, a 16-byte chunk
// boundary of the 128-byte row, so two threads can encode one record:
// features 0..31 = pos.x and pos.y frequencies, pos.z frequencies 0..7;
// features 32..63 = pos.z frequencies 8..11, the five one-blob groups, diffuse,
// specular and the two constant ones. Word j holds features 2j (low half) and
// 2j+1 of its half.
template <bool kBF16 = false>
__device__ __forceinline__ void encode_half0(const float (&r)[kInFloats], uint32_t* e) {
  enc_freq<0, 6, kBF16>(r[0], e + 0);
  enc_freq<0, 6, kBF16>(r[1], e + 6);
  enc_freq<0, 4, kBF16>(r[2], e + 12);
}

template <bool kBF16 = false>
__device__ __forceinline__ void encode_half1(const float (&r)[kInFloats], uint32_t* e) {
  enc_freq<8, 2, kBF16>(r[2], e + 0);
  enc_oneblob4<kBF16>(r[3], e[2], e[3]);
  enc_oneblob4<kBF16>(r[4], e[4], e[5]);
  enc_oneblob4<kBF16>(r[5], e[6], e[7]);
  enc_oneblob4<kBF16>(r[6], e[8], e[9]);
  enc_oneblob4<kBF16>(__fsub_rn(1.0f, enc_expf(-r[7])), e[10], e[11]);
  e[12] = pack2<kBF16>(r[8], r[9]);
  e[13] = pack2<kBF16>(r[10], r[11]);
  e[14] = pack2<kBF16>(r[12], r[13]);
  e[15] = pack2<kBF16>(1.0f, 1.0f);
}

// The whole record: 14 fp32 -> 64 16-bit features as 32 words.
template <bool kBF16 = false>
__device__ __forceinline__ void encode_input(const float (&r)[kInFloats], uint32_t (&e)[32]) {
  encode_half0<kBF16>(r, e);
  encode_half1<kBF16>(r, e + 16);
}

// The same features in E4M3 for the FP8 query: feature k, multiplied by inv_s
// (448 / the features' absmax scale), rounded to nearest even and saturated,
// in byte k % 4 of word k / 4 (the multiplies two per packed f32x2
// instruction, each rounded as one __fmul_rn). Split like the 16-bit encode at
// feature 32: half 0 gives words 0..7 (features 0..31), half 1 words 8..15.
__device__ __forceinline__ uint32_t e4m3_q4(float a, float b, float c, float d, float inv_s) {
  const uint64_t s2 = f32x2(inv_s, inv_s);
  float a0, a1, a2, a3;
  f32x2_split(mul_x2(f32x2(a, b), s2), a0, a1);
  f32x2_split(mul_x2(f32x2(c, d), s2), a2, a3);
  return pack4_e4m3(a0, a1, a2, a3);
}
// triangle-wave frequency k of coordinate p (the two forms agree; see enc_tri_h)
__device__ __forceinline__ float enc_tri_k(float p, int k) {
  return fabsf(p) < 0x1p100f ? enc_tri_h(p, 0.5f * static_cast<float>(1 << k)) : enc_tri(p, static_cast<float>(1 << k));
}
// four triangle-wave features of coordinate p, frequencies 4w..4w+3
__device__ __forceinline__ uint32_t enc_tri4_e4m3(float p, int w, float inv_s) {
  return e4m3_q4(enc_tri_k(p, 4 * w), enc_tri_k(p, 4 * w + 1), enc_tri_k(p, 4 * w + 2), enc_tri_k(p, 4 * w + 3), inv_s);
}
__device__ __forceinline__ uint32_t enc_blob_e4m3(float x, float inv_s) {
  float f0, f1, f2, f3;
  enc_qcdf_x2(0.0f, 1.0f, x, f0, f1);
  enc_qcdf_x2(2.0f, 3.0f, x, f2, f3);
  const float f4 = enc_qcdf(4.0f, x);
  return e4m3_q4(__fsub_rn(f1, f0), __fsub_rn(f2, f1), __fsub_rn(f3, f2), __fsub_rn(f4, f3), inv_s);
}

__device__ __forceinline__ void encode_e4m3_half0(const float (&r)[kInFloats], float inv_s, uint32_t* e) {
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int w = 0; w < 3; ++w) e[3 * c + w] = enc_tri4_e4m3(r[c], w, inv_s);
  e[6] = enc_tri4_e4m3(r[2], 0, inv_s);
  e[7] = enc_tri4_e4m3(r[2], 1, inv_s);
}

__device__ __forceinline__ void encode_e4m3_half1(const float (&r)[kInFloats], float inv_s, uint32_t* e) {
  e[0] = enc_tri4_e4m3(r[2], 2, inv_s);
  e[1] = enc_blob_e4m3(r[3], inv_s);
  e[2] = enc_blob_e4m3(r[4], inv_s);
  e[3] = enc_blob_e4m3(r[5], inv_s);
  e[4] = enc_blob_e4m3(r[6], inv_s);
  e[5] = enc_blob_e4m3(__fsub_rn(1.0f, enc_expf(-r[7])), inv_s);
  e[6] = e4m3_q4(r[8], r[9], r[10], r[11], inv_s);
  e[7] = e4m3_q4(r[12], r[13], 1.0f, 1.0f, inv_s);
}

__device__ __forceinline__ void encode_input_e4m3(const float (&r)[kInFloats], float inv_s, uint32_t (&e)[32]) {
  encode_e4m3_half0(r, inv_s, e);
  encode_e4m3_half1(r, inv_s, e + 8);
}

// Device-side error word bits (read back by nrc_get_error).
constexpr uint32_t kErrTimeout = 1u;

}  // namespace nrc
