/*
 * CPU oracle for the neural-radiance-cache hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's shader math, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg to check the GPU
 * path against. The product (libnrc.so) never links, loads or calls anything in
 * this directory.
 *
 * Parity status:
 *   - Record encoding: pinned against the reference's own NRCRecord.glsl compiled
 *     as C++ (oracle/ref/ref_glsl.cpp) through committed golden vectors.
 *   - MLP forward: pinned against the reference's own CPU MLP (test/main.cpp
 *     Evaluate()) through committed golden vectors.
 *   - Gradient / Adam: restated from shader/src/NN_nv.glsl, nrc_gradient.comp and
 *     nrc_optimize.comp. The reference's CPU Train() does not compute the shader's
 *     gradient (wrong loss seed, indicator instead of ReLU mask), so these are
 *     checked by a finite-difference test of the restated loss, not by reference
 *     outputs.
 *
 * Conventions (reference layout, src/VkNRCState.hpp:22-25, NN_nv.glsl:20,69-82):
 *   weights fp16[20672]: layer l<5 at l*4096, row-major W[out=64][in=64];
 *   output layer at 5*4096, row-major W[3][64]. y = W x.
 */
#ifndef NRC_ORACLE_H
#define NRC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_P 20672
#define ORACLE_IN_FLOATS 14

/* Scalar pieces (exported so tests can pin them individually). */
float oracle_expf(float x);
uint16_t oracle_f32_to_f16(float x);
float oracle_f16_to_f32(uint16_t h);

/* NRCSphEncode (NRCRecord.glsl:47-49): dirs n x 3 -> out n x 2. */
void oracle_sph_encode(const float* dirs, int64_t n, float* out);

/* NRCInputEncode (NRCRecord.glsl:51-95): records n x 14 -> enc n x 64 fp16 bits. */
void oracle_encode(const float* records, int64_t n, uint16_t* enc);

/* Forward, fp16 activations between layers, fp32 accumulation (the GPU path's
 * arithmetic). out: n x 3 fp32, unclamped. nthreads <= 0 means 1. */
void oracle_forward_f32(const uint16_t* w, const uint16_t* enc, int64_t n, float* out, int nthreads);

/* Forward in FP64 from the same fp16 weights/inputs, no intermediate rounding. */
void oracle_forward_f64(const uint16_t* w, const uint16_t* enc, int64_t n, double* out, int nthreads);

/* Gradient of the relative-L2 luminance loss (NN_nv.glsl:178-196, nrc_gradient.comp:26-58)
 * summed over n records, written to grad[20672] (not divided by n).
 *   mode 0: the GPU path's arithmetic: fp16 activations, fp16 dL/dout and fp16 dA
 *           (as the reference stores them), fp32 sums;
 *   mode 1: FP64 throughout (no fp16 rounding of activations or gradients).
 * target: n x 3. loss_sum (nullable): sum over records of the per-record loss
 * sum_c (p_c - t_c)^2 / (lum(max(p,0))^2 + 0.01), in double.
 * grad_abs (nullable): per-parameter sum of |term|, for error normalisation. */
void oracle_train_grad(const uint16_t* w, const uint16_t* enc, const float* target, int64_t n,
                       float loss_scale, int mode, double* grad, double* grad_abs, double* loss_sum,
                       int nthreads);
void oracle_train_grad_w64(const double* w, const uint16_t* enc, const float* target, int64_t n,
                           float loss_scale, double* grad, double* loss_sum, int nthreads);

/* The relative-L2 luminance loss gradient rows (NN_nv.glsl:178-196) for n
 * (prediction, target) pairs, each as the two 32-bit words (d0 | d1 << 16,
 * d2 | 0 << 16) of the reference's 16-bit row; fmt 0 fp16, 1 bf16. */
void oracle_loss_rows(const float* pred, const float* target, int64_t n, float loss_scale, int fmt, uint32_t* rows);

/* Optimizer state and entries (src/VkNRCState.cpp:25-31). */
typedef struct oracle_opt_state {
  uint32_t t;
  float beta1_t, beta2_t, alpha_t, alpha_t_1;
} oracle_opt_state;

typedef struct oracle_hparams {
  float learning_rate, beta1, beta2, epsilon, ema_alpha, loss_scale;
  uint32_t batch_cap;
} oracle_hparams;

/* nrc_train_prepare.comp:16-29: clamp the count, advance the step state if n > 0.
 * Returns the clamped count. */
uint32_t oracle_prepare(uint32_t count, const oracle_hparams* hp, oracle_opt_state* st);

/* nrc_optimize.comp:32-54 for all parameters. entries: P x {m, v, w, ema}.
 * grad: fp32 gradient sums. w16 receives fp16 weights; use16 (nullable) receives
 * fp16 of (use_ema ? ema : w). No-op when count == 0. */
void oracle_adam(float* entries, const float* grad, uint32_t count, const oracle_opt_state* st,
                 const oracle_hparams* hp, uint16_t* w16, uint16_t* use16, int use_ema);
void oracle_adam_fmt(float* entries, const float* grad, uint32_t count, const oracle_opt_state* st,
                     const oracle_hparams* hp, uint16_t* w16, uint16_t* use16, int use_ema, int fmt);

void oracle_scatter(const float* pred, const uint32_t* dst, int64_t n, float* bias_factor_r, const float* factor_gb,
                    uint32_t width, uint32_t height, float* const* train, const uint32_t* train_cap);

/* Precision forms: the same computations with every 16-bit quantity (weights,
 * encoded features, stored activations and gradients, the fp16 weight copies
 * Adam writes) in format fmt: 0 fp16 (the reference's), 1 bf16. */
uint16_t oracle_f32_to_bf16(float x);
float oracle_bf16_to_f32(uint16_t b);
void oracle_encode_fmt(const float* records, int64_t n, uint16_t* enc, int fmt);
void oracle_forward_f32_fmt(const uint16_t* w, const uint16_t* enc, int64_t n, float* out, int nthreads, int fmt);
void oracle_forward_f64_fmt(const uint16_t* w, const uint16_t* enc, int64_t n, double* out, int nthreads, int fmt);
void oracle_train_grad_fmt(const uint16_t* w, const uint16_t* enc, const float* target, int64_t n, float loss_scale,
                           int mode, double* grad, double* grad_abs, double* loss_sum, int nthreads, int fmt);

/* FP8 (E4M3) query form: conversions, fp32 features, the scales and E4M3
 * weights of the GPU's refresh, and the FP8 forward (see nrc_oracle.c). */
uint8_t oracle_f32_to_e4m3(float x);
float oracle_e4m3_to_f32(uint8_t b);
void oracle_encode_f32(const float* records, int64_t n, float* feats);
void oracle_fp8_quantize(const uint16_t* w16, int fmt, const float seen[6], float* state, uint8_t* w8);
void oracle_forward_fp8(const uint8_t* w8, const float c[6], float inv_sx0, const float* feats, int64_t n, float* out,
                        int nthreads);

/* Scene buffers for oracle_unpack, the host mirror of nrc_scene (include/nrc.h);
 * pointers are host pointers. */
typedef struct oracle_material {
  float diffuse[3];
  uint32_t diffuse_texture_id;
  float specular[3];
  uint32_t specular_texture_id;
  float emission[3];
  uint32_t emission_texture_id;
  float metallic, roughness, ior;
  uint32_t pad_;
} oracle_material;

typedef struct oracle_texture {
  const uint8_t* texels;
  uint32_t width, height;
} oracle_texture;

typedef struct oracle_scene {
  const float* vertices;
  const uint32_t* vertex_indices;
  const float* texcoords;
  const uint32_t* texcoord_indices;
  const oracle_material* materials;
  const uint32_t* material_ids;
  const float* transforms;
  const oracle_texture* textures;
  uint32_t vertex_count, texcoord_count, material_count, primitive_count, instance_count, texture_count;
} oracle_scene;

/* UnpackNRCInput (NRCRecord.glsl:97-125) of n packed inputs (4 words each,
 * records stride_words apart) into nrc_input floats (14 each, out_stride apart). */
void oracle_unpack(const oracle_scene* scene, const uint32_t* packed, int64_t n, int64_t stride_words, float* out,
                   int64_t out_stride);

/* Path tracer (shader/src/path_tracer.comp), nrc_trace_oracle.c. ranges: per
 * instance {first primitive, primitive count}. Outputs as the GPU's
 * nrc_trace_targets: eval records (5 words each, eval_capacity of them),
 * train records (10 words each, 16384 per batch), counters (start them at 0),
 * bias_factor_r (width x height x 4) and factor_gb (x 2) floats. */
typedef struct oracle_trace_params {
  float origin[3], look[3], side[3], up[3];
  uint32_t width, height, seed, left_method, right_method;
  float train_probability;
} oracle_trace_params;

typedef struct oracle_trace_out {
  uint32_t* eval_records;
  uint32_t eval_count, eval_capacity;
  uint32_t* train_records[4];
  uint32_t train_counts[4];
  float* bias_factor_r;
  float* factor_gb;
} oracle_trace_out;

void oracle_path_trace(const oracle_scene* scene, const uint32_t* ranges, const oracle_trace_params* p,
                       oracle_trace_out* o);

/* Screen pass (shader/src/screen.frag:10-31) over width x height rgba32f pixels:
 * color (rgb used) -> optional running average into accumulate (rgba32f, updated
 * in place when accumulate_on) -> Hejl 2015 filmic tone map (white 3.2) -> gamma
 * 1/2.2 -> out_rgba (float, alpha 1) and/or out_rgba8 (UNORM8, alpha 255). */
void oracle_screen(const float* color, float* accumulate, uint32_t width, uint32_t height, int accumulate_on,
                   uint32_t accumulate_count, uint8_t* out_rgba8, float* out_rgba);

#ifdef __cplusplus
}
#endif
#endif
