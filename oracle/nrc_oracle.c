/*
 * CPU oracle for the neural-radiance-cache hot path — TEST INFRASTRUCTURE ONLY.
 * See nrc_oracle.h for what is pinned against the reference and how.
 *
 * Build: oracle/build_oracle.sh (gcc -O2 -ffp-contract=off). Contraction is off so
 * that every fused multiply-add below is an explicit fmaf() and the op sequence is
 * the same on x86 and aarch64.
 */
#include "nrc_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------ fp16 -- */
uint16_t oracle_f32_to_f16(float x) {
  _Float16 h = (_Float16)x; /* IEEE round-to-nearest-even, as packHalf2x16 on the GPU */
  uint16_t b;
  memcpy(&b, &h, 2);
  return b;
}

float oracle_f16_to_f32(uint16_t b) {
  _Float16 h;
  memcpy(&h, &b, 2);
  return (float)h;
}

/* bf16: the upper half of an fp32, rounded to nearest even (NaN kept quiet). */
uint16_t oracle_f32_to_bf16(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7FFFFFFFu) > 0x7F800000u) return (uint16_t)((u >> 16) | 0x40u);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

float oracle_bf16_to_f32(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float x;
  memcpy(&x, &u, 4);
  return x;
}

/* The 16-bit storage format of a precision form: 0 fp16 (the reference's), 1 bf16. */
static inline uint16_t to16(float x, int fmt) { return fmt ? oracle_f32_to_bf16(x) : oracle_f32_to_f16(x); }
static inline float from16(uint16_t b, int fmt) { return fmt ? oracle_bf16_to_f32(b) : oracle_f16_to_f32(b); }
static inline float round16(float x, int fmt) { return from16(to16(x, fmt), fmt); }

/* ------------------------------------------------------------- exp -- */
/* e^x by Cody & Waite argument reduction (x = k ln2 + r, ln2 split into a
 * 16-bit-exact high part and a low correction) and the degree-7 Taylor
 * polynomial of e^r on |r| <= ln2/2 (truncation error < 6e-9 relative), then an
 * exact scale by 2^k. The GPU kernels use the same sequence, so the encoded
 * roughness feature is identical on both. GLSL's exp() is only specified to
 * 3 + 2|x| ulp, which this meets. */
float oracle_expf(float x) {
  x = fminf(fmaxf(x, -87.0f), 88.0f); /* NaN maps to -87, as on the GPU */
  const float k = rintf(x * 1.44269504f);
  float r = fmaf(k, -0.693145751953125f, x);
  r = fmaf(k, -1.42860677e-06f, r);
  float p = 1.98412698e-04f;       /* 1/7! */
  p = fmaf(p, r, 1.38888889e-03f); /* 1/6! */
  p = fmaf(p, r, 8.33333333e-03f); /* 1/5! */
  p = fmaf(p, r, 4.16666667e-02f); /* 1/4! */
  p = fmaf(p, r, 1.66666667e-01f); /* 1/3! */
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  const int32_t ki = (int32_t)k;
  const uint32_t sbits = (uint32_t)(ki + 127) << 23;
  float s;
  memcpy(&s, &sbits, 4);
  return p * s;
}

/* ---------------------------------------------------------- encode -- */
/* NRCSphEncode, NRCRecord.glsl:47-49 (M_PI in single precision as GLSL has it). */
void oracle_sph_encode(const float* dirs, int64_t n, float* out) {
  const float pi = 3.14159265358979323846f;
  for (int64_t i = 0; i < n; ++i) {
    const float x = dirs[3 * i], y = dirs[3 * i + 1], z = dirs[3 * i + 2];
    const float zc = z < -1.0f ? -1.0f : (z > 1.0f ? 1.0f : z);
    out[2 * i] = (x == 0.0f && y == 0.0f) ? 0.5f : 0.5f + atan2f(y, x) / (2.0f * pi);
    out[2 * i + 1] = acosf(zc) / pi;
  }
}

/* _nrc_tri, NRCRecord.glsl:65-68: 2|mod(x - 0.5, 2) - 1| - 1 with GLSL's
 * mod(a, b) = a - b floor(a / b). mod is exact here; m - 1 and the final -1 round. */
static inline float tri(float x) {
  const float y = x - 0.5f;
  const float f = floorf(y * 0.5f);
  const float m = fmaf(-2.0f, f, y);
  const float t = m - 1.0f;
  return fmaf(2.0f, fabsf(t), -1.0f);
}

/* _quartic_cdf at radius 1/4, NRCRecord.glsl:51-56:
 * clamp(15/16 u (1 - 2/3 u^2 + 1/5 u^4) + 1/2, 0, 1), u = 4 (edge - x),
 * evaluated in Horner form with fused multiply-adds. */
static inline float qcdf(float edge4, float x) {
  const float u = fmaf(x, -4.0f, edge4);
  const float u2 = u * u;
  const float s = fmaf(fmaf(u2, 0.2f, -0.6666667f), u2, 1.0f);
  const float c = fmaf(0.9375f * u, s, 0.5f);
  return fminf(fmaxf(c, 0.0f), 1.0f);
}

/* NRCOneBlob4Encode, NRCRecord.glsl:58-63: bins [0,.25),[.25,.5),[.5,.75),[.75,1]. */
static inline void oneblob4(float x, float* o) {
  const float f0 = qcdf(0.0f, x), f1 = qcdf(1.0f, x), f2 = qcdf(2.0f, x), f3 = qcdf(3.0f, x),
              f4 = qcdf(4.0f, x);
  o[0] = f1 - f0;
  o[1] = f2 - f1;
  o[2] = f3 - f2;
  o[3] = f4 - f3;
}

/* NRCInputEncode, NRCRecord.glsl:78-95. Feature order:
 *   [0,12) pos.x freq 2^0..2^11, [12,24) pos.y, [24,36) pos.z,
 *   [36,40) ob(dir.u), [40,44) ob(dir.v), [44,48) ob(normal.u), [48,52) ob(normal.v),
 *   [52,56) ob(1 - e^-roughness), [56,59) diffuse, [59,62) specular, 62, 63 = 1. */
void oracle_encode_fmt(const float* records, int64_t n, uint16_t* enc, int fmt) {
  for (int64_t i = 0; i < n; ++i) {
    const float* r = records + ORACLE_IN_FLOATS * i;
    float f[64];
    for (int c = 0; c < 3; ++c) {
      float scale = 1.0f;
      for (int k = 0; k < 12; ++k, scale *= 2.0f) f[12 * c + k] = tri(r[c] * scale);
    }
    oneblob4(r[3], f + 36);
    oneblob4(r[4], f + 40);
    oneblob4(r[5], f + 44);
    oneblob4(r[6], f + 48);
    oneblob4(1.0f - oracle_expf(-r[7]), f + 52);
    for (int c = 0; c < 6; ++c) f[56 + c] = r[8 + c];
    f[62] = 1.0f;
    f[63] = 1.0f;
    for (int c = 0; c < 64; ++c) enc[64 * i + c] = to16(f[c], fmt);
  }
}

void oracle_encode(const float* records, int64_t n, uint16_t* enc) { oracle_encode_fmt(records, n, enc, 0); }

/* ----------------------------------------------------------- threads -- */
typedef void (*range_fn)(void* ctx, int64_t begin, int64_t end, int tid);
typedef struct {
  range_fn fn;
  void* ctx;
  int64_t begin, end;
  int tid;
} range_job;

static void* range_trampoline(void* p) {
  range_job* j = (range_job*)p;
  j->fn(j->ctx, j->begin, j->end, j->tid);
  return NULL;
}

static void parallel_for(int64_t n, int nthreads, range_fn fn, void* ctx) {
  if (nthreads <= 1 || n < 2) {
    fn(ctx, 0, n, 0);
    return;
  }
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  range_job jobs[256];
  const int64_t chunk = (n + nthreads - 1) / nthreads;
  int used = 0;
  for (int t = 0; t < nthreads; ++t) {
    const int64_t b = t * chunk, e = b + chunk < n ? b + chunk : n;
    if (b >= e) break;
    jobs[t] = (range_job){fn, ctx, b, e, t};
    pthread_create(&th[t], NULL, range_trampoline, &jobs[t]);
    ++used;
  }
  for (int t = 0; t < used; ++t) pthread_join(th[t], NULL);
}

/* ---------------------------------------------------------- forward -- */
/* Weight layer l as float, transposed to wt[in][out] so that the inner loop runs
 * over outputs with each output summed in input order 0..63. */
typedef struct {
  float wt[5][64][64];
  float w5t[64][3];
  double wtd[5][64][64];
  double w5td[64][3];
  int fmt; /* 16-bit format of weights, inputs and stored activations/gradients */
} wcache;

static void load_weights(const uint16_t* w, wcache* c, int fmt) {
  c->fmt = fmt;
  for (int l = 0; l < 5; ++l)
    for (int o = 0; o < 64; ++o)
      for (int i = 0; i < 64; ++i) {
        const float v = from16(w[l * 4096 + o * 64 + i], fmt);
        c->wt[l][i][o] = v;
        c->wtd[l][i][o] = v;
      }
  for (int o = 0; o < 3; ++o)
    for (int i = 0; i < 64; ++i) {
      const float v = from16(w[5 * 4096 + o * 64 + i], fmt);
      c->w5t[i][o] = v;
      c->w5td[i][o] = v;
    }
}

/* One record forward, fp16 activations, fp32 sums. acts[l] receives the input of
 * layer l (l = 0..5), out the three fp32 outputs (no clamp). */
static void fwd_f32(const wcache* c, const uint16_t* e, float acts[6][64], float out[3]) {
  for (int i = 0; i < 64; ++i) acts[0][i] = from16(e[i], c->fmt);
  for (int l = 0; l < 5; ++l) {
    float z[64];
    for (int o = 0; o < 64; ++o) z[o] = 0.0f;
    for (int i = 0; i < 64; ++i) {
      const float a = acts[l][i];
      for (int o = 0; o < 64; ++o) z[o] += c->wt[l][i][o] * a;
    }
    for (int o = 0; o < 64; ++o) acts[l + 1][o] = round16(z[o] > 0.0f ? z[o] : 0.0f, c->fmt);
  }
  out[0] = out[1] = out[2] = 0.0f;
  for (int i = 0; i < 64; ++i)
    for (int o = 0; o < 3; ++o) out[o] += c->w5t[i][o] * acts[5][i];
}

static void fwd_f64(const wcache* c, const uint16_t* e, double acts[6][64], double out[3]) {
  for (int i = 0; i < 64; ++i) acts[0][i] = from16(e[i], c->fmt);
  for (int l = 0; l < 5; ++l) {
    double z[64];
    for (int o = 0; o < 64; ++o) z[o] = 0.0;
    for (int i = 0; i < 64; ++i) {
      const double a = acts[l][i];
      for (int o = 0; o < 64; ++o) z[o] += c->wtd[l][i][o] * a;
    }
    for (int o = 0; o < 64; ++o) acts[l + 1][o] = z[o] > 0.0 ? z[o] : 0.0;
  }
  out[0] = out[1] = out[2] = 0.0;
  for (int i = 0; i < 64; ++i)
    for (int o = 0; o < 3; ++o) out[o] += c->w5td[i][o] * acts[5][i];
}

typedef struct {
  const wcache* c;
  const uint16_t* enc;
  float* out32;
  double* out64;
} fwd_ctx;

static void fwd32_range(void* p, int64_t b, int64_t e, int tid) {
  (void)tid;
  fwd_ctx* x = (fwd_ctx*)p;
  float acts[6][64];
  for (int64_t i = b; i < e; ++i) fwd_f32(x->c, x->enc + 64 * i, acts, x->out32 + 3 * i);
}

static void fwd64_range(void* p, int64_t b, int64_t e, int tid) {
  (void)tid;
  fwd_ctx* x = (fwd_ctx*)p;
  double acts[6][64];
  for (int64_t i = b; i < e; ++i) fwd_f64(x->c, x->enc + 64 * i, acts, x->out64 + 3 * i);
}

void oracle_forward_f32_fmt(const uint16_t* w, const uint16_t* enc, int64_t n, float* out, int nthreads, int fmt) {
  wcache* c = (wcache*)malloc(sizeof(wcache));
  load_weights(w, c, fmt);
  fwd_ctx x = {c, enc, out, NULL};
  parallel_for(n, nthreads, fwd32_range, &x);
  free(c);
}

void oracle_forward_f32(const uint16_t* w, const uint16_t* enc, int64_t n, float* out, int nthreads) {
  oracle_forward_f32_fmt(w, enc, n, out, nthreads, 0);
}

void oracle_forward_f64_fmt(const uint16_t* w, const uint16_t* enc, int64_t n, double* out, int nthreads, int fmt) {
  wcache* c = (wcache*)malloc(sizeof(wcache));
  load_weights(w, c, fmt);
  fwd_ctx x = {c, enc, NULL, out};
  parallel_for(n, nthreads, fwd64_range, &x);
  free(c);
}

void oracle_forward_f64(const uint16_t* w, const uint16_t* enc, int64_t n, double* out, int nthreads) {
  oracle_forward_f64_fmt(w, enc, n, out, nthreads, 0);
}

/* ------------------------------------------------------------ train -- */
/* Relative-L2 luminance loss gradient, NN_nv.glsl:178-196: dL/dp = 2 s (p - t) /
 * (lum(max(p,0))^2 + 0.01), lum weights (0.299, 0.587, 0.114), the denominator
 * held constant. The GPU path evaluates it in fp32 in this order. */
static inline void loss_grad_f32(const float p[3], const float t[3], float s, float d[3]) {
  const float px = p[0] > 0.0f ? p[0] : 0.0f, py = p[1] > 0.0f ? p[1] : 0.0f, pz = p[2] > 0.0f ? p[2] : 0.0f;
  const float lum = fmaf(0.114f, pz, fmaf(0.587f, py, 0.299f * px));
  const float den = fmaf(lum, lum, 0.01f);
  const float s2 = 2.0f * s;
  for (int c = 0; c < 3; ++c) d[c] = (s2 * (p[c] - t[c])) / den;
}

/* The relative-L2 gradient rows as the reference stores them (NN_nv.glsl:185-186):
 * per record the words (d0 | d1 << 16, d2 | 0 << 16) of the 16-bit row, in
 * format fmt (0 fp16, 1 bf16); values beyond the format's range become inf. */
void oracle_loss_rows(const float* pred, const float* target, int64_t n, float loss_scale, int fmt, uint32_t* rows) {
  for (int64_t i = 0; i < n; ++i) {
    float d[3];
    loss_grad_f32(pred + 3 * i, target + 3 * i, loss_scale, d);
    rows[2 * i] = (uint32_t)to16(d[0], fmt) | ((uint32_t)to16(d[1], fmt) << 16);
    rows[2 * i + 1] = (uint32_t)to16(d[2], fmt);
  }
}

static inline double loss_value(const double p[3], const float t[3]) {
  const double px = p[0] > 0 ? p[0] : 0, py = p[1] > 0 ? p[1] : 0, pz = p[2] > 0 ? p[2] : 0;
  const double lum = 0.299 * px + 0.587 * py + 0.114 * pz;
  const double den = lum * lum + 0.01;
  double s = 0;
  for (int c = 0; c < 3; ++c) s += (p[c] - t[c]) * (p[c] - t[c]) / den;
  return s;
}

typedef struct {
  const wcache* c;
  const uint16_t* enc;
  const float* target;
  float loss_scale;
  int mode;
  double* grad[256];
  double* gabs[256];
  double loss[256];
} train_ctx;

static void train_range(void* p, int64_t b, int64_t e, int tid) {
  train_ctx* x = (train_ctx*)p;
  const wcache* c = x->c;
  double* G = x->grad[tid];
  double* A = x->gabs[tid];
  double loss = 0.0;
  for (int64_t r = b; r < e; ++r) {
    const float* t = x->target + 3 * r;
    /* acts[l] = input of layer l; g = gradient w.r.t. the output of the current layer */
    double acts[6][64], g[64], gn[64];
    double out[3];
    if (x->mode == 0) {
      float a32[6][64], o32[3], d[3];
      fwd_f32(c, x->enc + 64 * r, a32, o32);
      for (int l = 0; l < 6; ++l)
        for (int i = 0; i < 64; ++i) acts[l][i] = a32[l][i];
      loss_grad_f32(o32, t, x->loss_scale, d);
      for (int k = 0; k < 3; ++k) {
        out[k] = o32[k];
        g[k] = round16(d[k], c->fmt); /* packed to 16 bits, NN_nv.glsl:185-186 */
      }
    } else {
      fwd_f64(c, x->enc + 64 * r, acts, out);
      const double px = out[0] > 0 ? out[0] : 0, py = out[1] > 0 ? out[1] : 0, pz = out[2] > 0 ? out[2] : 0;
      const double lum = 0.299 * px + 0.587 * py + 0.114 * pz;
      const double den = lum * lum + 0.01;
      for (int k = 0; k < 3; ++k) g[k] = 2.0 * x->loss_scale * (out[k] - t[k]) / den;
    }
    loss += loss_value(out, t);
    /* output layer: dW5[k][i] += g[k] act5[i]; dA5 = W5^T g masked by act5 > 0 */
    for (int k = 0; k < 3; ++k)
      for (int i = 0; i < 64; ++i) {
        const double term = g[k] * acts[5][i];
        G[5 * 4096 + k * 64 + i] += term;
        if (A) A[5 * 4096 + k * 64 + i] += fabs(term);
      }
    for (int i = 0; i < 64; ++i) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += g[k] * c->w5td[i][k];
      /* ReLU mask; NaN sums are zeroed as the reference's NaN-mask trick does (NN_nv.glsl:240-243) */
      gn[i] = (acts[5][i] > 0.0 && s == s) ? s : 0.0;
      if (x->mode == 0) gn[i] = round16((float)gn[i], c->fmt);
    }
    for (int l = 4; l >= 0; --l) {
      for (int o = 0; o < 64; ++o) g[o] = gn[o];
      for (int o = 0; o < 64; ++o)
        for (int i = 0; i < 64; ++i) {
          const double term = g[o] * acts[l][i];
          G[l * 4096 + o * 64 + i] += term;
          if (A) A[l * 4096 + o * 64 + i] += fabs(term);
        }
      if (l == 0) break;
      for (int i = 0; i < 64; ++i) {
        double s = 0.0;
        for (int o = 0; o < 64; ++o) s += g[o] * c->wtd[l][i][o];
        gn[i] = (acts[l][i] > 0.0 && s == s) ? s : 0.0; /* NN_nv.glsl:272-277 */
        if (x->mode == 0) gn[i] = round16((float)gn[i], c->fmt);
      }
    }
  }
  x->loss[tid] = loss;
}

static void train_grad_cached(const wcache* c, const uint16_t* enc, const float* target, int64_t n,
                              float loss_scale, int mode, double* grad, double* grad_abs, double* loss_sum,
                              int nthreads) {
  if (nthreads <= 0) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  train_ctx* x = (train_ctx*)calloc(1, sizeof(train_ctx));
  x->c = c;
  x->enc = enc;
  x->target = target;
  x->loss_scale = loss_scale;
  x->mode = mode;
  for (int t = 0; t < nthreads; ++t) {
    x->grad[t] = (double*)calloc(ORACLE_P, sizeof(double));
    x->gabs[t] = grad_abs ? (double*)calloc(ORACLE_P, sizeof(double)) : NULL;
  }
  parallel_for(n, nthreads, train_range, x);
  /* fixed-order merge: the result does not depend on thread timing */
  for (int i = 0; i < ORACLE_P; ++i) {
    double s = 0.0, a = 0.0;
    for (int t = 0; t < nthreads; ++t) {
      s += x->grad[t][i];
      if (grad_abs) a += x->gabs[t][i];
    }
    grad[i] = s;
    if (grad_abs) grad_abs[i] = a;
  }
  if (loss_sum) {
    double l = 0.0;
    for (int t = 0; t < nthreads; ++t) l += x->loss[t];
    *loss_sum = l;
  }
  for (int t = 0; t < nthreads; ++t) {
    free(x->grad[t]);
    free(x->gabs[t]);
  }
  free(x);
}

void oracle_train_grad_fmt(const uint16_t* w, const uint16_t* enc, const float* target, int64_t n,
                           float loss_scale, int mode, double* grad, double* grad_abs, double* loss_sum,
                           int nthreads, int fmt) {
  wcache* c = (wcache*)malloc(sizeof(wcache));
  load_weights(w, c, fmt);
  train_grad_cached(c, enc, target, n, loss_scale, mode, grad, grad_abs, loss_sum, nthreads);
  free(c);
}

void oracle_train_grad(const uint16_t* w, const uint16_t* enc, const float* target, int64_t n,
                       float loss_scale, int mode, double* grad, double* grad_abs, double* loss_sum,
                       int nthreads) {
  oracle_train_grad_fmt(w, enc, target, n, loss_scale, mode, grad, grad_abs, loss_sum, nthreads, 0);
}

/* The FP64 oracle's training loop keeps its weights in FP64: the same gradient
 * and loss as oracle_train_grad in FP64 mode (mode 1), with the weights given as
 * double[ORACLE_P] in the parameter layout instead of fp16. */
void oracle_train_grad_w64(const double* w, const uint16_t* enc, const float* target, int64_t n,
                           float loss_scale, double* grad, double* loss_sum, int nthreads) {
  wcache* c = (wcache*)malloc(sizeof(wcache));
  c->fmt = 0; /* inputs are fp16 features */
  for (int l = 0; l < 5; ++l)
    for (int o = 0; o < 64; ++o)
      for (int i = 0; i < 64; ++i) {
        c->wtd[l][i][o] = w[l * 4096 + o * 64 + i];
        c->wt[l][i][o] = (float)w[l * 4096 + o * 64 + i];
      }
  for (int o = 0; o < 3; ++o)
    for (int i = 0; i < 64; ++i) {
      c->w5td[i][o] = w[5 * 4096 + o * 64 + i];
      c->w5t[i][o] = (float)w[5 * 4096 + o * 64 + i];
    }
  train_grad_cached(c, enc, target, n, loss_scale, 1, grad, NULL, loss_sum, nthreads);
  free(c);
}

/* -------------------------------------------------------- optimizer -- */
uint32_t oracle_prepare(uint32_t count, const oracle_hparams* hp, oracle_opt_state* st) {
  const uint32_t n = count < hp->batch_cap ? count : hp->batch_cap;
  if (n > 0) {
    st->t += 1;
    st->beta1_t *= hp->beta1;
    st->beta2_t *= hp->beta2;
    st->alpha_t_1 = st->alpha_t;
    st->alpha_t *= hp->ema_alpha;
  }
  return n;
}

/* nrc_optimize.comp:32-54, with its EMA formula kept as written:
 * ema = (1 - a)/eta_t * w + a * eta_{t-1} * ema, eta_t = 1 - a^t. */
void oracle_adam_fmt(float* entries, const float* grad, uint32_t count, const oracle_opt_state* st,
                     const oracle_hparams* hp, uint16_t* w16, uint16_t* use16, int use_ema, int fmt) {
  if (count == 0) return;
  const float b1 = hp->beta1, b2 = hp->beta2;
  const float omb1 = 1.0f - b1, omb2 = 1.0f - b2;
  const float c1 = 1.0f - st->beta1_t, c2 = 1.0f - st->beta2_t;
  const float eta_t = 1.0f - st->alpha_t, eta_t1 = 1.0f - st->alpha_t_1;
  const float ea = (1.0f - hp->ema_alpha) / eta_t, eb = hp->ema_alpha * eta_t1;
  const float fcount = (float)count;
  for (int i = 0; i < ORACLE_P; ++i) {
    float* e = entries + 4 * i;
    float g = grad[i] / fcount / hp->loss_scale;
    if (isnan(g) || isinf(g)) g = 0.0f;
    const float m = fmaf(b1, e[0], omb1 * g);
    const float v = fmaf(b2, e[1], omb2 * (g * g));
    const float hm = m / c1, hv = v / c2;
    const float w = e[2] - (hp->learning_rate * hm) / (sqrtf(hv) + hp->epsilon);
    const float ema = fmaf(ea, w, eb * e[3]);
    e[0] = m;
    e[1] = v;
    e[2] = w;
    e[3] = ema;
    w16[i] = to16(w, fmt);
    if (use16) use16[i] = to16(use_ema ? ema : w, fmt);
  }
}

void oracle_adam(float* entries, const float* grad, uint32_t count, const oracle_opt_state* st,
                 const oracle_hparams* hp, uint16_t* w16, uint16_t* use16, int use_ema) {
  oracle_adam_fmt(entries, grad, count, st, hp, w16, use16, use_ema, 0);
}

/* ------------------------------------------------ query destinations -- */
/* The destination epilogue of nrc_inference.comp:50-73 (word encoding
 * NRCRecord.glsl:19-33) applied in query order to predictions pred[n][3]
 * (already clamped at 0): a screen pixel of the rgba32f / rg32f images becomes
 * (bias + (factor.r, factor.g, factor.b) * pred, 0); a train word adds
 * factor * pred to the bias of records l..r of batch b. Each channel is one
 * fused multiply-add. Out-of-range pixels and records, and null batches, are
 * skipped. */
void oracle_scatter(const float* pred, const uint32_t* dst, int64_t n, float* bias_factor_r, const float* factor_gb,
                    uint32_t width, uint32_t height, float* const* train, const uint32_t* train_cap) {
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t d = dst[i];
    if (d == 0xFFFFFFFFu) continue;
    const uint32_t e = d >> 1;
    const float* p = pred + 3 * i;
    if ((d & 1u) == 0u) {
      const uint32_t x = e & 0x7FFFu, y = e >> 15;
      if (x >= width || y >= height) continue;
      const size_t px = (size_t)y * width + x;
      float* v = bias_factor_r + 4 * px;
      const float* gb = factor_gb + 2 * px;
      const float r = fmaf(v[3], p[0], v[0]), g = fmaf(gb[0], p[1], v[1]), b = fmaf(gb[1], p[2], v[2]);
      v[0] = r;
      v[1] = g;
      v[2] = b;
      v[3] = 0.0f;
    } else {
      const uint32_t b = e & 3u, l = (e >> 2) & 0x3FFFu, r = e >> 16;
      float* rec = train[b];
      if (rec == NULL) continue;
      for (uint32_t k = l; k <= r && k < train_cap[b]; ++k) {
        float* t = rec + 20 * (size_t)k;
        t[0] = fmaf(t[3], p[0], t[0]);
        t[1] = fmaf(t[4], p[1], t[1]);
        t[2] = fmaf(t[5], p[2], t[2]);
      }
    }
  }
}

/* ---------------------------------------------------------- screen -- */
/* The screen pass, shader/src/screen.frag:10-31: optional running average into
 * the accumulation image (:20-26), ToneMapFilmic_Hejl2015 with white point 3.2
 * (:10-15), gamma 1/2.2 (:29). GLSL leaves contraction to its compiler; this
 * restatement fixes one sequence (each `a * b + c` one fused multiply-add,
 * `color += acc * count` one too) that the GPU kernel repeats. pow() of a
 * negative base is undefined in GLSL; the tone curve dips below zero near black
 * (about -6e-4 at 0), so the base is clamped to zero first. rgba8 is the UNORM
 * conversion round(clamp(x, 0, 1) * 255), ties to even. */
static inline float hejl_curve(float x) {
  const float va = fmaf(1.425f, x, 0.05f);
  return fmaf(x, va, 0.004f) / fmaf(x, va + 0.55f, 0.0491f) - 0.0821f;
}

void oracle_screen(const float* color, float* accumulate, uint32_t width, uint32_t height, int accumulate_on,
                   uint32_t accumulate_count, uint8_t* out_rgba8, float* out_rgba) {
  const float wf = hejl_curve(3.2f); /* vf.w: the white point through the same curve */
  const int64_t n = (int64_t)width * height;
  for (int64_t i = 0; i < n; ++i) {
    float c[3] = {color[4 * i], color[4 * i + 1], color[4 * i + 2]};
    if (accumulate_on) {
      if (accumulate_count != 0) {
        const float k = (float)accumulate_count, k1 = (float)(accumulate_count + 1u);
        for (int j = 0; j < 3; ++j) c[j] = fmaf(accumulate[4 * i + j], k, c[j]) / k1;
      }
      for (int j = 0; j < 3; ++j) accumulate[4 * i + j] = c[j];
      accumulate[4 * i + 3] = 0.0f;
    }
    for (int j = 0; j < 3; ++j) {
      const float t = hejl_curve(c[j]) / wf;
      const float s = powf(fmaxf(t, 0.0f), 1.0f / 2.2f);
      if (out_rgba) out_rgba[4 * i + j] = s;
      if (out_rgba8) out_rgba8[4 * i + j] = (uint8_t)lrintf(fminf(fmaxf(s, 0.0f), 1.0f) * 255.0f);
    }
    if (out_rgba) out_rgba[4 * i + 3] = 1.0f;
    if (out_rgba8) out_rgba8[4 * i + 3] = 255;
  }
}

/* ---------------------------------------------------------- unpack -- */
/* UnpackNRCInput (shader/src/NRCRecord.glsl:97-125) over the scene buffers
 * (shader/src/Scene.glsl:50-71) and the reference's texture sampler (bilinear,
 * REPEAT, one level, R8G8B8A8_SRGB: src/rg/NRCRenderGraph.cpp:132,
 * src/VkScene.cpp:190). GLSL leaves the op sequence to its compiler; this
 * restatement fixes one that the GPU kernel repeats: dot products and
 * interpolations as fused multiply-add chains in component order, cross
 * products as multiply-then-subtract, normalize as a division by sqrt, unorm16
 * as u / 65535, lerp(x, y, t) = fma(t, y - x, x), exact fp32 filter weights
 * (hardware samplers quantise them), sRGB decoded per texel through a table
 * computed in double. Records with out-of-range indices unpack to zeros; a
 * texture id at or beyond the texture count reads as the constant colour. */
static float g_srgb[256];
static int g_srgb_ready = 0;

static void srgb_init(void) {
  if (g_srgb_ready) return;
  for (int i = 0; i < 256; ++i) {
    const double c = i / 255.0;
    g_srgb[i] = (float)(c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4));
  }
  g_srgb_ready = 1;
}

static inline float unorm16f(uint32_t u) { return (float)(u & 0xFFFFu) / 65535.0f; }
static inline float lerpf(float x, float y, float t) { return fmaf(t, y - x, x); }
static inline float interpf(float a, float b, float c, float w0, float w1, float w2) {
  return fmaf(c, w2, fmaf(b, w1, a * w0));
}

static uint32_t wrapf(float f, uint32_t n) {
  const float nf = (float)n;
  int r = (int)fmaf(-nf, floorf(f / nf), f);
  if (r < 0) r += (int)n;
  if (r >= (int)n) r -= (int)n;
  return (uint32_t)r;
}

static void sample_tex(const uint8_t* texels, uint32_t w, uint32_t h, float tu, float tv, float out[3]) {
  if (w == 0 || h == 0 || texels == NULL) {
    out[0] = out[1] = out[2] = 0.0f;
    return;
  }
  float u = fmaf(tu, (float)w, -0.5f), v = fmaf(tv, (float)h, -0.5f);
  if (!(fabsf(u) < 8388608.0f)) u = 0.0f;
  if (!(fabsf(v) < 8388608.0f)) v = 0.0f;
  const float fu = floorf(u), fv = floorf(v);
  const float a = u - fu, b = v - fv;
  const uint32_t i0 = wrapf(fu, w), j0 = wrapf(fv, h);
  const uint32_t i1 = i0 + 1 == w ? 0 : i0 + 1, j1 = j0 + 1 == h ? 0 : j0 + 1;
  const uint8_t* t00 = texels + 4 * ((size_t)j0 * w + i0);
  const uint8_t* t10 = texels + 4 * ((size_t)j0 * w + i1);
  const uint8_t* t01 = texels + 4 * ((size_t)j1 * w + i0);
  const uint8_t* t11 = texels + 4 * ((size_t)j1 * w + i1);
  for (int c = 0; c < 3; ++c)
    out[c] = lerpf(lerpf(g_srgb[t00[c]], g_srgb[t10[c]], a), lerpf(g_srgb[t01[c]], g_srgb[t11[c]], a), b);
}

void oracle_unpack(const oracle_scene* S, const uint32_t* packed, int64_t n, int64_t stride_words,
                   float* out, int64_t out_stride) {
  srgb_init();
  const float pi = 3.14159265358979323846f;
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t* in = packed + i * stride_words;
    float* r = out + i * out_stride;
    for (int k = 0; k < 14; ++k) r[k] = 0.0f;
    const uint32_t prim = in[0], inst = in[1] & 0x7FFFFFFFu;
    const int flip = (in[1] >> 31) != 0;
    if (prim >= S->primitive_count || inst >= S->instance_count) continue;
    uint32_t vi[3], ti[3];
    int ok = 1;
    for (int k = 0; k < 3; ++k) {
      vi[k] = S->vertex_indices[(size_t)prim * 3 + k];
      ti[k] = S->texcoord_indices[(size_t)prim * 3 + k];
      if (vi[k] >= S->vertex_count || ti[k] >= S->texcoord_count) ok = 0;
    }
    const uint32_t mid = S->material_ids[prim];
    if (!ok || mid >= S->material_count) continue;
    const float* T = S->transforms + (size_t)inst * 12;
    float v[3][3];
    for (int k = 0; k < 3; ++k) {
      const float* p = S->vertices + (size_t)vi[k] * 3;
      for (int c = 0; c < 3; ++c) {
        const float* col = T + 4 * c;
        v[k][c] = fmaf(p[2], col[2], fmaf(p[1], col[1], p[0] * col[0])) + col[3];
      }
    }
    float e1[3], e2[3], nn[3];
    for (int c = 0; c < 3; ++c) {
      e1[c] = v[1][c] - v[0][c];
      e2[c] = v[2][c] - v[0][c];
    }
    nn[0] = e1[1] * e2[2] - e1[2] * e2[1];
    nn[1] = e1[2] * e2[0] - e1[0] * e2[2];
    nn[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const float len = sqrtf(fmaf(nn[2], nn[2], fmaf(nn[1], nn[1], nn[0] * nn[0])));
    for (int c = 0; c < 3; ++c) nn[c] = flip ? -(nn[c] / len) : nn[c] / len;
    const float b1 = unorm16f(in[2]), b2 = unorm16f(in[2] >> 16);
    const float b0 = (1.0f - b1) - b2;
    for (int c = 0; c < 3; ++c) r[c] = interpf(v[0][c], v[1][c], v[2][c], b0, b1, b2);
    r[3] = unorm16f(in[3]);
    r[4] = unorm16f(in[3] >> 16);
    const float zc = nn[2] < -1.0f ? -1.0f : (nn[2] > 1.0f ? 1.0f : nn[2]);
    r[5] = (nn[0] == 0.0f && nn[1] == 0.0f) ? 0.5f : 0.5f + atan2f(nn[1], nn[0]) / (2.0f * pi);
    r[6] = acosf(zc) / pi;
    const oracle_material* m = S->materials + mid;
    r[7] = m->roughness;
    const float* tc[3];
    for (int k = 0; k < 3; ++k) tc[k] = S->texcoords + (size_t)ti[k] * 2;
    const float tu = interpf(tc[0][0], tc[1][0], tc[2][0], b0, b1, b2);
    const float tv = interpf(tc[0][1], tc[1][1], tc[2][1], b0, b1, b2);
    const uint32_t ids[2] = {m->diffuse_texture_id, m->specular_texture_id};
    const float* konst[2] = {m->diffuse, m->specular};
    for (int c = 0; c < 2; ++c) {
      float col[3] = {konst[c][0], konst[c][1], konst[c][2]};
      if (ids[c] != 0xFFFFFFFFu && ids[c] < S->texture_count) {
        const oracle_texture* t = S->textures + ids[c];
        sample_tex(t->texels, t->width, t->height, tu, tv, col);
      }
      for (int k = 0; k < 3; ++k) r[8 + 3 * c + k] = col[k];
    }
  }
}

/* ------------------------------------------------------------- fp8 -- */
/* E4M3 (bias 7, no infinities, max 448): round to nearest even, saturated to
 * +-448 (the GPU's cvt.rn.satfinite), NaN -> 0x7F. */
uint8_t oracle_f32_to_e4m3(float x) {
  if (isnan(x)) return 0x7F;
  const uint8_t sign = signbit(x) ? 0x80 : 0;
  float a = fabsf(x);
  if (a > 448.0f) a = 448.0f;
  if (a == 0.0f) return sign;
  int e;
  frexpf(a, &e);
  int ex = e - 1; /* floor(log2 a) */
  if (ex < -6) ex = -6;
  const float q = ldexpf(1.0f, ex - 3);
  const float r = rintf(a / q) * q; /* a / q is an exact power-of-two scaling */
  if (r == 0.0f) return sign;
  frexpf(r, &e);
  ex = e - 1;
  if (ex < -6) return (uint8_t)(sign | (int)(r / ldexpf(1.0f, -9)));
  const int m = (int)((r / ldexpf(1.0f, ex) - 1.0f) * 8.0f);
  return (uint8_t)(sign | ((ex + 7) << 3) | m);
}

float oracle_e4m3_to_f32(uint8_t b) {
  const int s = b >> 7, ex = (b >> 3) & 15, m = b & 7;
  float v;
  if (ex == 15 && m == 7) return NAN;
  if (ex == 0)
    v = ldexpf((float)m, -9);
  else
    v = ldexpf(1.0f + (float)m / 8.0f, ex - 7);
  return s ? -v : v;
}

/* NRCInputEncode's 64 features in fp32, before any rounding (the values
 * oracle_encode rounds to 16 bits). */
void oracle_encode_f32(const float* records, int64_t n, float* feats) {
  for (int64_t i = 0; i < n; ++i) {
    const float* r = records + ORACLE_IN_FLOATS * i;
    float* f = feats + 64 * i;
    for (int c = 0; c < 3; ++c) {
      float scale = 1.0f;
      for (int k = 0; k < 12; ++k, scale *= 2.0f) f[12 * c + k] = tri(r[c] * scale);
    }
    oneblob4(r[3], f + 36);
    oneblob4(r[4], f + 40);
    oneblob4(r[5], f + 44);
    oneblob4(r[6], f + 48);
    oneblob4(1.0f - oracle_expf(-r[7]), f + 52);
    for (int c = 0; c < 6; ++c) f[56 + c] = r[8 + c];
    f[62] = 1.0f;
    f[63] = 1.0f;
  }
}

/* The FP8 scales and E4M3 weights of the GPU's refresh (csrc/nrc_fp8.cu) from
 * 16-bit rendering weights w16 (format fmt) and the activation maxima seen
 * (0 = not seen: bounded from the previous layer). state: s_w[6], s_x[6],
 * c[6], 1/s_x[0], 448/max|W|[6]. w8: NRC_PARAM_COUNT bytes, parameter layout. */
void oracle_fp8_quantize(const uint16_t* w16, int fmt, const float seen[6], float* state, uint8_t* w8) {
  float amax_w[6] = {0}, rowsum[6] = {0};
  for (int row = 0; row < 323; ++row) {
    const int l = row < 320 ? row / 64 : 5;
    float s[32];
    for (int k = 0; k < 32; ++k) {
      const float a = fabsf(from16(w16[row * 64 + k], fmt)), b = fabsf(from16(w16[row * 64 + 32 + k], fmt));
      s[k] = a + b;
      const float m = a > b ? a : b;
      if (m > amax_w[l]) amax_w[l] = m;
    }
    for (int off = 16; off > 0; off >>= 1) { /* the GPU's butterfly: every lane ends with the same sum */
      float t[32];
      for (int k = 0; k < 32; ++k) t[k] = s[k] + s[k ^ off];
      memcpy(s, t, sizeof(t));
    }
    if (s[0] > rowsum[l]) rowsum[l] = s[0];
  }
  float ax[6], *sw = state, *sx = state + 6, *c = state + 12, *invw = state + 19;
  for (int l = 0; l < 6; ++l) {
    const float bound = l == 0 ? 1.0f : ax[l - 1] * rowsum[l - 1];
    ax[l] = seen[l] > 0.0f ? seen[l] : bound;
    if (!(ax[l] > 0.0f)) ax[l] = 1.0f;
    float aw = amax_w[l];
    if (!(aw > 0.0f)) aw = 1.0f;
    sw[l] = aw / 448.0f;
    invw[l] = 448.0f / aw;
    sx[l] = ax[l] / 448.0f;
  }
  for (int l = 0; l < 5; ++l) c[l] = (sw[l] * sx[l]) / sx[l + 1];
  c[5] = sw[5] * sx[5];
  state[18] = 1.0f / sx[0];
  for (int i = 0; i < ORACLE_P; ++i) {
    const int row = i / 64, l = row < 320 ? row / 64 : 5;
    w8[i] = oracle_f32_to_e4m3(from16(w16[i], fmt) * invw[l]);
  }
}

/* The FP8 query: features x8 = e4m3(f * inv_sx0); per hidden layer z = sum_i
 * w8 x8 (fp32, input order), x8' = e4m3(relu(z * c[l])); output z * c[5]
 * (unclamped). */
typedef struct {
  const uint8_t* w8;
  const float* c;
  float inv_sx0;
  const float* feats;
  float* out;
} fp8_ctx;

static void fp8_range(void* p, int64_t b, int64_t e, int tid) {
  (void)tid;
  fp8_ctx* x = (fp8_ctx*)p;
  for (int64_t r = b; r < e; ++r) {
    float a[64], z[64];
    for (int i = 0; i < 64; ++i) a[i] = oracle_e4m3_to_f32(oracle_f32_to_e4m3(x->feats[64 * r + i] * x->inv_sx0));
    for (int l = 0; l < 5; ++l) {
      for (int o = 0; o < 64; ++o) {
        float s = 0.0f;
        for (int i = 0; i < 64; ++i) s += oracle_e4m3_to_f32(x->w8[l * 4096 + o * 64 + i]) * a[i];
        z[o] = s;
      }
      for (int o = 0; o < 64; ++o) {
        const float y = z[o] * x->c[l];
        a[o] = oracle_e4m3_to_f32(oracle_f32_to_e4m3(y > 0.0f ? y : 0.0f));
      }
    }
    for (int k = 0; k < 3; ++k) {
      float s = 0.0f;
      for (int i = 0; i < 64; ++i) s += oracle_e4m3_to_f32(x->w8[5 * 4096 + k * 64 + i]) * a[i];
      x->out[3 * r + k] = s * x->c[5];
    }
  }
}

void oracle_forward_fp8(const uint8_t* w8, const float c[6], float inv_sx0, const float* feats, int64_t n, float* out,
                        int nthreads) {
  fp8_ctx x = {w8, c, inv_sx0, feats, out};
  parallel_for(n, nthreads, fp8_range, &x);
}
