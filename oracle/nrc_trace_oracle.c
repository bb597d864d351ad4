/*
 * CPU oracle of the record producer (the path tracer) — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of shader/src/path_tracer.comp (with CookTorranceBRDF.glsl,
 * Sample.glsl, RNG.glsl and Scene.glsl) used by tests/ to check the GPU tracer
 * against. GLSL leaves the order of floating-point operations and the accuracy of
 * its transcendental functions to the implementation; this restatement fixes one
 * choice: every expression is evaluated left to right with no contraction (built
 * with -ffp-contract=off), fused multiply-adds appear only as explicit fmaf, and
 * log, sin/cos, atan2, acos and exp are computed by the series and reductions
 * written below (a logarithm through atanh, sin/cos of 2 pi u by quadrant
 * reduction and Taylor series, atan by two argument reductions and its Taylor
 * series, exp by Cody-Waite reduction). The GPU tracer makes the same choices,
 * so images and records agree bit for bit; records appended through atomic
 * counters come in a different order, which the tests canonicalise.
 *
 * Hits: closest over all triangles (no BVH), ties to the lower triangle index.
 * Triangles are the instances' primitive ranges in instance order.
 * Primary hits: the camera ray from t = 0 without the secondary rays' 4.0 range
 * (the reference rasterises them into a V-buffer).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "nrc_oracle.h"

typedef struct {
  float x, y, z;
} V3;

static V3 v3(float x, float y, float z) {
  V3 r = {x, y, z};
  return r;
}
static V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static V3 scale(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static V3 divs(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
static V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
static float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static V3 normalize(V3 a) { return scale(a, 1.0f / sqrtf(dot(a, a))); }

static const float kPi = 3.14159265358979323846f;

static float bits_f(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static uint32_t f_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

static float t_log(float x) {
  if (x != x || x < 0.0f) return bits_f(0x7FC00000u);
  if (x == 0.0f) return -bits_f(0x7F800000u);
  if (x == bits_f(0x7F800000u)) return x;
  const uint32_t bits = f_bits(x);
  int e = (int)((bits >> 23) & 0xFF) - 127;
  float m = bits_f((bits & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e = e + 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f), s2 = s * s;
  float p = 1.0f / 15.0f;
  p = fmaf(p, s2, 1.0f / 13.0f);
  p = fmaf(p, s2, 1.0f / 11.0f);
  p = fmaf(p, s2, 1.0f / 9.0f);
  p = fmaf(p, s2, 1.0f / 7.0f);
  p = fmaf(p, s2, 1.0f / 5.0f);
  p = fmaf(p, s2, 1.0f / 3.0f);
  p = fmaf(p, s2, 1.0f);
  const float ef = (float)e;
  return fmaf(ef, 0.693145751953125f, fmaf(ef, 1.42860677e-06f, 2.0f * s * p));
}

static void t_sincos_turns(float u, float* so, float* co) {
  const float t = 4.0f * u;
  const float k = rintf(t);
  const float th = (t - k) * 1.57079637f;
  const float t2 = th * th;
  float sp = 1.0f / 362880.0f;
  sp = fmaf(sp, t2, -1.0f / 5040.0f);
  sp = fmaf(sp, t2, 1.0f / 120.0f);
  sp = fmaf(sp, t2, -1.0f / 6.0f);
  sp = fmaf(sp, t2, 1.0f);
  const float sn = th * sp;
  float cp = -1.0f / 3628800.0f;
  cp = fmaf(cp, t2, 1.0f / 40320.0f);
  cp = fmaf(cp, t2, -1.0f / 720.0f);
  cp = fmaf(cp, t2, 1.0f / 24.0f);
  cp = fmaf(cp, t2, -0.5f);
  const float cs = fmaf(cp, t2, 1.0f);
  const int q = (int)k & 3;
  *so = q == 0 ? sn : q == 1 ? cs : q == 2 ? -sn : -cs;
  *co = q == 0 ? cs : q == 1 ? -sn : q == 2 ? -cs : sn;
}

static float t_atan_pos(float z) {
  int inv = 0, shift = 0;
  if (z > 1.0f) {
    z = 1.0f / z;
    inv = 1;
  }
  if (z > 0.267949194f) {
    z = (z * 1.73205081f - 1.0f) / (z + 1.73205081f);
    shift = 1;
  }
  const float z2 = z * z;
  float p = 1.0f / 13.0f;
  p = fmaf(p, z2, -1.0f / 11.0f);
  p = fmaf(p, z2, 1.0f / 9.0f);
  p = fmaf(p, z2, -1.0f / 7.0f);
  p = fmaf(p, z2, 1.0f / 5.0f);
  p = fmaf(p, z2, -1.0f / 3.0f);
  p = fmaf(p, z2, 1.0f);
  float a = z * p;
  if (shift) a = a + 0.523598790f;
  if (inv) a = 1.57079637f - a;
  return a;
}

static float t_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  if (ax == 0.0f && ay == 0.0f) return 0.0f;
  float a = ay <= ax ? t_atan_pos(ay / ax) : 1.57079637f - t_atan_pos(ax / ay);
  if (x < 0.0f) a = kPi - a;
  return y < 0.0f ? -a : a;
}

static float t_acos(float x) { return t_atan2(sqrtf((1.0f - x) * (1.0f + x)), x); }

static float t_exp(float x) {
  x = fminf(fmaxf(x, -87.0f), 88.0f);
  const float k = rintf(x * 1.44269504f);
  float r = fmaf(k, -0.693145751953125f, x);
  r = fmaf(k, -1.42860677e-06f, r);
  float p = 1.98412698e-04f;
  p = fmaf(p, r, 1.38888889e-03f);
  p = fmaf(p, r, 8.33333333e-03f);
  p = fmaf(p, r, 4.16666667e-02f);
  p = fmaf(p, r, 1.66666667e-01f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  return p * bits_f((uint32_t)((int)k + 127) << 23);
}

/* RNG.glsl:6-13 */
static float rng_next(uint32_t* s) {
  *s = *s * 747796405u + 1u;
  uint32_t w = ((*s >> ((*s >> 28) + 4u)) ^ *s) * 277803737u;
  w = (w >> 22) ^ w;
  return (float)w / 4294967295.0f;
}

/* CookTorranceBRDF.glsl */
typedef struct {
  V3 diffuse, specular;
  float roughness, ior;
} Brdf;

static float ct_lum(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }
static float ct_spec_prob(const Brdf* b) {
  const float dl = ct_lum(b->diffuse), sl = ct_lum(b->specular);
  return sl / (dl + sl);
}
static float walter_g1(float v_dot_h, float v_dot_n, float ab2) {
  const float vn2 = v_dot_n * v_dot_n;
  const float a2 = 1.0f / (ab2 * (1.0f - vn2) / vn2), a = sqrtf(a2);
  return fmaxf(v_dot_h / v_dot_n, 0.0f) *
         (a >= 1.6f ? 1.0f : (3.535f * a + 2.181f * a2) / (1.0f + 2.276f * a + 2.577f * a2));
}
static float beckmann_d(float n_dot_h, float a2) {
  const float nh2 = n_dot_h * n_dot_h, nh4 = nh2 * nh2;
  return t_exp((nh2 - 1.0f) / (a2 * nh2)) / (kPi * a2 * nh4);
}
static float schlick(float v_dot_h, float ior) {
  float f0 = (ior - 1.0f) / (ior + 1.0f);
  f0 = f0 * f0;
  const float x = 1.0f - v_dot_h, x2 = x * x;
  return f0 + (1.0f - f0) * (x2 * x2 * x);
}
static V3 align_dir(V3 n, V3 d) {
  const V3 u = normalize(cross(fabsf(n.x) > 0.01f ? v3(0.f, 1.f, 0.f) : v3(1.f, 0.f, 0.f), n));
  const V3 v = cross(n, u);
  return add(add(scale(u, d.x), scale(v, d.y)), scale(n, d.z));
}
static V3 sample_cosine(V3 n, uint32_t* rng) {
  const float u1 = rng_next(rng), u2 = rng_next(rng);
  const float r = sqrtf(u1);
  float s, c;
  t_sincos_turns(u2, &s, &c);
  return align_dir(n, v3(r * c, r * s, sqrtf(1.0f - u1)));
}
static V3 ct_eval(const Brdf* b, V3 l, V3 v, V3 n) {
  const V3 h = normalize(add(l, v));
  const float n_dot_h = fmaxf(dot(n, h), 1e-8f);
  const float v_dot_h = fmaxf(dot(v, h), 1e-8f), l_dot_h = v_dot_h;
  const float n_dot_l = fminf(fmaxf(dot(n, l), 1e-8f), 1.0f - 1e-8f);
  const float n_dot_v = fminf(fmaxf(dot(n, v), 1e-8f), 1.0f - 1e-8f);
  const float a = b->roughness, a2 = a * a;
  const float G = walter_g1(v_dot_h, n_dot_v, a2) * walter_g1(l_dot_h, n_dot_l, a2);
  const float D = beckmann_d(n_dot_h, a2);
  const float F = schlick(v_dot_h, b->ior);
  const V3 spec = divs(scale(scale(scale(b->specular, D), G), F), 4.0f * n_dot_l * n_dot_v);
  return add(divs(b->diffuse, kPi), spec);
}
static float ct_pdf(const Brdf* b, V3 l, V3 v, V3 n) {
  const float n_dot_l = dot(l, n);
  if (n_dot_l < 0.0f) return 0.0f;
  const V3 h = normalize(add(l, v));
  const float a = b->roughness;
  const float p_h = beckmann_d(dot(n, h), a * a) * dot(n, h);
  const float p_ct = p_h / (4.0f * dot(v, h));
  const float p_l = n_dot_l / kPi;
  const float w = ct_spec_prob(b);
  return p_l * (1.0f - w) + p_ct * w;
}
static V3 ct_sample(const Brdf* b, V3 v, V3 n, uint32_t* rng) {
  const float a = b->roughness, a2 = a * a;
  float tan2 = -a2 * t_log(1.0f - rng_next(rng));
  if (tan2 != tan2) tan2 = 0.0f;
  const float n_dot_h = sqrtf(1.0f / (1.0f + tan2));
  float s, c;
  t_sincos_turns(rng_next(rng), &s, &c);
  const float r = sqrtf(1.0f - n_dot_h * n_dot_h);
  V3 h = align_dir(n, v3(r * c, r * s, n_dot_h));
  if (dot(v, h) < 0.0f) h = neg(h);
  const V3 iv = neg(v);
  V3 l = sub(iv, scale(h, 2.0f * dot(h, iv)));
  if (rng_next(rng) > ct_spec_prob(b)) l = sample_cosine(n, rng);
  return l;
}
static int is_inf(float f) { return fabsf(f) == bits_f(0x7F800000u); }
static V3 normalize_rgb(V3 c) {
  const int bad = c.x != c.x || c.y != c.y || c.z != c.z || is_inf(c.x) || is_inf(c.y) || is_inf(c.z);
  return bad ? v3(0.f, 0.f, 0.f) : v3(fmaxf(c.x, 0.f), fmaxf(c.y, 0.f), fmaxf(c.z, 0.f));
}

/* ------------------------------------------------------------ scene -- */
typedef struct {
  const oracle_scene* s;
  float lut[256];
  float* tri; /* 9 floats per triangle */
  uint32_t* tri_prim;
  uint32_t* tri_inst;
  uint32_t ntri;
} Scene;

static V3 xform(const float* T, V3 p) {
  return v3(p.x * T[0] + p.y * T[1] + p.z * T[2] + T[3], p.x * T[4] + p.y * T[5] + p.z * T[6] + T[7],
            p.x * T[8] + p.y * T[9] + p.z * T[10] + T[11]);
}
static V3 scene_vertex(const oracle_scene* S, uint32_t inst, uint32_t prim, int k) {
  const float* p = S->vertices + (size_t)S->vertex_indices[(size_t)prim * 3 + k] * 3;
  return xform(S->transforms + (size_t)inst * 12, v3(p[0], p[1], p[2]));
}
static float lerpf(float a, float b, float t) { return a + (b - a) * t; }
static uint32_t wrap_idx(float f, uint32_t n) {
  const float nf = (float)n;
  int r = (int)(f - nf * floorf(f / nf));
  if (r < 0) r += (int)n;
  if (r >= (int)n) r -= (int)n;
  return (uint32_t)r;
}
static V3 tex_sample(const oracle_texture* t, float tu, float tv, const float* lut) {
  const uint32_t w = t->width, h = t->height;
  if (w == 0 || h == 0 || t->texels == NULL) return v3(0.f, 0.f, 0.f);
  float u = tu * (float)w - 0.5f, v = tv * (float)h - 0.5f;
  if (!(fabsf(u) < 8388608.0f)) u = 0.0f;
  if (!(fabsf(v) < 8388608.0f)) v = 0.0f;
  const float fu = floorf(u), fv = floorf(v), a = u - fu, b = v - fv;
  const uint32_t i0 = wrap_idx(fu, w), j0 = wrap_idx(fv, h);
  const uint32_t i1 = i0 + 1 == w ? 0 : i0 + 1, j1 = j0 + 1 == h ? 0 : j0 + 1;
  const uint8_t* t00 = t->texels + 4 * ((size_t)j0 * w + i0);
  const uint8_t* t10 = t->texels + 4 * ((size_t)j0 * w + i1);
  const uint8_t* t01 = t->texels + 4 * ((size_t)j1 * w + i0);
  const uint8_t* t11 = t->texels + 4 * ((size_t)j1 * w + i1);
  float o[3];
  for (int c = 0; c < 3; ++c) o[c] = lerpf(lerpf(lut[t00[c]], lut[t10[c]], a), lerpf(lut[t01[c]], lut[t11[c]], a), b);
  return v3(o[0], o[1], o[2]);
}
static V3 mat_color(const oracle_scene* S, const float* konst, uint32_t id, float tu, float tv, const float* lut) {
  if (id != 0xFFFFFFFFu && id < S->texture_count) return tex_sample(S->textures + id, tu, tv, lut);
  return v3(konst[0], konst[1], konst[2]);
}

typedef struct {
  V3 position, normal, diffuse, specular, emission;
  float bu, bv, roughness, ior;
  uint32_t prim, inst;
  int flip;
} Hit;

typedef struct {
  V3 o, d;
} Ray;

static Hit make_hit(const Scene* SC, uint32_t prim, uint32_t inst, float bu, float bv, V3 v0, V3 v1, V3 v2,
                    V3 n_unnorm, Ray ray) {
  const oracle_scene* S = SC->s;
  Hit h;
  const V3 n = normalize(n_unnorm);
  h.flip = dot(n, ray.d) >= 0.0f;
  h.normal = h.flip ? neg(n) : n;
  h.prim = prim;
  h.inst = inst;
  h.bu = bu;
  h.bv = bv;
  const float b0 = 1.0f - bu - bv;
  h.position = add(add(scale(v0, b0), scale(v1, bu)), scale(v2, bv));
  const float* t0 = S->texcoords + (size_t)S->texcoord_indices[(size_t)prim * 3 + 0] * 2;
  const float* t1 = S->texcoords + (size_t)S->texcoord_indices[(size_t)prim * 3 + 1] * 2;
  const float* t2 = S->texcoords + (size_t)S->texcoord_indices[(size_t)prim * 3 + 2] * 2;
  const float tu = t0[0] * b0 + t1[0] * bu + t2[0] * bv, tv = t0[1] * b0 + t1[1] * bu + t2[1] * bv;
  const oracle_material* m = S->materials + S->material_ids[prim];
  h.diffuse = mat_color(S, m->diffuse, m->diffuse_texture_id, tu, tv, SC->lut);
  h.specular = mat_color(S, m->specular, m->specular_texture_id, tu, tv, SC->lut);
  h.emission = mat_color(S, m->emission, m->emission_texture_id, tu, tv, SC->lut);
  h.roughness = m->roughness;
  h.ior = m->ior;
  return h;
}

static int intersect(const float* T, Ray r, float tmin, float tmax, float* t, float* u, float* v) {
  const V3 v0 = v3(T[0], T[1], T[2]), e1 = sub(v3(T[3], T[4], T[5]), v0), e2 = sub(v3(T[6], T[7], T[8]), v0);
  const V3 p = cross(r.d, e2);
  const float det = dot(e1, p);
  if (det == 0.0f || det != det) return 0;
  const float inv = 1.0f / det;
  const V3 s = sub(r.o, v0);
  *u = dot(s, p) * inv;
  if (!(*u >= 0.0f && *u <= 1.0f)) return 0;
  const V3 q = cross(s, e1);
  *v = dot(r.d, q) * inv;
  if (!(*v >= 0.0f && *u + *v <= 1.0f)) return 0;
  *t = dot(e2, q) * inv;
  return *t >= tmin && *t <= tmax;
}

static int closest(const Scene* SC, Ray r, float tmin, float tmax, float* bt, float* bu, float* bv) {
  int best = -1;
  *bt = tmax;
  for (uint32_t i = 0; i < SC->ntri; ++i) {
    float t, u, v;
    if (intersect(SC->tri + (size_t)i * 9, r, tmin, *bt, &t, &u, &v) && (best < 0 || t < *bt)) {
      best = (int)i;
      *bt = t;
      *bu = u;
      *bv = v;
    }
  }
  return best;
}

/* ----------------------------------------------------------- tracer -- */
typedef struct {
  const Scene* sc;
  const oracle_trace_params* p;
  oracle_trace_out* o;
} Ctx;

typedef struct {
  V3 color;
  float cosine, pdf, dist2;
  Ray ray;
} Step;

typedef struct {
  uint32_t w[4];
} Packed;

static uint32_t pack_unorm2x16(float a, float b) {
  const float ca = fminf(fmaxf(a, 0.0f), 1.0f), cb = fminf(fmaxf(b, 0.0f), 1.0f);
  return (uint32_t)rintf(ca * 65535.0f) | ((uint32_t)rintf(cb * 65535.0f) << 16);
}
static Packed make_input(const Hit* h, V3 d) {
  Packed i;
  i.w[0] = h->prim;
  i.w[1] = h->inst | (h->flip ? 0x80000000u : 0u);
  i.w[2] = pack_unorm2x16(h->bu, h->bv);
  const float su = (d.x == 0.0f && d.y == 0.0f) ? 0.5f : 0.5f + t_atan2(d.y, d.x) / (2.0f * kPi);
  const float sv = t_acos(fminf(fmaxf(d.z, -1.0f), 1.0f)) / kPi;
  i.w[3] = pack_unorm2x16(su, sv);
  return i;
}
static Step brdf_step(const Hit* h, Ray ray, uint32_t* rng) {
  Brdf b = {h->diffuse, h->specular, fmaxf(h->roughness, 0.001f), fmaxf(h->ior, 1.5f)};
  const V3 v = neg(ray.d);
  const V3 dir = ct_sample(&b, v, h->normal, rng);
  const float pdf = ct_pdf(&b, dir, v, h->normal);
  const V3 f = ct_eval(&b, dir, v, h->normal);
  const float cosine = fabsf(dot(h->normal, dir));
  Step s;
  s.color = normalize_rgb(divs(scale(f, cosine), pdf));
  s.ray.o = h->position;
  s.ray.d = dir;
  s.cosine = cosine;
  s.pdf = pdf;
  const V3 dd = sub(ray.o, h->position);
  s.dist2 = dot(dd, dd);
  return s;
}
static int trace_hit(const Ctx* C, Ray ray, Hit* h) {
  float t, u, v;
  const int ti = closest(C->sc, ray, 1e-6f, 4.0f, &t, &u, &v);
  if (ti < 0) return 0;
  const uint32_t prim = C->sc->tri_prim[ti], inst = C->sc->tri_inst[ti];
  const oracle_scene* S = C->sc->s;
  const V3 v0 = scene_vertex(S, inst, prim, 0), v1 = scene_vertex(S, inst, prim, 1), v2 = scene_vertex(S, inst, prim, 2);
  *h = make_hit(C->sc, prim, inst, u, v, v0, v1, v2, cross(sub(v1, v0), sub(v2, v0)), ray);
  return 1;
}
static void push_eval(const Ctx* C, uint32_t dst, Packed in) {
  const uint32_t id = C->o->eval_count++;
  if (id >= C->o->eval_capacity) return;
  uint32_t* w = C->o->eval_records + (size_t)id * 5;
  w[0] = dst;
  memcpy(w + 1, in.w, 16);
}
static uint32_t dst_screen(uint32_t x, uint32_t y) { return (x | (y << 15)) << 1; }
static uint32_t dst_train(uint32_t b, uint32_t l, uint32_t r) { return ((b | (l << 2) | (r << 16)) << 1) | 1u; }

typedef struct {
  V3 bias, factor;
} Result;

static Result path_trace(const Ctx* C, Hit hit, Ray ray, uint32_t method, uint32_t* rng, uint32_t x, uint32_t y) {
  V3 radiance = v3(0.f, 0.f, 0.f), acc = v3(1.f, 1.f, 1.f);
  Step info = brdf_step(&hit, ray, rng);
  radiance = add(radiance, mul(acc, hit.emission));
  acc = mul(acc, info.color);
  ray = info.ray;
  const float c_a0 = method == 0 ? bits_f(0x7F800000u) : 0.01f * info.dist2 / (4.0f * kPi * info.cosine);
  float sqrt_a_sum = 0.0f;
  if (method != 2) {
    for (int bounce = 1; bounce < 8 && sqrt_a_sum * sqrt_a_sum <= c_a0; ++bounce) {
      if (trace_hit(C, ray, &hit)) {
        info = brdf_step(&hit, ray, rng);
        radiance = add(radiance, mul(acc, hit.emission));
        acc = mul(acc, info.color);
        ray = info.ray;
        sqrt_a_sum = sqrt_a_sum + sqrtf(info.dist2 / (info.pdf * info.cosine));
      } else {
        radiance = add(radiance, scale(acc, 10.0f));
        Result r = {radiance, acc};
        return r;
      }
    }
  }
  if (method != 0) push_eval(C, dst_screen(x, y), make_input(&hit, ray.d));
  Result r = {radiance, acc};
  return r;
}

static Result extended_trace(const Ctx* C, Hit hit, Ray ray, uint32_t method, uint32_t* rng, uint32_t x, uint32_t y) {
  V3 lights[8], colors[8];
  Packed inputs[8];
  for (int i = 0; i < 8; ++i) {
    colors[i] = v3(1.f, 1.f, 1.f);
    lights[i] = v3(0.f, 0.f, 0.f);
  }
  V3 acc = v3(1.f, 1.f, 1.f), radiance = v3(0.f, 0.f, 0.f);
  int light_terminate = 0;
  Step info = brdf_step(&hit, ray, rng);
  radiance = add(radiance, mul(acc, hit.emission));
  acc = mul(acc, info.color);
  ray = info.ray;
  Result result = {radiance, acc};
  inputs[0] = make_input(&hit, ray.d);
  const float c_a0 = 0.01f * info.dist2 / (4.0f * kPi * info.cosine);
  float sqrt_a_sum = 0.0f;
  int bounce = 1;
  for (; bounce < 8 && sqrt_a_sum * sqrt_a_sum <= c_a0; ++bounce) {
    if (trace_hit(C, ray, &hit)) {
      info = brdf_step(&hit, ray, rng);
      radiance = add(radiance, mul(acc, hit.emission));
      acc = mul(acc, info.color);
      ray = info.ray;
      sqrt_a_sum = sqrt_a_sum + sqrtf(info.dist2 / (info.pdf * info.cosine));
      lights[bounce - 1] = hit.emission;
      colors[bounce - 1] = info.color;
      inputs[bounce] = make_input(&hit, ray.d);
    } else {
      radiance = add(radiance, scale(acc, 10.0f));
      lights[bounce - 1] = v3(10.f, 10.f, 10.f);
      light_terminate = 1;
      break;
    }
  }
  if (method == 2) {
    push_eval(C, dst_screen(x, y), inputs[0]);
  } else {
    result.bias = radiance;
    result.factor = acc;
    if (!light_terminate) push_eval(C, dst_screen(x, y), inputs[bounce - 1]);
  }
  sqrt_a_sum = 0.0f;
  light_terminate = 0;
  for (; bounce < 8 && sqrt_a_sum * sqrt_a_sum <= c_a0; ++bounce) {
    if (trace_hit(C, ray, &hit)) {
      info = brdf_step(&hit, ray, rng);
      ray = info.ray;
      sqrt_a_sum = sqrt_a_sum + sqrtf(info.dist2 / (info.pdf * info.cosine));
      lights[bounce - 1] = hit.emission;
      colors[bounce - 1] = info.color;
      inputs[bounce] = make_input(&hit, ray.d);
    } else {
      lights[bounce - 1] = v3(10.f, 10.f, 10.f);
      light_terminate = 1;
      break;
    }
  }
  uint32_t batch = (uint32_t)(rng_next(rng) * 4.0f);
  batch = batch < 3 ? batch : 3;
  const uint32_t train_id = C->o->train_counts[batch];
  C->o->train_counts[batch] += (uint32_t)bounce;
  if (train_id < 16384) {
    for (int i = bounce - 2; i >= 0; --i) {
      lights[i] = add(lights[i], mul(colors[i], lights[i + 1]));
      colors[i] = mul(colors[i], colors[i + 1]);
    }
    const uint32_t count = (uint32_t)bounce < 16384 - train_id ? (uint32_t)bounce : 16384 - train_id;
    for (uint32_t i = 0; i < count; ++i) {
      uint32_t* w = C->o->train_records[batch] + (size_t)(train_id + i) * 10;
      const float f[6] = {lights[i].x, lights[i].y, lights[i].z, colors[i].x, colors[i].y, colors[i].z};
      memcpy(w, f, 24);
      memcpy(w + 6, inputs[i].w, 16);
    }
    if (!light_terminate) push_eval(C, dst_train(batch, train_id, train_id + count - 1), inputs[bounce - 1]);
  }
  return result;
}

void oracle_path_trace(const oracle_scene* S, const uint32_t* ranges, const oracle_trace_params* p,
                       oracle_trace_out* o) {
  Scene SC;
  SC.s = S;
  for (int i = 0; i < 256; ++i) {
    const double c = i / 255.0;
    SC.lut[i] = (float)(c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4));
  }
  /* world-space triangles: the instances' primitive ranges in instance order */
  uint64_t n = 0;
  for (uint32_t i = 0; i < S->instance_count; ++i) n += ranges[2 * i + 1];
  SC.ntri = (uint32_t)n;
  SC.tri = (float*)malloc((size_t)(n ? n : 1) * 9 * sizeof(float));
  SC.tri_prim = (uint32_t*)malloc((size_t)(n ? n : 1) * 4);
  SC.tri_inst = (uint32_t*)malloc((size_t)(n ? n : 1) * 4);
  uint32_t t = 0;
  for (uint32_t i = 0; i < S->instance_count; ++i)
    for (uint32_t k = 0; k < ranges[2 * i + 1]; ++k, ++t) {
      const uint32_t prim = ranges[2 * i] + k;
      for (int c = 0; c < 3; ++c) {
        const V3 v = scene_vertex(S, i, prim, c);
        SC.tri[(size_t)t * 9 + 3 * c] = v.x;
        SC.tri[(size_t)t * 9 + 3 * c + 1] = v.y;
        SC.tri[(size_t)t * 9 + 3 * c + 2] = v.z;
      }
      SC.tri_prim[t] = prim;
      SC.tri_inst[t] = i;
    }
  Ctx C = {&SC, p, o};
  const V3 look = v3(p->look[0], p->look[1], p->look[2]), side = v3(p->side[0], p->side[1], p->side[2]),
           up = v3(p->up[0], p->up[1], p->up[2]), org = v3(p->origin[0], p->origin[1], p->origin[2]);
  const uint32_t bw = (p->width + 7) / 8, bh = (p->height + 7) / 8;
  for (uint32_t by = 0; by < bh; ++by)
    for (uint32_t bx = 0; bx < bw; ++bx)
      for (int warp = 0; warp < 2; ++warp) {
        /* lanes: threadIdx.y = 4 warp + lane / 8, threadIdx.x = lane % 8 */
        uint32_t px[32], py[32], rng[32];
        int inside[32], first = -1, left_all = 1;
        for (int lane = 0; lane < 32; ++lane) {
          px[lane] = bx * 8 + (uint32_t)(lane % 8);
          py[lane] = by * 8 + (uint32_t)(4 * warp + lane / 8);
          rng[lane] = (((py[lane] & 0xFFu) << 8) | (px[lane] & 0xFFu)) + p->seed;
          inside[lane] = px[lane] < p->width && py[lane] < p->height;
          if (inside[lane] && first < 0) first = lane;
          if (inside[lane] && !(px[lane] <= p->width / 2)) left_all = 0;
        }
        if (first < 0) continue;
        const uint32_t method = left_all ? p->left_method : p->right_method;
        int train = 0;
        if (method != 0) train = rng_next(&rng[first]) < p->train_probability;
        for (int lane = 0; lane < 32; ++lane) {
          if (!inside[lane]) continue;
          const uint32_t x = px[lane], y = py[lane];
          const float cx = ((float)x + 0.5f) / (float)p->width * 2.0f - 1.0f;
          const float cy = ((float)y + 0.5f) / (float)p->height * 2.0f - 1.0f;
          Ray ray;
          ray.o = org;
          ray.d = normalize(add(add(look, scale(side, cx)), scale(up, cy)));
          Result res;
          float pt, pu, pv;
          const int ti = closest(&SC, ray, 0.0f, bits_f(0x7F800000u), &pt, &pu, &pv);
          if (ti < 0) {
            res.bias = v3(10.f, 10.f, 10.f);
            res.factor = v3(0.f, 0.f, 0.f);
          } else {
            const uint32_t prim = SC.tri_prim[ti], inst = SC.tri_inst[ti];
            const V3 v0 = scene_vertex(S, inst, prim, 0), v1 = scene_vertex(S, inst, prim, 1),
                     v2 = scene_vertex(S, inst, prim, 2);
            const V3 v01 = sub(v1, v0), v02 = sub(v2, v0), v0o = sub(ray.o, v0);
            const V3 nn = cross(v01, v02), q = cross(v0o, ray.d);
            const float d = 1.0f / dot(ray.d, nn);
            const float u = d * dot(neg(q), v02), v = d * dot(q, v01);
            const Hit hit = make_hit(&SC, prim, inst, u, v, v0, v1, v2, nn, ray);
            res = train ? extended_trace(&C, hit, ray, method, &rng[lane], x, y)
                        : path_trace(&C, hit, ray, method, &rng[lane], x, y);
          }
          res.bias = normalize_rgb(res.bias);
          res.factor = normalize_rgb(res.factor);
          const size_t pix = (size_t)y * p->width + x;
          o->bias_factor_r[4 * pix + 0] = res.bias.x;
          o->bias_factor_r[4 * pix + 1] = res.bias.y;
          o->bias_factor_r[4 * pix + 2] = res.bias.z;
          o->bias_factor_r[4 * pix + 3] = res.factor.x;
          o->factor_gb[2 * pix + 0] = res.factor.y;
          o->factor_gb[2 * pix + 1] = res.factor.z;
        }
      }
  free(SC.tri);
  free(SC.tri_prim);
  free(SC.tri_inst);
}
