// Record producer: the reference's path tracer (shader/src/path_tracer.comp)
// over a BVH built on the GPU. Host code (build, launch) and kernels.
//
// This file is compiled with -fmad=false: every multiply and add below is a
// separate IEEE operation unless written as fmaf, so the CPU oracle
// (oracle/nrc_trace_oracle.c), which repeats each expression in the same order
// with contraction off, produces the same floats. For the same reason the
// transcendental functions are this file's own (their methods are named where
// they are defined) rather than CUDA's, and a hit at equal distance from two
// triangles goes to the lower triangle index.
#include <cub/device/device_radix_sort.cuh>

#include <cmath>
#include <new>
#include <vector>

#include "nrc_common.cuh"
#include "nrc_kernels.h"

struct nrc_bvh {
  int device = 0;
  uint32_t tris = 0, nodes = 0;
  void* block = nullptr;  // triangles, then nodes
  const float4* tri = nullptr;  // 3 x float4 per triangle: v0.xyz prim, v1.xyz inst, v2.xyz pad
  const uint4* node = nullptr;  // 2 x uint4 per node: lo.xyz left, hi.xyz right
};

namespace nrc {
namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr uint32_t kLeaf = 0x80000000u;  // child index flag: a triangle
constexpr int kMaxBounce = 8;            // path_tracer.comp:11
constexpr float kTMin = 1e-6f, kTMax = 4.0f;  // path_tracer.comp:12-13
constexpr float kC = 0.01f;                   // path_tracer.comp:14
constexpr float kConstLight = 10.0f;          // path_tracer.comp:145

// ------------------------------------------------------------------ math --
struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 scale(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 divs(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3 normalize(V3 a) { return scale(a, 1.0f / sqrtf(dot(a, a))); }

// Natural logarithm: x = m 2^e with m in [1/sqrt(2), sqrt(2)), log m = 2 atanh(s),
// s = (m - 1) / (m + 1), by the odd series of atanh to s^15; e ln 2 in two parts.
__device__ float t_log(float x) {
  if (x != x || x < 0.0f) return __int_as_float(0x7FC00000);
  if (x == 0.0f) return -__int_as_float(0x7F800000);
  if (x == __int_as_float(0x7F800000)) return x;
  int bits = __float_as_int(x);
  int e = ((bits >> 23) & 0xFF) - 127;
  float m = __int_as_float((bits & 0x007FFFFF) | 0x3F800000);  // [1, 2)
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
  const float ef = static_cast<float>(e);
  return fmaf(ef, 0.693145751953125f, fmaf(ef, 1.42860677e-06f, 2.0f * s * p));
}

// sin and cos of 2 pi u: t = 4u = k + f with k = rint(t) (exact) and |f| <= 1/2,
// theta = f pi/2 in [-pi/4, pi/4]; Taylor series of sin to theta^9 and cos to
// theta^10, then the quadrant k mod 4.
__device__ void t_sincos_turns(float u, float& so, float& co) {
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
  const int q = static_cast<int>(k) & 3;
  so = q == 0 ? sn : q == 1 ? cs : q == 2 ? -sn : -cs;
  co = q == 0 ? cs : q == 1 ? -sn : q == 2 ? -cs : sn;
}

// atan on [0, inf): 1/z above 1 (pi/2 - atan), then atan z = pi/6 + atan((z sqrt3 - 1) / (z + sqrt3))
// above tan(pi/12), then the odd Taylor series to z^13.
__device__ float t_atan_pos(float z) {
  bool inv = false, shift = false;
  if (z > 1.0f) {
    z = 1.0f / z;
    inv = true;
  }
  if (z > 0.267949194f) {
    z = (z * 1.73205081f - 1.0f) / (z + 1.73205081f);
    shift = true;
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

__device__ float t_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  if (ax == 0.0f && ay == 0.0f) return 0.0f;
  float a = ay <= ax ? t_atan_pos(ay / ax) : 1.57079637f - t_atan_pos(ax / ay);
  if (x < 0.0f) a = kPi - a;
  return y < 0.0f ? -a : a;
}

__device__ float t_acos(float x) { return t_atan2(sqrtf((1.0f - x) * (1.0f + x)), x); }

// e^x: Cody-Waite reduction and the degree-7 Taylor polynomial (as the encoding's)
__device__ float t_exp(float x) {
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
  return p * __int_as_float((static_cast<int>(k) + 127) << 23);
}

// ------------------------------------------------------------------- rng --
// RNG.glsl:6-13: a condensed PCG (rxs-m-xs) step, then word / (2^32 - 1).
struct Rng {
  uint32_t s;
  __device__ float next() {
    s = s * 747796405u + 1u;
    uint32_t w = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
    w = (w >> 22) ^ w;
    return static_cast<float>(w) / 4294967295.0f;
  }
};

// ------------------------------------------------------------------ brdf --
// CookTorranceBRDF.glsl: Beckmann distribution, Walter's G1 approximation,
// Schlick's Fresnel, specular/diffuse lobe choice by luminance.
struct Brdf {
  V3 diffuse, specular;
  float roughness, ior;
};

__device__ __forceinline__ float ct_lum(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }
__device__ __forceinline__ float ct_spec_prob(const Brdf& b) {
  const float dl = ct_lum(b.diffuse), sl = ct_lum(b.specular);
  return sl / (dl + sl);
}
__device__ float walter_g1(float v_dot_h, float v_dot_n, float ab2) {
  const float vn2 = v_dot_n * v_dot_n;
  const float a2 = 1.0f / (ab2 * (1.0f - vn2) / vn2), a = sqrtf(a2);
  return fmaxf(v_dot_h / v_dot_n, 0.0f) *
         (a >= 1.6f ? 1.0f : (3.535f * a + 2.181f * a2) / (1.0f + 2.276f * a + 2.577f * a2));
}
__device__ float beckmann_d(float n_dot_h, float a2) {
  const float nh2 = n_dot_h * n_dot_h, nh4 = nh2 * nh2;
  return t_exp((nh2 - 1.0f) / (a2 * nh2)) / (kPi * a2 * nh4);
}
__device__ float schlick(float v_dot_h, float ior) {
  float f0 = (ior - 1.0f) / (ior + 1.0f);
  f0 = f0 * f0;
  const float x = 1.0f - v_dot_h, x2 = x * x;
  return f0 + (1.0f - f0) * (x2 * x2 * x);
}
// AlignDir (Sample.glsl:7-11)
__device__ V3 align_dir(V3 n, V3 d) {
  const V3 u = normalize(cross(fabsf(n.x) > 0.01f ? v3(0.f, 1.f, 0.f) : v3(1.f, 0.f, 0.f), n));
  const V3 v = cross(n, u);
  return add(add(scale(u, d.x), scale(v, d.y)), scale(n, d.z));
}
__device__ V3 sample_cosine(V3 n, Rng& rng) {  // Sample.glsl:13-20 (direction only)
  const float u1 = rng.next(), u2 = rng.next();
  const float r = sqrtf(u1);
  float s, c;
  t_sincos_turns(u2, s, c);
  return align_dir(n, v3(r * c, r * s, sqrtf(1.0f - u1)));
}
__device__ V3 ct_eval(const Brdf& b, V3 l, V3 v, V3 n) {
  const V3 h = normalize(add(l, v));
  const float n_dot_h = fmaxf(dot(n, h), 1e-8f);
  const float v_dot_h = fmaxf(dot(v, h), 1e-8f), l_dot_h = v_dot_h;
  const float n_dot_l = fminf(fmaxf(dot(n, l), 1e-8f), 1.0f - 1e-8f);
  const float n_dot_v = fminf(fmaxf(dot(n, v), 1e-8f), 1.0f - 1e-8f);
  const float a = b.roughness, a2 = a * a;
  const float G = walter_g1(v_dot_h, n_dot_v, a2) * walter_g1(l_dot_h, n_dot_l, a2);
  const float D = beckmann_d(n_dot_h, a2);
  const float F = schlick(v_dot_h, b.ior);
  // specular * D * G * F / (4 n.l n.v), left to right per channel; diffuse / pi
  const V3 spec = divs(scale(scale(scale(b.specular, D), G), F), 4.0f * n_dot_l * n_dot_v);
  return add(divs(b.diffuse, kPi), spec);
}
__device__ float ct_pdf(const Brdf& b, V3 l, V3 v, V3 n) {
  const float n_dot_l = dot(l, n);
  if (n_dot_l < 0.0f) return 0.0f;
  const V3 h = normalize(add(l, v));
  const float a = b.roughness;
  const float p_h = beckmann_d(dot(n, h), a * a) * dot(n, h);
  const float p_ct = p_h / (4.0f * dot(v, h));
  const float p_l = n_dot_l / kPi;
  const float w = ct_spec_prob(b);
  return p_l * (1.0f - w) + p_ct * w;  // mix(p_lambert, p_cook_torrance, w)
}
// CookTorranceSample: returns the incident direction; pdf via ct_pdf.
__device__ V3 ct_sample(const Brdf& b, V3 v, V3 n, Rng& rng) {
  const float a = b.roughness, a2 = a * a;
  float tan2 = -a2 * t_log(1.0f - rng.next());
  if (tan2 != tan2) tan2 = 0.0f;
  const float n_dot_h = sqrtf(1.0f / (1.0f + tan2));
  float s, c;
  t_sincos_turns(rng.next(), s, c);
  const float r = sqrtf(1.0f - n_dot_h * n_dot_h);
  V3 h = align_dir(n, v3(r * c, r * s, n_dot_h));
  if (dot(v, h) < 0.0f) h = neg(h);
  // reflect(-v, h) = -v - 2 dot(h, -v) h
  const V3 iv = neg(v);
  V3 l = sub(iv, scale(h, 2.0f * dot(h, iv)));
  if (rng.next() > ct_spec_prob(b)) l = sample_cosine(n, rng);
  return l;
}

__device__ __forceinline__ V3 normalize_rgb(V3 c) {  // NormalizeRGB, path_tracer.comp:147
  const bool bad = c.x != c.x || c.y != c.y || c.z != c.z || fabsf(c.x) == __int_as_float(0x7F800000) ||
                   fabsf(c.y) == __int_as_float(0x7F800000) || fabsf(c.z) == __int_as_float(0x7F800000);
  return bad ? v3(0.f, 0.f, 0.f) : v3(fmaxf(c.x, 0.f), fmaxf(c.y, 0.f), fmaxf(c.z, 0.f));
}

// ----------------------------------------------------------------- scene --
struct TraceScene {
  nrc_scene s;
  float lut[256];  // sRGB -> linear (texels decoded before filtering)
};

__device__ V3 xform(const float* T, V3 p) {  // vec4(p, 1) * mat3x4
  return v3(p.x * T[0] + p.y * T[1] + p.z * T[2] + T[3], p.x * T[4] + p.y * T[5] + p.z * T[6] + T[7],
            p.x * T[8] + p.y * T[9] + p.z * T[10] + T[11]);
}

__device__ V3 scene_vertex(const nrc_scene& S, uint32_t inst, uint32_t prim, int k) {
  const float* p = S.vertices + size_t(S.vertex_indices[size_t(prim) * 3 + k]) * 3;
  return xform(S.transforms + size_t(inst) * 12, v3(p[0], p[1], p[2]));
}

__device__ float lerpf(float a, float b, float t) { return a + (b - a) * t; }

__device__ uint32_t wrap_idx(float f, uint32_t n) {
  const float nf = static_cast<float>(n);
  int r = static_cast<int>(f - nf * floorf(f / nf));
  if (r < 0) r += static_cast<int>(n);
  if (r >= static_cast<int>(n)) r -= static_cast<int>(n);
  return static_cast<uint32_t>(r);
}

__device__ V3 tex_sample(const nrc_texture& t, float tu, float tv, const float* lut) {
  const uint32_t w = t.width, h = t.height;
  if (w == 0 || h == 0 || t.texels == nullptr) return v3(0.f, 0.f, 0.f);
  float u = tu * static_cast<float>(w) - 0.5f, v = tv * static_cast<float>(h) - 0.5f;
  if (!(fabsf(u) < 8388608.0f)) u = 0.0f;
  if (!(fabsf(v) < 8388608.0f)) v = 0.0f;
  const float fu = floorf(u), fv = floorf(v), a = u - fu, b = v - fv;
  const uint32_t i0 = wrap_idx(fu, w), j0 = wrap_idx(fv, h);
  const uint32_t i1 = i0 + 1 == w ? 0 : i0 + 1, j1 = j0 + 1 == h ? 0 : j0 + 1;
  const uchar4* px = reinterpret_cast<const uchar4*>(t.texels);
  const uchar4 t00 = px[size_t(j0) * w + i0], t10 = px[size_t(j0) * w + i1];
  const uchar4 t01 = px[size_t(j1) * w + i0], t11 = px[size_t(j1) * w + i1];
  auto ch = [&](unsigned char c00, unsigned char c10, unsigned char c01, unsigned char c11) {
    return lerpf(lerpf(lut[c00], lut[c10], a), lerpf(lut[c01], lut[c11], a), b);
  };
  return v3(ch(t00.x, t10.x, t01.x, t11.x), ch(t00.y, t10.y, t01.y, t11.y), ch(t00.z, t10.z, t01.z, t11.z));
}

__device__ V3 mat_color(const nrc_scene& S, const float* konst, uint32_t id, float tu, float tv, const float* lut) {
  if (id != 0xFFFFFFFFu && id < S.texture_count) return tex_sample(S.textures[id], tu, tv, lut);
  return v3(konst[0], konst[1], konst[2]);
}

struct Hit {
  V3 position, normal, diffuse, specular, emission;
  float bu, bv;  // barycentrics of vertices 1 and 2
  float roughness, ior;
  uint32_t prim, inst;
  bool flip;
};

struct Ray {
  V3 o, d;
};

// The hit record of (prim, inst) with barycentrics (bu, bv): GetRayQueryHit /
// GetVBufferHit (path_tracer.comp:66-131) after their barycentrics.
__device__ Hit make_hit(const nrc_scene& S, const float* lut, uint32_t prim, uint32_t inst, float bu, float bv,
                        V3 v0, V3 v1, V3 v2, V3 n_unnorm, Ray ray) {
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
  const float* t0 = S.texcoords + size_t(S.texcoord_indices[size_t(prim) * 3 + 0]) * 2;
  const float* t1 = S.texcoords + size_t(S.texcoord_indices[size_t(prim) * 3 + 1]) * 2;
  const float* t2 = S.texcoords + size_t(S.texcoord_indices[size_t(prim) * 3 + 2]) * 2;
  const float tu = t0[0] * b0 + t1[0] * bu + t2[0] * bv, tv = t0[1] * b0 + t1[1] * bu + t2[1] * bv;
  const nrc_material& m = S.materials[S.material_ids[prim]];
  h.diffuse = mat_color(S, m.diffuse, m.diffuse_texture_id, tu, tv, lut);
  h.specular = mat_color(S, m.specular, m.specular_texture_id, tu, tv, lut);
  h.emission = mat_color(S, m.emission, m.emission_texture_id, tu, tv, lut);
  h.roughness = m.roughness;
  h.ior = m.ior;
  return h;
}

// ------------------------------------------------------------- bvh trace --
struct TriView {
  const float4* tri;
  const uint4* node;
  uint32_t tris;
};

// Moller-Trumbore: t and barycentrics (u: vertex 1, v: vertex 2) when the ray
// meets the triangle with t in [tmin, tmax].
__device__ bool intersect(const float4* T, Ray r, float tmin, float tmax, float& t, float& u, float& v) {
  const float4 a = T[0], b = T[1], c = T[2];
  const V3 v0 = v3(a.x, a.y, a.z), e1 = sub(v3(b.x, b.y, b.z), v0), e2 = sub(v3(c.x, c.y, c.z), v0);
  const V3 p = cross(r.d, e2);
  const float det = dot(e1, p);
  if (det == 0.0f || det != det) return false;
  const float inv = 1.0f / det;
  const V3 s = sub(r.o, v0);
  u = dot(s, p) * inv;
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  const V3 q = cross(s, e1);
  v = dot(r.d, q) * inv;
  if (!(v >= 0.0f && u + v <= 1.0f)) return false;
  t = dot(e2, q) * inv;
  return t >= tmin && t <= tmax;
}

// Closest triangle along the ray in [tmin, tmax]; equal distances go to the lower
// triangle index. Returns the triangle index or -1. Kept out of line: the
// kernel traces from several call sites, and one shared copy of the traversal
// loop keeps the kernel's hot code within the instruction cache (measured 17%
// faster at 1080p than inlining it everywhere).
__device__ __noinline__ int trace_closest(const TriView& B, Ray r, float tmin, float tmax, float& bt, float& bu,
                                          float& bv) {
  if (B.tris == 0) return -1;
  const float ix = fabsf(r.d.x) > 1e-20f ? 1.0f / r.d.x : copysignf(1e20f, r.d.x);
  const float iy = fabsf(r.d.y) > 1e-20f ? 1.0f / r.d.y : copysignf(1e20f, r.d.y);
  const float iz = fabsf(r.d.z) > 1e-20f ? 1.0f / r.d.z : copysignf(1e20f, r.d.z);
  int best = -1;
  bt = tmax;
  uint32_t stack[64];
  int sp = 0;
  stack[sp++] = B.tris == 1 ? kLeaf : 0u;
  while (sp > 0) {
    const uint32_t id = stack[--sp];
    if (id & kLeaf) {
      const uint32_t ti = id & ~kLeaf;
      float t, u, v;
      if (intersect(B.tri + size_t(ti) * 3, r, tmin, bt, t, u, v) &&
          (t < bt || (t == bt && (best < 0 || static_cast<int>(ti) < best)))) {
        best = static_cast<int>(ti);
        bt = t;
        bu = u;
        bv = v;
      }
      continue;
    }
    const uint4 lo = B.node[size_t(id) * 2], hi = B.node[size_t(id) * 2 + 1];
    const float x0 = (__uint_as_float(lo.x) - r.o.x) * ix, x1 = (__uint_as_float(hi.x) - r.o.x) * ix;
    const float y0 = (__uint_as_float(lo.y) - r.o.y) * iy, y1 = (__uint_as_float(hi.y) - r.o.y) * iy;
    const float z0 = (__uint_as_float(lo.z) - r.o.z) * iz, z1 = (__uint_as_float(hi.z) - r.o.z) * iz;
    const float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
    const float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), bt));
    if (!(tn <= tf * 1.00001f + 1e-7f)) continue;  // conservative: the boxes are padded too
    if (sp + 2 > 64) continue;  // cannot happen for a radix tree of < 2^30 leaves (depth <= 63)
    stack[sp++] = lo.w;
    stack[sp++] = hi.w;
  }
  return best;
}

// --------------------------------------------------------------- records --
__device__ uint32_t pack_unorm2x16(float a, float b) {
  const float ca = fminf(fmaxf(a, 0.0f), 1.0f), cb = fminf(fmaxf(b, 0.0f), 1.0f);
  return static_cast<uint32_t>(rintf(ca * 65535.0f)) | (static_cast<uint32_t>(rintf(cb * 65535.0f)) << 16);
}

__device__ void sph_encode(V3 d, float& u, float& v) {  // NRCSphEncode with this file's atan2 / acos
  u = (d.x == 0.0f && d.y == 0.0f) ? 0.5f : 0.5f + t_atan2(d.y, d.x) / (2.0f * kPi);
  v = t_acos(fminf(fmaxf(d.z, -1.0f), 1.0f)) / kPi;
}

__device__ nrc_packed_input make_input(const Hit& h, V3 d) {  // MakeNRCInput, path_tracer.comp:158-165
  nrc_packed_input i;
  i.primitive_id = h.prim;
  i.flip_bit_instance_id = h.inst | (h.flip ? 0x80000000u : 0u);
  i.barycentric_2x16u = pack_unorm2x16(h.bu, h.bv);
  float su, sv;
  sph_encode(d, su, sv);
  i.scattered_dir_2x16u = pack_unorm2x16(su, sv);
  return i;
}

struct Step {  // BRDFStepInfo
  V3 color;
  float cosine, pdf, dist2;
  Ray ray;
};

__device__ Step brdf_step(const Hit& h, Ray ray, Rng& rng) {  // BRDFStep, path_tracer.comp:167-186
  Brdf b{h.diffuse, h.specular, fmaxf(h.roughness, 0.001f), fmaxf(h.ior, 1.5f)};
  const V3 v = neg(ray.d);
  const V3 dir = ct_sample(b, v, h.normal, rng);
  const float pdf = ct_pdf(b, dir, v, h.normal);
  const V3 f = ct_eval(b, dir, v, h.normal);
  const float cosine = fabsf(dot(h.normal, dir));
  Step s;
  s.color = normalize_rgb(divs(scale(f, cosine), pdf));  // brdf * cosine / pdf
  s.ray = Ray{h.position, dir};
  s.cosine = cosine;
  s.pdf = pdf;
  const V3 dd = sub(ray.o, h.position);
  s.dist2 = dot(dd, dd);
  return s;
}

struct TraceArgs {
  TraceScene sc;
  TriView bvh;
  nrc_trace_params p;
  nrc_trace_targets t;
};

__device__ void push_eval(const TraceArgs& A, uint32_t dst, const nrc_packed_input& in) {
  const uint32_t id = atomicAdd(A.t.eval_count, 1u);
  if (id >= A.t.eval_capacity) return;
  uint32_t* w = reinterpret_cast<uint32_t*>(A.t.eval_records + id);
  w[0] = dst;
  w[1] = in.primitive_id;
  w[2] = in.flip_bit_instance_id;
  w[3] = in.barycentric_2x16u;
  w[4] = in.scattered_dir_2x16u;
}

__device__ __forceinline__ uint32_t dst_screen(uint32_t x, uint32_t y) { return (x | (y << 15)) << 1; }
__device__ __forceinline__ uint32_t dst_train(uint32_t b, uint32_t l, uint32_t r) {
  return ((b | (l << 2) | (r << 16)) << 1) | 1u;
}

// The secondary hit of a traced ray (GetRayQueryHit) or false for a miss.
__device__ bool trace_hit(const TraceArgs& A, Ray ray, Hit& h) {
  float t, u, v;
  const int ti = trace_closest(A.bvh, ray, kTMin, kTMax, t, u, v);
  if (ti < 0) return false;
  const float4* T = A.bvh.tri + size_t(ti) * 3;
  const nrc_scene& S = A.sc.s;
  const uint32_t prim = __float_as_uint(T[0].w), inst = __float_as_uint(T[1].w);
  const V3 v0 = scene_vertex(S, inst, prim, 0), v1 = scene_vertex(S, inst, prim, 1), v2 = scene_vertex(S, inst, prim, 2);
  h = make_hit(S, A.sc.lut, prim, inst, u, v, v0, v1, v2, cross(sub(v1, v0), sub(v2, v0)), ray);
  return true;
}

struct Result {
  V3 bias, factor;
};

// PathTrace, path_tracer.comp:208-250 (the method is warp-uniform here).
__device__ Result path_trace(const TraceArgs& A, Hit hit, Ray ray, uint32_t method, Rng& rng, uint32_t x, uint32_t y) {
  V3 radiance = v3(0.f, 0.f, 0.f), acc = v3(1.f, 1.f, 1.f);
  Step info = brdf_step(hit, ray, rng);
  radiance = add(radiance, mul(acc, hit.emission));
  acc = mul(acc, info.color);
  ray = info.ray;
  const float c_a0 =
      method == NRC_METHOD_NONE ? __int_as_float(0x7F800000) : kC * info.dist2 / (4.0f * kPi * info.cosine);
  float sqrt_a_sum = 0.0f;
  if (method != NRC_METHOD_CACHE) {
    for (int bounce = 1; bounce < kMaxBounce && sqrt_a_sum * sqrt_a_sum <= c_a0; ++bounce) {
      if (trace_hit(A, ray, hit)) {
        info = brdf_step(hit, ray, rng);
        radiance = add(radiance, mul(acc, hit.emission));
        acc = mul(acc, info.color);
        ray = info.ray;
        sqrt_a_sum = sqrt_a_sum + sqrtf(info.dist2 / (info.pdf * info.cosine));
      } else {
        radiance = add(radiance, scale(acc, kConstLight));
        return Result{radiance, acc};
      }
    }
  }
  if (method != NRC_METHOD_NONE) push_eval(A, dst_screen(x, y), make_input(hit, ray.d));
  return Result{radiance, acc};
}

// ExtendedPathTrace, path_tracer.comp:252-375.
__device__ Result extended_trace(const TraceArgs& A, Hit hit, Ray ray, uint32_t method, Rng& rng, uint32_t x,
                                 uint32_t y) {
  V3 lights[kMaxBounce], colors[kMaxBounce];
  nrc_packed_input inputs[kMaxBounce];
  for (int i = 0; i < kMaxBounce; ++i) {
    colors[i] = v3(1.f, 1.f, 1.f);
    lights[i] = v3(0.f, 0.f, 0.f);
  }
  V3 acc = v3(1.f, 1.f, 1.f), radiance = v3(0.f, 0.f, 0.f);
  bool light_terminate = false;
  Step info = brdf_step(hit, ray, rng);
  radiance = add(radiance, mul(acc, hit.emission));
  acc = mul(acc, info.color);
  ray = info.ray;
  Result result{radiance, acc};
  inputs[0] = make_input(hit, ray.d);
  const float c_a0 = kC * info.dist2 / (4.0f * kPi * info.cosine);
  float sqrt_a_sum = 0.0f;
  int bounce = 1;
  for (; bounce < kMaxBounce && sqrt_a_sum * sqrt_a_sum <= c_a0; ++bounce) {
    if (trace_hit(A, ray, hit)) {
      info = brdf_step(hit, ray, rng);
      radiance = add(radiance, mul(acc, hit.emission));
      acc = mul(acc, info.color);
      ray = info.ray;
      sqrt_a_sum = sqrt_a_sum + sqrtf(info.dist2 / (info.pdf * info.cosine));
      lights[bounce - 1] = hit.emission;
      colors[bounce - 1] = info.color;
      inputs[bounce] = make_input(hit, ray.d);
    } else {
      radiance = add(radiance, scale(acc, kConstLight));
      lights[bounce - 1] = v3(kConstLight, kConstLight, kConstLight);
      light_terminate = true;
      break;
    }
  }
  if (method == NRC_METHOD_CACHE) {
    push_eval(A, dst_screen(x, y), inputs[0]);
  } else {
    result = Result{radiance, acc};
    if (!light_terminate) push_eval(A, dst_screen(x, y), inputs[bounce - 1]);
  }
  sqrt_a_sum = 0.0f;
  light_terminate = false;
  for (; bounce < kMaxBounce && sqrt_a_sum * sqrt_a_sum <= c_a0; ++bounce) {
    if (trace_hit(A, ray, hit)) {
      info = brdf_step(hit, ray, rng);
      ray = info.ray;
      sqrt_a_sum = sqrt_a_sum + sqrtf(info.dist2 / (info.pdf * info.cosine));
      lights[bounce - 1] = hit.emission;
      colors[bounce - 1] = info.color;
      inputs[bounce] = make_input(hit, ray.d);
    } else {
      lights[bounce - 1] = v3(kConstLight, kConstLight, kConstLight);
      light_terminate = true;
      break;
    }
  }
  // clamp(uint(u * 4), 0, 3) with u in [0, 1]
  uint32_t batch = static_cast<uint32_t>(rng.next() * static_cast<float>(NRC_TRAIN_BATCH_COUNT));
  batch = batch < NRC_TRAIN_BATCH_COUNT - 1 ? batch : NRC_TRAIN_BATCH_COUNT - 1;
  const uint32_t train_id = atomicAdd(A.t.train_counts[batch], static_cast<uint32_t>(bounce));
  if (train_id < NRC_TRAIN_BATCH_SIZE) {
    for (int i = bounce - 2; i >= 0; --i) {
      lights[i] = add(lights[i], mul(colors[i], lights[i + 1]));
      colors[i] = mul(colors[i], colors[i + 1]);
    }
    const uint32_t count = min(static_cast<uint32_t>(bounce), NRC_TRAIN_BATCH_SIZE - train_id);
    nrc_packed_train_record* rec = A.t.train_records[batch];
    for (uint32_t i = 0; i < count; ++i) {
      float* w = reinterpret_cast<float*>(rec + train_id + i);
      w[0] = lights[i].x;
      w[1] = lights[i].y;
      w[2] = lights[i].z;
      w[3] = colors[i].x;
      w[4] = colors[i].y;
      w[5] = colors[i].z;
      uint32_t* u = reinterpret_cast<uint32_t*>(w + 6);
      u[0] = inputs[i].primitive_id;
      u[1] = inputs[i].flip_bit_instance_id;
      u[2] = inputs[i].barycentric_2x16u;
      u[3] = inputs[i].scattered_dir_2x16u;
    }
    if (!light_terminate) push_eval(A, dst_train(batch, train_id, train_id + count - 1), inputs[bounce - 1]);
  }
  return result;
}

// main(), path_tracer.comp:377-420: 8 x 8 threads per block, warps of 32
// consecutive threads (4 rows), the warp standing in for the subgroup.
// 16 blocks of 64 threads per SM (64 registers): more warps to hide the BVH
// loads measured faster than fewer, spill-free warps (2.67 against 3.03 ms at
// 1080p with 12 blocks). A near-child-first traversal (both children's boxes
// tested at each node) measured slower here (2.79 ms).
__global__ void __launch_bounds__(64, 16) path_trace_kernel(const __grid_constant__ TraceArgs A) {
  extern __shared__ float lut_s[];
  for (int i = threadIdx.y * 8 + threadIdx.x; i < 256; i += 64) lut_s[i] = A.sc.lut[i];
  __syncthreads();
  const uint32_t x = blockIdx.x * 8 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  Rng rng{(((y & 0xFFu) << 8) | (x & 0xFFu)) + A.p.seed};
  const bool inside = x < A.p.width && y < A.p.height;
  const uint32_t active = __ballot_sync(0xffffffffu, inside);
  if (!inside) return;
  const int lane = (threadIdx.y * 8 + threadIdx.x) & 31;
  const bool left_all = __all_sync(active, x <= A.p.width / 2);
  const uint32_t method = left_all ? A.p.left_method : A.p.right_method;
  bool train = false;
  if (method != NRC_METHOD_NONE) {
    const int first = __ffs(active) - 1;  // subgroupElect: the lowest active lane
    if (lane == first) train = rng.next() < A.p.train_probability;
    train = __shfl_sync(active, train ? 1 : 0, first) != 0;
  }
  // primary hit (the V-buffer's primitive and instance), then GetVBufferHit
  const float cx = (static_cast<float>(x) + 0.5f) / static_cast<float>(A.p.width) * 2.0f - 1.0f;
  const float cy = (static_cast<float>(y) + 0.5f) / static_cast<float>(A.p.height) * 2.0f - 1.0f;
  const V3 look = v3(A.p.look[0], A.p.look[1], A.p.look[2]), side = v3(A.p.side[0], A.p.side[1], A.p.side[2]),
           up = v3(A.p.up[0], A.p.up[1], A.p.up[2]);
  Ray ray{v3(A.p.origin[0], A.p.origin[1], A.p.origin[2]), normalize(add(add(look, scale(side, cx)), scale(up, cy)))};
  Result res;
  float pt, pu, pv;
  const int ti = trace_closest(A.bvh, ray, 0.0f, __int_as_float(0x7F800000), pt, pu, pv);
  if (ti < 0) {
    res = Result{v3(kConstLight, kConstLight, kConstLight), v3(0.f, 0.f, 0.f)};
  } else {
    const float4* T = A.bvh.tri + size_t(ti) * 3;
    const nrc_scene& S = A.sc.s;
    const uint32_t prim = __float_as_uint(T[0].w), inst = __float_as_uint(T[1].w);
    const V3 v0 = scene_vertex(S, inst, prim, 0), v1 = scene_vertex(S, inst, prim, 1),
             v2 = scene_vertex(S, inst, prim, 2);
    // GetVBufferHit's barycentrics: the ray against the triangle's plane
    const V3 v01 = sub(v1, v0), v02 = sub(v2, v0), v0o = sub(ray.o, v0);
    const V3 n = cross(v01, v02), q = cross(v0o, ray.d);
    const float d = 1.0f / dot(ray.d, n);
    const float u = d * dot(neg(q), v02), v = d * dot(q, v01);
    const Hit hit = make_hit(S, lut_s, prim, inst, u, v, v0, v1, v2, n, ray);
    res = train ? extended_trace(A, hit, ray, method, rng, x, y) : path_trace(A, hit, ray, method, rng, x, y);
  }
  res.bias = normalize_rgb(res.bias);
  res.factor = normalize_rgb(res.factor);
  const size_t px = size_t(y) * A.p.width + x;
  reinterpret_cast<float4*>(A.t.bias_factor_r)[px] = make_float4(res.bias.x, res.bias.y, res.bias.z, res.factor.x);
  reinterpret_cast<float2*>(A.t.factor_gb)[px] = make_float2(res.factor.y, res.factor.z);
}

// ------------------------------------------------------------- bvh build --
struct BuildArgs {
  nrc_scene s;
  const nrc_instance_range* ranges;
  const uint32_t* first_tri;  // prefix sums of the ranges' counts (instances + 1)
  uint32_t instances, tris;
};

// World-space triangles and their centroids.
__global__ void tri_kernel(BuildArgs A, float4* tri, float* cent, uint32_t* bad) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.tris) return;
  uint32_t lo = 0, hi = A.instances;  // instance i holds triangles [first_tri[i], first_tri[i+1])
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (A.first_tri[mid] <= t) lo = mid; else hi = mid;
  }
  const uint32_t inst = lo, prim = A.ranges[inst].first_primitive + (t - A.first_tri[inst]);
  const nrc_scene& S = A.s;
  V3 v[3] = {v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
  bool ok = prim < S.primitive_count;
  for (int k = 0; k < 3 && ok; ++k) {
    const uint32_t vi = S.vertex_indices[size_t(prim) * 3 + k];
    if (vi >= S.vertex_count) { ok = false; break; }
    v[k] = scene_vertex(S, inst, prim, k);
  }
  if (!ok) atomicOr(bad, 1u);
  tri[size_t(t) * 3 + 0] = make_float4(v[0].x, v[0].y, v[0].z, __uint_as_float(prim));
  tri[size_t(t) * 3 + 1] = make_float4(v[1].x, v[1].y, v[1].z, __uint_as_float(inst));
  tri[size_t(t) * 3 + 2] = make_float4(v[2].x, v[2].y, v[2].z, 0.0f);
  cent[size_t(t) * 3 + 0] = (v[0].x + v[1].x + v[2].x) * (1.0f / 3.0f);
  cent[size_t(t) * 3 + 1] = (v[0].y + v[1].y + v[2].y) * (1.0f / 3.0f);
  cent[size_t(t) * 3 + 2] = (v[0].z + v[1].z + v[2].z) * (1.0f / 3.0f);
}

__device__ __forceinline__ uint32_t ordered(float f) {  // float -> uint32 preserving order
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__global__ void bounds_kernel(const float* cent, uint32_t n, uint32_t* box) {  // box: min xyz, max xyz (ordered)
  uint32_t mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const uint32_t o = ordered(cent[size_t(i) * 3 + k]);
      mn[k] = min(mn[k], o);
      mx[k] = max(mx[k], o);
    }
  for (int k = 0; k < 3; ++k) {
    atomicMin(&box[k], mn[k]);
    atomicMax(&box[3 + k], mx[k]);
  }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {  // 10 bits -> every third bit
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void morton_kernel(const float* cent, uint32_t n, const uint32_t* box, uint32_t* keys, uint32_t* vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t code = 0;
  for (int k = 0; k < 3; ++k) {
    const float lo = unordered(box[k]), hi = unordered(box[3 + k]);
    const float ext = hi - lo;
    float f = ext > 0.0f ? (cent[size_t(i) * 3 + k] - lo) / ext : 0.5f;
    f = fminf(fmaxf(f, 0.0f), 1.0f);
    const uint32_t q = min(static_cast<uint32_t>(f * 1024.0f), 1023u);
    code |= spread10(q) << (2 - k);
  }
  keys[i] = code;
  vals[i] = i;
}

// Common prefix of sorted keys i and j (the index breaks ties), -1 outside.
__device__ __forceinline__ int delta(const uint32_t* k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = k[i], b = k[j];
  return a != b ? __clz(a ^ b) : 32 + __clz(static_cast<uint32_t>(i) ^ static_cast<uint32_t>(j));
}

// Binary radix tree (Karras 2012): internal node i of n - 1.
__global__ void hierarchy_kernel(const uint32_t* keys, const uint32_t* order, int n, uint4* node, uint32_t* parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1) >= 0 ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int s = 0;
  for (int div = 2;; div *= 2) {
    const int t = (l + div - 1) / div;
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
  }
  const int gamma = i + s * d + min(d, 0);
  const int first = min(i, j), last = max(i, j);
  const uint32_t left = first == gamma ? (kLeaf | order[gamma]) : static_cast<uint32_t>(gamma);
  const uint32_t right = last == gamma + 1 ? (kLeaf | order[gamma + 1]) : static_cast<uint32_t>(gamma + 1);
  node[size_t(i) * 2].w = left;
  node[size_t(i) * 2 + 1].w = right;
  // parents: internal nodes at [0, n-1), leaves (by triangle) at n-1 + triangle
  parent[(left & kLeaf) ? (n - 1) + (left & ~kLeaf) : left] = static_cast<uint32_t>(i);
  parent[(right & kLeaf) ? (n - 1) + (right & ~kLeaf) : right] = static_cast<uint32_t>(i);
}

// Bottom-up bounds: each leaf climbs; the second child to arrive at a node
// computes its box (padded so the traversal's slab test is conservative).
__global__ void refit_kernel(const float4* tri, int n, uint4* node, const uint32_t* parent, uint32_t* visits) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint32_t cur = parent[(n - 1) + t];
  while (true) {
    __threadfence();
    if (atomicAdd(&visits[cur], 1u) == 0) return;  // the first to arrive leaves the node to the other
    __threadfence();
    float lo[3] = {__int_as_float(0x7F800000), __int_as_float(0x7F800000), __int_as_float(0x7F800000)};
    float hi[3] = {-__int_as_float(0x7F800000), -__int_as_float(0x7F800000), -__int_as_float(0x7F800000)};
    for (int c = 0; c < 2; ++c) {
      const uint32_t ch = c == 0 ? node[size_t(cur) * 2].w : node[size_t(cur) * 2 + 1].w;
      if (ch & kLeaf) {
        const float4* T = tri + size_t(ch & ~kLeaf) * 3;
        for (int v = 0; v < 3; ++v) {
          const float4 p = T[v];
          lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
          hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
        }
      } else {
        // the other child's box, written by another thread before its arrival
        const volatile uint32_t* a = reinterpret_cast<const volatile uint32_t*>(&node[size_t(ch) * 2]);
        const volatile uint32_t* b = reinterpret_cast<const volatile uint32_t*>(&node[size_t(ch) * 2 + 1]);
        lo[0] = fminf(lo[0], __uint_as_float(a[0])); lo[1] = fminf(lo[1], __uint_as_float(a[1]));
        lo[2] = fminf(lo[2], __uint_as_float(a[2]));
        hi[0] = fmaxf(hi[0], __uint_as_float(b[0])); hi[1] = fmaxf(hi[1], __uint_as_float(b[1]));
        hi[2] = fmaxf(hi[2], __uint_as_float(b[2]));
      }
    }
    for (int k = 0; k < 3; ++k) {  // pad by a relative and an absolute margin
      const float pad = (hi[k] - lo[k]) * 1e-5f + (fabsf(lo[k]) + fabsf(hi[k])) * 1e-6f + 1e-7f;
      lo[k] = lo[k] - pad;
      hi[k] = hi[k] + pad;
    }
    uint4* a = &node[size_t(cur) * 2];
    uint4* b = &node[size_t(cur) * 2 + 1];
    a->x = __float_as_uint(lo[0]); a->y = __float_as_uint(lo[1]); a->z = __float_as_uint(lo[2]);
    b->x = __float_as_uint(hi[0]); b->y = __float_as_uint(hi[1]); b->z = __float_as_uint(hi[2]);
    if (cur == 0) return;
    cur = parent[cur];
  }
}

float srgb_to_linear(int i) {
  const double c = i / 255.0;
  return static_cast<float>(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
}

}  // namespace
}  // namespace nrc

namespace {
int st(cudaError_t e) { return e == cudaSuccess ? NRC_OK : (e == cudaErrorMemoryAllocation ? NRC_ERROR_OUT_OF_MEMORY : NRC_ERROR_CUDA); }
}  // namespace

extern "C" {

int nrc_bvh_build(const nrc_scene* scene, const nrc_instance_range* d_ranges, nrc_bvh** out) {
  using namespace nrc;
  if (scene == nullptr || out == nullptr || (scene->instance_count > 0 && d_ranges == nullptr))
    return NRC_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  const uint32_t ni = scene->instance_count;
  std::vector<nrc_instance_range> ranges(ni);
  cudaError_t e = cudaSuccess;
  if (ni > 0) e = cudaMemcpy(ranges.data(), d_ranges, ni * sizeof(nrc_instance_range), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return st(e);
  std::vector<uint32_t> first(ni + 1, 0);
  uint64_t total = 0;
  for (uint32_t i = 0; i < ni; ++i) {
    if (uint64_t(ranges[i].first_primitive) + ranges[i].primitive_count > scene->primitive_count)
      return NRC_ERROR_INVALID_ARGUMENT;
    first[i] = static_cast<uint32_t>(total);
    total += ranges[i].primitive_count;
  }
  first[ni] = static_cast<uint32_t>(total);
  if (total >= (1u << 30)) return NRC_ERROR_TOO_LARGE;
  const uint32_t n = static_cast<uint32_t>(total);
  nrc_bvh* B = new (std::nothrow) nrc_bvh();
  if (B == nullptr) return NRC_ERROR_OUT_OF_MEMORY;
  cudaGetDevice(&B->device);
  B->tris = n;
  B->nodes = n > 1 ? n - 1 : 0;
  const size_t tri_bytes = size_t(n) * 3 * sizeof(float4), node_bytes = size_t(B->nodes) * 2 * sizeof(uint4);
  if ((e = cudaMalloc(&B->block, tri_bytes + node_bytes + 256)) != cudaSuccess) {
    delete B;
    return st(e);
  }
  float4* tri = static_cast<float4*>(B->block);
  uint4* node = reinterpret_cast<uint4*>(static_cast<uint8_t*>(B->block) + tri_bytes);
  B->tri = tri;
  B->node = node;
  // scratch for the build
  uint32_t *d_first = nullptr, *keys = nullptr, *vals = nullptr, *keys2 = nullptr, *vals2 = nullptr, *parent = nullptr,
           *visits = nullptr, *box = nullptr;
  float* cent = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  auto cleanup = [&]() {
    cudaFree(d_first); cudaFree(keys); cudaFree(vals); cudaFree(keys2); cudaFree(vals2);
    cudaFree(parent); cudaFree(visits); cudaFree(box); cudaFree(cent); cudaFree(tmp);
  };
  if (n > 0) {
    const size_t nn = n;
    if ((e = cudaMalloc(&d_first, (ni + 1) * 4)) == cudaSuccess && (e = cudaMalloc(&keys, nn * 4)) == cudaSuccess &&
        (e = cudaMalloc(&vals, nn * 4)) == cudaSuccess && (e = cudaMalloc(&keys2, nn * 4)) == cudaSuccess &&
        (e = cudaMalloc(&vals2, nn * 4)) == cudaSuccess && (e = cudaMalloc(&parent, (2 * nn) * 4)) == cudaSuccess &&
        (e = cudaMalloc(&visits, nn * 4 + 4)) == cudaSuccess && (e = cudaMalloc(&box, 64)) == cudaSuccess &&
        (e = cudaMalloc(&cent, nn * 12)) == cudaSuccess)
      e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, vals, vals2, static_cast<int>(n));
    if (e == cudaSuccess) e = cudaMalloc(&tmp, tmp_bytes ? tmp_bytes : 16);
    if (e == cudaSuccess) e = cudaMemcpy(d_first, first.data(), (ni + 1) * 4, cudaMemcpyHostToDevice);
    uint32_t box_init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    if (e == cudaSuccess) e = cudaMemcpy(box, box_init, 24, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(box + 8, 0, 4);  // the bad-index flag
    if (e == cudaSuccess) e = cudaMemset(visits, 0, nn * 4 + 4);
    BuildArgs A{*scene, d_ranges, d_first, ni, n};
    const uint32_t blocks = (n + 255) / 256;
    if (e == cudaSuccess) {
      tri_kernel<<<blocks, 256>>>(A, tri, cent, box + 8);
      bounds_kernel<<<blocks < 1024 ? blocks : 1024, 256>>>(cent, n, box);
      morton_kernel<<<blocks, 256>>>(cent, n, box, keys, vals);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, vals, vals2, static_cast<int>(n), 0, 30);
    if (e == cudaSuccess && n > 1) {
      hierarchy_kernel<<<(n - 1 + 255) / 256, 256>>>(keys2, vals2, static_cast<int>(n), node, parent);
      refit_kernel<<<blocks, 256>>>(tri, static_cast<int>(n), node, parent, visits);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    uint32_t bad = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&bad, box + 8, 4, cudaMemcpyDeviceToHost);
    cleanup();
    if (e == cudaSuccess && bad) {
      cudaFree(B->block);
      delete B;
      return NRC_ERROR_INVALID_ARGUMENT;  // an index past the scene's buffers
    }
  }
  if (e != cudaSuccess) {
    cudaFree(B->block);
    delete B;
    return st(e);
  }
  *out = B;
  return NRC_OK;
}

int nrc_bvh_destroy(nrc_bvh* B) {
  if (B == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  cudaFree(B->block);
  delete B;
  return NRC_OK;
}

int nrc_bvh_info(const nrc_bvh* B, uint32_t* tris, uint32_t* nodes) {
  if (B == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (tris) *tris = B->tris;
  if (nodes) *nodes = B->nodes;
  return NRC_OK;
}

int nrc_path_trace(const nrc_scene* scene, const nrc_bvh* bvh, const nrc_trace_params* p, const nrc_trace_targets* t,
                   void* stream) {
  using namespace nrc;
  if (scene == nullptr || bvh == nullptr || p == nullptr || t == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if (p->width == 0 || p->height == 0) return NRC_OK;
  if (p->width > 0x8000u || p->height > 0x10000u) return NRC_ERROR_INVALID_ARGUMENT;  // dst word's 15 / 16 bits
  if (p->left_method > 2 || p->right_method > 2) return NRC_ERROR_INVALID_ARGUMENT;
  if (t->eval_count == nullptr || (t->eval_capacity > 0 && t->eval_records == nullptr) ||
      t->bias_factor_r == nullptr || t->factor_gb == nullptr)
    return NRC_ERROR_INVALID_ARGUMENT;
  for (int b = 0; b < NRC_TRAIN_BATCH_COUNT; ++b)
    if (t->train_counts[b] == nullptr || t->train_records[b] == nullptr) return NRC_ERROR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(t->bias_factor_r) & 15u) || (reinterpret_cast<uintptr_t>(t->factor_gb) & 7u))
    return NRC_ERROR_MISALIGNED;
  TraceArgs A;
  A.sc.s = *scene;
  for (int i = 0; i < 256; ++i) A.sc.lut[i] = srgb_to_linear(i);
  A.bvh = TriView{bvh->tri, bvh->node, bvh->tris};
  A.p = *p;
  A.t = *t;
  dim3 grid((p->width + 7) / 8, (p->height + 7) / 8);
  path_trace_kernel<<<grid, dim3(8, 8), 256 * sizeof(float), static_cast<cudaStream_t>(stream)>>>(A);
  return st(cudaGetLastError());
}

}  // extern "C"
