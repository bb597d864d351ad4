// Scene unpack shared by the unpack kernel (nrc_unpack.cu) and the query
// kernel's packed-record form (nrc_infer.cu): UnpackNRCInput
// (shader/src/NRCRecord.glsl:97-125) over the scene buffers
// (shader/src/Scene.glsl:50-71).
//
// Per record: the primitive's three vertices through the instance transform
// (vec4(p, 1) * mat3x4), the face normal normalize(cross(v1 - v0, v2 - v0)),
// flipped when bit 31 of the instance word is set, sphere-encoded; barycentrics
// and the scattered direction from their unorm16 pairs; position and texcoord
// interpolated; roughness from the material; diffuse and specular from the
// material's constants or its textures.
//
// Textures are sampled as the reference's sampler is configured
// (src/rg/NRCRenderGraph.cpp:132; R8G8B8A8_SRGB, one level, src/VkScene.cpp:190):
// bilinear with REPEAT addressing, each texel sRGB-decoded before filtering.
// The filter weights are exact fp32 fractions here, where texture hardware
// quantises them (to 8 bits on current GPUs), so a hardware sample can differ
// from this one by up to about 1/256 of the texel contrast.
//
// Op sequence (the CPU oracle repeats it): dot products and interpolations are
// fused multiply-add chains in component order, cross products multiply then
// subtract, normalize divides by a correctly rounded square root, unorm16 is
// u / 65535 rounded once, lerp(x, y, t) = fma(t, y - x, x). Only the sphere
// encoding of the normal (atan2, acos) differs by a few ulp from the oracle.
#pragma once
#include "nrc_common.cuh"

namespace nrc {

struct SrgbLut {
  float v[256];
};

struct F3 {
  float x, y, z;
};

__device__ __forceinline__ float unorm16(uint32_t u) { return __fdiv_rn(static_cast<float>(u & 0xFFFFu), 65535.0f); }

// vec4(p, 1) * mat3x4: component i = dot((p, 1), column i).
__device__ __forceinline__ F3 xform(const float* __restrict__ T, F3 p) {
  float o[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float* c = T + 4 * i;
    o[i] = __fadd_rn(__fmaf_rn(p.z, c[2], __fmaf_rn(p.y, c[1], __fmul_rn(p.x, c[0]))), c[3]);
  }
  return F3{o[0], o[1], o[2]};
}

__device__ __forceinline__ float interp(float a, float b, float c, float w0, float w1, float w2) {
  return __fmaf_rn(c, w2, __fmaf_rn(b, w1, __fmul_rn(a, w0)));
}

__device__ __forceinline__ float lerp(float x, float y, float t) { return __fmaf_rn(t, __fsub_rn(y, x), x); }

// floor(f) mod n for REPEAT addressing; f integral, |f| < 2^23.
__device__ __forceinline__ uint32_t wrap(float f, uint32_t n) {
  const float nf = static_cast<float>(n);
  int r = static_cast<int>(__fmaf_rn(-nf, floorf(__fdiv_rn(f, nf)), f));
  if (r < 0) r += static_cast<int>(n);
  if (r >= static_cast<int>(n)) r -= static_cast<int>(n);
  return static_cast<uint32_t>(r);
}

__device__ inline F3 sample_texture(const nrc_texture& t, float tu, float tv, const float* lut) {
  const uint32_t w = t.width, h = t.height;
  if (w == 0 || h == 0 || t.texels == nullptr) return F3{0.f, 0.f, 0.f};
  float u = __fmaf_rn(tu, static_cast<float>(w), -0.5f), v = __fmaf_rn(tv, static_cast<float>(h), -0.5f);
  if (!(fabsf(u) < 8388608.0f)) u = 0.0f;  // NaN or beyond fp32's integer range: texel 0's neighbourhood
  if (!(fabsf(v) < 8388608.0f)) v = 0.0f;
  const float fu = floorf(u), fv = floorf(v);
  const float a = __fsub_rn(u, fu), b = __fsub_rn(v, fv);
  const uint32_t i0 = wrap(fu, w), j0 = wrap(fv, h);
  const uint32_t i1 = i0 + 1 == w ? 0 : i0 + 1, j1 = j0 + 1 == h ? 0 : j0 + 1;
  const uchar4* px = reinterpret_cast<const uchar4*>(t.texels);
  const uchar4 t00 = px[size_t(j0) * w + i0], t10 = px[size_t(j0) * w + i1];
  const uchar4 t01 = px[size_t(j1) * w + i0], t11 = px[size_t(j1) * w + i1];
  auto ch = [&](unsigned char c00, unsigned char c10, unsigned char c01, unsigned char c11) {
    return lerp(lerp(lut[c00], lut[c10], a), lerp(lut[c01], lut[c11], a), b);
  };
  return F3{ch(t00.x, t10.x, t01.x, t11.x), ch(t00.y, t10.y, t01.y, t11.y), ch(t00.z, t10.z, t01.z, t11.z)};
}

// UnpackNRCInput into 14 floats (nrc_input); false (and zeros) for a record
// whose indices fall outside the scene. `lut` is the sRGB decode table
// (srgb_lut()) in shared memory. The loads take no early exit: an out-of-range
// index is replaced by 0 (in range once the scene's counts are non-zero, checked
// first) and the record's outputs are zeroed at the end, so a thread can have
// the loads of several records in flight.
__device__ __forceinline__ bool unpack_one(const nrc_scene& S, const nrc_packed_input& in, const float* lut, float (&r)[kInFloats]) {
  if (S.primitive_count == 0 || S.instance_count == 0 || S.vertex_count == 0 || S.texcoord_count == 0 ||
      S.material_count == 0) {
#pragma unroll
    for (int k = 0; k < kInFloats; ++k) r[k] = 0.0f;
    return false;
  }
  const uint32_t prim = in.primitive_id, inst = in.flip_bit_instance_id & 0x7FFFFFFFu;
  const bool flip = (in.flip_bit_instance_id >> 31) != 0;
  bool ok = prim < S.primitive_count && inst < S.instance_count;
  const uint32_t pr = ok ? prim : 0u, in_id = ok ? inst : 0u;
  uint32_t vi[3], ti[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vi[k] = S.vertex_indices[size_t(pr) * 3 + k];
    ti[k] = S.texcoord_indices[size_t(pr) * 3 + k];
  }
  uint32_t mid = S.material_ids[pr];
#pragma unroll
  for (int k = 0; k < 3; ++k) ok = ok && vi[k] < S.vertex_count && ti[k] < S.texcoord_count;
  ok = ok && mid < S.material_count;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vi[k] = ok ? vi[k] : 0u;
    ti[k] = ok ? ti[k] : 0u;
  }
  mid = ok ? mid : 0u;
  const float* T = S.transforms + size_t(in_id) * 12;
  F3 v[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float* p = S.vertices + size_t(vi[k]) * 3;
    v[k] = xform(T, F3{p[0], p[1], p[2]});
  }
  // normal = normalize(cross(v1 - v0, v2 - v0)), negated when flipped
  const F3 e1{__fsub_rn(v[1].x, v[0].x), __fsub_rn(v[1].y, v[0].y), __fsub_rn(v[1].z, v[0].z)};
  const F3 e2{__fsub_rn(v[2].x, v[0].x), __fsub_rn(v[2].y, v[0].y), __fsub_rn(v[2].z, v[0].z)};
  F3 n{__fsub_rn(__fmul_rn(e1.y, e2.z), __fmul_rn(e1.z, e2.y)), __fsub_rn(__fmul_rn(e1.z, e2.x), __fmul_rn(e1.x, e2.z)),
       __fsub_rn(__fmul_rn(e1.x, e2.y), __fmul_rn(e1.y, e2.x))};
  const float len = __fsqrt_rn(__fmaf_rn(n.z, n.z, __fmaf_rn(n.y, n.y, __fmul_rn(n.x, n.x))));
  n = F3{__fdiv_rn(n.x, len), __fdiv_rn(n.y, len), __fdiv_rn(n.z, len)};
  if (flip) n = F3{-n.x, -n.y, -n.z};
  // barycentric = (1 - b1 - b2, b1, b2)
  const float b1 = unorm16(in.barycentric_2x16u), b2 = unorm16(in.barycentric_2x16u >> 16);
  const float b0 = __fsub_rn(__fsub_rn(1.0f, b1), b2);
  r[0] = interp(v[0].x, v[1].x, v[2].x, b0, b1, b2);
  r[1] = interp(v[0].y, v[1].y, v[2].y, b0, b1, b2);
  r[2] = interp(v[0].z, v[1].z, v[2].z, b0, b1, b2);
  r[3] = unorm16(in.scattered_dir_2x16u);
  r[4] = unorm16(in.scattered_dir_2x16u >> 16);
  // NRCSphEncode (NRCRecord.glsl:47-49)
  const float pi = 3.14159265358979323846f;
  r[5] = (n.x == 0.0f && n.y == 0.0f) ? 0.5f : __fadd_rn(0.5f, __fdiv_rn(atan2f(n.y, n.x), 2.0f * pi));
  r[6] = __fdiv_rn(acosf(fminf(fmaxf(n.z, -1.0f), 1.0f)), pi);
  const nrc_material& m = S.materials[mid];
  r[7] = m.roughness;
  const float* tc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) tc[k] = S.texcoords + size_t(ti[k]) * 2;
  const float tu = interp(tc[0][0], tc[1][0], tc[2][0], b0, b1, b2);
  const float tv = interp(tc[0][1], tc[1][1], tc[2][1], b0, b1, b2);
  const uint32_t ids[2] = {m.diffuse_texture_id, m.specular_texture_id};
  const float* konst[2] = {m.diffuse, m.specular};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    F3 col{konst[c][0], konst[c][1], konst[c][2]};
    if (ok && ids[c] != 0xFFFFFFFFu && ids[c] < S.texture_count) col = sample_texture(S.textures[ids[c]], tu, tv, lut);
    r[8 + 3 * c] = col.x;
    r[9 + 3 * c] = col.y;
    r[10 + 3 * c] = col.z;
  }
  if (!ok) {
#pragma unroll
    for (int k = 0; k < kInFloats; ++k) r[k] = 0.0f;
  }
  return ok;
}

// sRGB -> linear of the 256 byte values, in double, rounded once (host).
const SrgbLut& srgb_lut();

}  // namespace nrc
