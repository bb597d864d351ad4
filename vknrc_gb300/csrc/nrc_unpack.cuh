// Per-record arithmetic of the unpack kernels (nrc_unpack.cu): UnpackNRCInput
// (shader/src/NRCRecord.glsl:97-125) over the scene buffers
// (shader/src/Scene.glsl:50-71) or over the scene's gather tables
// (nrc_scene_prepare), which hold the same values laid out for the gathers.
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

static_assert(sizeof(nrc_material) == 64 && alignof(nrc_material) <= 16, "std430 Material: four 16-byte words");

struct SrgbLut {
  float v[256];
};

struct F3 {
  float x, y, z;
};

__device__ __forceinline__ float unorm16(uint32_t u) { return __fdiv_rn(static_cast<float>(u & 0xFFFFu), 65535.0f); }

// vec4(p, 1) * mat3x4: component i = dot((p, 1), column i); the three columns
// come in as 16-byte vectors (the transforms are 16-byte aligned).
__device__ __forceinline__ F3 xform(const float4 (&c)[3], F3 p) {
  float o[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    o[i] = __fadd_rn(__fmaf_rn(p.z, c[i].z, __fmaf_rn(p.y, c[i].y, __fmul_rn(p.x, c[i].x))), c[i].w);
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

// `lut` is this thread's copy of the sRGB decode table (srgb_lut()) in shared
// memory: entry c at lut[c * kLutCopies] (stage_lut). One copy: interleaved
// copies that spread a warp's lookups over the banks (16 or 32 of them) were
// measured no faster, and they take shared memory from the L1 capacity the
// scene gathers use.
constexpr uint32_t kLutCopies = 1;
// Bilinear footprint of (tu, tv) on a w x h texture with REPEAT addressing:
// texel (i0, j0), its neighbours i1 = i0 + 1 and j1 = j0 + 1 (wrapped), and
// the filter weights a (along u) and b (along v).
struct Footprint {
  uint32_t i0, j0, i1, j1;
  float a, b;
};

__device__ __forceinline__ Footprint footprint(uint32_t w, uint32_t h, float tu, float tv) {
  float u = __fmaf_rn(tu, static_cast<float>(w), -0.5f), v = __fmaf_rn(tv, static_cast<float>(h), -0.5f);
  if (!(fabsf(u) < 8388608.0f)) u = 0.0f;  // NaN or beyond fp32's integer range: texel 0's neighbourhood
  if (!(fabsf(v) < 8388608.0f)) v = 0.0f;
  const float fu = floorf(u), fv = floorf(v);
  Footprint f;
  f.a = __fsub_rn(u, fu);
  f.b = __fsub_rn(v, fv);
  f.i0 = wrap(fu, w);
  f.j0 = wrap(fv, h);
  f.i1 = f.i0 + 1 == w ? 0 : f.i0 + 1;
  f.j1 = f.j0 + 1 == h ? 0 : f.j0 + 1;
  return f;
}

// sRGB-decode and filter the four texels t00 (i0, j0), t10 (i1, j0), t01 (i0, j1), t11 (i1, j1).
__device__ __forceinline__ F3 filter(uchar4 t00, uchar4 t10, uchar4 t01, uchar4 t11, float a, float b,
                                     const float* lut) {
  auto ch = [&](unsigned char c00, unsigned char c10, unsigned char c01, unsigned char c11) {
    return lerp(lerp(lut[c00 * kLutCopies], lut[c10 * kLutCopies], a), lerp(lut[c01 * kLutCopies], lut[c11 * kLutCopies], a),
                b);
  };
  return F3{ch(t00.x, t10.x, t01.x, t11.x), ch(t00.y, t10.y, t01.y, t11.y), ch(t00.z, t10.z, t01.z, t11.z)};
}

__device__ __forceinline__ uchar4 as_uchar4(uint32_t v) {
  return make_uchar4(v & 0xFFu, (v >> 8) & 0xFFu, (v >> 16) & 0xFFu, v >> 24);
}

// A texture of the scene buffers: four texel loads.
__device__ inline F3 sample_texels(const uchar4* __restrict__ px, uint32_t w, uint32_t h, float tu, float tv,
                                   const float* lut) {
  if (w == 0 || h == 0 || px == nullptr) return F3{0.f, 0.f, 0.f};
  const Footprint f = footprint(w, h, tu, tv);
  const uchar4 t00 = px[size_t(f.j0) * w + f.i0], t10 = px[size_t(f.j0) * w + f.i1];
  const uchar4 t01 = px[size_t(f.j1) * w + f.i0], t11 = px[size_t(f.j1) * w + f.i1];
  return filter(t00, t10, t01, t11, f.a, f.b, lut);
}

// A texture of the gather tables, stored as footprints: entry (j, i) holds the
// texels (i, j), (i + 1, j), (i, j + 1), (i + 1, j + 1) (wrapped) in one
// 16-byte word, so a sample is one load.
__device__ inline F3 sample_quads(const uint4* __restrict__ q, uint32_t w, uint32_t h, float tu, float tv,
                                  const float* lut) {
  if (w == 0 || h == 0 || q == nullptr) return F3{0.f, 0.f, 0.f};
  const Footprint f = footprint(w, h, tu, tv);
  const uint4 t = q[size_t(f.j0) * w + f.i0];
  return filter(as_uchar4(t.x), as_uchar4(t.y), as_uchar4(t.z), as_uchar4(t.w), f.a, f.b, lut);
}

// The gather tables of nrc_scene_prepare (nrc_scene_tables), as 16-byte words.
// Primitive row (4 words): (v0.xyz, tc0.u), (v1.xyz, tc0.v), (v2.xyz, tc1.u),
// (tc1.v, tc2.u, tc2.v, material id), the vertices in object space; the
// material id is kInvalidRow when one of the primitive's indices is out of
// range. Material row (4 words): (diffuse.rgb, roughness), (specular.rgb,
// flags: bit 0 diffuse textured, bit 1 specular textured), then the diffuse and
// the specular texture as (footprint array address low, high, width, height);
// the footprint arrays (sample_quads) are part of the tables.
struct SceneRows {
  const uint4* prims;
  const uint4* mats;
};
constexpr uint32_t kInvalidRow = 0xFFFFFFFFu;

// What UnpackNRCInput reads for one record, gathered from either form of the scene.
struct Gathered {
  F3 p[3];         // object-space vertices
  float2 tc[3];    // texcoords
  uint4 col[2];    // diffuse / specular constant rgb in x..z
  float roughness;
  const void* tex[2];    // texture of each colour (sampled when `textured`): texels, or footprints with kRows
  uint32_t tw[2], th[2];
  bool textured[2];
  bool ok;         // every index in range
};

__device__ __forceinline__ bool scene_empty(const nrc_scene& S) {
  return S.primitive_count == 0 || S.instance_count == 0 || S.vertex_count == 0 || S.texcoord_count == 0 ||
         S.material_count == 0;
}

// Gathers from the scene buffers (Scene.glsl:50-58: indices, then vertices,
// texcoords and the material). An out-of-range index is replaced by 0 (in range
// once the scene's counts are non-zero) and clears `ok`; no early exit.
__device__ __forceinline__ void gather_buffers(const nrc_scene& S, uint32_t pr, bool ok, Gathered& g) {
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
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float* p = S.vertices + size_t(vi[k]) * 3;
    g.p[k] = F3{p[0], p[1], p[2]};
  }
  const float2* tc2 = reinterpret_cast<const float2*>(S.texcoords);
#pragma unroll
  for (int k = 0; k < 3; ++k) g.tc[k] = tc2[ti[k]];
  // the material's words 0..7 (diffuse, its texture, specular, its texture) and
  // 12..15 (metallic, roughness, ior) in three 16-byte loads (std430, 16-byte aligned)
  const uint4* m4 = reinterpret_cast<const uint4*>(S.materials + mid);
  const uint4 md = m4[0], ms = m4[1], mr = m4[3];
  g.roughness = __uint_as_float(mr.y);
  g.col[0] = md;
  g.col[1] = ms;
  const uint32_t ids[2] = {md.w, ms.w};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    g.textured[c] = ok && ids[c] != 0xFFFFFFFFu && ids[c] < S.texture_count;
    g.tex[c] = nullptr;
    g.tw[c] = g.th[c] = 0;
    if (g.textured[c]) {
      const nrc_texture t = S.textures[ids[c]];
      g.tex[c] = t.texels;
      g.tw[c] = t.width;
      g.th[c] = t.height;
    }
  }
  g.ok = ok;
}

// Gathers from the prepared rows: the record's primitive row (its four words
// q, loaded by the caller), then its material row.
__device__ __forceinline__ void gather_row(const uint4 (&q)[4], const uint4* __restrict__ mats, bool ok, Gathered& g) {
  ok = ok && q[3].w != kInvalidRow;
  const uint32_t mid = ok ? q[3].w : 0u;
  g.p[0] = F3{__uint_as_float(q[0].x), __uint_as_float(q[0].y), __uint_as_float(q[0].z)};
  g.p[1] = F3{__uint_as_float(q[1].x), __uint_as_float(q[1].y), __uint_as_float(q[1].z)};
  g.p[2] = F3{__uint_as_float(q[2].x), __uint_as_float(q[2].y), __uint_as_float(q[2].z)};
  g.tc[0] = make_float2(__uint_as_float(q[0].w), __uint_as_float(q[1].w));
  g.tc[1] = make_float2(__uint_as_float(q[2].w), __uint_as_float(q[3].x));
  g.tc[2] = make_float2(__uint_as_float(q[3].y), __uint_as_float(q[3].z));
  const uint4* m = mats + size_t(mid) * 4;
  const uint4 m0 = m[0], m1 = m[1], m2 = m[2], m3 = m[3];
  g.col[0] = m0;
  g.col[1] = m1;
  g.roughness = __uint_as_float(m0.w);
  const uint4 t[2] = {m2, m3};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    g.textured[c] = ok && ((m1.w >> c) & 1u);
    g.tex[c] = reinterpret_cast<const void*>((static_cast<uint64_t>(t[c].y) << 32) | t[c].x);
    g.tw[c] = t[c].z;
    g.th[c] = t[c].w;
  }
  g.ok = ok;
}

// A record's primitive and instance, clamped to 0 (in range once the scene is
// not empty) when out of range, which clears `ok`.
struct RecordRef {
  uint32_t prim, inst;
  bool ok, flip;
};

__device__ __forceinline__ RecordRef record_ref(const nrc_scene& S, const nrc_packed_input& in) {
  const uint32_t prim = in.primitive_id, inst = in.flip_bit_instance_id & 0x7FFFFFFFu;
  RecordRef f;
  f.flip = (in.flip_bit_instance_id >> 31) != 0;
  f.ok = prim < S.primitive_count && inst < S.instance_count;
  f.prim = f.ok ? prim : 0u;
  f.inst = f.ok ? inst : 0u;
  return f;
}

// The primitive rows of a warp's 32 records (lane l's row index `prim`),
// loaded cooperatively: load r fetches the rows of records 8r..8r+7, four
// lanes per row (16 bytes each), so each load instruction touches 8 rows
// instead of 32. warp_rows_load issues the loads; warp_rows_share passes the
// rows through `buf` (2 KB of the warp's shared memory, 16-byte slots swizzled
// so that neither the stores nor the loads conflict) to their lanes. Warp-wide.
__device__ __forceinline__ void warp_rows_load(const uint4* __restrict__ rows, uint32_t prim, uint4 (&v)[4]) {
  const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint32_t p = __shfl_sync(0xffffffffu, prim, 8 * r + (lane >> 2));
    v[r] = rows[size_t(p) * 4 + (lane & 3u)];
  }
}

__device__ __forceinline__ void warp_rows_share(const uint4 (&v)[4], uint4* __restrict__ buf, uint4 (&q)[4]) {
  const uint32_t lane = threadIdx.x & 31u;
  __syncwarp();  // the buffer's previous contents have been read
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint32_t rec = 8 * r + (lane >> 2);
    buf[rec * 4 + ((lane & 3u) ^ ((rec >> 1) & 3u))] = v[r];
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 4; ++k) q[k] = buf[lane * 4 + (k ^ ((lane >> 1) & 3u))];
}

// UnpackNRCInput into 14 floats (nrc_input) from a record's gathered scene
// data; false (and zeros) for a record whose indices fall outside the scene.
// `lut` is this thread's copy of the sRGB decode table (stage_lut). kRows: the
// textures are the tables' footprint arrays. The loads take no early exit: an
// out-of-range index is replaced by 0 and the record's outputs are zeroed at
// the end, so a thread can have the loads of several records in flight.
template <bool kRows>
__device__ __forceinline__ bool finish_unpack(const nrc_scene& S, const nrc_packed_input& in, const RecordRef& ref,
                                              const Gathered& g, const float* lut, float (&r)[kInFloats]) {
  const bool flip = ref.flip;
  const float4* T4 = reinterpret_cast<const float4*>(S.transforms + size_t(ref.inst) * 12);
  const float4 T[3] = {T4[0], T4[1], T4[2]};
  F3 v[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = xform(T, g.p[k]);
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
  r[7] = g.roughness;
  const float tu = interp(g.tc[0].x, g.tc[1].x, g.tc[2].x, b0, b1, b2);
  const float tv = interp(g.tc[0].y, g.tc[1].y, g.tc[2].y, b0, b1, b2);
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    F3 col{__uint_as_float(g.col[c].x), __uint_as_float(g.col[c].y), __uint_as_float(g.col[c].z)};
    if (g.textured[c]) {
      if constexpr (kRows)
        col = sample_quads(static_cast<const uint4*>(g.tex[c]), g.tw[c], g.th[c], tu, tv, lut);
      else
        col = sample_texels(static_cast<const uchar4*>(g.tex[c]), g.tw[c], g.th[c], tu, tv, lut);
    }
    r[8 + 3 * c] = col.x;
    r[9 + 3 * c] = col.y;
    r[10 + 3 * c] = col.z;
  }
  if (!g.ok) {
#pragma unroll
    for (int k = 0; k < kInFloats; ++k) r[k] = 0.0f;
  }
  return g.ok;
}

// UnpackNRCInput of one record from the scene buffers (one thread's gathers).
__device__ __forceinline__ bool unpack_one(const nrc_scene& S, const nrc_packed_input& in, const float* lut,
                                           float (&r)[kInFloats]) {
  if (scene_empty(S)) {
#pragma unroll
    for (int k = 0; k < kInFloats; ++k) r[k] = 0.0f;
    return false;
  }
  const RecordRef ref = record_ref(S, in);
  Gathered g;
  gather_buffers(S, ref.prim, ref.ok, g);
  return finish_unpack<false>(S, in, ref, g, lut, r);
}

// sRGB -> linear of the 256 byte values, in double, rounded once (host).
const SrgbLut& srgb_lut();

// The table into shared memory as kLutCopies interleaved copies (entry c of
// copy k at lut[c * kLutCopies + k]); returns this thread's copy
// (thread % kLutCopies). Block-wide.
__device__ __forceinline__ const float* stage_lut(float* lut, const SrgbLut& src) {
  for (uint32_t i = threadIdx.x; i < 256u * kLutCopies; i += blockDim.x) lut[i] = src.v[i / kLutCopies];
  __syncthreads();
  return lut + (threadIdx.x % kLutCopies);
}

}  // namespace nrc
