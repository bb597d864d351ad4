// Compiles the reference's record encoding (shader/src/NRCRecord.glsl) unchanged as
// C++ on top of the reference's vendored glm, so that the oracle's restatement of
// the encoding can be checked against the reference's own source. Test
// infrastructure only: built into oracle/_ref/ by oracle/ref/build_ref.sh, in the
// container that holds the reference tree; never shipped, never on the product path.
#define GLM_FORCE_SWIZZLE
#define GLM_FORCE_INTRINSICS
#include <glm/glm.hpp>
#include <glm/gtc/packing.hpp>
#include <cstdint>
#include <cstring>

namespace glsl {
using namespace glm;

// GLSL allows scalar-int op vector-float; glm does not.
inline vec4 operator-(int a, const vec4& b) { return float(a) - b; }
// GLSL compares a swizzle with a vector; glm's swizzle proxy converts to vec.
template <int N, typename T, qualifier Q, int E0, int E1, int E2, int E3>
inline bool operator==(const detail::_swizzle<N, T, Q, E0, E1, E2, E3>& a, const vec<N, T, Q>& b) {
	return vec<N, T, Q>(a) == b;
}
// GLSL's packHalf2x16 on the GPU rounds to nearest even; glm's rounds ties upward.
// The harness keeps the GPU built-in's rounding (IEEE conversion via _Float16).
inline uint pack_half2x16_rne(const vec2& v) {
	_Float16 lo = (_Float16)v.x, hi = (_Float16)v.y;
	uint16_t a, b;
	std::memcpy(&a, &lo, 2);
	std::memcpy(&b, &hi, 2);
	return uint(a) | (uint(b) << 16);
}
template <typename T, qualifier Q, int E0, int E1>
inline uint packHalf2x16(const detail::_swizzle<2, T, Q, E0, E1, -1, -2>& a) {
	return pack_half2x16_rne(vec2(a));
}
template <typename T, qualifier Q, int E0, int E1>
inline vec4 make_vec4(const detail::_swizzle<2, T, Q, E0, E1, -1, -2>& a, float z, float w) {
	return vec4(vec2(a), z, w);
}
// GLSL clamp(float, int, int)
inline float clamp(float x, int lo, int hi) { return glm::clamp(x, float(lo), float(hi)); }

#define in
#define inout
#define out
#include "NRCRecord.glsl"
#undef in
#undef inout
#undef out
} // namespace glsl

extern "C" {

// records: n x 14 floats laid out as UnpackedNRCInput (position, scattered_dir,
// normal, roughness, diffuse, specular); out: n x 64 fp16 bit patterns.
void ref_encode(const float* records, int64_t n, uint16_t* out) {
	for (int64_t i = 0; i < n; ++i) {
		const float* r = records + 14 * i;
		glsl::UnpackedNRCInput u;
		u.position = glm::vec3(r[0], r[1], r[2]);
		u.scattered_dir = glm::vec2(r[3], r[4]);
		u.normal = glm::vec2(r[5], r[6]);
		u.roughness = r[7];
		u.diffuse = glm::vec3(r[8], r[9], r[10]);
		u.specular = glm::vec3(r[11], r[12], r[13]);
		glm::uvec4 o[8];
		glsl::NRCInputEncode(u, o);
		std::memcpy(out + 64 * i, o, 128);
	}
}

// dirs: n x 3 unit vectors; out: n x 2 (NRCSphEncode)
void ref_sph_encode(const float* dirs, int64_t n, float* out) {
	for (int64_t i = 0; i < n; ++i) {
		glm::vec2 s = glsl::NRCSphEncode(glm::vec3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
		out[2 * i] = s.x;
		out[2 * i + 1] = s.y;
	}
}
}
