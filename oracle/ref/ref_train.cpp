// Compiles the reference's training arithmetic from its own shader source, so the
// oracle's restatement (and, through golden vectors, the GPU) can be checked
// against it:
//   - shader/src/nrc_train_prepare.comp  (count clamp, indirect size, step state)
//   - shader/src/nrc_optimize.comp       (NaN/Inf scrub, Adam, EMA, fp16 writes)
//   - NNLoadDA3_RelativeL2LuminanceLoss  (shader/src/NN_nv.glsl:178-196: the
//     relative-L2 luminance loss gradient packed to fp16 as one 16-wide row)
// oracle/ref/glsl_to_cpp.py turns each into C++ text in oracle/_ref/ (only the
// interface declarations change; every arithmetic line stays as written) and
// this file supplies what GLSL has built in. Test infrastructure only: built by
// oracle/ref/build_ref.sh where the reference tree is present, never shipped.
#define GLM_FORCE_SWIZZLE
#define GLM_FORCE_INTRINSICS
#include <glm/glm.hpp>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace glsl_rt {
using namespace glm;
typedef _Float16 float16_t;
// GLSL's packHalf2x16 rounds to nearest even (glm's rounds ties upward): an IEEE
// conversion through _Float16.
inline uint pack_half2x16_rne(const vec2& v) {
	_Float16 lo = (_Float16)v.x, hi = (_Float16)v.y;
	uint16_t a, b;
	std::memcpy(&a, &lo, 2);
	std::memcpy(&b, &hi, 2);
	return uint(a) | (uint(b) << 16);
}
template <typename T, qualifier Q, int E0, int E1>
inline uint pack_half2x16_rne(const detail::_swizzle<2, T, Q, E0, E1, -1, -2>& a) {
	return pack_half2x16_rne(vec2(a));
}
inline bool isnan(float x) { return std::isnan(x); }
inline bool isinf(float x) { return std::isinf(x); }
inline bool subgroupAll(bool b) { return b; }  // one invocation at a time
inline uint min(uint a, int b) { return a < uint(b) ? a : uint(b); }
} // namespace glsl_rt

namespace glsl_prepare {
using namespace glsl_rt;
using glsl_rt::min;
#include "nrc_train_prepare.inc"
} // namespace glsl_prepare

namespace glsl_optimize {
using namespace glsl_rt;
using glsl_rt::isinf;
using glsl_rt::isnan;
static uvec3 gl_GlobalInvocationID;
#define WRITE_USE_WEIGHTS
#include "nrc_optimize.inc"
#undef WRITE_USE_WEIGHTS
} // namespace glsl_optimize

namespace glsl_loss {
using namespace glsl_rt;
template <int A, int B, int C, int D>
struct fcoopmatNV {};
constexpr int gl_ScopeSubgroup = 3;
static uvec3 gl_LocalInvocationID;
static uint gl_SubgroupID;
static uvec4 g_shared[1024];
inline void barrier() {}
template <class... T>
inline void coopMatLoadNV(T&&...) {}
#define WORKGROUP_SIZE 128
#define SUBGROUP_SIZE 32
#define SHARED_BUFFER g_shared
#define packHalf2x16 pack_half2x16_rne
#define in
#define inout
#define out
#include "nn_loss.inc"
#undef in
#undef inout
#undef out
#undef packHalf2x16
} // namespace glsl_loss

extern "C" {

typedef struct ref_opt_state {
	uint32_t t;
	float beta1_t, beta2_t, alpha_t, alpha_t_1;
} ref_opt_state;

// nrc_train_prepare.comp on one count: returns the clamped count, writes the
// dispatch size (work groups of 128) and advances *st as the shader does.
uint32_t ref_prepare(uint32_t count, ref_opt_state* st, uint32_t* groups) {
	using namespace glsl_prepare;
	uCount = count;
	uStep = st->t;
	uBeta1_T = st->beta1_t;
	uBeta2_T = st->beta2_t;
	uAlpha_T = st->alpha_t;
	uAlpha_T_1 = st->alpha_t_1;
	ref_prepare_main();
	st->t = uStep;
	st->beta1_t = uBeta1_T;
	st->beta2_t = uBeta2_T;
	st->alpha_t = uAlpha_T;
	st->alpha_t_1 = uAlpha_T_1;
	*groups = uCommand.x;
	return uCount;
}

// nrc_optimize.comp over n parameters: entries n x {m, v, w, ema} updated in
// place, w16 / use16 receive the fp16 weights (untouched when count == 0, as the
// shader returns early). `st` is the state after the prepare pass.
void ref_optimize(float* entries, const float* grad, int64_t n, uint32_t count, const ref_opt_state* st,
                  uint32_t use_ema, uint16_t* w16, uint16_t* use16) {
	using namespace glsl_optimize;
	static_assert(sizeof(OptimizerEntry) == 16, "entry layout");
	uWeights = reinterpret_cast<float16_t*>(w16);
	uUseWeights = reinterpret_cast<float16_t*>(use16);
	uGradients = const_cast<float*>(grad);
	uOptimizerEntries = reinterpret_cast<OptimizerEntry*>(entries);
	uBatchTrainCount = count;
	uStep = st->t;
	uBeta1_T = st->beta1_t;
	uBeta2_T = st->beta2_t;
	uAlpha_T = st->alpha_t;
	uAlpha_T_1 = st->alpha_t_1;
	uUseEMAWeights = use_ema;
	for (int64_t i = 0; i < n; ++i) {
		gl_GlobalInvocationID = uvec3(uint(i), 0u, 0u);
		ref_optimize_main();
	}
}

// NNLoadDA3_RelativeL2LuminanceLoss for n (prediction, target) pairs: rows
// receives, per pair, the first two words of the fp16 gradient row (d0|d1<<16,
// d2|0<<16); the shader zeroes the rest of the 16-wide row.
void ref_loss_rows(const float* pred, const float* target, int64_t n, float loss_scale, uint32_t* rows) {
	using namespace glsl_loss;
	fcoopmatNV<16, gl_ScopeSubgroup, 16, 16> unused[8];
	gl_SubgroupID = 0;
	for (int64_t i = 0; i < n; ++i) {
		gl_LocalInvocationID = uvec3(0u);
		NNLoadDA3_RelativeL2LuminanceLoss(vec3(pred[3 * i], pred[3 * i + 1], pred[3 * i + 2]),
		                                  vec3(target[3 * i], target[3 * i + 1], target[3 * i + 2]), loss_scale,
		                                  unused);
		rows[2 * i] = g_shared[0].x;
		rows[2 * i + 1] = g_shared[0].y;
	}
}
}
