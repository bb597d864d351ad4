// Compiles the reference's CPU MLP (test/main.cpp: Evaluate() and Train()) unchanged,
// with a stub device runtime, and exposes them through a C interface for fixture
// generation and cost timing. Test infrastructure only (built into oracle/_ref/).
#define main vknrc_reference_test_main
#include "main.cpp"
#undef main

extern "C" {

// weights: 20672 fp16 (a8 layout); inputs: n x 64 fp16 (column-major 64 x n);
// out: n x 3 fp16. Returns 0.
int ref_evaluate(const uint16_t *weights, const uint16_t *inputs, int64_t n, uint16_t *out) {
	std::vector<half> w(64 * 64 * 5 + 64 * kOutputCount), x((size_t)n * 64);
	std::memcpy(w.data(), weights, w.size() * sizeof(half));
	std::memcpy(x.data(), inputs, x.size() * sizeof(half));
	auto y = Evaluate(w, x);
	std::memcpy(out, y.data(), y.size() * sizeof(half));
	return 0;
}

// Reference Train() (prints layer shapes; its math is not the shader's). Used for
// cost timing only. dw: 20672 floats.
int ref_train(const uint16_t *weights, const uint16_t *inputs, const uint16_t *targets, int64_t n, float *dw) {
	std::vector<half> w(64 * 64 * 5 + 64 * kOutputCount), x((size_t)n * 64), t((size_t)n * 3);
	std::memcpy(w.data(), weights, w.size() * sizeof(half));
	std::memcpy(x.data(), inputs, x.size() * sizeof(half));
	std::memcpy(t.data(), targets, t.size() * sizeof(half));
	auto g = Train(w, x, t);
	std::memcpy(dw, g.data(), g.size() * sizeof(float));
	return 0;
}
}
