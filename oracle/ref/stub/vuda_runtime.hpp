// Stand-in for the reference's Vulkan-backed CUDA-like runtime (test/vuda), so that
// the reference's CPU MLP in test/main.cpp compiles without a graphics stack. The
// device calls do nothing: only Evaluate() and Train() are used from that file.
#pragma once
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <span>
#include <string>
#include <vector>

enum vuda_stub_copy_kind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };
inline int cudaMalloc(void **p, size_t) { *p = nullptr; return 0; }
inline int cudaMemcpy(void *, const void *, size_t, int) { return 0; }
inline int cudaStreamSynchronize(int) { return 0; }
inline int cudaSetDevice(int) { return 0; }
namespace vuda {
template <typename... A> inline void launchKernel(A &&...) {}
} // namespace vuda
