// Reference input streams that need the C++ standard library.
// TEST INFRASTRUCTURE ONLY.
#include <cstddef>
#include <cstdint>
#include <functional>
#include <random>

#include "umi_oracle.h"

// main/fprop.cu:41-47 draws the input tensor and then the weights from one
// std::default_random_engine with the default seed through
// uniform_int_distribution<int>(0, 10).  Drawing from the same standard
// library engine and distribution reproduces the stream exactly.
extern "C" void oracle_ref_fprop_inputs(int32_t* in, size_t n_in, int32_t* wt, size_t n_wt) {
	std::default_random_engine gen;
	std::uniform_int_distribution<int> dist(0, 10);
	for (size_t i = 0; i < n_in; ++i) in[i] = dist(gen);
	for (size_t i = 0; i < n_wt; ++i) wt[i] = dist(gen);
}
