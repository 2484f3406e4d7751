// Checked build of the generic path (-DUMI_CHECKED): an output view that
// maps points outside the output's physical extent must raise the flag and
// skip those writes (guard words after the buffer stay intact); a valid call
// must leave the flag clear.  Prints one JSON line.
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "umi/UMI_gpu.h"

using namespace UMI;

namespace {

const auto PAD = PhysicalDim::PAD;

struct Copy {
	int v;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(1, 0) { v = IMEM(0, 0); }
	STRATEGY_LOOP_STUB_
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = v; }
};

}  // namespace

int main() {
	const int w = 64, guard = 256;
	std::vector<int> in(w), host(w + guard);
	for (int i = 0; i < w; ++i) in[i] = i + 1;
	int *din = nullptr, *dout = nullptr;
	cudaMalloc(&din, w * sizeof(int));
	cudaMalloc(&dout, (w + guard) * sizeof(int));
	cudaMemcpy(din, in.data(), w * sizeof(int), cudaMemcpyHostToDevice);
	auto run = [&](int out_stride) {
		cudaMemset(dout, 0x5a, (w + guard) * sizeof(int));
		const umi_status st = Execute<Copy, 0x11>(
			{{{1, 1, 1, 1}, {1, 1, 1, 1}, {1, 1, 1, 1}, {w, 32, 32, 1}}}, {{{1, 1}, {1, 1}, {1, 1}, {1, 1}}},
			{{{{{{}, {}, {}, {3, 0, 1}}}, {}, {{{1, PAD}, {1, PAD}, {1, PAD}, {w, PAD}}}, DEFAULT_SHM, {din}, {}}}},
			{{{{{{}, {}, {}, {3, 0, out_stride}}}, {}, {{{}, {}, {}, {w, PAD}}}, {dout}}}});
		const unsigned flags = checked_flags();
		cudaMemcpy(host.data(), dout, (w + guard) * sizeof(int), cudaMemcpyDeviceToHost);
		bool guard_ok = true;
		for (int i = w; i < w + guard; ++i) guard_ok &= host[i] == 0x5a5a5a5a;
		int written = 0;
		for (int i = 0; i < w; ++i) written += host[i] != 0x5a5a5a5a;
		return std::make_tuple((int)st, flags, guard_ok, written);
	};
	const auto [st1, f1, g1, n1] = run(1);  // valid: every point writes its own element
	const auto [st2, f2, g2, n2] = run(3);  // stride 3: points p >= 22 map past the 64 elements
	std::printf("{\"valid\": {\"status\": %d, \"flags\": %u, \"guard_ok\": %d, \"written\": %d}, "
	            "\"oob\": {\"status\": %d, \"flags\": %u, \"guard_ok\": %d, \"written\": %d}}\n",
	            st1, f1, (int)g1, n1, st2, f2, (int)g2, n2);
	cudaFree(din);
	cudaFree(dout);
	return 0;
}
