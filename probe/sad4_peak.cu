// Peak-throughput probe for the packed-byte SAD instruction used by the
// motion-estimation kernels (benchmark helper, not part of the operator ABI;
// built by __graft_entry__.build() into probe/libumi_probe.so).
//
// umi_probe_sad4_peak launches `ctas` CTAs of 256 threads.  In mode 0 the
// timed loop of every thread is nothing but `vabsdiff4.u32.u32.u32.add`
// instructions: 8 independent accumulator chains, each against its own pair
// of operands that stay fixed in registers (the chains differ in their
// operands, so no two instructions compute the same value).  Nothing else
// issues on the integer ALU pipe inside the loop: the loop counter of the
// outer loop runs once per 16 x 8 = 128 SAD instructions.  Mode 1 runs the
// two-instruction alternative (__vabsdiffu4 then __dp4a against 0x01010101)
// for comparison.  The caller times the launch.
#include <cuda_runtime.h>
#include <cstdint>

namespace {

__device__ __forceinline__ uint32_t sad4_acc(uint32_t a, uint32_t b, uint32_t c) {
	uint32_t d;
	asm volatile("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
	return d;
}

template <int MODE>
__global__ void __launch_bounds__(256) sad4_peak_kernel(uint32_t seed, int iters, uint32_t* out) {
	const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t a[8], b[8], acc[8];
#pragma unroll
	for (int k = 0; k < 8; ++k) {
		a[k] = (seed ^ (t * 2654435761u)) + 0x01020304u * (uint32_t)k;
		b[k] = seed * 747796405u + t * 0x9E3779B9u + 0x10203040u * (uint32_t)k;
		acc[k] = 0;
	}
#pragma unroll 1
	for (int i = 0; i < iters; ++i) {
#pragma unroll
		for (int u = 0; u < 16; ++u) {
#pragma unroll
			for (int k = 0; k < 8; ++k) {
				if (MODE == 0) acc[k] = sad4_acc(a[k], b[k], acc[k]);
				else acc[k] = (uint32_t)__dp4a(__vabsdiffu4(a[k], b[k]), 0x01010101u, acc[k]);
			}
		}
	}
	uint32_t s = 0;
#pragma unroll
	for (int k = 0; k < 8; ++k) s ^= acc[k];
	out[t] = s;
}

}  // namespace

// Returns cudaError_t as int.  out must hold ctas*256 uint32.
extern "C" int umi_probe_sad4_peak(int mode, int ctas, int iters, uint32_t* out, void* stream) {
	const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
	if (mode == 0) sad4_peak_kernel<0><<<ctas, 256, 0, st>>>(12345u, iters, out);
	else sad4_peak_kernel<1><<<ctas, 256, 0, st>>>(12345u, iters, out);
	return (int)cudaGetLastError();
}

// Byte absolute differences performed by one launch.
extern "C" double umi_probe_sad4_ops(int ctas, int iters) { return 4.0 * 8.0 * 16.0 * 256.0 * (double)ctas * iters; }
