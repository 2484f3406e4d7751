// 3x3 weighted filter on float32 images, sm_103a.
//
// Replaces the Execute calls of main/filter3x3.cu:37-58 (Filter3x3: sum of a
// 3x3 neighbourhood, PAD value outside the image) and main/wfilter3x3.cu:39-69
// (WFilter3x3: the same with a 3x3 weight memory) for float images.
//
// HBM-bound: 4 bytes read + 4 bytes written per pixel.  A warp owns a
// 128-column strip and RY output rows; each lane keeps 4 adjacent columns of
// three input rows in registers, loads every input row once with one 128-bit
// load, takes the x-1 / x+4 neighbours from the adjacent lanes by shuffle
// (the strip's edge lanes load one extra float), and writes 4 outputs with
// one 128-bit store.  Accumulation order per output: (dy, dx) row-major, FMA.
#include "common.h"

namespace {

constexpr int RY = 4;     // output rows per warp
constexpr int WARPS = 8;  // warps per CTA, stacked vertically
constexpr int TWC = 128;  // columns per warp

struct Weights9 {
	float w[9];
};

struct FilterGeom {
	int h, w;
	float pad;
	int vec;  // in/out 16-byte aligned and w % 4 == 0
};

// Row y, columns x .. x+3 of this lane, plus the strip-edge neighbour (x0-1
// for lane 0, x0+TWC for lane 31) in `edge`.
__device__ __forceinline__ float4 load_row(const float* __restrict__ in, const FilterGeom& g, int y, int x0, int lane,
                                           float& edge) {
	const int x = x0 + 4 * lane;
	float4 v = make_float4(g.pad, g.pad, g.pad, g.pad);
	edge = g.pad;
	if (y >= 0 && y < g.h) {
		const float* row = in + (size_t)y * g.w;
		if (g.vec && x + 3 < g.w) {
			v = __ldg(reinterpret_cast<const float4*>(row + x));
		} else {
			if (x + 0 < g.w) v.x = __ldg(row + x + 0);
			if (x + 1 < g.w) v.y = __ldg(row + x + 1);
			if (x + 2 < g.w) v.z = __ldg(row + x + 2);
			if (x + 3 < g.w) v.w = __ldg(row + x + 3);
		}
		const int xe = lane == 0 ? x0 - 1 : x0 + TWC;
		if ((lane == 0 || lane == 31) && xe >= 0 && xe < g.w) edge = __ldg(row + xe);
	}
	return v;
}

// Columns x-1 .. x+4 of a loaded row: neighbours come from the adjacent lanes.
__device__ __forceinline__ void spread(float4 v, float edge, int lane, float r[6]) {
	float left = __shfl_up_sync(0xffffffffu, v.w, 1);
	float right = __shfl_down_sync(0xffffffffu, v.x, 1);
	if (lane == 0) left = edge;
	if (lane == 31) right = edge;
	r[0] = left; r[1] = v.x; r[2] = v.y; r[3] = v.z; r[4] = v.w; r[5] = right;
}

__global__ void __launch_bounds__(WARPS * 32) filter3x3_f32_kernel(const float* __restrict__ in, float* __restrict__ out,
                                                                   const FilterGeom g, const Weights9 wt) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
	// Programmatic dependent launch: let the next launch in the stream start
	// its CTAs early, and wait for the previous one before touching memory.
	asm volatile("griddepcontrol.launch_dependents;");
	asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int x0 = blockIdx.x * TWC;
	const int y0 = (blockIdx.y * WARPS + warp) * RY;
	if (y0 >= g.h) return;  // whole warp leaves together
	// Issue all RY + 2 row loads before any use.
	float4 raw[RY + 2];
	float edge[RY + 2];
#pragma unroll
	for (int i = 0; i < RY + 2; ++i) raw[i] = load_row(in, g, y0 - 1 + i, x0, lane, edge[i]);
	float r0[6], r1[6], r2[6];
	spread(raw[0], edge[0], lane, r0);
	spread(raw[1], edge[1], lane, r1);
	const int x = x0 + 4 * lane;
#pragma unroll
	for (int i = 0; i < RY; ++i) {
		const int y = y0 + i;
		if (y >= g.h) break;
		spread(raw[i + 2], edge[i + 2], lane, r2);
		float o[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			float s = 0.0f;
			s = fmaf(wt.w[0], r0[k], s); s = fmaf(wt.w[1], r0[k + 1], s); s = fmaf(wt.w[2], r0[k + 2], s);
			s = fmaf(wt.w[3], r1[k], s); s = fmaf(wt.w[4], r1[k + 1], s); s = fmaf(wt.w[5], r1[k + 2], s);
			s = fmaf(wt.w[6], r2[k], s); s = fmaf(wt.w[7], r2[k + 1], s); s = fmaf(wt.w[8], r2[k + 2], s);
			o[k] = s;
		}
		float* dst = out + (size_t)y * g.w + x;
		if (g.vec && x + 3 < g.w) {
			*reinterpret_cast<float4*>(dst) = make_float4(o[0], o[1], o[2], o[3]);
		} else {
#pragma unroll
			for (int k = 0; k < 4; ++k)
				if (x + k < g.w) dst[k] = o[k];
		}
#pragma unroll
		for (int k = 0; k < 6; ++k) { r0[k] = r1[k]; r1[k] = r2[k]; }
	}
}

}  // namespace

extern "C" umi_status umi_filter3x3_f32(const float* in, float* out, int32_t h, int32_t w, const float* w9, float pad,
                                        void* stream) {
	if (h < 0 || w < 0) return umi::fail(UMI_ERR_INVALID_ARG, "filter3x3: negative size %dx%d", h, w);
	if (h == 0 || w == 0) return umi::ok();
	if (!in || !out || !w9) return umi::fail(UMI_ERR_INVALID_ARG, "filter3x3: null pointer");
	if (in == out) return umi::fail(UMI_ERR_INVALID_ARG, "filter3x3: in and out alias");
	FilterGeom g{h, w, pad, umi::aligned(in, 16) && umi::aligned(out, 16) && (w % 4) == 0};
	Weights9 wt;
	for (int i = 0; i < 9; ++i) wt.w[i] = w9[i];
	cudaLaunchConfig_t cfg{};
	cfg.gridDim = dim3(umi::ceil_div(w, TWC), umi::ceil_div(h, WARPS * RY));
	cfg.blockDim = dim3(WARPS * 32);
	cfg.stream = umi::as_stream(stream);
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	UMI_TRY(umi::cuda_status(cudaLaunchKernelEx(&cfg, filter3x3_f32_kernel, in, out, g, wt), "filter3x3_f32_kernel"));
	return umi::ok();
}
