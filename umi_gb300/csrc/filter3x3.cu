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
// This form reaches the HBM copy rate on large frames (7.0 TB/s at 8192^2).
//
// umi_filter3x3_f32_tma is the same filter with TMA-staged halo tiles
// (filter3x3_tma_kernel: one box per tile with the tensor map's zero fill as
// the padding, double-buffered, TMA tile stores).  Measured on GB300 it is
// slower than the register form at every size from 1024^2 to 8192^2 (5.6 vs
// 7.0 TB/s at 8192^2): each input is used by three rows of one warp already,
// so staging adds shared-memory traffic without saving DRAM traffic.  It is
// kept as a separate entry point, not the default.
#include <cudaTypedefs.h>

#include <algorithm>

#include "common.h"
#include "tc_common.cuh"

namespace umi {
void* tma_encode_fn();  // cuTensorMapEncodeTiled (gemm_tc.cu)
}

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

// ---- TMA-staged halo tiles (zero padding, 16-byte aligned rows).
// Persistent CTAs walk tiles t = blockIdx.x, + gridDim.x, ... of TW x TH
// outputs.  One TMA box brings a tile's input with its halo, (TW + 8) x
// (TH + 2) floats from (x0 - 4, y0 - 1): the box's x stays on a 16-byte
// boundary (4 floats left of the tile instead of 1), and the tensor map's
// zero fill outside the image is the reference's PAD 0.  Two input buffers:
// the next tile's box is in flight while this one is computed.  Thread t owns
// column t % TW and TH / 2 rows: a 3 x 3 register window slides down its
// column.  Outputs go to one of two shared tiles and leave by one TMA tile
// store each (clipped at the image edge by the tensor map), overlapping the
// next tile.  Waits are bounded (1 s): a CTA whose box never lands writes
// NaN into that tile, lets its copies finish and returns.
constexpr int TTW = 128, TTH = 16, TNT = 256;
constexpr int TIN_W = TTW + 8, TIN_H = TTH + 2;
constexpr int TROWS = TTH / (TNT / TTW);  // output rows per thread
constexpr int TIN_WORDS = (TIN_W * TIN_H + 31) & ~31;  // input tile, rounded to 128 bytes
constexpr int TOUT_WORDS = TTW * TTH;
constexpr size_t TSMEM = (size_t)4 * (2 * TIN_WORDS + 2 * TOUT_WORDS) + 128;
static_assert(TIN_WORDS % 32 == 0 && TOUT_WORDS % 32 == 0, "TMA tiles in shared memory start on 128-byte boundaries");

__global__ void __launch_bounds__(TNT) filter3x3_tma_kernel(const __grid_constant__ CUtensorMap tin,
                                                             const __grid_constant__ CUtensorMap tout, float* __restrict__ out,
                                                             const FilterGeom g, const Weights9 wt, int tiles_x,
                                                             int ntiles) {
	using namespace umi_tc;
	extern __shared__ __align__(128) uint8_t smem_raw[];
	float* sin = reinterpret_cast<float*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
	float* sout = sin + 2 * TIN_WORDS;  // 128-byte aligned (TMA store sources)
	__shared__ __align__(8) uint64_t bar[2];
	__shared__ int abort_sh;
	if (threadIdx.x == 0) {
		mbar_init(&bar[0], 1);
		mbar_init(&bar[1], 1);
		abort_sh = 0;
		fence_mbar_init();
	}
	__syncthreads();
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
	asm volatile("griddepcontrol.launch_dependents;");
	asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
	auto load = [&](int t, int b) {
		const int ty = t / tiles_x, tx = t - ty * tiles_x;
		mbar_arrive_expect_tx(&bar[b], (uint32_t)(4 * TIN_W * TIN_H));
		tma_load_2d(sin + b * TIN_WORDS, &tin, &bar[b], tx * TTW - 4, ty * TTH - 1);
	};
	const int c = threadIdx.x % TTW, r0 = (threadIdx.x / TTW) * TROWS;
	int i = 0;
	if (threadIdx.x == 0 && (int)blockIdx.x < ntiles) load(blockIdx.x, 0);
	for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
		const int b = i & 1;
		const int tn = t + gridDim.x;
		if (threadIdx.x == 0) {
			if (tn < ntiles) load(tn, b ^ 1);  // its buffer was last read in iteration i - 1 (barrier below)
			bulk_wait_read_1();                // the store that used sout[b] (iteration i - 2) has read it
		}
		mbar_wait(&bar[b], (uint32_t)(i >> 1) & 1u, &abort_sh, nullptr, 0);
		__syncthreads();  // every thread sees the same abort flag; sout[b] is free
		const int ty = t / tiles_x, tx = t - ty * tiles_x;
		const int x0 = tx * TTW, y0 = ty * TTH;
		if (abort_sh) {  // a box never landed: mark the tile, let the copies finish, return (uniform)
			for (int r = r0; r < r0 + TROWS; ++r)
				if (y0 + r < g.h && x0 + c < g.w) out[(size_t)(y0 + r) * g.w + x0 + c] = __int_as_float(0x7fc00000);
			if (threadIdx.x == 0) {
				volatile int own = 0;
				mbar_wait(&bar[b], (uint32_t)(i >> 1) & 1u, &own, nullptr, 0);
				if (tn < ntiles) mbar_wait(&bar[b ^ 1], (uint32_t)((i + 1) >> 1) & 1u, &own, nullptr, 0);
				bulk_wait_all();
			}
			return;
		}
		// input column of output column c, dx = -1: tile column c + 3
		const float* col = sin + b * TIN_WORDS + c + 3;
		float* o = sout + b * TOUT_WORDS;
		float a0 = col[r0 * TIN_W], a1 = col[r0 * TIN_W + 1], a2 = col[r0 * TIN_W + 2];
		float b0 = col[(r0 + 1) * TIN_W], b1 = col[(r0 + 1) * TIN_W + 1], b2 = col[(r0 + 1) * TIN_W + 2];
#pragma unroll
		for (int k = 0; k < TROWS; ++k) {
			const float* rr = col + (r0 + k + 2) * TIN_W;
			const float c0 = rr[0], c1 = rr[1], c2 = rr[2];
			float s = 0.0f;
			s = fmaf(wt.w[0], a0, s); s = fmaf(wt.w[1], a1, s); s = fmaf(wt.w[2], a2, s);
			s = fmaf(wt.w[3], b0, s); s = fmaf(wt.w[4], b1, s); s = fmaf(wt.w[5], b2, s);
			s = fmaf(wt.w[6], c0, s); s = fmaf(wt.w[7], c1, s); s = fmaf(wt.w[8], c2, s);
			o[(r0 + k) * TTW + c] = s;
			a0 = b0; a1 = b1; a2 = b2;
			b0 = c0; b1 = c1; b2 = c2;
		}
		fence_proxy_async_smem();  // the tile's generic stores before the async-proxy store reads them
		__syncthreads();           // also: every thread is done reading sin[b]
		if (threadIdx.x == 0) {
			tma_store_2d(&tout, o, x0, y0);
			bulk_commit();
		}
	}
	if (threadIdx.x == 0) bulk_wait_all();
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

extern "C" umi_status umi_filter3x3_f32_tma(const float* in, float* out, int32_t h, int32_t w, const float* w9,
                                            void* stream) {
	if (h < 0 || w < 0) return umi::fail(UMI_ERR_INVALID_ARG, "filter3x3_tma: negative size %dx%d", h, w);
	if (h == 0 || w == 0) return umi::ok();
	if (!in || !out || !w9) return umi::fail(UMI_ERR_INVALID_ARG, "filter3x3_tma: null pointer");
	if (in == out) return umi::fail(UMI_ERR_INVALID_ARG, "filter3x3_tma: in and out alias");
	const float pad = 0.0f;
	FilterGeom g{h, w, pad, umi::aligned(in, 16) && umi::aligned(out, 16) && (w % 4) == 0};
	Weights9 wt;
	for (int i = 0; i < 9; ++i) wt.w[i] = w9[i];
	auto enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(umi::tma_encode_fn());
	if (!enc) return umi::fail(UMI_ERR_CUDA, "filter3x3_tma: cuTensorMapEncodeTiled unavailable");
	if (!g.vec) return umi::fail(UMI_ERR_UNSUPPORTED, "filter3x3_tma: needs 16-byte aligned in/out and w %% 4 == 0");
	{
		CUtensorMap tin, tout;
		const cuuint64_t dims[2] = {(cuuint64_t)w, (cuuint64_t)h};
		const cuuint64_t strides[1] = {(cuuint64_t)w * 4};
		const cuuint32_t es[2] = {1, 1};
		const cuuint32_t bin[2] = {(cuuint32_t)TIN_W, (cuuint32_t)TIN_H};
		const cuuint32_t bout[2] = {(cuuint32_t)TTW, (cuuint32_t)TTH};
		CUresult r = enc(&tin, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(in), dims, strides, bin, es,
		                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
		                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (r == CUDA_SUCCESS)
			r = enc(&tout, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, out, dims, strides, bout, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
			        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (r == CUDA_SUCCESS) {
			UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(filter3x3_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                                              (int)TSMEM), "cudaFuncSetAttribute"));
			int dev = 0, sms = 0, per_sm = 0;
			UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
			UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
			                         "cudaDeviceGetAttribute"));
			UMI_TRY(umi::cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, filter3x3_tma_kernel, TNT, TSMEM),
			                         "cudaOccupancyMaxActiveBlocksPerMultiprocessor"));
			const int tiles_x = umi::ceil_div(w, TTW), ntiles = tiles_x * umi::ceil_div(h, TTH);
			cudaLaunchConfig_t cfg{};
			cfg.gridDim = dim3(std::max(1, std::min(ntiles, sms * std::max(per_sm, 1))));
			cfg.blockDim = dim3(TNT);
			cfg.dynamicSmemBytes = TSMEM;
			cfg.stream = umi::as_stream(stream);
			cudaLaunchAttribute attr[1];
			attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
			attr[0].val.programmaticStreamSerializationAllowed = 1;
			cfg.attrs = attr;
			cfg.numAttrs = 1;
			UMI_TRY(umi::cuda_status(cudaLaunchKernelEx(&cfg, filter3x3_tma_kernel, tin, tout, out, g, wt, tiles_x, ntiles),
			                         "filter3x3_tma_kernel"));
			return umi::ok();
		}
		return umi::fail(UMI_ERR_CUDA, "filter3x3_tma: tensor map (%d)", (int)r);
	}
}
