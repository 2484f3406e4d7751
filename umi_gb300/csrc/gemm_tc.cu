// Tensor-core GEMM on sm_103a (tcgen05 + TMA), C[M,N] (fp32) = A[M,K] * B[N,K]^T
// with bf16 or f16 operands and fp32 accumulation in tensor memory.
//
// Replaces the Execute call of main/gemm.cu:37-67 (Gemm strategy,
// main/gemm.cu:8-15: accum += A * B through shared memory, scalar) for the
// half-precision operand types, plus a split-precision FP32 emulation.
//
// One CTA computes a 128 x 256 tile of C:
//   warp 0, one lane  : TMA producer, K-slices of 64 into a 4-stage ring
//                       (A 16 KB + B 32 KB per stage, 128-byte swizzle);
//   warp 1            : allocates 256 TMEM columns; one lane issues the
//                       tcgen05.mma (M=128, N=256, K=16, 4 per slice) and
//                       commits each slice back to the producer;
//   warps 2..5        : epilogue, tcgen05.ld of their 32 TMEM lanes (rows),
//                       fp32 stores.
// All mbarrier waits are bounded (tc_common.cuh); on timeout the kernel
// records an error bit in *err, drains its own copies and MMAs, frees TMEM
// and returns.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.h"
#include "tc_common.cuh"

namespace {

using namespace umi_tc;

constexpr int BM = 128, BK = 64;
constexpr int NTHREADS = 192;

// Tile policies: where the K-slices of A and B come from and where the
// 128 x BN fp32 tile goes.
struct GemmArgs {
	float* C;
	int M, N, K, ldc;
	int vec;   // C 16-byte aligned and ldc % 4 == 0
	int* err;  // optional: error bits of bounded waits that gave up
};

// C[M,N] = A[M,K] B[N,K]^T: grid (N/BN, M/BM).
struct GemmPolicy {
	static constexpr int BN = 256, STAGES = 4;
	using Args = GemmArgs;
	struct Tile { int m0, n0; };
	__device__ static Tile tile(const Args&) { return {(int)blockIdx.y * BM, (int)blockIdx.x * BN}; }
	__device__ static int nk(const Args& g) { return (g.K + BK - 1) / BK; }
	__device__ static void load(const CUtensorMap* ta, const CUtensorMap* tb, const Args&, const Tile& t, int ks,
	                            void* a, void* b, uint64_t* bar) {
		tma_load_2d(a, ta, bar, ks * BK, t.m0);
		tma_load_2d(b, tb, bar, ks * BK, t.n0);
	}
	// this thread's row of the tile, columns [c, c+32)
	__device__ static void store(const Args& g, const Tile& t, int rl, int c, const float (&v)[32]) {
		const int row = t.m0 + rl;
		if (row >= g.M) return;
		float* dst = g.C + (size_t)row * g.ldc + t.n0 + c;
		if (g.vec && t.n0 + c + 31 < g.N) {
#pragma unroll
			for (int i = 0; i < 32; i += 4)
				*reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
		} else {
#pragma unroll
			for (int i = 0; i < 32; ++i)
				if (t.n0 + c + i < g.N) dst[i] = v[i];
		}
	}
};

// 2-D convolution, stride 1, zero padding r/2, as an implicit GEMM:
// rows = 128 output pixels of one image row (n, y, x0..x0+127), columns =
// output channels, K = (tap, input-channel slice of 64).  A slice is one TMA
// box of the NHWC input at (c0, x0+dx-pad, y+dy-pad, n): the box's
// out-of-bounds zero fill is the padding.  B slices come from the KRSC
// weights viewed as (k, r*r*c).  Output NCHW fp32.
struct ConvArgs {
	float* out;
	int n, c, h, w, k, r;
	int xtiles;
	int* err;
};
struct ConvPolicy {
	static constexpr int BN = 128, STAGES = 3;
	using Args = ConvArgs;
	struct Tile { int n, y, x0, k0; };
	__device__ static Tile tile(const Args& g) {
		const int b = blockIdx.x;
		const int xt = b % g.xtiles, rest = b / g.xtiles;
		return {rest / g.h, rest % g.h, xt * BM, (int)blockIdx.y * BN};
	}
	__device__ static int nk(const Args& g) { return g.r * g.r * (g.c / BK); }
	__device__ static void load(const CUtensorMap* ta, const CUtensorMap* tb, const Args& g, const Tile& t, int ks,
	                            void* a, void* b, uint64_t* bar) {
		const int cs = g.c / BK;
		const int tap = ks / cs, c0 = (ks - tap * cs) * BK;
		const int dy = tap / g.r, dx = tap - dy * g.r, pad = g.r / 2;
		tma_load_4d(a, ta, bar, c0, t.x0 + dx - pad, t.y + dy - pad, t.n);
		tma_load_2d(b, tb, bar, tap * g.c + c0, t.k0);
	}
	// this thread's pixel (row rl of the tile), output channels [k0+c, +32)
	__device__ static void store(const Args& g, const Tile& t, int rl, int c, const float (&v)[32]) {
		const int x = t.x0 + rl;
		if (x >= g.w) return;
		const size_t plane = (size_t)g.h * g.w;
		float* dst = g.out + ((size_t)t.n * g.k) * plane + (size_t)t.y * g.w + x;
#pragma unroll
		for (int i = 0; i < 32; ++i) {
			const int kk = t.k0 + c + i;
			if (kk < g.k) dst[(size_t)kk * plane] = v[i];
		}
	}
};

// One CTA computes one 128 x BN tile:
//   warp 0, one lane : TMA producer into a STAGES-deep ring (A 16 KB, B BN*128 B);
//   warp 1           : allocates BN TMEM columns; one lane issues tcgen05.mma
//                      (M=128, N=BN, K=16, 4 per slice), commits each slice
//                      back to the producer;
//   warps 2..5       : epilogue, tcgen05.ld of their 32 TMEM lanes, stores.
template <class P>
__global__ void __launch_bounds__(NTHREADS, 1)
	tc_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, const typename P::Args g,
	          const uint32_t idesc) {
	constexpr int BN = P::BN, STAGES = P::STAGES;
	constexpr uint32_t A_TILE = BM * BK * 2, B_TILE = BN * BK * 2, STAGE_BYTES = A_TILE + B_TILE;
	extern __shared__ uint8_t smem_raw[];
	uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
	uint64_t* full = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
	uint64_t* empty = full + STAGES;
	uint64_t* accum = empty + STAGES;
	uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
	volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const typename P::Tile t = P::tile(g);
	const int nk = P::nk(g);

	if (threadIdx.x == 0) {
		for (int s = 0; s < STAGES; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], 1);
		}
		mbar_init(accum, 1);
		*abort_flag = 0;
		fence_mbar_init();
		tma_prefetch(&ta);
		tma_prefetch(&tb);
	}
	if (warp == 1) {
		tmem_alloc(tmem_slot, BN);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;

	if (warp == 0 && lane == 0) {
		// ---- producer
		int armed[STAGES];
		for (int s = 0; s < STAGES; ++s) armed[s] = -1;
		for (int ks = 0; ks < nk; ++ks) {
			const int s = ks % STAGES;
			const uint32_t round = ks / STAGES;
			if (!mbar_wait(&empty[s], (round & 1) ^ 1, abort_flag, g.err, kErrTimeoutEmpty)) break;
			mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
			armed[s] = (int)round;
			P::load(&ta, &tb, g, t, ks, base + s * STAGE_BYTES, base + s * STAGE_BYTES + A_TILE, &full[s]);
		}
		if (*abort_flag) {
			// let every copy this thread started land before the CTA exits
			volatile int own = 0;
			for (int s = 0; s < STAGES; ++s)
				if (armed[s] >= 0) mbar_wait(&full[s], (uint32_t)armed[s] & 1, &own, g.err, kErrTimeoutFull);
		}
	} else if (warp == 1 && lane == 0) {
		// ---- MMA issuer
		for (int ks = 0; ks < nk; ++ks) {
			const int s = ks % STAGES;
			const uint32_t round = ks / STAGES;
			if (!mbar_wait(&full[s], round & 1, abort_flag, g.err, kErrTimeoutFull)) break;
			tc_fence_after();
			const uint64_t ad = desc_kmajor_sw128(smem_u32(base + s * STAGE_BYTES));
			const uint64_t bd = desc_kmajor_sw128(smem_u32(base + s * STAGE_BYTES + A_TILE));
#pragma unroll
			for (int kk = 0; kk < BK / 16; ++kk) mma_f16(tmem, ad + 2 * kk, bd + 2 * kk, idesc, ks > 0 || kk > 0);
			mma_commit(&empty[s]);
		}
		mma_commit(accum);
		// the MMAs issued above finish before TMEM is freed
		volatile int own = 0;
		mbar_wait(accum, 0, &own, g.err, kErrTimeoutAccum);
	} else if (warp >= 2) {
		// ---- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 (rows of the tile)
		const bool ok = mbar_wait(accum, 0, abort_flag, g.err, kErrTimeoutAccum);
		tc_fence_after();
		if (ok && !*abort_flag) {
			const int q = warp & 3;
#pragma unroll 1
			for (int c = 0; c < BN; c += 32) {
				float v[32];
				tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c, v);
				P::store(g, t, 32 * q + lane, c, v);
			}
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 1) {
		tc_fence_after();
		tmem_dealloc(tmem, BN);
	}
}

template <class P>
constexpr size_t smem_bytes() {
	return (size_t)P::STAGES * (BM * BK * 2 + P::BN * BK * 2) + 1024 + 256;
}

// ---- split of fp32 operands into bf16 hi/lo parts, concatenated along K:
// A' = [A_hi | A_lo | A_hi], B' = [B_hi | B_hi | B_lo]  =>  A' B'^T =
// A_hi B_hi^T + A_lo B_hi^T + A_hi B_lo^T  (bf16x3 of Henry, Tang & Heinecke,
// "Leveraging the bfloat16 Artificial Intelligence Datatype For
// Higher-Precision Computations", ARITH 2019; the lo*lo term is dropped).
__global__ void split_bf16x3_kernel(const float* __restrict__ X, __nv_bfloat16* __restrict__ Y, int rows, int K,
                                    int lo_block) {
	const size_t n = (size_t)rows * K;
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const size_t r = i / K, k = i - r * K;
		const float x = X[i];
		const __nv_bfloat16 hi = __float2bfloat16_rn(x);
		const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
		__nv_bfloat16* y = Y + r * (size_t)(3 * K) + k;
		y[0] = hi;
		y[K] = lo_block == 1 ? lo : hi;
		y[2 * K] = lo_block == 2 ? lo : hi;
	}
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
	static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
	static std::once_flag once;
	std::call_once(once, [] {
		cudaDriverEntryPointQueryResult q;
		void* p = nullptr;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
	});
	return fn;
}

umi_status map_kmajor(CUtensorMap* m, const void* ptr, CUtensorMapDataType dt, int rows, int K, int box_rows) {
	auto enc = encode_fn();
	if (!enc) return umi::fail(UMI_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
	const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
	const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
	const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
	const cuuint32_t es[2] = {1, 1};
	const CUresult r = enc(m, dt, 2, const_cast<void*>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
	                       CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
	                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	if (r != CUDA_SUCCESS) return umi::fail(UMI_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
	return UMI_OK;
}

umi_status gemm_launch(const void* A, const void* B, float* C, int M, int N, int K, int ab_type, int* err,
                       cudaStream_t st) {
	if (M < 0 || N < 0 || K < 0) return umi::fail(UMI_ERR_INVALID_ARG, "gemm: negative size");
	if (M == 0 || N == 0) return UMI_OK;
	if (!A || !B || !C) return umi::fail(UMI_ERR_INVALID_ARG, "gemm: null pointer");
	if (K == 0) return umi::cuda_status(cudaMemsetAsync(C, 0, (size_t)M * N * sizeof(float), st), "cudaMemsetAsync");
	if (K % 8 != 0) return umi::fail(UMI_ERR_UNSUPPORTED, "gemm: K = %d must be a multiple of 8 (16-byte rows)", K);
	if (!umi::aligned(A, 16) || !umi::aligned(B, 16))
		return umi::fail(UMI_ERR_INVALID_ARG, "gemm: A and B must be 16-byte aligned");
	const CUtensorMapDataType dt = ab_type ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
	CUtensorMap ta, tb;
	UMI_TRY(map_kmajor(&ta, A, dt, M, K, BM));
	UMI_TRY(map_kmajor(&tb, B, dt, N, K, GemmPolicy::BN));
	GemmArgs g{C, M, N, K, N, umi::aligned(C, 16) && N % 4 == 0, err};
	constexpr size_t SMEM = smem_bytes<GemmPolicy>();
	auto kern = tc_kernel<GemmPolicy>;
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM),
	                         "cudaFuncSetAttribute"));
	const dim3 grid(umi::ceil_div(N, GemmPolicy::BN), umi::ceil_div(M, BM));
	kern<<<grid, NTHREADS, SMEM, st>>>(ta, tb, g, idesc_f16((uint32_t)ab_type, BM, GemmPolicy::BN));
	return umi::launch_status("tc_kernel<gemm>");
}

}  // namespace

extern "C" umi_status umi_gemm_bf16(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t* err,
                                    void* stream) {
	const umi_status s = gemm_launch(A, B, C, M, N, K, 1, err, umi::as_stream(stream));
	return s == UMI_OK ? umi::ok() : s;
}

extern "C" umi_status umi_gemm_f16(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t* err,
                                   void* stream) {
	const umi_status s = gemm_launch(A, B, C, M, N, K, 0, err, umi::as_stream(stream));
	return s == UMI_OK ? umi::ok() : s;
}

extern "C" size_t umi_gemm_f32_bf16x3_workspace_bytes(int32_t M, int32_t N, int32_t K) {
	if (M <= 0 || N <= 0 || K <= 0) return 0;
	const size_t a = ((size_t)M * 3 * K * 2 + 255) & ~size_t(255);
	return a + (size_t)N * 3 * K * 2;
}

extern "C" umi_status umi_gemm_f32_bf16x3(const float* A, const float* B, float* C, int32_t M, int32_t N, int32_t K,
                                          void* workspace, size_t workspace_bytes, int32_t* err, void* stream) {
	if (M < 0 || N < 0 || K < 0) return umi::fail(UMI_ERR_INVALID_ARG, "gemm_bf16x3: negative size");
	if (M == 0 || N == 0 || K == 0) return gemm_launch(A, B, C, M, N, 0, 1, err, umi::as_stream(stream));
	if (!A || !B || !C || !workspace) return umi::fail(UMI_ERR_INVALID_ARG, "gemm_bf16x3: null pointer");
	if (workspace_bytes < umi_gemm_f32_bf16x3_workspace_bytes(M, N, K))
		return umi::fail(UMI_ERR_NO_MEMORY, "gemm_bf16x3: workspace too small");
	if (!umi::aligned(workspace, 256)) return umi::fail(UMI_ERR_INVALID_ARG, "gemm_bf16x3: workspace not 256-byte aligned");
	const cudaStream_t st = umi::as_stream(stream);
	__nv_bfloat16* As = static_cast<__nv_bfloat16*>(workspace);
	__nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(workspace) +
	                                                     (((size_t)M * 3 * K * 2 + 255) & ~size_t(255)));
	split_bf16x3_kernel<<<1024, 256, 0, st>>>(A, As, M, K, 1);
	UMI_TRY(umi::launch_status("split_bf16x3_kernel"));
	split_bf16x3_kernel<<<1024, 256, 0, st>>>(B, Bs, N, K, 2);
	UMI_TRY(umi::launch_status("split_bf16x3_kernel"));
	const umi_status s = gemm_launch(As, Bs, C, M, N, 3 * K, 1, err, st);
	return s == UMI_OK ? umi::ok() : s;
}

namespace {

umi_status conv_launch(const void* x, const void* wt, float* out, int n, int c, int h, int w, int k, int r, int* err,
                       cudaStream_t st) {
	if (n < 0 || c < 0 || h < 0 || w < 0 || k < 0) return umi::fail(UMI_ERR_INVALID_ARG, "conv: negative size");
	if (n == 0 || h == 0 || w == 0 || k == 0) return UMI_OK;
	if (!x || !wt || !out) return umi::fail(UMI_ERR_INVALID_ARG, "conv: null pointer");
	if (r != 1 && r != 3 && r != 5 && r != 7) return umi::fail(UMI_ERR_UNSUPPORTED, "conv: filter %dx%d (1, 3, 5, 7)", r, r);
	if (c % BK != 0) return umi::fail(UMI_ERR_UNSUPPORTED, "conv: %d input channels (a multiple of %d)", c, BK);
	if (!umi::aligned(x, 16) || !umi::aligned(wt, 16)) return umi::fail(UMI_ERR_INVALID_ARG, "conv: misaligned input");
	auto enc = encode_fn();
	if (!enc) return umi::fail(UMI_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
	CUtensorMap ta, tb;
	{
		const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
		const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)w * c * 2, (cuuint64_t)h * w * c * 2};
		const cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)BM, 1, 1};
		const cuuint32_t es[4] = {1, 1, 1, 1};
		const CUresult rr = enc(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, es,
		                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
		                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (rr != CUDA_SUCCESS) return umi::fail(UMI_ERR_CUDA, "conv: input tensor map (%d)", (int)rr);
	}
	UMI_TRY(map_kmajor(&tb, wt, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, k, r * r * c, ConvPolicy::BN));
	ConvArgs g{out, n, c, h, w, k, r, umi::ceil_div(w, BM), err};
	constexpr size_t SMEM = smem_bytes<ConvPolicy>();
	auto kern = tc_kernel<ConvPolicy>;
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM),
	                         "cudaFuncSetAttribute"));
	const int64_t tiles = (int64_t)n * h * g.xtiles;
	if (tiles > INT32_MAX) return umi::fail(UMI_ERR_UNSUPPORTED, "conv: too many tiles");
	const dim3 grid((unsigned)tiles, umi::ceil_div(k, ConvPolicy::BN));
	kern<<<grid, NTHREADS, SMEM, st>>>(ta, tb, g, idesc_f16(1u, BM, ConvPolicy::BN));
	return umi::launch_status("tc_kernel<conv>");
}

}  // namespace

extern "C" umi_status umi_conv2d_fprop_bf16(const void* x_nhwc, const void* w_krsc, float* out_nchw, int32_t n, int32_t c,
                                            int32_t h, int32_t w, int32_t k, int32_t r, int32_t* err, void* stream) {
	const umi_status s = conv_launch(x_nhwc, w_krsc, out_nchw, n, c, h, w, k, r, err, umi::as_stream(stream));
	return s == UMI_OK ? umi::ok() : s;
}
