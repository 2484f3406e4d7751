// Tensor-core GEMM on sm_103a (tcgen05 + TMA), C[M,N] (fp32) = A[M,K] * B[N,K]^T
// with bf16 or f16 operands and fp32 accumulation in tensor memory.
//
// Replaces the Execute call of main/gemm.cu:37-67 (Gemm strategy,
// main/gemm.cu:8-15: accum += A * B through shared memory, scalar) for the
// half-precision operand types, plus a split-precision FP32 emulation.
//
// Persistent CTAs compute 128 x 256 tiles of C:
//   warp 0, one lane  : TMA producer, K-slices of 64 into a 4-stage ring
//                       (A 16 KB + B 32 KB per stage, 128-byte swizzle);
//   warp 1            : allocates 512 TMEM columns (two accumulators); one
//                       lane issues the tcgen05.mma (M=128, N=256, K=16, 4 per
//                       slice) and commits each slice back to the producer;
//   warps 2..5        : epilogue, tcgen05.ld of their 32 TMEM lanes (rows),
//                       fp32 stores, overlapping the next tile's MMAs.
// All mbarrier waits are bounded (tc_common.cuh); on timeout the kernel
// records an error bit in *err, drains its own copies and MMAs, frees TMEM
// and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "common.h"
#include "tc_common.cuh"
#include "menet_roll.h"

namespace {

using namespace umi_tc;

constexpr int BM = 128, BK = 64;
constexpr int NTHREADS = 192;

// Tile policies: where the K-slices of A and B come from and where the
// 128 x BN fp32 tile goes.
struct GemmArgs {
	float* C;
	int M, N, K, ldc;
	int vec;   // C 16-byte aligned and ldc % 4 == 0: stores through the C tensor map
	int* err;  // optional: error bits of bounded waits that gave up
	unsigned long long acc_wait_ns;  // limit of the epilogue's wait for a finished accumulator (kWaitNs)
};

// C[M,N] = A[M,K] B[N,K]^T: grid (N/BN, M/BM).  BN = 256, or 224 where it
// fills the last round of persistent tiles better (gemm_launch chooses).
template <int BN_>
struct GemmPolicyT {
	static constexpr int BN = BN_, STAGES = 4;
	static constexpr bool RESIDENT_B = false;
	static constexpr int NK_RES = 0;
	static constexpr bool EPI_TMA = true;  // epilogue through shared memory + TMA tile stores
	__device__ static unsigned long long acc_wait_ns(const GemmArgs& g) { return g.acc_wait_ns; }
	using Args = GemmArgs;
	struct Tile { int m0, n0; };
	// tiles in row-major order of (m-block, n-block): CTAs working at the same
	// time share A row-blocks in L2
	__host__ __device__ static int ntiles(const Args& g) { return ((g.M + BM - 1) / BM) * ((g.N + BN - 1) / BN); }
	__device__ static Tile tile(const Args& g, int id) {
		const int nt = (g.N + BN - 1) / BN;
		return {(id / nt) * BM, (id % nt) * BN};
	}
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
using GemmPolicy = GemmPolicyT<256>;
using GemmPolicy224 = GemmPolicyT<224>;

// TMEM columns of two accumulators of BN columns: the allocation unit is a
// power of two of at least 32 columns.
__host__ __device__ constexpr uint32_t tmem_cols_for(int bn) {
	uint32_t c = 32;
	while (c < 2u * (uint32_t)bn) c <<= 1;
	return c;
}

// 2-D convolution, stride 1, zero padding r/2, as an implicit GEMM:
// rows = 128 output pixels of one image row (n, y, x0..x0+127), columns =
// output channels, K = (tap, input-channel slice of 64).  A slice is one TMA
// box of the NHWC input at (c0, x0+dx-pad, y+dy-pad, n): the box's
// out-of-bounds zero fill is the padding.  B slices come from the KRSC
// weights viewed as (k, r*r*c).  Output NCHW fp32.
struct ConvArgs {
	float* out;
	int n, c, h, w, k, r;
	int xtiles, ktiles;
	int vec4;  // out 16-byte aligned and w % 4 == 0: float4 stores along x
	int* err;
};
struct ConvPolicy {
	static constexpr int BN = 128, STAGES = 3;
	static constexpr bool RESIDENT_B = false;
	static constexpr int NK_RES = 0;
	static constexpr bool EPI_TMA = false;
	template <class A> __device__ static unsigned long long acc_wait_ns(const A&) { return kWaitNs; }
	using Args = ConvArgs;
	struct Tile { int n, y, x0, k0; };
	// tile id = ((n*h + y)*xtiles + xt)*ktiles + kt
	__host__ __device__ static int ntiles(const Args& g) { return g.n * g.h * g.xtiles * g.ktiles; }
	__device__ static Tile tile(const Args& g, int id) {
		const int kt = id % g.ktiles, b = id / g.ktiles;
		const int xt = b % g.xtiles, rest = b / g.xtiles;
		return {rest / g.h, rest % g.h, xt * BM, kt * BN};
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
	// resident-weight form: the A slice alone, and B slice ks of output-channel block 0
	__device__ static void load_a(const CUtensorMap* ta, const Args& g, const Tile& t, int ks, void* a, uint64_t* bar) {
		const int cs = g.c / BK;
		const int tap = ks / cs, c0 = (ks - tap * cs) * BK;
		const int dy = tap / g.r, dx = tap - dy * g.r, pad = g.r / 2;
		tma_load_4d(a, ta, bar, c0, t.x0 + dx - pad, t.y + dy - pad, t.n);
	}
	__device__ static void load_b(const CUtensorMap* tb, const Args& g, int ks, void* b, uint64_t* bar) {
		const int cs = g.c / BK;
		const int tap = ks / cs, c0 = (ks - tap * cs) * BK;
		tma_load_2d(b, tb, bar, tap * g.c + c0, 0);
	}
	// This thread holds pixel x0 + rl of the tile for output channels
	// [k0+c, +32).  Groups of 4 channels are transposed across the 4 lanes of
	// each quad (two butterfly shuffle stages), after which lane 4j+m holds
	// channel 4*grp+m of pixels 4j..4j+3: one 16-byte store per lane and
	// group instead of four 4-byte stores.  Every lane takes part in the
	// shuffles; bounds are checked at the stores.
	__device__ static void store(const Args& g, const Tile& t, int rl, int c, const float (&v)[32]) {
		const int lane = rl & 31, m = lane & 3;
		const bool b1 = (m >> 1) & 1, b0 = m & 1;
		const int xq = t.x0 + (rl - m);  // first pixel of this lane's quad
		const size_t plane = (size_t)g.h * g.w;
		float* base = g.out + ((size_t)t.n * g.k) * plane + (size_t)t.y * g.w + xq;
		const bool vec = g.vec4 && xq + 3 < g.w;
#pragma unroll
		for (int grp = 0; grp < 8; ++grp) {
			// r[k] = channel 4grp+k of this lane's pixel
			float r0 = v[4 * grp], r1 = v[4 * grp + 1], r2 = v[4 * grp + 2], r3 = v[4 * grp + 3];
			// stage 1 (lanes m, m^2): keep the channel pair whose high bit is b1, swap the other
			{
				const float s0 = b1 ? r0 : r2, s1 = b1 ? r1 : r3;
				const float y0 = __shfl_xor_sync(0xffffffffu, s0, 2), y1 = __shfl_xor_sync(0xffffffffu, s1, 2);
				// now (row p1, col c0): own row for p1 == b1, partner's row otherwise; channels (b1, c0)
				const float k0 = b1 ? r2 : r0, k1 = b1 ? r3 : r1;  // own values of channels (b1, 0), (b1, 1)
				r0 = b1 ? y0 : k0;  // pixel (0, b0), channel (b1, 0)
				r1 = b1 ? y1 : k1;  // pixel (0, b0), channel (b1, 1)
				r2 = b1 ? k0 : y0;  // pixel (1, b0), channel (b1, 0)
				r3 = b1 ? k1 : y1;  // pixel (1, b0), channel (b1, 1)
			}
			// stage 2 (lanes m, m^1): keep channel low bit b0, swap the other
			{
				const float s0 = b0 ? r0 : r1, s1 = b0 ? r2 : r3;
				const float y0 = __shfl_xor_sync(0xffffffffu, s0, 1), y1 = __shfl_xor_sync(0xffffffffu, s1, 1);
				const float k0 = b0 ? r1 : r0, k1 = b0 ? r3 : r2;  // own: pixels (0, b0), (1, b0), channel (b1, b0)
				// pixel (p1, p0) of channel (b1, b0): own when p0 == b0
				const float q00 = b0 ? y0 : k0, q01 = b0 ? k0 : y0;  // p1 = 0: p0 = 0, 1
				const float q10 = b0 ? y1 : k1, q11 = b0 ? k1 : y1;  // p1 = 1: p0 = 0, 1
				r0 = q00; r1 = q01; r2 = q10; r3 = q11;             // pixels 0, 1, 2, 3 of the quad
			}
			const int kk = t.k0 + c + 4 * grp + m;
			if (kk < g.k) {
				float* dst = base + (size_t)kk * plane;
				if (vec) {
					*reinterpret_cast<float4*>(dst) = make_float4(r0, r1, r2, r3);
				} else {
					if (xq < g.w) dst[0] = r0;
					if (xq + 1 < g.w) dst[1] = r1;
					if (xq + 2 < g.w) dst[2] = r2;
					if (xq + 3 < g.w) dst[3] = r3;
				}
			}
		}
	}
};

// The same convolution with every weight slice resident in shared memory for
// the CTA's lifetime (output channels <= BN and at most NK_RES slices: 3x3 x
// 64 channels is 9 slices, 144 KB): only input slices stream through the ring,
// halving the operand traffic from L2.
struct ConvResPolicy : ConvPolicy {
	static constexpr int STAGES = 4;
	static constexpr bool RESIDENT_B = true;
	static constexpr int NK_RES = 9;
};

// 3x3 convolution over 64 input channels with resident weights and one A
// load per filter row (strip_run_kernel with ConvRun, below): the strip of
// BM + 2 input pixels of row y + dy - 1 (one TMA box, zero fill outside the
// image) serves the three horizontal taps, whose operands start 0, 1 and 2
// rows into the strip.
struct ConvStripPolicy : ConvResPolicy {
	static constexpr int R = 3;
	static constexpr int STRIP_ROWS = BM + R - 1;                          // 130
	static constexpr uint32_t STRIP_BYTES = STRIP_ROWS * BK * 2;          // 16 640 (the box)
	static constexpr uint32_t STRIP_STAGE = (STRIP_BYTES + 1023) & ~1023u;  // 17 408
};

// Arguments of one motion-proposal layer (MenetRun, below).
struct MenetArgs {
	__nv_bfloat16* out;  // (h, w, 32) bf16
	const float* bias;   // 32
	int h, w, dil, xtiles;
	int* err;
};

// Persistent CTAs, each looping over tiles id = blockIdx.x, +gridDim.x, ...:
//   warp 0, one lane : TMA producer into a STAGES-deep ring (A 16 KB, B BN*128 B),
//                      running ahead across tile boundaries;
//   warp 1           : allocates 2*BN TMEM columns (two accumulators); one lane
//                      issues tcgen05.mma (M=128, N=BN, K=16, 4 per slice) into
//                      accumulator (tile & 1), commits each slice back to the
//                      producer and each finished tile to the epilogue;
//   warps 2..5       : epilogue, tcgen05.ld of their 32 TMEM lanes, stores,
//                      then release the accumulator to the MMA warp.
// The epilogue of tile i runs while the MMAs of tile i+1 fill the other
// accumulator.  Every wait is bounded (tc_common.cuh); on a timeout every
// role stops, the producer drains its copies, the MMA lane waits for its
// issued MMAs, and TMEM is freed.
template <class P>
__global__ void __launch_bounds__(NTHREADS, 1)
	tc_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
	          const __grid_constant__ CUtensorMap tcm, const typename P::Args g, const uint32_t idesc) {
	constexpr int BN = P::BN, STAGES = P::STAGES;
	constexpr bool RES = P::RESIDENT_B;
	constexpr uint32_t A_TILE = BM * BK * 2, B_TILE = BN * BK * 2;
	constexpr uint32_t STAGE_BYTES = RES ? A_TILE : A_TILE + B_TILE;  // bytes one ring load brings
	extern __shared__ uint8_t smem_raw[];
	// 1024-byte aligned start (128-byte swizzled TMA tiles), formed by indexing
	// the shared array so that the compiler keeps shared-memory accesses
	uint8_t* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
	uint8_t* bres = base + STAGES * STAGE_BYTES;  // resident B slices (RES only)
	uint8_t* ebuf = bres + (RES ? P::NK_RES * B_TILE : 0);  // epilogue staging, 2 x 4 KB per epilogue warp (EPI_TMA)
	uint64_t* full = reinterpret_cast<uint64_t*>(ebuf + (P::EPI_TMA ? 8 * 4096 : 0));
	uint64_t* empty = full + STAGES;
	uint64_t* accfull = empty + STAGES;  // [2]
	uint64_t* accempty = accfull + 2;    // [2]
	uint64_t* drain = accempty + 2;
	uint64_t* bready = drain + 1;        // resident B loaded (RES only)
	uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bready + 1);
	volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int ntiles = P::ntiles(g);
	const int nk = P::nk(g);  // K-slices of A and B: ring loads per tile

	if (threadIdx.x == 0) {
		for (int s = 0; s < STAGES; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], 1);
		}
		for (int a = 0; a < 2; ++a) {
			mbar_init(&accfull[a], 1);
			mbar_init(&accempty[a], 4);  // one arrive per epilogue warp
		}
		mbar_init(drain, 1);
		mbar_init(bready, 1);
		*abort_flag = 0;
		fence_mbar_init();
		tma_prefetch(&ta);
		tma_prefetch(&tb);
	}
	if (warp == 1) {
		tmem_alloc(tmem_slot, tmem_cols_for(BN));
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
		if constexpr (RES) {
			mbar_arrive_expect_tx(bready, (uint32_t)nk * B_TILE);
			for (int ks = 0; ks < nk; ++ks) P::load_b(&tb, g, ks, bres + ks * B_TILE, bready);
		}
		uint32_t q = 0;  // slices issued by this CTA
		for (int id = blockIdx.x; id < ntiles && !*abort_flag; id += gridDim.x) {
			const typename P::Tile t = P::tile(g, id);
			for (int ks = 0; ks < nk; ++ks, ++q) {
				const int s = (int)(q % STAGES);
				const uint32_t round = q / STAGES;
				if (!mbar_wait(&empty[s], (round & 1) ^ 1, abort_flag, g.err, kErrTimeoutEmpty)) break;
				mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
				armed[s] = (int)round;
				if constexpr (RES)
					P::load_a(&ta, g, t, ks, base + s * STAGE_BYTES, &full[s]);
				else
					P::load(&ta, &tb, g, t, ks, base + s * STAGE_BYTES, base + s * STAGE_BYTES + A_TILE, &full[s]);
			}
		}
		if (*abort_flag) {
			// let every copy this thread started land before the CTA exits
			volatile int own = 0;
			for (int s = 0; s < STAGES; ++s)
				if (armed[s] >= 0) mbar_wait(&full[s], (uint32_t)armed[s] & 1, &own, g.err, kErrTimeoutFull);
			if constexpr (RES) mbar_wait(bready, 0, &own, g.err, kErrTimeoutFull);
		}
	} else if (warp == 1 && lane == 0) {
		// ---- MMA issuer
		bool ready = true;
		if constexpr (RES) ready = mbar_wait(bready, 0, abort_flag, g.err, kErrTimeoutFull);
		uint32_t q = 0;
		int i = 0;  // local tile count
		for (int id = blockIdx.x; ready && id < ntiles && !*abort_flag; id += gridDim.x, ++i) {
			const int a = i & 1;
			const uint32_t use = (uint32_t)(i >> 1);
			if (!mbar_wait(&accempty[a], (use & 1) ^ 1, abort_flag, g.err, kErrTimeoutAccEmpty)) break;
			tc_fence_after();
			const uint32_t acc = tmem + (uint32_t)(a * BN);
			bool ok = true;
			for (int ks = 0; ks < nk; ++ks, ++q) {
				const int s = (int)(q % STAGES);
				const uint32_t round = q / STAGES;
				if (!mbar_wait(&full[s], round & 1, abort_flag, g.err, kErrTimeoutFull)) { ok = false; break; }
				tc_fence_after();
				const uint64_t ad = desc_kmajor_sw128(smem_u32(base + s * STAGE_BYTES));
				const uint64_t bd =
					desc_kmajor_sw128(smem_u32(RES ? bres + ks * B_TILE : base + s * STAGE_BYTES + A_TILE));
#pragma unroll
				for (int kk = 0; kk < BK / 16; ++kk) mma_f16(acc, ad + 2 * kk, bd + 2 * kk, idesc, ks > 0 || kk > 0);
				mma_commit(&empty[s]);
			}
			if (!ok) break;
			mma_commit(&accfull[a]);
		}
		// every MMA issued above finishes before TMEM is freed
		mma_commit(drain);
		volatile int own = 0;
		mbar_wait(drain, 0, &own, g.err, kErrTimeoutAccum);
	} else if (warp >= 2) {
		// ---- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 (rows of the tile)
		const int qd = warp & 3;
		int i = 0;
		uint32_t nst = 0;  // TMA stores issued by this warp
		for (int id = blockIdx.x; id < ntiles; id += gridDim.x, ++i) {
			const int a = i & 1;
			const uint32_t use = (uint32_t)(i >> 1);
			if (!mbar_wait(&accfull[a], use & 1, abort_flag, g.err, kErrTimeoutAccum, P::acc_wait_ns(g))) break;
			tc_fence_after();
			const typename P::Tile t = P::tile(g, id);
#pragma unroll 1
			for (int c = 0; c < BN; c += 32) {
				float v[32];
				tmem_ld32(tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(a * BN + c), v);
				if constexpr (P::EPI_TMA) {
					if (g.vec) {
						// 32 rows x 32 columns through a 4 KB buffer with the 128-byte
						// swizzle of the C tensor map (chunk j of row r at j ^ (r & 7):
						// conflict-free), then one TMA store; out-of-range rows and
						// columns are clipped by the TMA.
						const int row0 = t.m0 + 32 * qd, col0 = t.n0 + c;
						if (row0 < g.M && col0 < g.N) {
							uint8_t* sb = ebuf + (qd * 2 + (nst & 1)) * 4096;
							if (lane == 0) bulk_wait_read_1();  // the store that last used sb has read it
							__syncwarp();
#pragma unroll
							for (int j = 0; j < 8; ++j)
								*reinterpret_cast<float4*>(sb + lane * 128 + ((j ^ (lane & 7)) << 4)) =
									make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
							fence_proxy_async_smem();
							__syncwarp();
							if (lane == 0) {
								tma_store_2d(&tcm, sb, col0, row0);
								bulk_commit();
							}
							++nst;
						}
						continue;
					}
				}
				P::store(g, t, 32 * qd + lane, c, v);
			}
			tc_fence_before();
			__syncwarp();
			if (lane == 0) mbar_arrive(&accempty[a]);
		}
		if constexpr (P::EPI_TMA) {
			if (lane == 0) bulk_wait_all();  // stores done before the CTA exits
			__syncwarp();
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 1) {
		tc_fence_after();
		tmem_dealloc(tmem, tmem_cols_for(BN));
	}
}

template <class P>
constexpr size_t smem_bytes() {
	const size_t stage = (size_t)(BM * BK * 2);
	const size_t epi = P::EPI_TMA ? 8 * 4096 : 0;
	return P::RESIDENT_B
	           ? (size_t)P::STAGES * stage + (size_t)P::NK_RES * (P::BN * BK * 2) + epi + 1024 + 256
	           : (size_t)P::STAGES * (BM * BK * 2 + P::BN * BK * 2) + epi + 1024 + 256;
}

// 3x3 convolution in the strip form (64 input channels, at most 128 outputs,
// resident weights, one TMA box per filter row) walking output rows in runs;
// T supplies the geometry (ConvRun).  The tiles of a block of columns (image
// and x tile) are ordered by row class (y mod d, one class for d = 1) and
// then by y, id = block * h + pos, and CTA c takes the contiguous run
// [c * per, (c + 1) * per); a run splits into segments of consecutive
// positions of one block and one class, whose output rows step by d.  Output
// row y reads the strips of input rows y - d, y, y + d, so consecutive rows of
// a segment share two of their three: the producer loads each strip of a
// segment once (rows y_a - d .. y_b + d) and the MMA warp frees a strip's
// ring slot after the last row that reads it (a row's MMAs complete in issue
// order, so committing after row y frees the strip of row y - d, and after a
// segment's last row the two strips below it).  One strip load per row
// instead of three.  The epilogue, whose NCHW stores (256 MiB at the
// benchmark shape) bound the kernel, runs on T::EPI_WARPS warps,
// T::EPI_WARPS / 4 per TMEM lane quadrant, each storing an equal share of the
// output channels.  Waits, abort and drain as in tc_kernel.
struct ConvRun {
	using Args = ConvArgs;
	static constexpr int BN = ConvStripPolicy::BN, STAGES = ConvStripPolicy::STAGES, NK_RES = 9, EPI_WARPS = 8;
	static constexpr int KT = BK;          // K per tap: 64 channels, 128-byte rows
	static constexpr int ROW_BYTES = 128;  // one strip row (pixel) in shared memory
	static constexpr uint32_t STRIP_STAGE = ConvStripPolicy::STRIP_STAGE;
	__device__ static uint64_t desc_a(uint32_t strip, int row) { return desc_kmajor_sw128_rows(strip, row); }
	__device__ static uint64_t desc_b(uint32_t slice) { return desc_kmajor_sw128(slice); }
	__device__ static uint32_t strip_bytes(const Args&) { return ConvStripPolicy::STRIP_BYTES; }
	__device__ static int dil(const Args&) { return 1; }
	__host__ __device__ static int rows(const Args& g) { return g.h; }
	__host__ __device__ static int blocks(const Args& g) { return g.n * g.xtiles; }
	// output row of position pos, and the end of its row class (one class)
	__device__ static void row_of(const Args& g, int pos, int& y, int& class_end) {
		y = pos;
		class_end = g.h;
	}
	__device__ static void load_strip(const CUtensorMap* ta, const Args& g, int blk, int row, void* dst, uint64_t* bar) {
		const int n = blk / g.xtiles, x0 = (blk - n * g.xtiles) * BM;
		tma_load_4d(dst, ta, bar, 0, x0 - 1, row, n);
	}
	__device__ static void load_b(const CUtensorMap* tb, const Args& g, int ks, void* b, uint64_t* bar) {
		ConvStripPolicy::load_b(tb, g, ks, b, bar);
	}
	__device__ static void store(const Args& g, int blk, int y, int rl, int c, const float (&v)[32]) {
		ConvPolicy::Tile t;
		t.n = blk / g.xtiles;
		t.y = y;
		t.x0 = (blk - t.n * g.xtiles) * BM;
		t.k0 = 0;
		ConvPolicy::store(g, t, rl, c, v);
	}
	struct Epi {
		__device__ explicit Epi(const Args&) {}
		__device__ void store(const Args& g, int blk, int y, int rl, int c, const float (&v)[32]) const {
			ConvRun::store(g, blk, y, rl, c, v);
		}
	};
};
// One 3x3 layer of the motion-proposal network (32 -> 32 channels, dilation
// d <= 8) in the same run order (menet_rows_kernel below).  Activations are
// bf16 NHWC with 32-channel pixels (64 bytes, TMA boxes with the 64-byte
// swizzle), so a tap is one K = 32 slice.  The strip of input row y' holds
// its 128 + 2d pixels around the block; taps dx = 0, 1, 2 start 0, d, 2d rows
// into it.  Epilogue: + bias, ReLU, bf16, one 64-byte pixel per thread.
struct MenetRun {
	using Args = MenetArgs;
	static constexpr int STAGES = 16, NK_RES = 9, MAXD = 8;
	static constexpr int KT = 32;         // K per tap: 32 channels, 64-byte rows
	static constexpr int ROW_BYTES = 64;  // one strip row (pixel) in shared memory
	static constexpr uint32_t STRIP_STAGE = ((BM + 2 * MAXD) * KT * 2 + 1023) & ~1023u;  // 9 216
	__device__ static uint64_t desc_a(uint32_t strip, int row) { return desc_kmajor_sw64(strip + 64u * (uint32_t)row); }
	__device__ static uint64_t desc_b(uint32_t slice) { return desc_kmajor_sw64(slice); }
	__device__ static uint32_t strip_bytes(const Args& g) { return (uint32_t)(BM + 2 * g.dil) * KT * 2; }
	// classes c = y mod d in order, y ascending within a class: classes
	// 0 .. rm-1 hold q+1 rows, the others q (q = h / d, rm = h mod d)
	__device__ static void row_of(const Args& g, int pos, int& y, int& class_end) {
		const int d = g.dil, q = g.h / d, rm = g.h - q * d, big = rm * (q + 1);
		if (pos < big) {
			const int c = pos / (q + 1), k = pos - c * (q + 1);
			y = c + k * d;
			class_end = (c + 1) * (q + 1);
		} else {
			const int p2 = pos - big, c = p2 / q, k = p2 - c * q;
			y = rm + c + k * d;
			class_end = big + (c + 1) * q;
		}
	}
	__device__ static void load_strip(const CUtensorMap* ta, const Args& g, int blk, int row, void* dst, uint64_t* bar) {
		tma_load_4d(dst, ta, bar, 0, blk * BM - g.dil, row, 0);
	}
	__device__ static void load_b(const CUtensorMap* tb, const Args&, int ks, void* b, uint64_t* bar) {
		tma_load_2d(b, tb, bar, ks * KT, 0);
	}
	// epilogue: the layer's 32 biases held in registers, + bias, ReLU, bf16,
	// one 64-byte pixel per thread
	struct Epi {
		float bias[32];
		__device__ explicit Epi(const Args& g) {
#pragma unroll
			for (int i = 0; i < 32; ++i) bias[i] = g.bias[i];
		}
		__device__ void store(const Args& g, int blk, int y, int rl, int c, const float (&v)[32]) const {
			const int x = blk * BM + rl;
			if (c != 0 || x >= g.w) return;
			uint32_t q[16];
#pragma unroll
			for (int i = 0; i < 16; ++i) {
				const float a0 = fmaxf(v[2 * i] + bias[2 * i], 0.0f), a1 = fmaxf(v[2 * i + 1] + bias[2 * i + 1], 0.0f);
				const __nv_bfloat162 b2 = __floats2bfloat162_rn(a0, a1);
				q[i] = *reinterpret_cast<const uint32_t*>(&b2);
			}
			uint4* dst = reinterpret_cast<uint4*>(g.out + ((size_t)y * g.w + x) * 32);
#pragma unroll
			for (int i = 0; i < 4; ++i) dst[i] = make_uint4(q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]);
		}
	};
};

template <class T>
constexpr int run_threads() { return 64 + 32 * T::EPI_WARPS; }
template <class T>
constexpr size_t run_smem_bytes() {
	return (size_t)T::STAGES * T::STRIP_STAGE + (size_t)T::NK_RES * (T::BN * T::KT * 2) + 1024 + 256;
}

template <class T>
__global__ void __launch_bounds__(run_threads<T>(), 1)
	strip_run_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
	                 const typename T::Args g, const uint32_t idesc, const int per) {
	constexpr int BN = T::BN, STAGES = T::STAGES, NKR = T::NK_RES;
	constexpr uint32_t B_TILE = BN * T::KT * 2, SS = T::STRIP_STAGE;
	static_assert(STAGES >= 3, "an output row reads three strips at once");
	static_assert(SS % 1024 == 0 && B_TILE % 512 == 0, "operand tiles start on a swizzle atom");
	constexpr uint32_t TCOLS = tmem_cols_for(BN);
	extern __shared__ uint8_t smem_raw[];
	uint8_t* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
	uint8_t* bres = base + STAGES * SS;
	uint64_t* full = reinterpret_cast<uint64_t*>(bres + NKR * B_TILE);
	uint64_t* empty = full + STAGES;
	uint64_t* accfull = empty + STAGES;  // [2]
	uint64_t* accempty = accfull + 2;    // [2]
	uint64_t* drain = accempty + 2;
	uint64_t* bready = drain + 1;
	uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bready + 1);
	volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int H = T::rows(g), ntiles = T::blocks(g) * H, d = T::dil(g);
	const int t0 = blockIdx.x * per, t1 = min(ntiles, t0 + per);
	// the segment of the run starting at tile s0: block, first output row, end
	auto segment = [&](int s0, int& blk, int& y0, int& s1) {
		blk = s0 / H;
		int pend;
		T::row_of(g, s0 - blk * H, y0, pend);
		s1 = min(t1, blk * H + pend);
	};

	if (threadIdx.x == 0) {
		for (int s = 0; s < STAGES; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], 1);
		}
		for (int a = 0; a < 2; ++a) {
			mbar_init(&accfull[a], 1);
			mbar_init(&accempty[a], T::EPI_WARPS);
		}
		mbar_init(drain, 1);
		mbar_init(bready, 1);
		*abort_flag = 0;
		fence_mbar_init();
		tma_prefetch(&ta);
		tma_prefetch(&tb);
	}
	if (warp == 1) {
		tmem_alloc(tmem_slot, TCOLS);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;

	if (warp == 0 && lane == 0) {
		// ---- producer: weights once, then every strip of every segment once
		int armed[STAGES];
		for (int s = 0; s < STAGES; ++s) armed[s] = -1;
		mbar_arrive_expect_tx(bready, (uint32_t)NKR * B_TILE);
		for (int ks = 0; ks < NKR; ++ks) T::load_b(&tb, g, ks, bres + ks * B_TILE, bready);
		const uint32_t sbytes = T::strip_bytes(g);
		uint32_t q = 0;
		bool go = true;
		for (int s0 = t0; go && s0 < t1 && !*abort_flag;) {
			int blk, y0, s1;
			segment(s0, blk, y0, s1);
			for (int i = 0; i < s1 - s0 + 2; ++i, ++q) {  // input row y0 + (i - 1) d
				const int s = (int)(q % STAGES);
				const uint32_t round = q / STAGES;
				if (!mbar_wait(&empty[s], (round & 1) ^ 1, abort_flag, g.err, kErrTimeoutEmpty)) { go = false; break; }
				mbar_arrive_expect_tx(&full[s], sbytes);
				armed[s] = (int)round;
				T::load_strip(&ta, g, blk, y0 + (i - 1) * d, base + s * SS, &full[s]);
			}
			s0 = s1;
		}
		if (*abort_flag) {
			volatile int own = 0;
			for (int s = 0; s < STAGES; ++s)
				if (armed[s] >= 0) mbar_wait(&full[s], (uint32_t)armed[s] & 1, &own, g.err, kErrTimeoutFull);
			mbar_wait(bready, 0, &own, g.err, kErrTimeoutFull);
		}
	} else if (warp == 1 && lane == 0) {
		// ---- MMA issuer
		bool ok = mbar_wait(bready, 0, abort_flag, g.err, kErrTimeoutFull);
		// Descriptors of strip slot 0, row 0 and of weight slice 0; every
		// operand below is one of them plus a byte offset / 16 in the start
		// address field (bits 0-13: shared addresses stay below 2^18, so the
		// sum never carries out of the field).
		const uint64_t a_base = T::desc_a(smem_u32(base), 0), b_base = T::desc_b(smem_u32(bres));
		const uint32_t a_row = (uint32_t)(d * T::ROW_BYTES) >> 4;
		uint32_t q0 = 0;      // first strip of the segment
		uint32_t waited = 0;  // strips 0 .. waited - 1 have landed
		int i = 0;            // tiles so far (accumulator a = i & 1)
		for (int s0 = t0; ok && s0 < t1 && !*abort_flag;) {
			int blk, y0, s1;
			segment(s0, blk, y0, s1);
			const int rows = s1 - s0;
			for (int k = 0; ok && k < rows; ++k, ++i) {  // output row y0 + k d: strips q0 + k .. q0 + k + 2
				const int a = i & 1;
				const uint32_t use = (uint32_t)(i >> 1);
				if (!mbar_wait(&accempty[a], (use & 1) ^ 1, abort_flag, g.err, kErrTimeoutAccEmpty)) { ok = false; break; }
				tc_fence_after();
				const uint32_t acc = tmem + (uint32_t)(a * BN);
#pragma unroll 1
				for (int dy = 0; dy < 3; ++dy) {
					const uint32_t q = q0 + (uint32_t)(k + dy);
					const int s = (int)(q % STAGES);
					if (q >= waited) {  // the row before waited for the first two strips of this one
						if (!mbar_wait(&full[s], (q / STAGES) & 1, abort_flag, g.err, kErrTimeoutFull)) { ok = false; break; }
						tc_fence_after();
						waited = q + 1;
					}
					const uint64_t as = a_base + ((uint32_t)s * (SS >> 4));
					const uint64_t bs = b_base + (uint32_t)dy * (3 * B_TILE >> 4);
#pragma unroll
					for (int dx = 0; dx < 3; ++dx) {
						const uint64_t ad = as + (uint32_t)dx * a_row, bd = bs + (uint32_t)dx * (B_TILE >> 4);
#pragma unroll
						for (int kk = 0; kk < T::KT / 16; ++kk)
							mma_f16(acc, ad + 2 * kk, bd + 2 * kk, idesc, dy > 0 || dx > 0 || kk > 0);
					}
				}
				if (!ok) break;
				mma_commit(&empty[(q0 + (uint32_t)k) % STAGES]);  // the strip of row y0 + (k - 1) d: last read here
				if (k == rows - 1) {
					mma_commit(&empty[(q0 + (uint32_t)k + 1) % STAGES]);
					mma_commit(&empty[(q0 + (uint32_t)k + 2) % STAGES]);
				}
				mma_commit(&accfull[a]);
			}
			q0 += (uint32_t)(rows + 2);
			s0 = s1;
		}
		mma_commit(drain);
		volatile int own = 0;
		mbar_wait(drain, 0, &own, g.err, kErrTimeoutAccum);
	} else if (warp >= 2) {
		// ---- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 (pixels of the
		// row), output channels [part * SPAN, +SPAN) with part = (w - 2) / 4
		constexpr int SPAN = BN / (T::EPI_WARPS / 4);
		static_assert(T::EPI_WARPS % 4 == 0 && SPAN % 32 == 0, "whole 32-column TMEM loads per warp");
		const int qd = warp & 3, part = (warp - 2) >> 2;
		const typename T::Epi epi(g);
		int i = 0;
		for (int id = t0; id < t1; ++id, ++i) {
			const int a = i & 1;
			const uint32_t use = (uint32_t)(i >> 1);
			if (!mbar_wait(&accfull[a], use & 1, abort_flag, g.err, kErrTimeoutAccum)) break;
			tc_fence_after();
			const int blk = id / H;
			int y, pend;
			T::row_of(g, id - blk * H, y, pend);
#pragma unroll 1
			for (int c = part * SPAN; c < (part + 1) * SPAN; c += 32) {
				float v[32];
				tmem_ld32(tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(a * BN + c), v);
				epi.store(g, blk, y, 32 * qd + lane, c, v);
			}
			tc_fence_before();
			__syncwarp();
			if (lane == 0) mbar_arrive(&accempty[a]);
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 1) {
		tc_fence_after();
		tmem_dealloc(tmem, TCOLS);
	}
}

// Launch of strip_run_kernel<T> over `tiles` tiles: one CTA per SM, each a
// contiguous run of ceil(tiles / CTAs) tiles.
template <class T>
umi_status launch_strip_run(const CUtensorMap& ta, const CUtensorMap& tb, const typename T::Args& g, int64_t tiles,
                            cudaStream_t st, const char* what) {
	constexpr size_t SMEM = run_smem_bytes<T>();
	auto kern = strip_run_kernel<T>;
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM),
	                         "cudaFuncSetAttribute"));
	int dev = 0, sms = 0, per_sm = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	UMI_TRY(umi::cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, run_threads<T>(), SMEM),
	                         "cudaOccupancyMaxActiveBlocksPerMultiprocessor"));
	per_sm = std::min(per_sm, 512 / (int)tmem_cols_for(T::BN));
	if (per_sm < 1) return umi::fail(UMI_ERR_UNSUPPORTED, "%s: does not fit an SM", what);
	int grid = (int)std::min<int64_t>(tiles, (int64_t)per_sm * sms);
	const int per = (int)umi::ceil_div(tiles, (int64_t)grid);
	grid = (int)umi::ceil_div(tiles, (int64_t)per);
	kern<<<grid, run_threads<T>(), SMEM, st>>>(ta, tb, g, idesc_f16(1u, BM, T::BN), per);
	return umi::launch_status(what);
}

// Persistent grid: as many CTAs as fit on the GPU at once (each holds 2*BN of
// the 512 TMEM columns of its SM; shared memory admits at most two CTAs per
// SM, so the columns always suffice), at most one per tile.
template <class K>
umi_status persistent_grid(K kern, size_t smem, int ntiles, int tmem_cols, int* grid) {
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
	                         "cudaFuncSetAttribute"));
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
	                                              (int)cudaSharedmemCarveoutMaxShared), "cudaFuncSetAttribute"));
	int dev = 0, sms = 0, per_sm = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	UMI_TRY(umi::cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NTHREADS, smem),
	                         "cudaOccupancyMaxActiveBlocksPerMultiprocessor"));
	per_sm = std::min(per_sm, 512 / tmem_cols);  // co-resident CTAs never wait for TMEM columns
	if (per_sm < 1) return umi::fail(UMI_ERR_UNSUPPORTED, "tc_kernel: does not fit an SM");
	*grid = std::max(1, std::min(ntiles, per_sm * sms));
	return UMI_OK;
}

// ---- FP32 products at FP32-level accuracy on the FP16 tensor cores.
//
// Operand splitting with error correction (Ootomo & Yokota, "Recovering
// single precision accuracy from Tensor Cores while surpassing the FP32
// theoretical peak performance", IJHPCA 2022): x = x_hi + 2^-11 x_lo with
// x_hi = rn_f16(x), x_lo = rn_f16((x - x_hi) 2^11), and
//   a b ~= a_hi b_hi + 2^-11 (a_hi b_lo + a_lo b_hi)       (a_lo b_lo dropped).
// Measured on GB300, the tensor core's fp32 accumulation truncates (the
// error of a bf16 GEMM with exact products is biased toward zero and grows
// with K: median 4.2e-6 relative at K = 4096 against 4.4e-7 for a plain
// fp32 sum), so, as the paper prescribes, the large term is not accumulated
// over all of K in the tensor core: a_hi b_hi of every `kc` K-slices goes to
// a fresh TMEM chunk (two, ping-ponged) that the epilogue warps add into fp32
// registers with round-to-nearest adds while the MMAs fill the other chunk.
// The correction terms (2^-11 smaller) accumulate over all of K in a third
// TMEM accumulator; their truncation is scaled down by 2^-11.
//
// Tile 128 x 128, K-slices of 64 fp16: a stage holds a_hi, a_lo, b_hi, b_lo
// (16 KB each, 128-byte swizzle), three stages.  TMEM: chunks at columns
// 0 and 128, correction accumulators (per tile parity) at 256 and 384.
// Roles as in tc_kernel: warp 0 TMA producer, warp 1 MMA issuer (3 MMAs per
// K-step of 16), warps 2..5 epilogue (each owns 32 rows: 128 fp32 running
// sums per thread).  Every wait is bounded; on a timeout every role stops,
// copies and MMAs drain, TMEM is freed.
struct SplitMaps {
	CUtensorMap ah, al, bh, bl;
};
constexpr uint32_t SPLIT_TILE = BM * BK * 2;      // 16 KB: 128 rows x 64 fp16
constexpr uint32_t SPLIT_STAGE = 4 * SPLIT_TILE;  // a_hi, a_lo, b_hi, b_lo
constexpr int SPLIT_STAGES = 3, SPLIT_BN = 128;
constexpr float kSplitLoScale = 1.0f / 2048.0f;

struct GemmSplitPolicy {
	static constexpr bool EPI_TMA = true;
	using Args = GemmArgs;
	using Tile = GemmPolicy::Tile;
	__host__ __device__ static int ntiles(const Args& g) {
		return ((g.M + BM - 1) / BM) * ((g.N + SPLIT_BN - 1) / SPLIT_BN);
	}
	// grouped order: 8 row-blocks at a time, column by column, so that the
	// tiles in flight at once (one per CTA) share 8 blocks of A and a short
	// run of B in L2 instead of sweeping all of B for every row of tiles
	static constexpr int GROUP_M = 8;
	__device__ static Tile tile(const Args& g, int id) {
		const int nt = (g.N + SPLIT_BN - 1) / SPLIT_BN, mt = (g.M + BM - 1) / BM;
		const int per_group = GROUP_M * nt;
		const int first_m = (id / per_group) * GROUP_M;
		const int gsz = min(mt - first_m, GROUP_M);
		const int r = id - (id / per_group) * per_group;
		return {(first_m + r % gsz) * BM, (r / gsz) * SPLIT_BN};
	}
	__device__ static int nk(const Args& g) { return (g.K + BK - 1) / BK; }
	__device__ static void load4(const SplitMaps& m, const Args&, const Tile& t, int ks, uint8_t* dst, uint64_t* bar) {
		tma_load_2d(dst, &m.ah, bar, ks * BK, t.m0);
		tma_load_2d(dst + SPLIT_TILE, &m.al, bar, ks * BK, t.m0);
		tma_load_2d(dst + 2 * SPLIT_TILE, &m.bh, bar, ks * BK, t.n0);
		tma_load_2d(dst + 3 * SPLIT_TILE, &m.bl, bar, ks * BK, t.n0);
	}
	__device__ static void store(const Args& g, const Tile& t, int rl, int c, const float (&v)[32]) {
		GemmPolicy::store(g, t, rl, c, v);
	}
};

// The convolution (ConvPolicy's tiles: 128 pixels of a row x 128 output
// channels, K-slices (tap, 64 input channels)) with split operands.
struct ConvSplitPolicy {
	static constexpr bool EPI_TMA = false;
	using Args = ConvArgs;
	using Tile = ConvPolicy::Tile;
	static_assert(ConvPolicy::BN == SPLIT_BN, "tile width");
	__host__ __device__ static int ntiles(const Args& g) { return ConvPolicy::ntiles(g); }
	__device__ static Tile tile(const Args& g, int id) { return ConvPolicy::tile(g, id); }
	__device__ static int nk(const Args& g) { return ConvPolicy::nk(g); }
	__device__ static void load4(const SplitMaps& m, const Args& g, const Tile& t, int ks, uint8_t* dst, uint64_t* bar) {
		const int cs = g.c / BK;
		const int tap = ks / cs, c0 = (ks - tap * cs) * BK;
		const int dy = tap / g.r, dx = tap - dy * g.r, pad = g.r / 2;
		tma_load_4d(dst, &m.ah, bar, c0, t.x0 + dx - pad, t.y + dy - pad, t.n);
		tma_load_4d(dst + SPLIT_TILE, &m.al, bar, c0, t.x0 + dx - pad, t.y + dy - pad, t.n);
		tma_load_2d(dst + 2 * SPLIT_TILE, &m.bh, bar, tap * g.c + c0, t.k0);
		tma_load_2d(dst + 3 * SPLIT_TILE, &m.bl, bar, tap * g.c + c0, t.k0);
	}
	__device__ static void store(const Args& g, const Tile& t, int rl, int c, const float (&v)[32]) {
		ConvPolicy::store(g, t, rl, c, v);
	}
};

template <class P>
__global__ void __launch_bounds__(NTHREADS, 1)
	tc_split_kernel(const __grid_constant__ SplitMaps maps, const __grid_constant__ CUtensorMap tcm,
	                const typename P::Args g, const uint32_t idesc, const int kc) {
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	uint8_t* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
	uint8_t* ebuf = base + SPLIT_STAGES * SPLIT_STAGE;  // epilogue staging, 2 x 4 KB per epilogue warp (EPI_TMA)
	uint64_t* full = reinterpret_cast<uint64_t*>(ebuf + (P::EPI_TMA ? 8 * 4096 : 0));
	uint64_t* empty = full + SPLIT_STAGES;
	uint64_t* hifull = empty + SPLIT_STAGES;  // [2] chunk of a_hi b_hi complete
	uint64_t* hiempty = hifull + 2;           // [2] chunk added into the registers
	uint64_t* accfull = hiempty + 2;          // [2] correction accumulator complete
	uint64_t* accempty = accfull + 2;         // [2] correction accumulator read
	uint64_t* drain = accempty + 2;
	uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
	volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int ntiles = P::ntiles(g);
	const int nk = P::nk(g);
	const int nchunk = (nk + kc - 1) / kc;

	if (threadIdx.x == 0) {
		for (int s = 0; s < SPLIT_STAGES; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], 1);
		}
		for (int a = 0; a < 2; ++a) {
			mbar_init(&hifull[a], 1);
			mbar_init(&hiempty[a], 4);
			mbar_init(&accfull[a], 1);
			mbar_init(&accempty[a], 4);
		}
		mbar_init(drain, 1);
		*abort_flag = 0;
		fence_mbar_init();
		tma_prefetch(&maps.ah);
		tma_prefetch(&maps.al);
		tma_prefetch(&maps.bh);
		tma_prefetch(&maps.bl);
	}
	if (warp == 1) {
		tmem_alloc(tmem_slot, 512);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;

	if (warp == 0 && lane == 0) {
		// ---- producer
		int armed[SPLIT_STAGES];
		for (int s = 0; s < SPLIT_STAGES; ++s) armed[s] = -1;
		uint32_t q = 0;
		for (int id = blockIdx.x; id < ntiles && !*abort_flag; id += gridDim.x) {
			const typename P::Tile t = P::tile(g, id);
			for (int ks = 0; ks < nk; ++ks, ++q) {
				const int s = (int)(q % SPLIT_STAGES);
				const uint32_t round = q / SPLIT_STAGES;
				if (!mbar_wait(&empty[s], (round & 1) ^ 1, abort_flag, g.err, kErrTimeoutEmpty)) break;
				mbar_arrive_expect_tx(&full[s], SPLIT_STAGE);
				armed[s] = (int)round;
				P::load4(maps, g, t, ks, base + s * SPLIT_STAGE, &full[s]);
			}
		}
		if (*abort_flag) {
			volatile int own = 0;
			for (int s = 0; s < SPLIT_STAGES; ++s)
				if (armed[s] >= 0) mbar_wait(&full[s], (uint32_t)armed[s] & 1, &own, g.err, kErrTimeoutFull);
		}
	} else if (warp == 1 && lane == 0) {
		// ---- MMA issuer
		uint32_t q = 0, cq = 0;
		int i = 0;
		bool ok = true;
		for (int id = blockIdx.x; ok && id < ntiles && !*abort_flag; id += gridDim.x, ++i) {
			const int a = i & 1;
			if (!mbar_wait(&accempty[a], ((uint32_t)(i >> 1) & 1) ^ 1, abort_flag, g.err, kErrTimeoutAccEmpty)) break;
			tc_fence_after();
			const uint32_t cacc = tmem + 256u + (uint32_t)(a * SPLIT_BN);
			uint32_t hacc = 0;
			for (int ks = 0; ks < nk; ++ks, ++q) {
				const bool first = ks % kc == 0;
				if (first) {
					const uint32_t hb = cq & 1;
					if (!mbar_wait(&hiempty[hb], ((cq >> 1) & 1) ^ 1, abort_flag, g.err, kErrTimeoutAccEmpty)) {
						ok = false;
						break;
					}
					tc_fence_after();
					hacc = tmem + hb * (uint32_t)SPLIT_BN;
				}
				const int s = (int)(q % SPLIT_STAGES);
				if (!mbar_wait(&full[s], (q / SPLIT_STAGES) & 1, abort_flag, g.err, kErrTimeoutFull)) {
					ok = false;
					break;
				}
				tc_fence_after();
				const uint32_t sa = smem_u32(base + s * SPLIT_STAGE);
				const uint64_t dah = desc_kmajor_sw128(sa), dal = desc_kmajor_sw128(sa + SPLIT_TILE);
				const uint64_t dbh = desc_kmajor_sw128(sa + 2 * SPLIT_TILE), dbl = desc_kmajor_sw128(sa + 3 * SPLIT_TILE);
#pragma unroll
				for (int kk = 0; kk < BK / 16; ++kk) {
					mma_f16(hacc, dah + 2 * kk, dbh + 2 * kk, idesc, !first || kk > 0);
					mma_f16(cacc, dah + 2 * kk, dbl + 2 * kk, idesc, ks > 0 || kk > 0);
					mma_f16(cacc, dal + 2 * kk, dbh + 2 * kk, idesc, true);
				}
				mma_commit(&empty[s]);
				if (ks % kc == kc - 1 || ks == nk - 1) {
					mma_commit(&hifull[cq & 1]);
					++cq;
				}
			}
			if (!ok) break;
			mma_commit(&accfull[a]);
		}
		mma_commit(drain);
		volatile int own = 0;
		mbar_wait(drain, 0, &own, g.err, kErrTimeoutAccum);
	} else if (warp >= 2) {
		// ---- epilogue: warp w owns TMEM lanes 32*(w%4) .. +31 (rows of the tile)
		const int qd = warp & 3;
		const uint32_t lane_base = (uint32_t)(32 * qd) << 16;
		uint32_t cq = 0, nst = 0;
		int i = 0;
		bool ok = true;
		for (int id = blockIdx.x; ok && id < ntiles; id += gridDim.x, ++i) {
			const int a = i & 1;
			float run[SPLIT_BN];
#pragma unroll
			for (int c = 0; c < SPLIT_BN; ++c) run[c] = 0.0f;
			for (int ch = 0; ch < nchunk; ++ch, ++cq) {
				const uint32_t hb = cq & 1;
				if (!mbar_wait(&hifull[hb], (cq >> 1) & 1, abort_flag, g.err, kErrTimeoutAccum)) {
					ok = false;
					break;
				}
				tc_fence_after();
#pragma unroll
				for (int c = 0; c < SPLIT_BN; c += 32) {
					float v[32];
					tmem_ld32(tmem + lane_base + hb * (uint32_t)SPLIT_BN + (uint32_t)c, v);
#pragma unroll
					for (int j = 0; j < 32; ++j) run[c + j] += v[j];
				}
				tc_fence_before();
				__syncwarp();
				if (lane == 0) mbar_arrive(&hiempty[hb]);
			}
			if (!ok) break;
			if (!mbar_wait(&accfull[a], ((uint32_t)i >> 1) & 1, abort_flag, g.err, kErrTimeoutAccum)) break;
			tc_fence_after();
			const typename P::Tile t = P::tile(g, id);
#pragma unroll
			for (int c = 0; c < SPLIT_BN; c += 32) {
				float v[32];
				tmem_ld32(tmem + lane_base + 256u + (uint32_t)(a * SPLIT_BN + c), v);
#pragma unroll
				for (int j = 0; j < 32; ++j) v[j] = fmaf(v[j], kSplitLoScale, run[c + j]);  // exact scaling, one rounding
				if constexpr (P::EPI_TMA) {
					if (g.vec) {
						const int row0 = t.m0 + 32 * qd, col0 = t.n0 + c;
						if (row0 < g.M && col0 < g.N) {
							uint8_t* sb = ebuf + (qd * 2 + (nst & 1)) * 4096;
							if (lane == 0) bulk_wait_read_1();
							__syncwarp();
#pragma unroll
							for (int j = 0; j < 8; ++j)
								*reinterpret_cast<float4*>(sb + lane * 128 + ((j ^ (lane & 7)) << 4)) =
									make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
							fence_proxy_async_smem();
							__syncwarp();
							if (lane == 0) {
								tma_store_2d(&tcm, sb, col0, row0);
								bulk_commit();
							}
							++nst;
						}
						continue;
					}
				}
				P::store(g, t, 32 * qd + lane, c, v);
			}
			tc_fence_before();
			__syncwarp();
			if (lane == 0) mbar_arrive(&accempty[a]);
		}
		if constexpr (P::EPI_TMA) {
			if (lane == 0) bulk_wait_all();
			__syncwarp();
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 1) {
		tc_fence_after();
		tmem_dealloc(tmem, 512);
	}
}

template <class P>
constexpr size_t split_smem_bytes() {
	return (size_t)SPLIT_STAGES * SPLIT_STAGE + (P::EPI_TMA ? 8 * 4096 : 0) + 1024 + 256;
}

// x (rows x K fp32) -> hi = rn_f16(x), lo = rn_f16((x - hi) 2^11), both (rows x K) fp16.
__global__ void split_f16_kernel(const float4* __restrict__ X, uint2* __restrict__ Hi, uint2* __restrict__ Lo, size_t n4) {
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
		const float4 x = X[i];
		const float xs[4] = {x.x, x.y, x.z, x.w};
		__half h[4], l[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			h[k] = __float2half_rn(xs[k]);
			l[k] = __float2half_rn((xs[k] - __half2float(h[k])) * 2048.0f);
		}
		Hi[i] = make_uint2((uint32_t)__half_as_ushort(h[0]) | ((uint32_t)__half_as_ushort(h[1]) << 16),
		                   (uint32_t)__half_as_ushort(h[2]) | ((uint32_t)__half_as_ushort(h[3]) << 16));
		Lo[i] = make_uint2((uint32_t)__half_as_ushort(l[0]) | ((uint32_t)__half_as_ushort(l[1]) << 16),
		                   (uint32_t)__half_as_ushort(l[2]) | ((uint32_t)__half_as_ushort(l[3]) << 16));
	}
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
                       cudaStream_t st, unsigned long long acc_wait_ns = kWaitNs) {
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
	GemmArgs g{C, M, N, K, N, umi::aligned(C, 16) && N % 4 == 0, err, acc_wait_ns};
	CUtensorMap tc;
	std::memset(&tc, 0, sizeof(tc));
	if (g.vec) {
		auto enc = encode_fn();
		const cuuint64_t dims[2] = {(cuuint64_t)N, (cuuint64_t)M};
		const cuuint64_t strides[1] = {(cuuint64_t)N * 4};
		const cuuint32_t box[2] = {32, 32};
		const cuuint32_t es[2] = {1, 1};
		const CUresult r = enc(&tc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, es,
		                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
		                       CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (r != CUDA_SUCCESS) return umi::fail(UMI_ERR_CUDA, "gemm: C tensor map (%d)", (int)r);
	}
	if ((int64_t)umi::ceil_div(M, BM) * umi::ceil_div(N, GemmPolicy224::BN) > INT32_MAX)
		return umi::fail(UMI_ERR_UNSUPPORTED, "gemm: too many tiles");
	// One CTA per SM works through the tiles in rounds; a round costs about the
	// same for every tile (the MMAs run the full width), so pick the width
	// whose rounds x width is smaller: 4096^3 is 512 tiles of 256 (3.4 rounds
	// on 152 SMs, 4 x 256 column-units) or 608 of 224 (exactly 4 rounds,
	// 4 x 224).
	int dev = 0, sms = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	const int64_t mt = umi::ceil_div(M, BM);
	const int64_t r256 = umi::ceil_div(mt * umi::ceil_div(N, 256), (int64_t)sms);
	const int64_t r224 = umi::ceil_div(mt * umi::ceil_div(N, 224), (int64_t)sms);
	if (r224 * 224 < r256 * 256) {
		UMI_TRY(map_kmajor(&tb, B, dt, N, K, GemmPolicy224::BN));
		constexpr size_t SMEM = smem_bytes<GemmPolicy224>();
		auto kern = tc_kernel<GemmPolicy224>;
		int grid = 0;
		UMI_TRY(persistent_grid(kern, SMEM, GemmPolicy224::ntiles(g), tmem_cols_for(GemmPolicy224::BN), &grid));
		kern<<<grid, NTHREADS, SMEM, st>>>(ta, tb, tc, g, idesc_f16((uint32_t)ab_type, BM, GemmPolicy224::BN));
		return umi::launch_status("tc_kernel<gemm 224>");
	}
	UMI_TRY(map_kmajor(&tb, B, dt, N, K, GemmPolicy::BN));
	constexpr size_t SMEM = smem_bytes<GemmPolicy>();
	auto kern = tc_kernel<GemmPolicy>;
	int grid = 0;
	UMI_TRY(persistent_grid(kern, SMEM, GemmPolicy::ntiles(g), tmem_cols_for(GemmPolicy::BN), &grid));
	kern<<<grid, NTHREADS, SMEM, st>>>(ta, tb, tc, g, idesc_f16((uint32_t)ab_type, BM, GemmPolicy::BN));
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

extern "C" umi_status umi_gemm_bf16_wait_limit(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K,
                                               int32_t* err, unsigned long long epilogue_wait_ns, void* stream) {
	const umi_status s = gemm_launch(A, B, C, M, N, K, 1, err, umi::as_stream(stream), epilogue_wait_ns);
	return s == UMI_OK ? umi::ok() : s;
}

extern "C" umi_status umi_err_status(int32_t err_bits) {
	if (err_bits == 0) return umi::ok();
	return umi::fail(UMI_ERR_TIMEOUT,
	                 "a bounded device wait gave up (error bits 0x%x: 1 slice not loaded, 2 ring slot not released, "
	                 "4 accumulator not finished, 8 accumulator not released)",
	                 (unsigned)err_bits);
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

constexpr int kSplitChunkDefault = 2;  // K-slices of 64 per TMEM chunk of a_hi b_hi

size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

umi_status split_operand(const float* X, size_t n, __half* hi, __half* lo, cudaStream_t st) {
	const size_t n4 = n / 4;
	const int blocks = (int)std::min<size_t>(4096, std::max<size_t>(1, (n4 + 255) / 256));
	split_f16_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const float4*>(X), reinterpret_cast<uint2*>(hi),
	                                          reinterpret_cast<uint2*>(lo), n4);
	return umi::launch_status("split_f16_kernel");
}

template <class P>
umi_status split_launch(const SplitMaps& maps, const CUtensorMap& tc, const typename P::Args& g, int kc,
                        cudaStream_t st, const char* what) {
	constexpr size_t SMEM = split_smem_bytes<P>();
	auto kern = tc_split_kernel<P>;
	int grid = 0;
	UMI_TRY(persistent_grid(kern, SMEM, P::ntiles(g), 512, &grid));
	kern<<<grid, NTHREADS, SMEM, st>>>(maps, tc, g, idesc_f16(0u, BM, SPLIT_BN), kc);
	return umi::launch_status(what);
}

umi_status check_chunk(int32_t chunk, int* kc) {
	if (chunk < 0 || chunk > 64) return umi::fail(UMI_ERR_INVALID_ARG, "split: chunk of %d K-slices (0..64)", chunk);
	*kc = chunk == 0 ? kSplitChunkDefault : chunk;
	return UMI_OK;
}

}  // namespace

extern "C" size_t umi_gemm_f32_f16x3_workspace_bytes(int32_t M, int32_t N, int32_t K) {
	if (M <= 0 || N <= 0 || K <= 0) return 0;
	return 2 * al256((size_t)M * K * 2) + 2 * al256((size_t)N * K * 2);
}

extern "C" umi_status umi_gemm_f32_f16x3(const float* A, const float* B, float* C, int32_t M, int32_t N, int32_t K,
                                         int32_t chunk, void* workspace, size_t workspace_bytes, int32_t* err,
                                         void* stream) {
	if (M < 0 || N < 0 || K < 0) return umi::fail(UMI_ERR_INVALID_ARG, "gemm_f16x3: negative size");
	const cudaStream_t st = umi::as_stream(stream);
	int kc = 0;
	UMI_TRY(check_chunk(chunk, &kc));
	if (M == 0 || N == 0) return umi::ok();
	if (!A || !B || !C) return umi::fail(UMI_ERR_INVALID_ARG, "gemm_f16x3: null pointer");
	if (K == 0) {
		const umi_status s = umi::cuda_status(cudaMemsetAsync(C, 0, (size_t)M * N * sizeof(float), st), "cudaMemsetAsync");
		return s == UMI_OK ? umi::ok() : s;
	}
	if (K % 8 != 0) return umi::fail(UMI_ERR_UNSUPPORTED, "gemm_f16x3: K = %d must be a multiple of 8", K);
	if (!umi::aligned(A, 16) || !umi::aligned(B, 16))
		return umi::fail(UMI_ERR_INVALID_ARG, "gemm_f16x3: A and B must be 16-byte aligned");
	if (!workspace) return umi::fail(UMI_ERR_INVALID_ARG, "gemm_f16x3: null workspace");
	if (!umi::aligned(workspace, 256)) return umi::fail(UMI_ERR_INVALID_ARG, "gemm_f16x3: workspace not 256-byte aligned");
	if (workspace_bytes < umi_gemm_f32_f16x3_workspace_bytes(M, N, K))
		return umi::fail(UMI_ERR_NO_MEMORY, "gemm_f16x3: workspace of %zu bytes, need %zu", workspace_bytes,
		                 umi_gemm_f32_f16x3_workspace_bytes(M, N, K));
	if ((int64_t)umi::ceil_div(M, BM) * umi::ceil_div(N, SPLIT_BN) > INT32_MAX)
		return umi::fail(UMI_ERR_UNSUPPORTED, "gemm_f16x3: too many tiles");
	char* ws = static_cast<char*>(workspace);
	__half* ah = reinterpret_cast<__half*>(ws);
	__half* al = reinterpret_cast<__half*>(ws + al256((size_t)M * K * 2));
	__half* bh = reinterpret_cast<__half*>(ws + 2 * al256((size_t)M * K * 2));
	__half* bl = reinterpret_cast<__half*>(ws + 2 * al256((size_t)M * K * 2) + al256((size_t)N * K * 2));
	UMI_TRY(split_operand(A, (size_t)M * K, ah, al, st));
	UMI_TRY(split_operand(B, (size_t)N * K, bh, bl, st));
	SplitMaps maps;
	UMI_TRY(map_kmajor(&maps.ah, ah, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, M, K, BM));
	UMI_TRY(map_kmajor(&maps.al, al, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, M, K, BM));
	UMI_TRY(map_kmajor(&maps.bh, bh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, N, K, SPLIT_BN));
	UMI_TRY(map_kmajor(&maps.bl, bl, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, N, K, SPLIT_BN));
	GemmArgs g{C, M, N, K, N, umi::aligned(C, 16) && N % 4 == 0, err, kWaitNs};
	CUtensorMap tc;
	std::memset(&tc, 0, sizeof(tc));
	if (g.vec) {
		auto enc = encode_fn();
		const cuuint64_t dims[2] = {(cuuint64_t)N, (cuuint64_t)M};
		const cuuint64_t strides[1] = {(cuuint64_t)N * 4};
		const cuuint32_t box[2] = {32, 32};
		const cuuint32_t es[2] = {1, 1};
		const CUresult r = enc(&tc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, es,
		                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
		                       CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (r != CUDA_SUCCESS) return umi::fail(UMI_ERR_CUDA, "gemm_f16x3: C tensor map (%d)", (int)r);
	}
	const umi_status s = split_launch<GemmSplitPolicy>(maps, tc, g, kc, st, "tc_split_kernel<gemm>");
	return s == UMI_OK ? umi::ok() : s;
}

extern "C" size_t umi_conv2d_fprop_f32_f16x3_workspace_bytes(int32_t n, int32_t c, int32_t h, int32_t w, int32_t k,
                                                             int32_t r) {
	if (n <= 0 || c <= 0 || h <= 0 || w <= 0 || k <= 0 || r <= 0) return 0;
	return 2 * al256((size_t)n * h * w * c * 2) + 2 * al256((size_t)k * r * r * c * 2);
}

extern "C" umi_status umi_conv2d_fprop_f32_f16x3(const float* x_nhwc, const float* w_krsc, float* out_nchw, int32_t n,
                                                 int32_t c, int32_t h, int32_t w, int32_t k, int32_t r, int32_t chunk,
                                                 void* workspace, size_t workspace_bytes, int32_t* err, void* stream) {
	if (n < 0 || c < 0 || h < 0 || w < 0 || k < 0) return umi::fail(UMI_ERR_INVALID_ARG, "conv_f16x3: negative size");
	int kc = 0;
	UMI_TRY(check_chunk(chunk, &kc));
	if (n == 0 || h == 0 || w == 0 || k == 0) return umi::ok();
	if (!x_nhwc || !w_krsc || !out_nchw || !workspace) return umi::fail(UMI_ERR_INVALID_ARG, "conv_f16x3: null pointer");
	if (r != 1 && r != 3 && r != 5 && r != 7)
		return umi::fail(UMI_ERR_UNSUPPORTED, "conv_f16x3: filter %dx%d (1, 3, 5, 7)", r, r);
	if (c % BK != 0) return umi::fail(UMI_ERR_UNSUPPORTED, "conv_f16x3: %d input channels (a multiple of %d)", c, BK);
	if (!umi::aligned(x_nhwc, 16) || !umi::aligned(w_krsc, 16))
		return umi::fail(UMI_ERR_INVALID_ARG, "conv_f16x3: misaligned input");
	if (!umi::aligned(workspace, 256)) return umi::fail(UMI_ERR_INVALID_ARG, "conv_f16x3: workspace not 256-byte aligned");
	if (workspace_bytes < umi_conv2d_fprop_f32_f16x3_workspace_bytes(n, c, h, w, k, r))
		return umi::fail(UMI_ERR_NO_MEMORY, "conv_f16x3: workspace too small");
	auto enc = encode_fn();
	if (!enc) return umi::fail(UMI_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
	const cudaStream_t st = umi::as_stream(stream);
	const size_t nx = (size_t)n * h * w * c, nw = (size_t)k * r * r * c;
	char* ws = static_cast<char*>(workspace);
	__half* xh = reinterpret_cast<__half*>(ws);
	__half* xl = reinterpret_cast<__half*>(ws + al256(nx * 2));
	__half* wh = reinterpret_cast<__half*>(ws + 2 * al256(nx * 2));
	__half* wl = reinterpret_cast<__half*>(ws + 2 * al256(nx * 2) + al256(nw * 2));
	UMI_TRY(split_operand(x_nhwc, nx, xh, xl, st));
	UMI_TRY(split_operand(w_krsc, nw, wh, wl, st));
	SplitMaps maps;
	for (int part = 0; part < 2; ++part) {
		const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
		const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)w * c * 2, (cuuint64_t)h * w * c * 2};
		const cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)BM, 1, 1};
		const cuuint32_t es[4] = {1, 1, 1, 1};
		const CUresult rr = enc(part ? &maps.al : &maps.ah, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 4, part ? xl : xh, dims,
		                        strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
		                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (rr != CUDA_SUCCESS) return umi::fail(UMI_ERR_CUDA, "conv_f16x3: input tensor map (%d)", (int)rr);
	}
	UMI_TRY(map_kmajor(&maps.bh, wh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, k, r * r * c, SPLIT_BN));
	UMI_TRY(map_kmajor(&maps.bl, wl, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, k, r * r * c, SPLIT_BN));
	ConvArgs g{out_nchw, n, c, h, w, k, r, umi::ceil_div(w, BM), umi::ceil_div(k, SPLIT_BN),
	           umi::aligned(out_nchw, 16) && w % 4 == 0, err};
	if ((int64_t)n * h * g.xtiles * g.ktiles > INT32_MAX) return umi::fail(UMI_ERR_UNSUPPORTED, "conv_f16x3: too many tiles");
	CUtensorMap unused;
	std::memset(&unused, 0, sizeof(unused));
	const umi_status s = split_launch<ConvSplitPolicy>(maps, unused, g, kc, st, "tc_split_kernel<conv>");
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
	const bool strip = r == 3 && c == BK && k <= ConvStripPolicy::BN;
	{
		const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
		const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)w * c * 2, (cuuint64_t)h * w * c * 2};
		const cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)(strip ? ConvStripPolicy::STRIP_ROWS : BM), 1, 1};
		const cuuint32_t es[4] = {1, 1, 1, 1};
		const CUresult rr = enc(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, es,
		                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
		                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (rr != CUDA_SUCCESS) return umi::fail(UMI_ERR_CUDA, "conv: input tensor map (%d)", (int)rr);
	}
	UMI_TRY(map_kmajor(&tb, wt, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, k, r * r * c, ConvPolicy::BN));
	ConvArgs g{out, n, c, h, w, k, r, umi::ceil_div(w, BM), umi::ceil_div(k, ConvPolicy::BN),
	           umi::aligned(out, 16) && w % 4 == 0, err};
	const int64_t tiles = (int64_t)n * h * g.xtiles * g.ktiles;
	if (tiles > INT32_MAX) return umi::fail(UMI_ERR_UNSUPPORTED, "conv: too many tiles");
	int grid = 0;
	if (strip)  // k <= BN: one output-channel block; runs of output rows, each input row's strip loaded once per run
		return launch_strip_run<ConvRun>(ta, tb, g, tiles, st, "strip_run_kernel<conv>");
	if (g.ktiles == 1 && r * r * (c / BK) <= ConvResPolicy::NK_RES) {
		constexpr size_t SMEM = smem_bytes<ConvResPolicy>();
		auto kern = tc_kernel<ConvResPolicy>;
		UMI_TRY(persistent_grid(kern, SMEM, (int)tiles, tmem_cols_for(ConvResPolicy::BN), &grid));
		kern<<<grid, NTHREADS, SMEM, st>>>(ta, tb, tb, g, idesc_f16(1u, BM, ConvResPolicy::BN));
		return umi::launch_status("tc_kernel<conv, resident weights>");
	}
	constexpr size_t SMEM = smem_bytes<ConvPolicy>();
	auto kern = tc_kernel<ConvPolicy>;
	UMI_TRY(persistent_grid(kern, SMEM, (int)tiles, tmem_cols_for(ConvPolicy::BN), &grid));
	kern<<<grid, NTHREADS, SMEM, st>>>(ta, tb, tb, g, idesc_f16(1u, BM, ConvPolicy::BN));
	return umi::launch_status("tc_kernel<conv>");
}

}  // namespace

extern "C" umi_status umi_conv2d_fprop_bf16(const void* x_nhwc, const void* w_krsc, float* out_nchw, int32_t n, int32_t c,
                                            int32_t h, int32_t w, int32_t k, int32_t r, int32_t* err, void* stream) {
	const umi_status s = conv_launch(x_nhwc, w_krsc, out_nchw, n, c, h, w, k, r, err, umi::as_stream(stream));
	return s == UMI_OK ? umi::ok() : s;
}

namespace umi {

// cuTensorMapEncodeTiled for the other translation units (full_me.cu).
void* tma_encode_fn() { return reinterpret_cast<void*>(encode_fn()); }

// One tensor-core layer of the motion-proposal network (see MenetRun):
// in/out (h, w, 32) bf16 NHWC, wpack (32, 9*32) bf16 K-major (tap-major, then
// input channel), bias 32 fp32.  Used by learned_me.cu.
// The 32-channel layers in rolling-accumulator form.  A tcgen05.mma of
// M = 128, K = 16 takes the same 75 clocks for every N up to 144 (then about
// half a clock per column), so an N = 32 MMA runs at a fifth of the tensor
// rate.  Here each strip (input row m of a run) is multiplied once by the
// stacked weights of every filter row that reads it: for tap column dx,
// B = [W(dy, dx) for dy = lo .. hi] (32 rows each, N = 32 (hi - lo + 1))
// and D = the accumulators of output rows m - lo .. m - hi side by side.
// Sixteen 32-column accumulators (all of TMEM) take consecutive output rows
// in descending column order (row r at 32 (15 - r mod 16)), so those rows
// are adjacent columns except where the ring wraps (then two MMAs).  Every
// MMA accumulates: the accumulators are cleared at launch and by the
// epilogue after it drains one.  Six MMAs per output row (3 dx x 2 K = 16
// slices) instead of 18; a strip is read by its own six MMAs only.
namespace {
constexpr int ROLL_SLOTS = umi_roll::kSlots;
constexpr int ROLL_EPI_WARPS = 8;  // two groups of four, taking alternate rows
__host__ __device__ constexpr int roll_threads() { return 64 + 32 * ROLL_EPI_WARPS; }
constexpr size_t roll_smem_bytes() {
	return (size_t)MenetRun::STAGES * MenetRun::STRIP_STAGE + (size_t)MenetRun::NK_RES * (32 * MenetRun::KT * 2) + 1024 +
	       1024;
}
__device__ __forceinline__ int roll_slot(int r) { return umi_roll::slot(r); }

__global__ void __launch_bounds__(roll_threads(), 1)
	menet_rows_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, const MenetArgs g,
	                  const int per) {
	using T = MenetRun;
	constexpr int STAGES = T::STAGES, NKR = T::NK_RES;
	constexpr uint32_t B_TILE = 32 * T::KT * 2, SS = T::STRIP_STAGE;  // 2 KB per tap, 9 KB per strip
	static_assert(ROLL_SLOTS * 32 == 512 && ROLL_EPI_WARPS == 8, "sixteen accumulators fill TMEM; two epilogue groups");
	extern __shared__ uint8_t smem_raw[];
	uint8_t* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
	uint8_t* bres = base + STAGES * SS;  // tap (dy, dx) at (3 dx + dy) * 2 KB: the dy of one dx adjacent
	uint64_t* full = reinterpret_cast<uint64_t*>(bres + NKR * B_TILE);
	uint64_t* empty = full + STAGES;
	uint64_t* accfull = empty + STAGES;          // [ROLL_SLOTS]
	uint64_t* accempty = accfull + ROLL_SLOTS;  // [ROLL_SLOTS]
	uint64_t* drain = accempty + ROLL_SLOTS;
	uint64_t* bready = drain + 1;
	uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bready + 1);
	volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int H = g.h, ntiles = g.xtiles * H, d = g.dil;
	const int t0 = blockIdx.x * per, t1 = min(ntiles, t0 + per);
	auto segment = [&](int s0, int& blk, int& y0, int& s1) {
		blk = s0 / H;
		int pend;
		T::row_of(g, s0 - blk * H, y0, pend);
		s1 = min(t1, blk * H + pend);
	};

	if (threadIdx.x == 0) {
		for (int s = 0; s < STAGES; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], 1);
		}
		for (int a = 0; a < ROLL_SLOTS; ++a) {
			mbar_init(&accfull[a], 1);
			mbar_init(&accempty[a], 4);
		}
		mbar_init(drain, 1);
		mbar_init(bready, 1);
		*abort_flag = 0;
		fence_mbar_init();
		tma_prefetch(&ta);
		tma_prefetch(&tb);
	}
	if (warp == 1) {
		tmem_alloc(tmem_slot, 512);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;
	if (warp >= 2 && warp < 6) {  // one warp per lane quadrant clears every accumulator
#pragma unroll 1
		for (uint32_t c = 0; c < 512; c += 32) tmem_zero32(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + c);
		tmem_wait_st();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();

	if (warp == 0 && lane == 0) {
		// ---- producer: weights once (tap ks = 3 dy + dx to slot 3 dx + dy), then every strip once
		int armed[STAGES];
		for (int s = 0; s < STAGES; ++s) armed[s] = -1;
		mbar_arrive_expect_tx(bready, (uint32_t)NKR * B_TILE);
		for (int ks = 0; ks < NKR; ++ks) T::load_b(&tb, g, ks, bres + (3 * (ks % 3) + ks / 3) * B_TILE, bready);
		const uint32_t sbytes = T::strip_bytes(g);
		uint32_t q = 0;
		bool go = true;
		for (int s0 = t0; go && s0 < t1 && !*abort_flag;) {
			int blk, y0, s1;
			segment(s0, blk, y0, s1);
			for (int i = 0; i < s1 - s0 + 2; ++i, ++q) {  // input row y0 + (i - 1) d
				const int s = (int)(q % STAGES);
				const uint32_t round = q / STAGES;
				if (!mbar_wait(&empty[s], (round & 1) ^ 1, abort_flag, g.err, kErrTimeoutEmpty)) { go = false; break; }
				mbar_arrive_expect_tx(&full[s], sbytes);
				armed[s] = (int)round;
				T::load_strip(&ta, g, blk, y0 + (i - 1) * d, base + s * SS, &full[s]);
			}
			s0 = s1;
		}
		if (*abort_flag) {
			volatile int own = 0;
			for (int s = 0; s < STAGES; ++s)
				if (armed[s] >= 0) mbar_wait(&full[s], (uint32_t)armed[s] & 1, &own, g.err, kErrTimeoutFull);
			mbar_wait(bready, 0, &own, g.err, kErrTimeoutFull);
		}
	} else if (warp == 1 && lane == 0) {
		// ---- MMA issuer: strip m of a run of `rows` output rows feeds rows
		// m - dy for dy in [lo, hi] = [max(0, m - rows + 1), min(2, m)]
		bool ok = mbar_wait(bready, 0, abort_flag, g.err, kErrTimeoutFull);
		const uint64_t a_base = T::desc_a(smem_u32(base), 0), b_base = T::desc_b(smem_u32(bres));
		const uint32_t a_row = (uint32_t)(d * T::ROW_BYTES) >> 4;
		uint32_t q = 0;  // strips so far
		int r0 = 0;      // output rows of the earlier runs
		for (int s0 = t0; ok && s0 < t1 && !*abort_flag;) {
			int blk, y0, s1;
			segment(s0, blk, y0, s1);
			const int rows = s1 - s0;
			for (int m = 0; m < rows + 2; ++m, ++q) {
				const umi_roll::Step st = umi_roll::step(m, rows, r0);
				const int lo = st.lo, cnt = st.hi - st.lo + 1;
				if (lo == 0) {  // row r0 + m starts here: its accumulator must be drained and cleared
					const int r = r0 + m;
					if (!mbar_wait(&accempty[roll_slot(r)], ((uint32_t)(r / ROLL_SLOTS) & 1) ^ 1, abort_flag, g.err,
					               kErrTimeoutAccEmpty)) {
						ok = false;
						break;
					}
					tc_fence_after();
				}
				const int s = (int)(q % STAGES);
				if (!mbar_wait(&full[s], (q / STAGES) & 1, abort_flag, g.err, kErrTimeoutFull)) {
					ok = false;
					break;
				}
				tc_fence_after();
				const int first = st.first, c1 = st.c1;  // c1 blocks before the ring wraps to column 0
				const uint32_t id1 = idesc_f16(1u, BM, 32 * c1), id2 = idesc_f16(1u, BM, 32 * (cnt - c1));
				const uint64_t as = a_base + ((uint32_t)s * (SS >> 4));
#pragma unroll
				for (int dx = 0; dx < 3; ++dx) {
					const uint64_t ad = as + (uint32_t)dx * a_row;
					const uint64_t bd = b_base + (uint32_t)(3 * dx + lo) * (B_TILE >> 4);
#pragma unroll
					for (int kk = 0; kk < T::KT / 16; ++kk) {
						mma_f16(tmem + 32u * (uint32_t)first, ad + 2 * kk, bd + 2 * kk, id1, true);
						if (c1 < cnt) mma_f16(tmem, ad + 2 * kk, bd + (uint32_t)c1 * (B_TILE >> 4) + 2 * kk, id2, true);
					}
				}
				mma_commit(&empty[s]);                                      // the strip's only reader
				if (m >= 2) mma_commit(&accfull[roll_slot(r0 + m - 2)]);  // row m - 2 has all nine taps
			}
			r0 += rows;
			s0 = s1;
		}
		mma_commit(drain);
		volatile int own = 0;
		mbar_wait(drain, 0, &own, g.err, kErrTimeoutAccum);
	} else if (warp >= 2) {
		// ---- epilogue: group (w - 2) / 4 takes rows r = group mod 2; warp w
		// reads TMEM lanes 32 (w%4) .. +31 (pixels), clears the accumulator,
		// releases it, then + bias, ReLU, bf16 and the 64-byte pixel store
		const int qd = warp & 3, grp = (warp - 2) >> 2;
		const T::Epi epi(g);
		for (int r = grp; t0 + r < t1; r += 2) {
			const int id = t0 + r, sl = roll_slot(r);
			if (!mbar_wait(&accfull[sl], (uint32_t)(r / ROLL_SLOTS) & 1, abort_flag, g.err, kErrTimeoutAccum)) break;
			tc_fence_after();
			const uint32_t ta_ = tmem + ((uint32_t)(32 * qd) << 16) + 32u * (uint32_t)sl;
			float v[32];
			tmem_ld32(ta_, v);
			tmem_zero32(ta_);
			tmem_wait_st();
			tc_fence_before();
			__syncwarp();
			if (lane == 0) mbar_arrive(&accempty[sl]);
			const int blk = id / H;
			int y, pend;
			T::row_of(g, id - blk * H, y, pend);
			epi.store(g, blk, y, 32 * qd + lane, 0, v);
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 1) {
		tc_fence_after();
		tmem_dealloc(tmem, 512);
	}
}

umi_status launch_menet_rows(const CUtensorMap& ta, const CUtensorMap& tb, const MenetArgs& g, int64_t tiles,
                             cudaStream_t st) {
	constexpr size_t SMEM = roll_smem_bytes();
	UMI_TRY(umi::cuda_status(
		cudaFuncSetAttribute(menet_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM),
		"cudaFuncSetAttribute"));
	int dev = 0, sms = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	int grid = (int)std::min<int64_t>(tiles, (int64_t)sms);  // all of TMEM: one CTA per SM
	const int per = (int)umi::ceil_div(tiles, (int64_t)grid);
	grid = (int)umi::ceil_div(tiles, (int64_t)per);
	menet_rows_kernel<<<grid, roll_threads(), SMEM, st>>>(ta, tb, g, per);
	return umi::launch_status("menet_rows_kernel");
}
}  // namespace

umi_status menet_conv_tc(const void* in, void* out, const void* wpack, const float* bias, int h, int w, int dil,
                         int* err, cudaStream_t st) {
	if (dil < 1 || dil > MenetRun::MAXD) return umi::fail(UMI_ERR_UNSUPPORTED, "menet conv: dilation %d", dil);
	if (!umi::aligned(in, 16) || !umi::aligned(out, 16) || !umi::aligned(wpack, 16))
		return umi::fail(UMI_ERR_INVALID_ARG, "menet conv: misaligned buffer");
	auto enc = encode_fn();
	if (!enc) return umi::fail(UMI_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
	CUtensorMap ta, tb;
	{
		const cuuint64_t dims[4] = {32, (cuuint64_t)w, (cuuint64_t)h, 1};
		const cuuint64_t strides[3] = {64, (cuuint64_t)w * 64, (cuuint64_t)h * w * 64};
		const cuuint32_t box[4] = {32, (cuuint32_t)(BM + 2 * dil), 1, 1};
		const cuuint32_t es[4] = {1, 1, 1, 1};
		const CUresult rr = enc(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(in), dims, strides, box, es,
		                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
		                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (rr != CUDA_SUCCESS) return umi::fail(UMI_ERR_CUDA, "menet conv: activation tensor map (%d)", (int)rr);
	}
	{
		const cuuint64_t dims[2] = {9 * 32, 32};
		const cuuint64_t strides[1] = {9 * 32 * 2};
		const cuuint32_t box[2] = {32, 32};
		const cuuint32_t es[2] = {1, 1};
		const CUresult rr = enc(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(wpack), dims, strides, box, es,
		                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
		                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		if (rr != CUDA_SUCCESS) return umi::fail(UMI_ERR_CUDA, "menet conv: weight tensor map (%d)", (int)rr);
	}
	MenetArgs g{static_cast<__nv_bfloat16*>(out), bias, h, w, dil, umi::ceil_div(w, BM), err};
	// runs of output rows y, y + d, y + 2d, ...: each input row's strip loaded once per run
	return launch_menet_rows(ta, tb, g, (int64_t)h * g.xtiles, st);
}

}  // namespace umi
