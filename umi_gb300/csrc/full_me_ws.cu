// Full-search motion estimation, 16x16 blocks, search range +-R for the
// benchmark ranges R = 32 and R = 64: a warp-specialised persistent kernel.
//
// Same operator as full_me.cu (main/full_me.cu:8-64: SAD of a block of `cur`
// against `ref` at every displacement, reference pixels clamped to the frame;
// argmin first in raster order of (dy, dx), main/full_me.cu:70-71), laid out
// so that the integer ALU pipe does little but `vabsdiff4`:
//
//  * one CTA per SM: warps 0..3 produce, warps 4..19 search.  Every SM
//    sub-partition gets one producer and four search warps, so the four ALU
//    pipes get equal work;
//  * the producer brings each macroblock's reference window into a ring of
//    NB shared-memory buffers (one TMA box when the window lies inside the
//    frame on a 16-byte boundary, else 4-byte cp.async with rows clamped to
//    the frame, single bytes where a word crosses the left or right edge or
//    is not 4-byte aligned (a window moved by its search centre)),
//    then writes the three byte-shifted copies of the window (copy s, word k
//    = bytes [4k+s, 4k+s+4) of a row) with integer multiplies: lo >> 8s is
//    the high word of lo * 2^(32-8s) and hi << (32-8s) its low word, two FMA-
//    pipe instructions per output word that leave the ALU pipe to the SADs;
//  * the producers load PD macroblocks ahead of the one they shift and may
//    run up to NB - PD macroblocks ahead of the search;
//  * hand-off by mbarriers: `full[b]` (128 producer arrivals) when buffer b
//    holds a macroblock's window, block and copies; `empty[b]` (one arrival per
//    search task) when every task of it is done.  No CTA-wide barrier in the
//    loop: a search warp that finishes its tasks of one macroblock goes on to
//    the next one whose buffer is full;
//  * the search tasks of all the CTA's macroblocks form one stream: task L is
//    (macroblock L / TPM, column ix, rows 13q .. 13q+12) with TPM = (2R+1) x
//    ceil((2R+1)/13) tasks per macroblock, and search thread c takes tasks
//    c, c + 512, ...: every thread does the same number of equal tasks, and a
//    warp whose 32 tasks straddle two macroblocks reads two buffers without
//    diverging;
//  * a task keeps 13 window rows of 4 words in a register ring and streams the
//    block's 16 rows (one broadcast 16-byte shared load each): 16 x 4 x 13 =
//    832 `vabsdiff4.add` per task against 5 shared loads per block row.  All
//    shared-memory offsets are compile-time constants (R is a template
//    parameter), so the loads need no address arithmetic;
//  * argmin: per task, key = sad * 16 + q (an IMAD) and 12 minima; the task's
//    key (sad << 15) | raster index goes to a shared atomicMin per macroblock;
//    the producer writes (mv_y, mv_x, sad) when it recycles the buffer.
//
// Waits sleep in hardware between tests (mbarrier.try_wait with a suspend-
// time hint), so a warp that ran ahead takes no issue slots from the SADs.
// Every mbarrier wait is bounded (1 s of %globaltimer).  A wait that gives up
// raises the CTA's abort flag and ORs an error bit into a library-wide device
// word (read and cleared by umi_full_me_error); the producer then lets its
// own copies land, marks every macroblock of the CTA that it did not finish
// with sad = -1 and returns.  No wait can hang the GPU.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>

#include "common.h"
#include "tc_common.cuh"

namespace umi {
void* tma_encode_fn();  // cuTensorMapEncodeTiled (gemm_tc.cu)
}

// Error bits of the motion-estimation kernels (bounded waits that gave up).
__device__ int g_full_me_err;

namespace {

using namespace umi_tc;

enum : int { kMeErrFull = 1, kMeErrEmpty = 2, kMeErrLoad = 4 };

__device__ __forceinline__ uint32_t sad4_acc(uint32_t a, uint32_t b, uint32_t c) {
	uint32_t d;
	asm("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
	return d;
}

__device__ __forceinline__ void cp_async4(uint32_t* dst, const void* src) {
	asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
	asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <int R> struct WsGeom {
	static constexpr int ND = 2 * R + 1;           // displacements per axis
	static constexpr int G = 13;                    // vertical displacements per task
	static constexpr int NG = (ND + G - 1) / G;     // tasks per column
	static constexpr int WR = NG * G + 15;          // window rows staged
	static constexpr int WRAW = R / 2 + 5;          // raw words of a row the copies read
	static constexpr int S = (WRAW + 3) & ~3;       // row stride in words (TMA box rows: 16-byte multiple)
	static constexpr int WC = R / 2 + 4;            // words per row of the shifted copies
	static constexpr int COPY = WR * S + ((8 - (WR * S) % 32) + 32) % 32;  // copies 8 banks apart
	static constexpr int CB = 4 * COPY;             // the current block: 16 rows x 4 words
	static constexpr int BUF = (CB + 64 + 31) & ~31;  // words per buffer (128-byte multiple)
	static constexpr int TPM = ND * NG;             // search tasks per macroblock
	static constexpr int NB = R == 32 ? 6 : 2;      // buffers in the ring
	static constexpr int PD = R == 32 ? 2 : 1;      // macroblocks whose loads are issued ahead of the shift
	static constexpr size_t SMEM = (size_t)NB * BUF * 4 + 128;
	static_assert(ND * ND < (1 << 15), "raster index fits the key's low 15 bits");
	static_assert(COPY % 32 == 8 && COPY >= WR * S, "copy layout");
	static_assert(WR <= 256 && 4 * S <= 256, "TMA box");
};

constexpr int kProdWarps = 4, kProdThreads = 32 * kProdWarps;
constexpr int kSearchWarps = 16, kSearchThreads = 32 * kSearchWarps;
constexpr int kThreads = kProdThreads + kSearchThreads;

// Named barrier 1 among the producer warps only (warps 0..3).
__device__ __forceinline__ void bar_producers() { asm volatile("bar.sync 1, %0;" ::"n"(kProdThreads) : "memory"); }

struct WsArgs {
	const uint8_t* cur;
	const uint8_t* ref;
	const int32_t* centers;     // optional: per-block search centres (cy, cx)
	int32_t* out;               // (nblk, 3): mv_y, mv_x, sad
	int h, w, nbx, nblk;
	const int32_t* list;        // optional: search only these blocks (slot i -> block list[i])
	const int32_t* list_count;  // number of valid slots of `list` (device word)
	int slots;                  // slots covered by the grid (nblk, or the list's capacity)
	int tma;                    // the tensor map over ref is valid
	uint32_t mul[3];            // 2^24, 2^16, 2^8: multipliers of the shifted copies (runtime values)
	uint32_t mul16;             // 16 (runtime: the argmin key stays an IMAD)
};

__device__ __forceinline__ int ws_block(const WsArgs& a, int slot) { return a.list ? a.list[slot] : slot; }

// One search task: column ix, vertical displacements iy0 .. iy0+12 (those
// < ND); returns the argmin key (sad << 15) | (iy * ND + ix).
template <int R>
__device__ __forceinline__ uint32_t ws_task(const uint32_t* __restrict__ buf, int ix, int iy0, uint32_t mul16) {
	using Gm = WsGeom<R>;
	constexpr int S = Gm::S, G = Gm::G;
	const uint32_t* cb = buf + Gm::CB;
	const uint32_t* wp = buf + (ix & 3) * Gm::COPY + (ix >> 2) + iy0 * S;
	uint32_t ring[G][4], acc[G];
#pragma unroll
	for (int q = 0; q < G; ++q) acc[q] = 0;
#pragma unroll
	for (int q = 0; q < G - 1; ++q)
#pragma unroll
		for (int k = 0; k < 4; ++k) ring[q][k] = wp[q * S + k];
#pragma unroll
	for (int py = 0; py < 16; ++py) {
		const uint4 c4 = *reinterpret_cast<const uint4*>(cb + 4 * py);  // same address in every lane
		const uint32_t cv[4] = {c4.x, c4.y, c4.z, c4.w};
		const int r = py + G - 1;
#pragma unroll
		for (int k = 0; k < 4; ++k) ring[r % G][k] = wp[r * S + k];
#pragma unroll
		for (int k = 0; k < 4; ++k)
#pragma unroll
			for (int q = 0; q < G; ++q) acc[q] = sad4_acc(cv[k], ring[(py + q) % G][k], acc[q]);
	}
	uint32_t kmin = 0xffffffffu;
	if (iy0 + G <= Gm::ND) {
#pragma unroll
		for (int q = 0; q < G; ++q) kmin = min(kmin, acc[q] * mul16 + (uint32_t)q);
	} else {  // the last row group of a range whose 2R+1 rows are not a multiple of 13
#pragma unroll
		for (int q = 0; q < G; ++q)
			if (iy0 + q < Gm::ND) kmin = min(kmin, acc[q] * mul16 + (uint32_t)q);
	}
	return ((kmin >> 4) << 15) | (uint32_t)((iy0 + (int)(kmin & 15u)) * Gm::ND + ix);
}

template <int R>
__global__ void __launch_bounds__(kThreads, 1)
full_me_ws_kernel(const WsArgs a, const __grid_constant__ CUtensorMap tref) {
	using Gm = WsGeom<R>;
	constexpr int NB = Gm::NB, PD = Gm::PD, S = Gm::S, TPM = Gm::TPM;
	extern __shared__ __align__(128) uint8_t smem_raw[];
	// 128-byte aligned start (TMA destinations), formed by indexing the shared
	// array so that the compiler keeps shared-memory loads and stores
	uint32_t* bufs = reinterpret_cast<uint32_t*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
	__shared__ __align__(8) uint64_t full[NB], empty[NB], tbar[NB];
	__shared__ uint32_t best[NB];
	__shared__ int abort_sh;
	volatile int* abort_flag = &abort_sh;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	int slots = a.slots;
	if (a.list) slots = min(slots, *a.list_count);
	const int nj = (int)blockIdx.x < slots ? (slots - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;
	if (nj == 0) return;  // uniform over the CTA
	if (tid == 0) {
		for (int b = 0; b < NB; ++b) {
			mbar_init(&full[b], kProdThreads);
			mbar_init(&empty[b], TPM);
			mbar_init(&tbar[b], 1);
			best[b] = 0xffffffffu;
		}
		abort_sh = 0;
		fence_mbar_init();
		if (a.tma) tma_prefetch(&tref);
	}
	__syncthreads();

	if (warp < kProdWarps) {
		// ------------------------------------------------------------ producer
		// Decisions after a wait are taken by all producer threads together:
		// each thread waits (bounded; a timeout raises the abort flag), then
		// the producers' named barrier, then every thread reads the abort flag,
		// so that all of them take the same branch and reach the same barriers.
		const int pt = tid, pw = warp;
		uint32_t tma_pending = 0;  // bit b: buffer b's current fill came by TMA and was not yet waited for
		uint32_t tma_phase = 0;    // bit b: parity of buffer b's next TMA completion
		auto origin = [&](int j, int& blk, int& gy0, int& gx0, int& cy, int& cx) {
			blk = ws_block(a, (int)blockIdx.x + j * (int)gridDim.x);
			const int by = blk / a.nbx, bx = blk - by * a.nbx;
			cy = a.centers ? a.centers[2 * blk] : 0;
			cx = a.centers ? a.centers[2 * blk + 1] : 0;
			gy0 = 16 * by + cy - R;
			gx0 = 16 * bx + cx - R;
		};
		// Loads of macroblock j into buffer j % NB; every producer thread commits one cp.async group.
		auto issue = [&](int j) {
			const int b = j % NB;
			uint32_t* buf = bufs + b * Gm::BUF;
			int blk, gy0, gx0, cy, cx;
			origin(j, blk, gy0, gx0, cy, cx);
			const bool box = a.tma && gx0 >= 0 && (gx0 & 15) == 0 && gx0 + 2 * R + 16 <= a.w && gy0 >= 0 &&
			                 gy0 + 2 * R + 16 <= a.h;
			fence_proxy_async_smem();  // earlier generic accesses of the buffer before the async-proxy writes
			if (box) {
				if (pt == 0) {
					mbar_arrive_expect_tx(&tbar[b], (uint32_t)(4 * S * Gm::WR));
					tma_load_2d(buf, &tref, &tbar[b], gx0, gy0);
				}
				tma_pending |= 1u << b;
			} else {
				for (int r = pw; r < Gm::WR; r += kProdWarps) {
					const int gy = min(max(gy0 + r, 0), a.h - 1);
					const uint8_t* row = a.ref + (size_t)gy * a.w;
					for (int k = lane; k < Gm::WRAW; k += 32) {
						const int gx = gx0 + 4 * k;
						// 4-byte copies need a 4-byte-aligned source: a window moved
						// off the 4-byte grid by its search centre takes single bytes
						if (gx >= 0 && gx + 4 <= a.w && (gx & 3) == 0) {
							cp_async4(buf + r * S + k, row + gx);
						} else {
							uint32_t v = 0;
#pragma unroll
							for (int t = 0; t < 4; ++t)
								v |= (uint32_t)__ldg(row + min(max(gx + t, 0), a.w - 1)) << (8 * t);
							buf[r * S + k] = v;
						}
					}
				}
			}
			if (pt < 64) {
				const int by = blk / a.nbx, bx = blk - by * a.nbx;
				cp_async4(buf + Gm::CB + pt, a.cur + (size_t)(16 * by + (pt >> 2)) * a.w + 16 * bx + 4 * (pt & 3));
			}
			cp_async_commit();
		};
		// Waits for macroblock j's loads, writes the shifted copies, marks the buffer full.
		auto finish = [&](int j) -> bool {
			const int b = j % NB;
			uint32_t* buf = bufs + b * Gm::BUF;
			cp_async_wait<PD - 1>();  // one group per macroblock; PD - 1 newer ones may stay in flight
			if (tma_pending >> b & 1u) {
				mbar_wait_sleep(&tbar[b], tma_phase >> b & 1u, abort_flag, &g_full_me_err, kMeErrLoad, 2000);
				tma_phase ^= 1u << b;
				tma_pending &= ~(1u << b);
			}
			bar_producers();
			if (*abort_flag) return false;
			const uint32_t m1 = a.mul[0], m2 = a.mul[1], m3 = a.mul[2];
			// rows pw, pw + 4, ...: fully unrolled from one base pointer, so every
			// shared-memory offset is an immediate (no address arithmetic per word)
			constexpr int RPW = (Gm::WR + kProdWarps - 1) / kProdWarps;
			uint32_t* rb = buf + pw * S + lane;
#pragma unroll
			for (int i = 0; i < RPW; ++i) {
				if (Gm::WR % kProdWarps == 0 || pw + kProdWarps * i < Gm::WR) {
#pragma unroll
					for (int kc = 0; kc < Gm::WC; kc += 32) {
						if (lane + kc < Gm::WC) {
							const int o = kProdWarps * i * S + kc;
							const uint32_t lo = rb[o], hi = rb[o + 1];
							rb[Gm::COPY + o] = __umulhi(lo, m1) + hi * m1;
							rb[2 * Gm::COPY + o] = __umulhi(lo, m2) + hi * m2;
							rb[3 * Gm::COPY + o] = __umulhi(lo, m3) + hi * m3;
						}
					}
				}
			}
			mbar_arrive(&full[b]);
			return true;
		};
		// Waits until every task of macroblock x is done, writes its result, resets its key.
		auto retire = [&](int x) -> bool {
			const int b = x % NB;
			mbar_wait_sleep(&empty[b], (uint32_t)(x / NB) & 1u, abort_flag, &g_full_me_err, kMeErrEmpty);
			bar_producers();
			if (*abort_flag) return false;
			if (pt == 0) {
				const uint32_t key = best[b];
				best[b] = 0xffffffffu;
				int blk, gy0, gx0, cy, cx;
				origin(x, blk, gy0, gx0, cy, cx);
				const int idx = (int)(key & 0x7fffu), iy = idx / Gm::ND, ix = idx - iy * Gm::ND;
				a.out[3 * blk + 0] = cy + iy - R;
				a.out[3 * blk + 1] = cx + ix - R;
				a.out[3 * blk + 2] = (int32_t)(key >> 15);
			}
			return true;
		};
		int retired = 0;
		bool ok = true;
		for (int p = 0; p < PD; ++p) {
			if (p < nj) issue(p);
			else cp_async_commit();
		}
		for (int j = 0; j < nj && ok; ++j) {
			ok = finish(j);
			const int jj = j + PD;
			if (ok && jj < nj && jj >= NB) {
				ok = retire(jj - NB);
				if (ok) ++retired;
			}
			if (ok && jj < nj) issue(jj);
			else cp_async_commit();
		}
		for (; ok && retired < nj; ++retired) ok = retire(retired);
		if (!ok) {
			// let this thread's copies land before the CTA exits; mark the
			// macroblocks the CTA did not finish
			asm volatile("cp.async.wait_all;" ::: "memory");
			volatile int own = 0;
			for (int b = 0; b < NB; ++b)
				if (tma_pending >> b & 1u) mbar_wait(&tbar[b], tma_phase >> b & 1u, &own, &g_full_me_err, kMeErrLoad);
			for (int x = retired + pt; x < nj; x += kProdThreads) {
				int blk, gy0, gx0, cy, cx;
				origin(x, blk, gy0, gx0, cy, cx);
				a.out[3 * blk + 0] = cy;
				a.out[3 * blk + 1] = cx;
				a.out[3 * blk + 2] = -1;
			}
		}
	} else {
		// ------------------------------------------------------------ search
		// task L = c, c + 512, ...: macroblock j = L / TPM (buffer b = j % NB, its
		// use j / NB), task t = L % TPM, kept incrementally (512 < 2 TPM)
		static_assert(kSearchThreads < 2 * TPM, "one wrap per step");
		const int c = tid - kProdThreads;
		int j = c / TPM, t = c - j * TPM;
		int b = j % NB;
		uint32_t use = (uint32_t)(j / NB);
		for (; j < nj;) {
			if (!mbar_wait_sleep(&full[b], use & 1u, abort_flag, &g_full_me_err, kMeErrFull, 2000)) break;
			const int q = t / Gm::ND, ix = t - q * Gm::ND;
			const uint32_t key = ws_task<R>(bufs + b * Gm::BUF, ix, q * Gm::G, a.mul16);
			atomicMin(&best[b], key);
			mbar_arrive(&empty[b]);
			t += kSearchThreads - TPM;  // one macroblock forward, then the remainder
			++j;
			if (++b == NB) { b = 0; ++use; }
			if (t < 0) {  // the step did not reach the next macroblock
				t += TPM;
				--j;
				if (--b < 0) { b = NB - 1; --use; }
			} else if (t >= TPM) {
				t -= TPM;
				++j;
				if (++b == NB) { b = 0; ++use; }
			}
		}
	}
}

template <int R>
umi_status launch_ws(const WsArgs& a0, cudaStream_t st) {
	using Gm = WsGeom<R>;
	WsArgs a = a0;
	CUtensorMap tref;
	std::memset(&tref, 0, sizeof(tref));
	a.tma = 0;
	auto enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(umi::tma_encode_fn());
	if (enc && umi::aligned(a.ref, 16) && a.w % 16 == 0) {
		const cuuint64_t dims[2] = {(cuuint64_t)a.w, (cuuint64_t)a.h};
		const cuuint64_t strides[1] = {(cuuint64_t)a.w};
		const cuuint32_t box[2] = {(cuuint32_t)(4 * Gm::S), (cuuint32_t)Gm::WR};
		const cuuint32_t es[2] = {1, 1};
		const CUresult cr = enc(&tref, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t*>(a.ref), dims, strides, box,
		                        es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
		                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
		a.tma = cr == CUDA_SUCCESS;
	}
	auto kern = full_me_ws_kernel<R>;
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Gm::SMEM),
	                         "cudaFuncSetAttribute"));
	int dev = 0, sms = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	const int grid = std::max(1, std::min(a.slots, sms));
	kern<<<grid, kThreads, Gm::SMEM, st>>>(a, tref);
	return umi::launch_status("full_me_ws_kernel");
}

}  // namespace

namespace umi {

// The warp-specialised search serves 16x16 blocks, r = 32 or 64, argmin
// output, 4-byte-aligned frames with w % 4 == 0.  Returns UMI_ERR_UNSUPPORTED
// (without launching) for anything else: the caller then uses the general
// kernels.
umi_status full_me_ws(const uint8_t* cur, const uint8_t* ref, int h, int w, int b, int r, const int32_t* centers,
                      int32_t* out, const int32_t* list, const int32_t* list_count, int max_slots, cudaStream_t st) {
	if (b != 16 || (r != 32 && r != 64)) return UMI_ERR_UNSUPPORTED;
	if (!aligned(cur, 4) || !aligned(ref, 4) || w % 4 != 0) return UMI_ERR_UNSUPPORTED;
	WsArgs a{};
	a.cur = cur; a.ref = ref; a.centers = centers; a.out = out;
	a.h = h; a.w = w; a.nbx = w / 16; a.nblk = (h / 16) * (w / 16);
	a.list = list; a.list_count = list_count;
	a.slots = list ? std::min(max_slots, a.nblk) : a.nblk;
	a.mul[0] = 1u << 24; a.mul[1] = 1u << 16; a.mul[2] = 1u << 8;
	a.mul16 = 16;
	if (a.nblk == 0 || a.slots <= 0) return UMI_OK;
	return r == 32 ? launch_ws<32>(a, st) : launch_ws<64>(a, st);
}

}  // namespace umi

extern "C" umi_status umi_full_me_error(int32_t* bits, void* stream) {
	const cudaStream_t st = umi::as_stream(stream);
	int v = 0;
	UMI_TRY(umi::cuda_status(cudaMemcpyFromSymbolAsync(&v, g_full_me_err, sizeof(int), 0, cudaMemcpyDeviceToHost, st),
	                         "cudaMemcpyFromSymbolAsync"));
	UMI_TRY(umi::cuda_status(cudaStreamSynchronize(st), "cudaStreamSynchronize"));
	if (bits) *bits = v;
	if (v == 0) return umi::ok();
	const int zero = 0;
	UMI_TRY(umi::cuda_status(cudaMemcpyToSymbolAsync(g_full_me_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st),
	                         "cudaMemcpyToSymbolAsync"));
	UMI_TRY(umi::cuda_status(cudaStreamSynchronize(st), "cudaStreamSynchronize"));
	return umi::fail(UMI_ERR_TIMEOUT,
	                 "full_me: a bounded wait gave up (bits 0x%x: 1 window not full, 2 tasks not done, 4 copy not "
	                 "landed); the affected blocks hold sad = -1",
	                 (unsigned)v);
}
