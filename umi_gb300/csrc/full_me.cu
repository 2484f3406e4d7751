// Full-search block motion estimation on uint8 frames, sm_103a.
//
// Replaces the Execute call of main/full_me.cu:34-64 (MotionEst strategy,
// main/full_me.cu:8-15: sad += |cur - ref| over a b x b block for every
// displacement, reference pixels clamped to the frame) and adds the argmin
// the reference leaves to the caller.
//
// Design (integer pipe, everything on-chip):
//  * one CTA searches M macroblocks; the reference window of each
//    ((b + 2r) x (b + 2r) bytes, edge-replicated) is staged once in shared
//    memory, in four copies shifted by 0..3 bytes so that any horizontal
//    displacement reads whole aligned 32-bit words;
//  * a thread owns one horizontal displacement ix and G consecutive vertical
//    displacements; it keeps a ring of G window rows in registers and streams
//    the current block's rows through one broadcast 128-bit shared load each
//    (5G+4 live words), so two CTAs fit an SM; every (block row, window row)
//    pair costs b/4 `vabsdiff4 ... .add` instructions (4 byte |a-b| plus
//    accumulate in one instruction, the native packed-SAD path);
//  * the argmin is fused: key = (sad << 15) | raster index of (dy, dx), a
//    shared-memory atomicMin per macroblock gives the minimum SAD with the
//    first displacement in raster order (the reference's output order
//    (..., sy, sx), main/full_me.cu:70-71).
//  * the argmin search runs persistent CTAs with two window buffers: the
//    next macroblocks' windows are copied (4-byte cp.async by all threads)
//    while the current ones are searched (full_me_pipe_kernel); the
//    SAD-volume output keeps one CTA per group of macroblocks
//    (full_me_kernel).  The benchmark shapes (16x16 blocks, r = 32 and 64,
//    argmin) go to the warp-specialised kernel of full_me_ws.cu instead.
#include <algorithm>
#include <cstring>

#include <cudaTypedefs.h>

#include "common.h"
#include "tc_common.cuh"

namespace umi {
// Warp-specialised search for 16x16 blocks at r = 32, 64 (full_me_ws.cu);
// UMI_ERR_UNSUPPORTED (nothing launched) for other shapes.
umi_status full_me_ws(const uint8_t* cur, const uint8_t* ref, int h, int w, int b, int r, const int32_t* centers,
                      int32_t* out, const int32_t* list, const int32_t* list_count, int max_slots, cudaStream_t st);
}

namespace {

constexpr int kMaxR = 64;

__device__ __forceinline__ uint32_t sad4_acc(uint32_t a, uint32_t b, uint32_t c) {
	uint32_t d;
	asm("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
	return d;
}

struct MeGeom {
	int h, w, b, r;
	int nbx, nblk;
	int ndx;          // 2r + 1 displacements per axis
	int ng;           // groups of G vertical displacements
	int win_rows;     // rows staged per window (ng*G + b - 1)
	int win_words;    // 32-bit words per staged row
	int win_need;     // words of a row the search reads: (2r + b + 3) / 4 + 1
	int copy_stride;  // words between the four shifted copies
	int mb_stride;    // words per macroblock (4 copies + current block)
	int m;            // macroblocks per CTA
	int tasks_per_mb; // ndx * ng
	int vec_ok;       // ref and cur are 4-byte aligned and w % 4 == 0: word loads / 4-byte cp.async allowed
	int nx32;         // largest multiple of 32 <= ndx: displacements served by whole warps
	int ng2;          // argmin search: groups of G2 vertical displacements for the ndx - nx32 leftover columns (0: none)
	int tasks_pipe;   // argmin search tasks per macroblock: ng*nx32 + ng2*(ndx - nx32), or ndx*ng when ng2 == 0
	const int32_t* list;        // optional: search only these blocks (slot i -> block list[i])
	const int32_t* list_count;  // number of valid slots of `list` (device word)
	int slots;                  // slots covered by the grid (nblk, or the list's capacity)
};

// Block searched by slot `slot`, or -1 past the last slot.
__device__ __forceinline__ int slot_block(const MeGeom& g, int slot) {
	if (g.list) return slot < *g.list_count ? g.list[slot] : -1;
	return slot < g.nblk ? slot : -1;
}

// Register budget per instantiation: the benchmark shape (b = 16, G = 13,
// 352 threads) is held to 80 registers so that two CTAs (6 warps per SM
// sub-partition x 80 x 32 <= 16K registers) fit an SM.
// The other shapes get a budget of about 5G + 30 (ring + accumulators + addressing).
template <int B, int G> struct MeRegs { static constexpr int value = B == 16 ? (5 * G + 31) / 8 * 8 + 8 : 64; };
template <> struct MeRegs<16, 13> { static constexpr int value = 80; };

template <int B, int G, bool VOLUME>
__global__ void __launch_bounds__(512) __maxnreg__((MeRegs<B, G>::value))
full_me_kernel(const uint8_t* __restrict__ cur, const uint8_t* __restrict__ ref, const int32_t* __restrict__ centers,
               int32_t* __restrict__ out, const MeGeom g) {
	extern __shared__ __align__(128) uint32_t smem[];
	constexpr int BW = B / 4;  // words per block row
	__shared__ uint32_t best[64];
	const int tid = threadIdx.x;
	const int mb0 = blockIdx.x * g.m;

	// Staging walks (row, word) pairs: a thread starts at word t % win_words of
	// row t / win_words and advances by whole rows (one division per thread).
	const int rstep = blockDim.x / g.win_words;  // host guarantees blockDim >= win_words
	const int wd0 = tid - (tid / g.win_words) * g.win_words;
	const int row0 = tid / g.win_words;
	const bool stager = row0 < rstep;  // threads past rstep*win_words idle while staging
	// 1. Stage windows (copy 0) and current blocks.
	for (int m = 0; m < g.m; ++m) {
		const int blk = slot_block(g, mb0 + m);
		if (blk < 0) break;
		const int by = blk / g.nbx, bx = blk - by * g.nbx;
		const int cy = centers ? centers[2 * blk] : 0, cx = centers ? centers[2 * blk + 1] : 0;
		const int gy0 = by * B + cy - g.r, gx0 = bx * B + cx - g.r;
		uint32_t* win = smem + m * g.mb_stride;
		const int gx = gx0 + 4 * wd0;
		const bool vec = g.vec_ok && gx >= 0 && gx + 3 < g.w && (gx & 3) == 0;
		int xs[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) xs[k] = min(max(gx + k, 0), g.w - 1);
		if (stager) {
			for (int row = row0; row < g.win_rows; row += rstep) {
				const int gy = min(max(gy0 + row, 0), g.h - 1);
				const uint8_t* src = ref + (size_t)gy * g.w;
				uint32_t v;
				if (vec) {
					v = __ldg(reinterpret_cast<const uint32_t*>(src + gx));
				} else {
					v = 0;
#pragma unroll
					for (int k = 0; k < 4; ++k) v |= (uint32_t)__ldg(src + xs[k]) << (8 * k);
				}
				win[row * g.win_words + wd0] = v;
			}
		}
		uint32_t* cb = win + 4 * g.copy_stride;
		if (tid < B * BW) {
			const int row = tid / BW, wd = tid - row * BW;
			const uint8_t* src = cur + (size_t)(by * B + row) * g.w + bx * B + 4 * wd;
			uint32_t v = 0;
#pragma unroll
			for (int k = 0; k < 4; ++k) v |= (uint32_t)__ldg(src + k) << (8 * k);
			cb[tid] = v;
		}
		if (tid == 0) best[m] = 0xffffffffu;
	}
	__syncthreads();
	// 2. Shifted copies s = 1..3: word k holds bytes [4k+s, 4k+s+4) of the row.
	for (int m = 0; m < g.m; ++m) {
		if (slot_block(g, mb0 + m) < 0 || !stager) break;
		uint32_t* win = smem + m * g.mb_stride;
		const bool last = wd0 + 1 == g.win_words;
		for (int row = row0; row < g.win_rows; row += rstep) {
			const int j = row * g.win_words + wd0;
			const uint32_t lo = win[j], hi = last ? 0u : win[j + 1];
			win[g.copy_stride + j] = __funnelshift_r(lo, hi, 8);
			win[2 * g.copy_stride + j] = __funnelshift_r(lo, hi, 16);
			win[3 * g.copy_stride + j] = __funnelshift_r(lo, hi, 24);
		}
	}
	__syncthreads();

	// 3. Search.
	const int total = g.m * g.tasks_per_mb;
	for (int t = tid; t < total; t += blockDim.x) {
		const int m = t / g.tasks_per_mb;
		const int rem = t - m * g.tasks_per_mb;
		// Tasks [0, ng*nx32) cover ix < nx32 with whole warps per group (one
		// row per warp-wide load: conflict-free); the remaining columns of all
		// groups follow.
		int grp, ix;
		const int main_tasks = g.ng * g.nx32;
		if (rem < main_tasks) {
			grp = rem / g.nx32;
			ix = rem - grp * g.nx32;
		} else {
			const int rw = g.ndx - g.nx32, r2 = rem - main_tasks;
			grp = r2 / rw;
			ix = g.nx32 + (r2 - grp * rw);
		}
		const int blk = slot_block(g, mb0 + m);
		if (blk < 0) continue;
		const uint32_t* win = smem + m * g.mb_stride;
		const uint32_t* cb = win + 4 * g.copy_stride;
		const uint32_t* wp = win + (ix & 3) * g.copy_stride + (ix >> 2) + grp * G * g.win_words;
		// ring[s] holds window row r with r % G == s; at block row py the G
		// candidates q = 0..G-1 need window rows py .. py+G-1.
		uint32_t ring[G][BW];
		uint32_t acc[G];
#pragma unroll
		for (int q = 0; q < G; ++q) {
			acc[q] = 0;
#pragma unroll
			for (int k = 0; k < BW; ++k) ring[q][k] = wp[q * g.win_words + k];
		}
#pragma unroll
		for (int py = 0; py < B; ++py) {
			uint32_t cv[BW];
			if (BW == 4) {
				const uint4 c4 = *reinterpret_cast<const uint4*>(cb + py * BW);  // same address in every lane
				cv[0] = c4.x; cv[1] = c4.y; cv[2 % BW] = c4.z; cv[3 % BW] = c4.w;
			} else {
#pragma unroll
				for (int k = 0; k < BW; ++k) cv[k] = cb[py * BW + k];
			}
			if (py > 0) {
				const int r = py + G - 1;
#pragma unroll
				for (int k = 0; k < BW; ++k) ring[r % G][k] = wp[r * g.win_words + k];
			}
			// k outer, q inner: consecutive instructions update different accumulators.
#pragma unroll
			for (int k = 0; k < BW; ++k)
#pragma unroll
				for (int q = 0; q < G; ++q) acc[q] = sad4_acc(cv[k], ring[(py + q) % G][k], acc[q]);
		}
		const int iy0 = grp * G;
		if (VOLUME) {
			int32_t* o = out + (size_t)blk * g.ndx * g.ndx;
#pragma unroll
			for (int q = 0; q < G; ++q)
				if (iy0 + q < g.ndx) o[(iy0 + q) * g.ndx + ix] = (int32_t)acc[q];
		} else {
			uint32_t key = 0xffffffffu;
#pragma unroll
			for (int q = 0; q < G; ++q)
				if (iy0 + q < g.ndx) key = min(key, (acc[q] << 15) | (uint32_t)((iy0 + q) * g.ndx + ix));
			atomicMin(&best[m], key);
		}
	}
	if (VOLUME) return;
	__syncthreads();
	for (int m = tid; m < g.m; m += blockDim.x) {
		const int blk = slot_block(g, mb0 + m);
		if (blk < 0) break;
		const uint32_t key = best[m];
		const int idx = (int)(key & 0x7fffu);
		const int iy = idx / g.ndx, ix = idx - iy * g.ndx;
		const int cy = centers ? centers[2 * blk] : 0, cx = centers ? centers[2 * blk + 1] : 0;
		out[3 * blk + 0] = cy + iy - g.r;
		out[3 * blk + 1] = cx + ix - g.r;
		out[3 * blk + 2] = (int32_t)(key >> 15);
	}
}

// ---- Persistent, double-buffered form of the argmin search.
// Each CTA walks groups of g.m macroblocks (group gi = blockIdx.x, +gridDim.x,
// ...).  While it searches group gi out of one shared-memory buffer, the
// windows of its next group are copied into the other buffer with cp.async
// (windows wholly inside the frame; windows that need edge replication are
// staged with clamped loads as before), so the copy latency hides behind the
// search.  Same tasks, same arithmetic, same argmin key: results are
// identical to full_me_kernel.

__device__ __forceinline__ void cp_async4(uint32_t* dst, const void* src) {
	const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
	asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Stage copy 0 of every window of group gi (and its current blocks) into buf.
// Stage copy 0 of every window of group gi (and its current blocks) into buf.
template <int B>
__device__ __forceinline__ void me_stage_group(const MeGeom& g, uint32_t* buf, int gi, const uint8_t* __restrict__ cur,
                                               const uint8_t* __restrict__ ref, const int32_t* __restrict__ centers,
                                               int tid, int row0, int wd0, int rstep, bool stager) {
	constexpr int BW = B / 4;
	for (int m = 0; m < g.m; ++m) {
		const int blk = slot_block(g, gi * g.m + m);
		if (blk < 0) break;
		const int by = blk / g.nbx, bx = blk - by * g.nbx;
		const int cy = centers ? centers[2 * blk] : 0, cx = centers ? centers[2 * blk + 1] : 0;
		const int gy0 = by * B + cy - g.r, gx0 = bx * B + cx - g.r;
		uint32_t* win = buf + m * g.mb_stride;
		const bool inside = g.vec_ok && gy0 >= 0 && gy0 + g.win_rows <= g.h && gx0 >= 0 &&
		                    gx0 + 4 * g.win_words <= g.w && (gx0 & 3) == 0;
		if (stager) {
			if (inside) {
				const uint8_t* src = ref + (size_t)gy0 * g.w + gx0 + 4 * wd0;
				for (int row = row0; row < g.win_rows; row += rstep)
					cp_async4(win + row * g.win_words + wd0, src + (size_t)row * g.w);
			} else {
				const int gx = gx0 + 4 * wd0;
				const bool vec = g.vec_ok && gx >= 0 && gx + 3 < g.w && (gx & 3) == 0;
				int xs[4];
#pragma unroll
				for (int k = 0; k < 4; ++k) xs[k] = min(max(gx + k, 0), g.w - 1);
				for (int row = row0; row < g.win_rows; row += rstep) {
					const int gy = min(max(gy0 + row, 0), g.h - 1);
					const uint8_t* src = ref + (size_t)gy * g.w;
					uint32_t v;
					if (vec) {
						v = __ldg(reinterpret_cast<const uint32_t*>(src + gx));
					} else {
						v = 0;
#pragma unroll
						for (int k = 0; k < 4; ++k) v |= (uint32_t)__ldg(src + xs[k]) << (8 * k);
					}
					win[row * g.win_words + wd0] = v;
				}
			}
		}
		uint32_t* cb = win + 4 * g.copy_stride;
		if (tid < B * BW) {
			const int row = tid / BW, wd = tid - row * BW;
			const uint8_t* src = cur + (size_t)(by * B + row) * g.w + bx * B + 4 * wd;
			if (g.vec_ok) {
				cp_async4(cb + tid, src);
			} else {
				uint32_t v = 0;
#pragma unroll
				for (int k = 0; k < 4; ++k) v |= (uint32_t)__ldg(src + k) << (8 * k);
				cb[tid] = v;
			}
		}
	}
}

// Window origin of slot `slot`'s block, or false past the last slot.
template <int B>
__device__ __forceinline__ bool me_window(const MeGeom& g, const int32_t* __restrict__ centers, int slot, int& blk,
                                          int& gy0, int& gx0) {
	blk = slot_block(g, slot);
	if (blk < 0) return false;
	const int by = blk / g.nbx, bx = blk - by * g.nbx;
	const int cy = centers ? centers[2 * blk] : 0, cx = centers ? centers[2 * blk + 1] : 0;
	gy0 = by * B + cy - g.r;
	gx0 = bx * B + cx - g.r;
	return true;
}

// Copies 1..3 of every window of group gi (word k of copy s holds bytes
// [4k+s, 4k+s+4) of the row).
__device__ __forceinline__ void me_shift_group(const MeGeom& g, uint32_t* buf, int gi, int row0, int wd0, int rstep,
                                               bool stager) {
	if (!stager) return;
	for (int m = 0; m < g.m; ++m) {
		if (slot_block(g, gi * g.m + m) < 0) break;
		uint32_t* win = buf + m * g.mb_stride;
		const bool last = wd0 + 1 == g.win_words;
		for (int row = row0; row < g.win_rows; row += rstep) {
			const int j = row * g.win_words + wd0;
			const uint32_t lo = win[j], hi = last ? 0u : win[j + 1];
			win[g.copy_stride + j] = __funnelshift_r(lo, hi, 8);
			win[2 * g.copy_stride + j] = __funnelshift_r(lo, hi, 16);
			win[3 * g.copy_stride + j] = __funnelshift_r(lo, hi, 24);
		}
	}
}

// One search task: horizontal displacement ix, vertical displacements
// iy0 .. iy0+GG-1 (those < ndx) of the window at `win`; returns the argmin key.
template <int B, int GG>
__device__ __forceinline__ uint32_t me_task(const MeGeom& g, const uint32_t* win, int ix, int iy0) {
	constexpr int BW = B / 4;
	const uint32_t* cb = win + 4 * g.copy_stride;
	const uint32_t* wp = win + (ix & 3) * g.copy_stride + (ix >> 2) + iy0 * g.win_words;
	uint32_t ring[GG][BW];
	uint32_t acc[GG];
#pragma unroll
	for (int q = 0; q < GG; ++q) {
		acc[q] = 0;
#pragma unroll
		for (int k = 0; k < BW; ++k) ring[q][k] = wp[q * g.win_words + k];
	}
#pragma unroll
	for (int py = 0; py < B; ++py) {
		uint32_t cv[BW];
		if (BW == 4) {
			const uint4 c4 = *reinterpret_cast<const uint4*>(cb + py * BW);
			cv[0] = c4.x; cv[1] = c4.y; cv[2 % BW] = c4.z; cv[3 % BW] = c4.w;
		} else {
#pragma unroll
			for (int k = 0; k < BW; ++k) cv[k] = cb[py * BW + k];
		}
		if (py > 0) {
			const int r = py + GG - 1;
#pragma unroll
			for (int k = 0; k < BW; ++k) ring[r % GG][k] = wp[r * g.win_words + k];
		}
#pragma unroll
		for (int k = 0; k < BW; ++k)
#pragma unroll
			for (int q = 0; q < GG; ++q) acc[q] = sad4_acc(cv[k], ring[(py + q) % GG][k], acc[q]);
	}
	uint32_t key = 0xffffffffu;
#pragma unroll
	for (int q = 0; q < GG; ++q)
		if (iy0 + q < g.ndx) key = min(key, (acc[q] << 15) | (uint32_t)((iy0 + q) * g.ndx + ix));
	return key;
}

// Vertical displacements per task of the leftover columns (ix >= nx32): at
// most one warp of short tasks instead of a warp of full-length tasks with
// few lanes active.
constexpr int G2 = 5;

template <int B, int G>
__global__ void __launch_bounds__(512) __maxnreg__((MeRegs<B, G>::value))
full_me_pipe_kernel(const uint8_t* __restrict__ cur, const uint8_t* __restrict__ ref,
                    const int32_t* __restrict__ centers, int32_t* __restrict__ out, const MeGeom g) {
	extern __shared__ __align__(128) uint32_t smem[];
	__shared__ uint32_t best[2][64];
	const int tid = threadIdx.x;
	const int ngroups = (g.slots + g.m - 1) / g.m;
	const int rstep = blockDim.x / g.win_words;  // host guarantees blockDim >= win_words
	const int row0 = tid / g.win_words;
	const int wd0 = tid - row0 * g.win_words;
	const bool stager = row0 < rstep;
	const int buf_words = g.m * g.mb_stride;
	int gi = blockIdx.x;
	if (gi >= ngroups || slot_block(g, gi * g.m) < 0) return;  // uniform over the CTA
	if (tid < 64) best[0][tid] = best[1][tid] = 0xffffffffu;
	me_stage_group<B>(g, smem, gi, cur, ref, centers, tid, row0, wd0, rstep, stager);
	cp_async_wait_all();
	__syncthreads();
	me_shift_group(g, smem, gi, row0, wd0, rstep, stager);
	__syncthreads();
	int cbuf = 0;
	const int total = g.m * g.tasks_pipe;
	while (true) {
		const int ngi = gi + gridDim.x;
		const bool has_next = ngi < ngroups && slot_block(g, ngi * g.m) >= 0;
		uint32_t* cur_buf = smem + cbuf * buf_words;
		uint32_t* next_buf = smem + (cbuf ^ 1) * buf_words;
		if (has_next) me_stage_group<B>(g, next_buf, ngi, cur, ref, centers, tid, row0, wd0, rstep, stager);
		// Search group gi: tasks [0, ng*nx32) are whole-warp columns with G
		// vertical displacements each; the leftover columns follow in tasks of G2.
		for (int t = tid; t < total; t += blockDim.x) {
			const int m = t / g.tasks_pipe;
			const int rem = t - m * g.tasks_pipe;
			if (slot_block(g, gi * g.m + m) < 0) continue;
			const uint32_t* win = cur_buf + m * g.mb_stride;
			const int main_tasks = g.ng * g.nx32;
			uint32_t key;
			if (rem < main_tasks) {
				const int grp = rem / g.nx32;
				const int ix = rem - grp * g.nx32;
				key = me_task<B, G>(g, win, ix, grp * G);
			} else {
				const int rw = g.ndx - g.nx32, r2 = rem - main_tasks;
				const int grp = r2 / rw;
				const int ix = g.nx32 + (r2 - grp * rw);
				key = g.ng2 ? me_task<B, G2>(g, win, ix, grp * G2) : me_task<B, G>(g, win, ix, grp * G);
			}
			atomicMin(&best[cbuf][m], key);
		}
		cp_async_wait_all();
		__syncthreads();  // search of gi done; this thread's copies for ngi landed (all threads: barrier)
		if (tid < g.m) {
			const int blk = slot_block(g, gi * g.m + tid);
			if (blk >= 0) {
				const uint32_t key = best[cbuf][tid];
				const int idx = (int)(key & 0x7fffu);
				const int iy = idx / g.ndx, ix = idx - iy * g.ndx;
				const int cy = centers ? centers[2 * blk] : 0, cx = centers ? centers[2 * blk + 1] : 0;
				out[3 * blk + 0] = cy + iy - g.r;
				out[3 * blk + 1] = cx + ix - g.r;
				out[3 * blk + 2] = (int32_t)(key >> 15);
			}
			best[cbuf][tid] = 0xffffffffu;
		}
		if (!has_next) break;
		me_shift_group(g, next_buf, ngi, row0, wd0, rstep, stager);
		__syncthreads();
		gi = ngi;
		cbuf ^= 1;
	}
}

// ---- Small-range argmin search (16x16 blocks, r <= 7): the refine around
// proposal centres.  A warp serves floor(32 / (2r + 1)) blocks.  It first
// stages, for each of them, the (16 + 2r)-row window (rows clamped to the
// frame, words from a 4-byte-aligned left edge, bytes outside the frame
// replicated) and the current block in its shared-memory slice: all loads in
// flight at once.  Then a lane owns one horizontal displacement of one block
// and walks the block's 16 rows once, keeping the 2r + 1 window rows that
// the current block row meets (at the 2r + 1 vertical displacements) in a
// register ring: per block row one window row enters (four words realigned by
// prmt from five) and the block row (one broadcast 16-byte load) is compared
// with every ring row: 16 (2r + 1) x 4 vabsdiff4 per lane.  The argmin key
// (sad << 8) | raster index is reduced over each block's lanes by shuffles.
// Same candidates, clamping and tie-break as full_me_kernel.  Nine CTAs per
// SM (56 registers, no spills): the 10 800 warps of a 4K +-4 refine run in
// two waves of 36 warps per SM instead of three of 32 (28 us instead of 32).
template <int R>
__global__ void __launch_bounds__(128, 9) me_small_kernel(const uint8_t* __restrict__ cur, const uint8_t* __restrict__ ref,
                                                       const int32_t* __restrict__ centers, int32_t* __restrict__ out,
                                                       int h, int w, int nbx, int nblk) {
	constexpr int ND = 2 * R + 1, BPW = 32 / ND, WR = 16 + 2 * R;
	constexpr int WW = (2 * R + 22) / 4;          // words per window row: 16 + 2r bytes from an offset 0..3
	constexpr int WIN = (WR * WW + 3) & ~3;       // window words, rounded so the block starts 16-byte aligned
	constexpr int SEG = WIN + 64;                 // window + current block
	constexpr int RPP = 32 / WW;                  // window rows staged per pass
	static_assert(ND <= 16 && ND * ND <= 256, "key layout and segment reduction");
	__shared__ __align__(16) uint32_t sm[4][BPW * SEG];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int blk0 = (int)((size_t)blockIdx.x * 4 + warp) * BPW;
	uint32_t* ws = sm[warp];
	// 1. Staging (lane -> (row rr + RPP * pass, word kk) of the window, (row, word) of the block).
	const int kk = lane % WW, rr = lane / WW;
#pragma unroll
	for (int s = 0; s < BPW; ++s) {
		const int b = blk0 + s;
		if (b >= nblk) break;  // warp-uniform
		const int by = b / nbx, bx = b - by * nbx;
		const int cy = centers ? __ldg(centers + 2 * b) : 0, cx = centers ? __ldg(centers + 2 * b + 1) : 0;
		const int xa0 = (16 * bx + cx - R) & ~3, gx = xa0 + 4 * kk;
		const bool word = gx >= 0 && gx + 4 <= w;  // 4-byte aligned: ref aligned, w % 4 == 0
		const int y0 = 16 * by + cy - R;
		uint32_t* dst = ws + s * SEG;
		if (rr < RPP) {
#pragma unroll
			for (int pass = 0; pass < (WR + RPP - 1) / RPP; ++pass) {
				const int r = rr + RPP * pass;
				if (r < WR) {
					const uint8_t* row = ref + (size_t)min(max(y0 + r, 0), h - 1) * w;
					uint32_t v;
					if (word) {
						v = __ldg(reinterpret_cast<const uint32_t*>(row + gx));
					} else {
						v = 0;
#pragma unroll
						for (int j = 0; j < 4; ++j) v |= (uint32_t)__ldg(row + min(max(gx + j, 0), w - 1)) << (8 * j);
					}
					dst[r * WW + kk] = v;
				}
			}
		}
		const uint32_t* cb = reinterpret_cast<const uint32_t*>(cur + (size_t)(16 * by) * w + 16 * bx);
#pragma unroll
		for (int pass = 0; pass < 2; ++pass) {
			const int r = (lane >> 2) + 8 * pass, k = lane & 3;
			dst[WIN + 4 * r + k] = __ldg(cb + (size_t)r * (w >> 2) + k);
		}
	}
	__syncwarp();
	// 2. Search.
	const int seg = lane / ND, dx = lane - seg * ND;
	const int blk = blk0 + seg;
	const bool active = seg < BPW && blk < nblk;
	uint32_t key = 0xffffffffu;
	int cy = 0, cx = 0;
	if (active) {
		const int bx = blk - (blk / nbx) * nbx;
		if (centers) { cy = __ldg(centers + 2 * blk); cx = __ldg(centers + 2 * blk + 1); }
		const int off = ((16 * bx + cx - R) & 3) + dx;  // byte of this lane's first column in a staged row
		const uint32_t sel = 0x3210u + 0x1111u * (uint32_t)(off & 3);
		const uint32_t* win = ws + seg * SEG + (off >> 2);  // words off/4 .. off/4 + 4 < WW
		const uint4* blkrows = reinterpret_cast<const uint4*>(ws + seg * SEG + WIN);
		auto window_row = [&](int wr, uint32_t (&v)[4]) {
			uint32_t u[5];
#pragma unroll
			for (int k = 0; k < 5; ++k) u[k] = win[wr * WW + k];
#pragma unroll
			for (int k = 0; k < 4; ++k) v[k] = __byte_perm(u[k], u[k + 1], sel);
		};
		uint32_t ring[ND][4], cost[ND];
#pragma unroll
		for (int d = 0; d < ND; ++d) cost[d] = 0;
#pragma unroll
		for (int wr = 0; wr < ND - 1; ++wr) window_row(wr, ring[wr]);
#pragma unroll
		for (int br = 0; br < 16; ++br) {
			window_row(br + ND - 1, ring[(br + ND - 1) % ND]);
			const uint4 cv = blkrows[br];
			const uint32_t c[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
			for (int d = 0; d < ND; ++d)  // block row br meets window row br + d at vertical displacement d - R
#pragma unroll
				for (int k = 0; k < 4; ++k) cost[d] = sad4_acc(c[k], ring[(br + d) % ND][k], cost[d]);
		}
#pragma unroll
		for (int d = 0; d < ND; ++d) key = min(key, (cost[d] << 8) | (uint32_t)(d * ND + dx));
	}
#pragma unroll
	for (int o = 1; o < 16; o <<= 1) {  // segmented min over the block's ND <= 16 lanes
		const uint32_t v = __shfl_down_sync(0xffffffffu, key, o);
		if (dx + o < ND) key = min(key, v);
	}
	if (active && dx == 0) {
		const int idx = (int)(key & 0xffu), iy = idx / ND, ix = idx - iy * ND;
		out[3 * blk + 0] = cy + iy - R;
		out[3 * blk + 1] = cx + ix - R;
		out[3 * blk + 2] = (int32_t)(key >> 8);
	}
}

template <int R>
umi_status launch_small_r(const uint8_t* cur, const uint8_t* ref, const int32_t* centers, int32_t* out, const MeGeom& g,
                          cudaStream_t st) {
	constexpr int BPW = 32 / (2 * R + 1);
	const int warps = (g.nblk + BPW - 1) / BPW;
	me_small_kernel<R><<<(warps + 3) / 4, 128, 0, st>>>(cur, ref, centers, out, g.h, g.w, g.nbx, g.nblk);
	return umi::launch_status("me_small_kernel");
}

umi_status launch_small(const uint8_t* cur, const uint8_t* ref, const int32_t* centers, int32_t* out, const MeGeom& g,
                        cudaStream_t st) {
	switch (g.r) {
		case 1: return launch_small_r<1>(cur, ref, centers, out, g, st);
		case 2: return launch_small_r<2>(cur, ref, centers, out, g, st);
		case 3: return launch_small_r<3>(cur, ref, centers, out, g, st);
		case 4: return launch_small_r<4>(cur, ref, centers, out, g, st);
		case 5: return launch_small_r<5>(cur, ref, centers, out, g, st);
		case 6: return launch_small_r<6>(cur, ref, centers, out, g, st);
		default: return launch_small_r<7>(cur, ref, centers, out, g, st);
	}
}

// Vertical displacements per thread: the candidate that wastes the fewest
// padded rows (ng*G - ndx), larger G on ties (fewer window-row loads).
int pick_g(int ndx) {
	const int cands[] = {15, 13, 9, 5};
	int best = cands[0], waste = 1 << 30;
	for (int gcand : cands) {
		const int ng = (ndx + gcand - 1) / gcand;
		const int wst = ng * gcand - ndx;
		if (wst < waste) { waste = wst; best = gcand; }
	}
	return best;
}

template <int B, int G, bool V>
umi_status launch_g(const uint8_t* cur, const uint8_t* ref, const int32_t* centers, int32_t* out, const MeGeom& g,
                    int threads, size_t smem, cudaStream_t st) {
	auto kern = full_me_kernel<B, G, V>;
	if (smem > 48 * 1024) UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                                                 (int)smem), "cudaFuncSetAttribute"));
	// Without this the driver may pick a small shared-memory carveout and
	// allow only one CTA per SM.
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
	                                              (int)cudaSharedmemCarveoutMaxShared), "cudaFuncSetAttribute"));
	const int grid = (g.slots + g.m - 1) / g.m;
	kern<<<grid, threads, smem, st>>>(cur, ref, centers, out, g);
	return umi::launch_status("full_me_kernel");
}

template <int B, int G>
umi_status launch_pipe_g(const uint8_t* cur, const uint8_t* ref, const int32_t* centers, int32_t* out, const MeGeom& g,
                         int threads, size_t smem, cudaStream_t st) {
	auto kern = full_me_pipe_kernel<B, G>;
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
	                         "cudaFuncSetAttribute"));
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
	                                              (int)cudaSharedmemCarveoutMaxShared), "cudaFuncSetAttribute"));
	int dev = 0, sms = 0, per_sm = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	UMI_TRY(umi::cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem),
	                         "cudaOccupancyMaxActiveBlocksPerMultiprocessor"));
	if (per_sm < 1) return umi::fail(UMI_ERR_UNSUPPORTED, "full_me: %zu bytes of shared memory per CTA do not fit", smem);
	const int ngroups = (g.slots + g.m - 1) / g.m;
	const int grid = std::min(ngroups, per_sm * sms);
	kern<<<grid, threads, smem, st>>>(cur, ref, centers, out, g);
	return umi::launch_status("full_me_pipe_kernel");
}

template <int B>
umi_status launch_pipe_b(int G, const uint8_t* cur, const uint8_t* ref, const int32_t* centers, int32_t* out,
                         const MeGeom& g, int threads, size_t smem, cudaStream_t st) {
	switch (G) {
		case 5: return launch_pipe_g<B, 5>(cur, ref, centers, out, g, threads, smem, st);
		case 9: return launch_pipe_g<B, 9>(cur, ref, centers, out, g, threads, smem, st);
		case 13: return launch_pipe_g<B, 13>(cur, ref, centers, out, g, threads, smem, st);
		default: return launch_pipe_g<B, 15>(cur, ref, centers, out, g, threads, smem, st);
	}
}

template <int B, bool V>
umi_status launch_b(int G, const uint8_t* cur, const uint8_t* ref, const int32_t* centers, int32_t* out,
                    const MeGeom& g, int threads, size_t smem, cudaStream_t st) {
	switch (G) {
		case 5: return launch_g<B, 5, V>(cur, ref, centers, out, g, threads, smem, st);
		case 9: return launch_g<B, 9, V>(cur, ref, centers, out, g, threads, smem, st);
		case 13: return launch_g<B, 13, V>(cur, ref, centers, out, g, threads, smem, st);
		default: return launch_g<B, 15, V>(cur, ref, centers, out, g, threads, smem, st);
	}
}

umi_status full_me_common(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b, int32_t r,
                          const int32_t* centers, int32_t* out, bool volume, void* stream,
                          const int32_t* list = nullptr, const int32_t* list_count = nullptr, int32_t max_slots = 0) {
	if (!cur || !ref || !out) return umi::fail(UMI_ERR_INVALID_ARG, "full_me: null pointer");
	if (h < 0 || w < 0) return umi::fail(UMI_ERR_INVALID_ARG, "full_me: negative size %dx%d", h, w);
	if (b != 8 && b != 16) return umi::fail(UMI_ERR_UNSUPPORTED, "full_me: block size %d (supported: 8, 16)", b);
	if (r < 1 || r > kMaxR) return umi::fail(UMI_ERR_UNSUPPORTED, "full_me: search range %d (supported 1..%d)", r, kMaxR);
	MeGeom g{};
	g.h = h; g.w = w; g.b = b; g.r = r;
	g.nbx = w / b;
	g.nblk = (h / b) * g.nbx;
	if (g.nblk == 0) return umi::ok();
	g.list = list;
	g.list_count = list_count;
	g.slots = list ? std::min(max_slots, g.nblk) : g.nblk;
	if (g.slots <= 0) return umi::ok();
	g.ndx = 2 * r + 1;
	const int G = pick_g(g.ndx);
	g.ng = (g.ndx + G - 1) / G;
	g.win_rows = g.ng * G + b - 1;
	g.win_need = (2 * r + b + 3) / 4 + 1;
	g.vec_ok = umi::aligned(ref, 4) && umi::aligned(cur, 4) && (w % 4) == 0;
	if (!volume) {  // the benchmark ranges: warp-specialised kernel (full_me_ws.cu)
		const umi_status rc = umi::full_me_ws(cur, ref, h, w, b, r, centers, out, list, list_count, max_slots,
		                                      umi::as_stream(stream));
		if (rc != UMI_ERR_UNSUPPORTED) return rc == UMI_OK ? umi::ok() : rc;
	}
	if (!volume && !list && b == 16 && r <= 7 && g.vec_ok) {  // small windows: registers only
		const umi_status rc = launch_small(cur, ref, centers, out, g, umi::as_stream(stream));
		return rc == UMI_OK ? umi::ok() : rc;
	}
	g.win_words = g.win_need;
	const int copy = g.win_rows * g.win_words;
	g.copy_stride = ((copy + 31) / 32) * 32 + 8;  // copies land 8 banks apart
	g.mb_stride = 4 * g.copy_stride + b * b / 4 + 4;
	g.mb_stride = (g.mb_stride + 3) & ~3;  // current block 16-byte aligned
	g.tasks_per_mb = g.ndx * g.ng;
	g.nx32 = (g.ndx / 32) * 32;
	g.ng2 = (g.nx32 > 0 && g.ndx > g.nx32) ? (g.ndx + G2 - 1) / G2 : 0;
	g.tasks_pipe = g.ng2 ? g.ng * g.nx32 + g.ng2 * (g.ndx - g.nx32) : g.tasks_per_mb;
	// Macroblocks per CTA: enough tasks to fill at least ~256 threads, within
	// 96 KB of shared memory (the argmin search keeps two such buffers) and
	// the 64-slot argmin table.
	int m = std::max(1, 256 / g.tasks_per_mb);
	// Argmin search with one macroblock's tasks filling the CTA: two per group
	// when two CTAs still fit an SM (half the group barriers per macroblock).
	if (!volume && m == 1 && 2 * 2 * (size_t)g.mb_stride * 4 <= 112 * 1024) m = 2;
	const int max_m_smem = std::max(1, (int)((96 * 1024) / (g.mb_stride * 4)));
	m = std::min(std::min(m, max_m_smem), 64);
	g.m = m;
	// Threads: one task each when they fit 512, else as few rounds as possible.
	// Staging needs one thread per current-block word (b*b/4 <= 64) and per
	// window word of a row (<= 37).
	auto threads_for = [](int total) {
		int t = ((total + 31) / 32) * 32;
		if (t > 512) {
			const int iters = (total + 511) / 512;
			t = (((total + iters - 1) / iters) + 31) / 32 * 32;
		}
		return std::max(t, 64);
	};
	const int threads = threads_for(m * g.tasks_per_mb);
	const size_t smem = (size_t)m * g.mb_stride * 4;
	const cudaStream_t st = umi::as_stream(stream);
	umi_status rc;
	if (!volume && 2 * smem <= 200 * 1024) {  // double-buffered persistent search
		const int tp = threads_for(m * g.tasks_pipe);
		rc = b == 16 ? launch_pipe_b<16>(G, cur, ref, centers, out, g, tp, 2 * smem, st)
		             : launch_pipe_b<8>(G, cur, ref, centers, out, g, tp, 2 * smem, st);
	} else if (b == 16)
		rc = volume ? launch_b<16, true>(G, cur, ref, centers, out, g, threads, smem, st)
		            : launch_b<16, false>(G, cur, ref, centers, out, g, threads, smem, st);
	else
		rc = volume ? launch_b<8, true>(G, cur, ref, centers, out, g, threads, smem, st)
		            : launch_b<8, false>(G, cur, ref, centers, out, g, threads, smem, st);
	return rc == UMI_OK ? umi::ok() : rc;
}

}  // namespace

extern "C" umi_status umi_full_me_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b,
                                     int32_t r, const int32_t* centers, int32_t* mv, void* stream) {
	return full_me_common(cur, ref, h, w, b, r, centers, mv, false, stream);
}

extern "C" umi_status umi_full_me_sad_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b,
                                         int32_t r, int32_t* sad, void* stream) {
	return full_me_common(cur, ref, h, w, b, r, nullptr, sad, true, stream);
}

extern "C" umi_status umi_full_me_u8_list(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b,
                                          int32_t r, const int32_t* centers, const int32_t* blocks,
                                          const int32_t* n_blocks, int32_t max_blocks, int32_t* mv, void* stream) {
	if (!blocks || !n_blocks) return umi::fail(UMI_ERR_INVALID_ARG, "full_me_list: null block list");
	if (max_blocks < 0) return umi::fail(UMI_ERR_INVALID_ARG, "full_me_list: negative capacity");
	return full_me_common(cur, ref, h, w, b, r, centers, mv, false, stream, blocks, n_blocks, max_blocks);
}
