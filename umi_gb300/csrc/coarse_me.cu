// Coarse-to-fine motion proposal for block motion estimation (sm_103a).
//
// No counterpart in the reference.  Every 16x16 block of `cur` is reduced to
// 4 x 4 cells, each the rounded mean of a 4x4 pixel patch, and `ref` is
// reduced the same way at every even pixel position:
//   q(img, y, x) = (sum_{u,v < 4} img[clamp(y + u)][clamp(x + v)] + 8) >> 4
// (coordinates clamped to the frame: edge replication, the boundary rule of
// the exhaustive search).  The proposal for block (by, bx) is the
// displacement (dy, dx), both even and within +-range, that minimises
//   sum_{i,j < 4} | q(cur, 16by + 4i, 16bx + 4j) - q(ref, 16by + 4i + dy, 16bx + 4j + dx) |,
// ties to the first displacement in raster order of (dy, dx).  A search on a
// 2-pixel grid over box-filtered frames: 1/64 of the absolute differences of
// the exhaustive search over the same range.  The refine, audit and fallback
// stage (me_pipeline.h) then turns it into the final vectors.
//
// Layout.  The reference cells at even positions (2 y2, 2 x2) are split by the
// parities (py, px) of (y2, x2) into four u8 planes with 16-cell margins,
//   plane[2 py + px][16 + a][16 + b] = q(ref, 4a + 2py, 4b + 2px),
//   a in [-16, 4 nby + 16), b in [-16, 4 nbx + 16),
// so that candidate (dy, dx) = (2 (2A + py), 2 (2B + px)) reads row
// 16 + 4by + i + A, bytes 16 + 4bx + B .. +3 of plane 2py + px for cell row i:
// the four cells of a row are one unaligned word, one vabsdiff4 per cell row.
// cur's cells are four words per block.
//
// Search kernel: one CTA per run of three vertically adjacent blocks, one
// warp per plane, one lane per candidate column B holding 32 candidate rows of
// each block in registers; the argmin key (sad << 12) | raster index is
// reduced per warp, then over the four warps.
#include <algorithm>
#include <climits>

#include "common.h"
#include "me_pipeline.h"

namespace {

constexpr int NT = 256;
constexpr int MARGIN = 16;  // cells on each side of a plane
constexpr int WIN_ROWS = 35;  // plane rows a block's candidates touch: 4 cell rows + A in [-16, 15]
constexpr int WIN_WORDS = 9;  // words of a plane row a block's candidates touch: 4 cells + B in [-16, 15]

__device__ __forceinline__ uint32_t sad4_acc(uint32_t a, uint32_t b, uint32_t c) {
	uint32_t d;
	asm("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
	return d;
}

// Four cells q(img, y0, x0 + 4 j), j = 0..3, packed little-endian.
__device__ uint32_t box_word(const uint8_t* __restrict__ img, int h, int w, int y0, int x0, bool words) {
	uint32_t s[4] = {0, 0, 0, 0};
	if (words && x0 >= 0 && x0 + 16 <= w) {
		// the 16 columns lie inside the row: aligned word loads, realigned by prmt
		const int xa = x0 & ~3, sh = x0 & 3;
		const uint32_t sel = 0x3210u + 0x1111u * (uint32_t)sh;
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const uint32_t* row = reinterpret_cast<const uint32_t*>(img + (size_t)min(max(y0 + u, 0), h - 1) * w + xa);
			uint32_t v[5];
#pragma unroll
			for (int k = 0; k < 4; ++k) v[k] = __ldg(row + k);
			v[4] = sh ? __ldg(row + 4) : 0u;  // in the row: xa + 20 <= w when sh != 0 (w % 4 == 0)
#pragma unroll
			for (int j = 0; j < 4; ++j) s[j] = sad4_acc(__byte_perm(v[j], v[j + 1], sel), 0u, s[j]);
		}
	} else {
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const uint8_t* row = img + (size_t)min(max(y0 + u, 0), h - 1) * w;
#pragma unroll
			for (int j = 0; j < 4; ++j)
#pragma unroll
				for (int v = 0; v < 4; ++v) s[j] += __ldg(row + min(max(x0 + 4 * j + v, 0), w - 1));
		}
	}
	return ((s[0] + 8) >> 4) | (((s[1] + 8) >> 4) << 8) | (((s[2] + 8) >> 4) << 16) | (((s[3] + 8) >> 4) << 24);
}

struct CoarseGeom {
	int h, w, nby, nbx, nblk, pr, pw;  // pr x pw: rows x bytes of one plane
	size_t plane_bytes;
	CoarseGeom(int h_, int w_) : h(h_), w(w_) {
		nby = h / 16; nbx = w / 16; nblk = nby * nbx;
		pr = 4 * nby + 2 * MARGIN; pw = 4 * nbx + 2 * MARGIN;
		plane_bytes = (size_t)pr * pw;
	}
};

// Bytes x0 .. x0 + 19 of a row as five words, columns clamped to the row.
__device__ __forceinline__ void row_words5(const uint8_t* __restrict__ row, int w, int x0, bool fast, uint32_t (&v)[5]) {
	if (fast) {  // 4-byte aligned and inside the row
		const uint32_t* p = reinterpret_cast<const uint32_t*>(row + x0);
#pragma unroll
		for (int k = 0; k < 5; ++k) v[k] = __ldg(p + k);
	} else {
#pragma unroll
		for (int k = 0; k < 5; ++k) {
			uint32_t t = 0;
#pragma unroll
			for (int b = 0; b < 4; ++b) t |= (uint32_t)__ldg(row + min(max(x0 + 4 * k + b, 0), w - 1)) << (8 * b);
			v[k] = t;
		}
	}
}

__device__ __forceinline__ uint32_t pack_cells(const uint32_t (&s)[4]) {
	return ((s[0] + 8) >> 4) | (((s[1] + 8) >> 4) << 8) | (((s[2] + 8) >> 4) << 16) | (((s[3] + 8) >> 4) << 24);
}

// cells[4 blk + i] = cells of cur's block row i; planes as described above.
// A plane thread owns word k of plane row `row` in all four planes: the cells
// q(4 (row - 16) + 2 py, 16 k - 64 + 2 px + 4 j) for py, px in {0, 1} and
// j = 0..3 cover pixel rows 4 row - 64 .. +5 and bytes 16 k - 64 .. +19, so
// the thread reads six rows of five words once (row sums by vabsdiff4
// against zero; rows 2-3 are shared by both row parities).  A cell thread
// owns one word of cur's cells.
__global__ void __launch_bounds__(NT) coarse_cells_kernel(const uint8_t* __restrict__ cur, const uint8_t* __restrict__ ref,
                                                          CoarseGeom g, bool words, uint32_t* __restrict__ cells,
                                                          uint32_t* __restrict__ planes) {
	const int pww = g.pw / 4;
	const int nplane = g.pr * pww, n = nplane + 4 * g.nblk;  // < 2^31: frames up to 2^30 pixels
	const size_t plane_words = (size_t)nplane;
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
		if (e < nplane) {
			const int row = e / pww, k = e - row * pww;
			const int y0 = 4 * (row - MARGIN), x0 = 16 * k - 4 * MARGIN;
			const bool fast = words && x0 >= 0 && x0 + 20 <= g.w;
			uint32_t acc[3][2][4];  // [pixel row pair][px][j]
#pragma unroll
			for (int u = 0; u < 6; ++u) {
				uint32_t v[5];
				row_words5(ref + (size_t)min(max(y0 + u, 0), g.h - 1) * g.w, g.w, x0, fast, v);
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					const uint32_t odd = __byte_perm(v[j], v[j + 1], 0x5432u);  // bytes 4j + 2 .. 4j + 5
					acc[u >> 1][0][j] = sad4_acc(v[j], 0u, (u & 1) ? acc[u >> 1][0][j] : 0u);
					acc[u >> 1][1][j] = sad4_acc(odd, 0u, (u & 1) ? acc[u >> 1][1][j] : 0u);
				}
			}
#pragma unroll
			for (int py = 0; py < 2; ++py)
#pragma unroll
				for (int px = 0; px < 2; ++px) {
					uint32_t s[4];
#pragma unroll
					for (int j = 0; j < 4; ++j) s[j] = acc[py][px][j] + acc[py + 1][px][j];
					planes[(2 * py + px) * plane_words + e] = pack_cells(s);
				}
		} else {
			const int c = e - nplane, blk = c >> 2, i = c & 3;
			const int by = blk / g.nbx, bx = blk - by * g.nbx;
			cells[c] = box_word(cur, g.h, g.w, 16 * by + 4 * i, 16 * bx, words);
		}
	}
}

// Minimum of cost[a] * 32 + a over the candidate rows a whose vertical
// displacement 2 (a - 16) + PY lies in [-m, m]: the first row wins ties.
// Runtime range (M < 0): masks per row.
template <int M, int PY>
__device__ __forceinline__ uint32_t first_min_row(const uint32_t (&cost)[32], int m) {
	uint32_t mn = 0xffffffffu;
#pragma unroll
	for (int a = 0; a < 32; ++a) {
		const int dy2 = 2 * (a - 16) + PY;
		if (M >= 0 ? (dy2 >= -M && dy2 <= M) : (dy2 >= -m && dy2 <= m)) mn = min(mn, cost[a] * 32u + (uint32_t)a);
	}
	return mn;
}

__device__ __forceinline__ uint32_t min_u16x2(uint32_t a, uint32_t b) {
	uint32_t d;
	asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
	return d;
}

// The same minimum for a range fixed at compile time, on 16-bit keys: a cost
// is at most 16 * 255 = 4080 < 0xfff, so cost * 16 + (a & 15) fits 16 bits
// and rows a and a + 16 share one word, reduced by 15 packed minima; a row
// outside the range holds 0xffff, above every real key.  The words are formed
// by multiply-adds with multipliers the compiler cannot see (k16 = 16,
// k20 = 1 << 20), which keeps them on the FMA pipe beside the SADs.
template <int M, int PY>
__device__ __forceinline__ uint32_t first_min_row_packed(const uint32_t (&cost)[32], uint32_t k16, uint32_t k20) {
	static_assert(M >= 1, "every row parity has a row inside the range");
	auto in = [](int a) { const int dy2 = 2 * (a - 16) + PY; return dy2 >= -M && dy2 <= M; };
	uint32_t w[16];
#pragma unroll
	for (int a = 0; a < 16; ++a) {
		const bool lo = in(a), hi = in(a + 16);
		const uint32_t c = (uint32_t)a | ((uint32_t)a << 16);
		if (lo && hi) w[a] = cost[a] * k16 + (cost[a + 16] * k20 + c);
		else if (lo) w[a] = cost[a] * k16 + (0xffff0000u | (uint32_t)a);
		else if (hi) w[a] = cost[a + 16] * k20 + (((uint32_t)a << 16) | 0xffffu);
		else w[a] = 0xffffffffu;
	}
#pragma unroll
	for (int s = 8; s > 0; s >>= 1)
#pragma unroll
		for (int a = 0; a < s; ++a) w[a] = min_u16x2(w[a], w[a + s]);
	const uint32_t klo = w[0] & 0xffffu, khi = w[0] >> 16;
	const uint32_t kl = ((klo >> 4) << 5) | (klo & 15u), kh = ((khi >> 4) << 5) | 16u | (khi & 15u);
	return min(kl, kh);  // equal costs: the row of the low half comes first
}

// Key of a lane's best candidate: (sad << 12) | raster index of (dy, dx).
__device__ __forceinline__ uint32_t cand_key(uint32_t mn, int py, int dx2, int m) {
	const int a = (int)(mn & 31u), dy2 = 2 * (a - 16) + py, nd = 2 * m + 1;
	return ((mn >> 5) << 12) | (uint32_t)((dy2 + m) * nd + dx2 + m);
}

// One CTA per run of NBK vertically adjacent blocks (NBK p .. NBK p + NBK - 1)
// of one block column, one warp per plane (py, px), one lane per candidate
// column B = lane - 16.  The lane streams the 35 + 4 (NBK - 1) plane rows the
// run's windows cover once: one realigned word per row (two shared loads and
// a prmt) meets the four cell rows i of block bb at candidate rows
// A = row - 16 - 4 bb - i, so a candidate costs four vabsdiff4 and a small
// share of a prmt; 32 NBK costs stay in registers.  M = range / 2 at compile
// time (the default range 60: packed 16-bit argmin), or M < 0 for any range
// (runtime masks).  Three blocks per CTA: 61.5 us at 4K against 65.6 us for
// two (four: the same as three, with 159 registers).
constexpr int NBK = 3;
constexpr int RUN_ROWS = WIN_ROWS + 4 * (NBK - 1);
template <int M>
__global__ void __launch_bounds__(128) coarse_search_kernel(const uint32_t* __restrict__ cells,
                                                            const uint32_t* __restrict__ planes, CoarseGeom g, int m_rt,
                                                            uint32_t k16, uint32_t k20, int32_t* __restrict__ centers) {
	const int m = M >= 0 ? M : m_rt;
	__shared__ uint32_t win[4][RUN_ROWS][WIN_WORDS];
	__shared__ uint32_t best[NBK][4];
	const int run = blockIdx.x / g.nbx, bx = blockIdx.x - run * g.nbx, by0 = NBK * run;
	const int pww = g.pw / 4;
	const size_t plane_words = (size_t)g.pr * pww;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, py = warp >> 1, px = warp & 1;
	{  // warp p stages plane p: lane -> word lane % 9 of rows lane / 9 + 3 j (27 lanes)
		constexpr int RPP = 32 / WIN_WORDS;
		const int kk = lane % WIN_WORDS, rr = lane / WIN_WORDS;
		if (rr < RPP) {
			// word bx + k <= nbx + 7 < pww; plane row 4 by0 + r < pr except the last
			// rows of a run whose lower blocks do not exist (those stay zero)
			const uint32_t* src = planes + warp * plane_words + (size_t)(4 * by0 + rr) * pww + bx + kk;
#pragma unroll
			for (int j = 0; j < (RUN_ROWS + RPP - 1) / RPP; ++j) {
				const int r = rr + RPP * j;
				if (r < RUN_ROWS) win[warp][r][kk] = 4 * by0 + r < g.pr ? __ldg(src + (size_t)RPP * j * pww) : 0u;
			}
		}
	}
	uint32_t c[NBK][4];
#pragma unroll
	for (int bb = 0; bb < NBK; ++bb)
#pragma unroll
		for (int i = 0; i < 4; ++i)
			c[bb][i] = by0 + bb < g.nby ? __ldg(cells + 4 * (size_t)((by0 + bb) * g.nbx + bx) + i) : 0u;
	__syncwarp();
	const int dx2 = 2 * (lane - 16) + px;
	uint32_t key[NBK];
#pragma unroll
	for (int bb = 0; bb < NBK; ++bb) key[bb] = 0xffffffffu;
	if (dx2 >= -m && dx2 <= m) {
		uint32_t cost[NBK][32];  // candidate rows A = a - 16 of block bb
#pragma unroll
		for (int bb = 0; bb < NBK; ++bb)
#pragma unroll
			for (int a = 0; a < 32; ++a) cost[bb][a] = 0;
		const uint32_t* wrow = &win[warp][0][lane >> 2];  // bytes lane .. lane + 3 of each row
		const uint32_t sel = 0x3210u + 0x1111u * (uint32_t)(lane & 3);
#pragma unroll
		for (int r = 0; r < RUN_ROWS; ++r) {
			const uint32_t v = __byte_perm(wrow[r * WIN_WORDS], wrow[r * WIN_WORDS + 1], sel);
#pragma unroll
			for (int bb = 0; bb < NBK; ++bb)
#pragma unroll
				for (int i = 0; i < 4; ++i) {
					const int a = r - 4 * bb - i;  // window row r = 16 + 4 bb + A + i
					if (a >= 0 && a < 32) cost[bb][a] = sad4_acc(c[bb][i], v, cost[bb][a]);
				}
		}
#pragma unroll
		for (int bb = 0; bb < NBK; ++bb) {
			uint32_t mn;
			if constexpr (M >= 0)
				mn = py ? first_min_row_packed<M, 1>(cost[bb], k16, k20) : first_min_row_packed<M, 0>(cost[bb], k16, k20);
			else
				mn = py ? first_min_row<M, 1>(cost[bb], m) : first_min_row<M, 0>(cost[bb], m);
			if (mn != 0xffffffffu) key[bb] = cand_key(mn, py, dx2, m);
		}
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1)
#pragma unroll
		for (int bb = 0; bb < NBK; ++bb) key[bb] = min(key[bb], __shfl_xor_sync(0xffffffffu, key[bb], o));
	if (lane == 0)
#pragma unroll
		for (int bb = 0; bb < NBK; ++bb) best[bb][warp] = key[bb];
	__syncthreads();
	if (threadIdx.x < NBK && by0 + (int)threadIdx.x < g.nby) {
		const int t = threadIdx.x, blk = (by0 + t) * g.nbx + bx;
		const uint32_t k = min(min(best[t][0], best[t][1]), min(best[t][2], best[t][3]));
		const int idx = (int)(k & 4095u), nd = 2 * m + 1;
		centers[2 * blk] = 2 * (idx / nd - m);
		centers[2 * blk + 1] = 2 * (idx % nd - m);
	}
}

// ---- workspace
struct CoarseWork {
	size_t cells, planes, centers, list, count, alist, amv, bytes;
	explicit CoarseWork(const CoarseGeom& g) {
		size_t o = 0;
		auto take = [&](size_t n) { size_t r = o; o += (n + 255) & ~size_t(255); return r; };
		cells = take(16 * (size_t)g.nblk);
		planes = take(4 * g.plane_bytes);
		centers = take(sizeof(int32_t) * 2 * g.nblk);
		list = take(sizeof(int32_t) * g.nblk);
		count = take(sizeof(int32_t) * 4);
		alist = take(sizeof(int32_t) * g.nblk);
		amv = take(sizeof(int32_t) * 3 * g.nblk);
		bytes = o;
	}
	template <class T> T* at(void* ws, size_t off) const { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }
};

umi_status check_frame(int h, int w) {
	if (h < 16 || w < 16) return umi::fail(UMI_ERR_INVALID_ARG, "coarse ME: frame %dx%d smaller than one block", h, w);
	if (h % 16 || w % 16) return umi::fail(UMI_ERR_UNSUPPORTED, "coarse ME: frame %dx%d not a multiple of 16", h, w);
	if ((size_t)h * w > (size_t)1 << 30) return umi::fail(UMI_ERR_UNSUPPORTED, "coarse ME: frame %dx%d too large", h, w);
	return UMI_OK;
}

umi_status centers_impl(const uint8_t* cur, const uint8_t* ref, int h, int w, int range, int32_t* centers, void* ws,
                        cudaStream_t st) {
	const CoarseGeom g(h, w);
	const CoarseWork K(g);
	const bool words = umi::aligned(cur, 4) && umi::aligned(ref, 4);
	const size_t items = (size_t)g.pr * (g.pw / 4) + 4 * (size_t)g.nblk;
	const int grid = (int)std::min<size_t>((items + NT - 1) / NT, 152 * 16);
	coarse_cells_kernel<<<grid, NT, 0, st>>>(cur, ref, g, words, K.at<uint32_t>(ws, K.cells), K.at<uint32_t>(ws, K.planes));
	UMI_TRY(umi::launch_status("coarse_cells_kernel"));
	auto kern = range == 60 ? coarse_search_kernel<30> : coarse_search_kernel<-1>;
	const int runs = (g.nby + NBK - 1) / NBK * g.nbx;
	kern<<<runs, 128, 0, st>>>(K.at<uint32_t>(ws, K.cells), K.at<uint32_t>(ws, K.planes), g, range / 2, 16u, 1u << 20,
	                           centers);
	return umi::launch_status("coarse_search_kernel");
}

umi_status check_common(const uint8_t* cur, const uint8_t* ref, int h, int w, void* ws, size_t bytes) {
	UMI_TRY(check_frame(h, w));
	if (!cur || !ref || !ws) return umi::fail(UMI_ERR_INVALID_ARG, "coarse ME: null pointer");
	if (bytes < CoarseWork(CoarseGeom(h, w)).bytes) return umi::fail(UMI_ERR_NO_MEMORY, "coarse ME: workspace too small");
	if (!umi::aligned(ws, 256)) return umi::fail(UMI_ERR_INVALID_ARG, "coarse ME: workspace alignment");
	return UMI_OK;
}

}  // namespace

extern "C" size_t umi_me_coarse_workspace_bytes(int32_t h, int32_t w) {
	if (check_frame(h, w) != UMI_OK) return 0;
	return CoarseWork(CoarseGeom(h, w)).bytes;
}

extern "C" umi_status umi_me_coarse_centers_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w,
                                               int32_t range, int32_t* centers, void* workspace,
                                               size_t workspace_bytes, void* stream) {
	UMI_TRY(check_common(cur, ref, h, w, workspace, workspace_bytes));
	if (!centers) return umi::fail(UMI_ERR_INVALID_ARG, "coarse ME: null pointer");
	if (range < 0 || range > 62 || range % 2)
		return umi::fail(UMI_ERR_UNSUPPORTED, "coarse ME: range %d (even, 0..62)", range);
	UMI_TRY(centers_impl(cur, ref, h, w, range, centers, workspace, umi::as_stream(stream)));
	return umi::ok();
}

extern "C" umi_status umi_me_coarse_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t refine_r,
                                       int32_t full_r, int32_t sad_threshold, int32_t audit_stride, int32_t* mv,
                                       unsigned long long* audit_sums, int32_t* n_fallback, void* workspace,
                                       size_t workspace_bytes, void* stream) {
	UMI_TRY(check_common(cur, ref, h, w, workspace, workspace_bytes));
	if (!mv) return umi::fail(UMI_ERR_INVALID_ARG, "coarse ME: null pointer");
	if (refine_r < 1 || full_r < refine_r || full_r > 64)
		return umi::fail(UMI_ERR_UNSUPPORTED, "coarse ME: refine %d / full %d ranges", refine_r, full_r);
	if (audit_stride < 0) return umi::fail(UMI_ERR_INVALID_ARG, "coarse ME: negative audit stride");
	const cudaStream_t st = umi::as_stream(stream);
	const CoarseWork K{CoarseGeom(h, w)};
	const umi::MeFinishBuffers fb{K.at<int32_t>(workspace, K.list), K.at<int32_t>(workspace, K.count),
	                              K.at<int32_t>(workspace, K.alist), K.at<int32_t>(workspace, K.amv)};
	umi::MeAudit audit;  // the audited blocks' exhaustive search runs beside the proposal and the refine
	UMI_TRY(umi::me_audit_begin(cur, ref, h, w, full_r, audit_stride, fb, st, &audit));
	int32_t* centers = K.at<int32_t>(workspace, K.centers);
	UMI_TRY(centers_impl(cur, ref, h, w, (full_r - refine_r) & ~1, centers, workspace, st));
	return umi::me_refine_fallback_finish(cur, ref, h, w, centers, refine_r, full_r, sad_threshold, audit_stride, mv,
	                                      audit_sums, n_fallback, fb, audit, st);
}
