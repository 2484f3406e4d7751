// Integral image uint8 -> int32, sm_103a.
//
// Replaces the two Execute calls of main/iimg.cu:37-82 (a Loop-output prefix
// scan along x written transposed, applied twice) with one read of the uint8
// frame from HBM and one write of the int32 result.
//
// Two forms share this file.  umi_iimg_u8_i32 uses the band form (further
// down: column sums per group of bands, then one output pass).
// umi_iimg_u8_i32_noalloc keeps the tile form below, whose small tile sums
// fit the library's built-in scratch:
// the frame is cut into TH x TW tiles (64 x 256: a 1080p frame is 136 tiles,
// about one per SM).  With the inclusive integral image ii and a tile at
// (Y0, X0):
//   ii[y][x] = corner + sum_{X0<=x'<=x} top[x'] + sum_{Y0<=y'<=y} left[y'] + local[y][x]
//   top[x]   = sum over all rows above the tile of column x,
//   left[y]  = sum over all columns left of the tile of row y,
//   corner   = sum over the whole rectangle above-left of the tile,
//   local    = the 2-D prefix inside the tile.
// Kernel 1 (iimg_tile_sums) writes per-tile row sums, column sums and tile
// totals to a small workspace (about 3% of the output).  Kernel 2
// (iimg_tiles) loads its tile and computes the local prefix with warp-shuffle
// scans, then waits for kernel 1 (programmatic dependent launch: the wait is
// griddepcontrol.wait, so everything before it overlaps kernel 1), adds the
// carries (at most nty + ntx + nty*ntx small-array reads per tile, issued as
// independent loads) and writes the tile with 16-byte stores.
#include <cuda.h>

#include <mutex>

#include "common.h"

namespace {

constexpr int NT = 256;         // threads: 8 warps
constexpr int NW = NT / 32;
constexpr int RPW = 8;          // rows per warp
constexpr int TH = NW * RPW;    // 64 tile rows
constexpr int CPL = 8;          // columns per lane
constexpr int TW = 32 * CPL;    // 256 tile columns
constexpr int MAXNTY = 64;      // carries unrolled up to this many tile rows (frames up to 4096 rows)

struct IimgGeom {
	int h, w, ntx, nty;
	int vec_in;   // in is 8-byte aligned and w % 8 == 0
	int vec_out;  // out is 16-byte aligned and w % 4 == 0
	int32_t* rowsum;   // [h][ntx]
	int32_t* colsum;   // [nty][w]
	int32_t* tilesum;  // [nty][ntx]
};

__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
	asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}
__device__ __forceinline__ void pdl_trigger() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
	asm volatile("griddepcontrol.launch_dependents;");
#endif
}

// The lane's 8 pixels of row y starting at column x, zeros past the edges.
__device__ __forceinline__ uint2 load8(const uint8_t* __restrict__ in, const IimgGeom& g, int y, int x) {
	if (y >= g.h) return make_uint2(0, 0);
	const uint8_t* row = in + (size_t)y * g.w;
	if (g.vec_in && x + 7 < g.w) return __ldg(reinterpret_cast<const uint2*>(row + x));
	uint32_t lo = 0, hi = 0;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		if (x + k < g.w) lo |= (uint32_t)__ldg(row + x + k) << (8 * k);
		if (x + 4 + k < g.w) hi |= (uint32_t)__ldg(row + x + 4 + k) << (8 * k);
	}
	return make_uint2(lo, hi);
}

__device__ __forceinline__ void unpack8(uint2 p, uint32_t v[8]) {
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		v[k] = (p.x >> (8 * k)) & 0xffu;
		v[4 + k] = (p.y >> (8 * k)) & 0xffu;
	}
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
		if (lane >= o) v += n;
	}
	return v;
}

__global__ void __launch_bounds__(NT) iimg_tile_sums(const uint8_t* __restrict__ in, const IimgGeom g) {
	__shared__ uint32_t colpart[NW][TW];
	__shared__ uint32_t warptot[NW];
	pdl_wait();  // when launched after an earlier kernel that may write `in`
	pdl_trigger();
	const int tx = blockIdx.x, ty = blockIdx.y;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int X0 = tx * TW, Y0 = ty * TH;
	const int y0 = Y0 + warp * RPW, x = X0 + CPL * lane;
	uint2 raw[RPW];
#pragma unroll
	for (int r = 0; r < RPW; ++r) raw[r] = load8(in, g, y0 + r, x);
	uint32_t col[CPL] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
	for (int r = 0; r < RPW; ++r) {
		uint32_t v[CPL];
		unpack8(raw[r], v);
		uint32_t s = 0;
#pragma unroll
		for (int k = 0; k < CPL; ++k) { s += v[k]; col[k] += v[k]; }
		s = __reduce_add_sync(0xffffffffu, s);
		if (lane == 0 && y0 + r < g.h) g.rowsum[(size_t)(y0 + r) * g.ntx + tx] = (int32_t)s;
	}
#pragma unroll
	for (int k = 0; k < CPL; ++k) colpart[warp][CPL * lane + k] = col[k];
	__syncthreads();
	{
		const int c = threadIdx.x;  // NT == TW: one column per thread
		uint32_t s = 0;
#pragma unroll
		for (int i = 0; i < NW; ++i) s += colpart[i][c];
		if (X0 + c < g.w) g.colsum[(size_t)ty * g.w + X0 + c] = (int32_t)s;
		s = __reduce_add_sync(0xffffffffu, s);
		if (lane == 0) warptot[warp] = s;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t t = 0;
#pragma unroll
		for (int i = 0; i < NW; ++i) t += warptot[i];
		g.tilesum[(size_t)ty * g.ntx + tx] = (int32_t)t;
	}
}

__global__ void __launch_bounds__(NT) iimg_tiles(const uint8_t* __restrict__ in, int32_t* __restrict__ out,
                                                 const IimgGeom g) {
	__shared__ uint32_t wtot[NW][TW];  // per-warp column totals, then their exclusive prefix over warps
	__shared__ uint32_t topw[NW];      // per-warp totals of the top-carry x-scan
	__shared__ uint32_t lefty[TH];     // inclusive y-prefix of the left carries
	__shared__ uint32_t cornerp[NW];
	const int tx = blockIdx.x, ty = blockIdx.y;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int X0 = tx * TW, Y0 = ty * TH;
	const int y0 = Y0 + warp * RPW, x = X0 + CPL * lane;

	// Local 2-D prefix.  The input is not written by kernel 1, so it is read
	// before the dependency wait and overlaps kernel 1.
	uint2 raw[RPW];
#pragma unroll
	for (int r = 0; r < RPW; ++r) raw[r] = load8(in, g, y0 + r, x);
	uint32_t loc[RPW][CPL];
	uint32_t col[CPL] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
	for (int r = 0; r < RPW; ++r) {
		uint32_t v[CPL];
		unpack8(raw[r], v);
#pragma unroll
		for (int k = 1; k < CPL; ++k) v[k] += v[k - 1];
		const uint32_t excl = warp_incl_scan(v[CPL - 1], lane) - v[CPL - 1];
#pragma unroll
		for (int k = 0; k < CPL; ++k) {
			col[k] += v[k] + excl;
			loc[r][k] = col[k];
		}
	}
#pragma unroll
	for (int k = 0; k < CPL; ++k) wtot[warp][CPL * lane + k] = col[k];
	__syncthreads();
	{
		const int c = threadIdx.x;
		uint32_t run = 0;
#pragma unroll
		for (int i = 0; i < NW; ++i) {
			const uint32_t t = wtot[i][c];
			wtot[i][c] = run;
			run += t;
		}
	}

	// Carries from kernel 1.
	pdl_wait();
	pdl_trigger();
	uint32_t topc;  // inclusive x-prefix (within this warp's 32 columns) of the top carries
	{
		const int c = threadIdx.x, xc = X0 + c;
		uint32_t s = 0;
		if (xc < g.w) {
#pragma unroll
			for (int t = 0; t < MAXNTY; ++t)
				if (t < ty) s += (uint32_t)__ldcg(g.colsum + (size_t)t * g.w + xc);
		}
		topc = warp_incl_scan(s, lane);
		if (lane == 31) topw[warp] = topc;
	}
	if (threadIdx.x < TH) {
		const int y = Y0 + threadIdx.x;
		uint32_t s = 0;
		if (y < g.h) {
#pragma unroll 8
			for (int t = 0; t < tx; ++t) s += (uint32_t)__ldcg(g.rowsum + (size_t)y * g.ntx + t);
		}
		// rows are spread over warps 0 and 1: scan within each, stitch below
		lefty[threadIdx.x] = warp_incl_scan(s, lane);
	}
	{
		uint32_t s = 0;
		const int n = ty * tx;
		for (int i = threadIdx.x; i < n; i += NT) {
			const int a = i / tx, b = i - a * tx;
			s += (uint32_t)__ldcg(g.tilesum + (size_t)a * g.ntx + b);
		}
		s = __reduce_add_sync(0xffffffffu, s);
		if (lane == 0) cornerp[warp] = s;
	}
	__syncthreads();
	uint32_t corner = 0;
#pragma unroll
	for (int i = 0; i < NW; ++i) corner += cornerp[i];
	// Top carry prefix for this lane's 8 columns: the warp-level scans of
	// columns [32*wv, 32*wv+32) are in topc of warp wv; columns of this lane
	// are CPL*lane .. CPL*lane+7, owned by warp (CPL*lane)/32.
	__shared__ uint32_t topx[TW];
	topx[threadIdx.x] = topc;
	__syncthreads();
	uint32_t topv[CPL];
#pragma unroll
	for (int k = 0; k < CPL; ++k) {
		const int c = CPL * lane + k;
		uint32_t t = topx[c];
		const int seg = c >> 5;
		for (int sgi = 0; sgi < seg; ++sgi) t += topw[sgi];
		topv[k] = t + corner + wtot[warp][c];
	}
	uint32_t lbase = 0;
	if (warp * RPW >= 32) lbase = lefty[31];  // rows 32..63: add the total of rows 0..31
#pragma unroll
	for (int r = 0; r < RPW; ++r) {
		const int y = y0 + r;
		if (y >= g.h) break;
		const uint32_t lv = lefty[warp * RPW + r] + lbase;
		int32_t o[CPL];
#pragma unroll
		for (int k = 0; k < CPL; ++k) o[k] = (int32_t)(loc[r][k] + topv[k] + lv);
		int32_t* dst = out + (size_t)y * g.w + x;
		if (g.vec_out && x + 7 < g.w) {
			reinterpret_cast<int4*>(dst)[0] = make_int4(o[0], o[1], o[2], o[3]);
			reinterpret_cast<int4*>(dst)[1] = make_int4(o[4], o[5], o[6], o[7]);
		} else {
#pragma unroll
			for (int k = 0; k < CPL; ++k)
				if (x + k < g.w) dst[k] = o[k];
		}
	}
}

size_t ws_bytes(int h, int w) {
	const size_t ntx = umi::ceil_div(w, TW), nty = umi::ceil_div(h, TH);
	auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
	return al((size_t)h * ntx * 4) + al(nty * (size_t)w * 4) + al(nty * ntx * 4);
}

// ---------------------------------------------------------------------------
// Band form (umi_iimg_u8_i32).  The frame is cut into bands of RB rows over
// the full width and the bands into groups of GB bands (128 rows).  With
// V[b][x] = sum of column x over all rows above band b,
//   ii[y][x] = sum_{x'<=x} V[b][x'] + sum_{band rows y'<=y} sum_{x'<=x} in[y'][x'],
//   V[b][x]  = sum_{groups g' above the group of b} S[g'][x] + W[b][x],
// where S[g][x] is the column sum of group g and W[b][x] the column sum of the
// bands of its group above b.  Kernel 1 (one CTA per group and 128 columns)
// reads every group once and writes W and S (uint16: at most 128 * 255).
// Kernel 2 (one CTA per band) loads its band's pixels, waits for kernel 1
// (programmatic dependent launch: its launch and pixel loads overlap kernel
// 1), forms V from at most ceil(h / 128) independent loads per column, scans
// its RB rows and its V row along x with one block-wide scan of RB + 1
// values per thread, and writes the band.  Two launches, both parallel over
// the whole frame; no grid-wide wait.
constexpr int RB = 8;          // rows per band
constexpr int GB = 16;         // bands per group
constexpr int GCT = 16;        // kernel-1 threads across the columns of a group (x CPL = 128 columns)
constexpr int SEG = NT * CPL;  // columns per kernel-2 pass (2048)
static_assert(GB * GCT == NT, "kernel 1: one thread per band and 8 columns");

struct BandGeom {
	int h, w, nb, ng, wpad, nseg;
	int vec_in, vec_out;
	uint16_t* wsum;  // [ng * GB][wpad]  W
	uint16_t* gsum;  // [ng][wpad]       S
};

size_t band_ws_bytes(int h, int w) {
	const size_t nb = umi::ceil_div(h, RB), ng = umi::ceil_div(nb, (size_t)GB), wpad = (size_t)umi::ceil_div(w, CPL) * CPL;
	auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
	return al(ng * GB * wpad * 2) + al(ng * wpad * 2);
}

__global__ void __launch_bounds__(NT) iimg_group_sums(const uint8_t* __restrict__ in, const BandGeom g) {
	__shared__ __align__(16) uint32_t cs[GB][GCT * CPL];
	pdl_trigger();
	const int gi = blockIdx.y, j = threadIdx.x / GCT, c = threadIdx.x % GCT;
	const int xs = blockIdx.x * GCT * CPL, x0 = xs + c * CPL;
	IimgGeom ig{};
	ig.h = g.h; ig.w = g.w; ig.vec_in = g.vec_in;
	uint32_t s[CPL] = {};
	if (x0 < g.w) {
		const int y0 = (gi * GB + j) * RB;
		uint2 raw[RB];
#pragma unroll
		for (int r = 0; r < RB; ++r) raw[r] = load8(in, ig, y0 + r, x0);
#pragma unroll
		for (int r = 0; r < RB; ++r) {
			uint32_t v[CPL];
			unpack8(raw[r], v);
#pragma unroll
			for (int k = 0; k < CPL; ++k) s[k] += v[k];
		}
	}
	*reinterpret_cast<uint4*>(&cs[j][c * CPL]) = make_uint4(s[0], s[1], s[2], s[3]);
	*reinterpret_cast<uint4*>(&cs[j][c * CPL + 4]) = make_uint4(s[4], s[5], s[6], s[7]);
	__syncthreads();
	if (threadIdx.x < GCT * CPL) {  // one column per thread: exclusive prefix over the group's bands
		const int x = xs + threadIdx.x;
		if (x < g.w) {
			uint32_t run = 0;
#pragma unroll
			for (int k = 0; k < GB; ++k) {
				g.wsum[(size_t)(gi * GB + k) * g.wpad + x] = (uint16_t)run;
				run += cs[k][threadIdx.x];
			}
			g.gsum[(size_t)gi * g.wpad + x] = (uint16_t)run;
		}
	}
}

__device__ __forceinline__ void add_u16x8(uint32_t (&v)[CPL], uint4 p) {
	v[0] += p.x & 0xffffu; v[1] += p.x >> 16;
	v[2] += p.y & 0xffffu; v[3] += p.y >> 16;
	v[4] += p.z & 0xffffu; v[5] += p.z >> 16;
	v[6] += p.w & 0xffffu; v[7] += p.w >> 16;
}

__global__ void __launch_bounds__(NT) iimg_band_out(const uint8_t* __restrict__ in, int32_t* __restrict__ out,
                                                     const BandGeom g) {
	__shared__ uint32_t wtot[NW][RB + 1];
	const int b = blockIdx.x, lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
	const int y0 = b * RB;
	IimgGeom ig{};
	ig.h = g.h; ig.w = g.w; ig.vec_in = g.vec_in;
	uint32_t carry[RB + 1] = {};  // totals of the segments to the left (rows, then the V row)
	uint2 raw[RB];
	{
		const int x0 = threadIdx.x * CPL;
#pragma unroll
		for (int r = 0; r < RB; ++r) raw[r] = x0 < g.w ? load8(in, ig, y0 + r, x0) : make_uint2(0, 0);
	}
	pdl_wait();
	for (int seg = 0; seg < g.nseg; ++seg) {
		const int x0 = seg * SEG + threadIdx.x * CPL;
		const bool live = x0 < g.w;
		if (seg > 0) {
#pragma unroll
			for (int r = 0; r < RB; ++r) raw[r] = live ? load8(in, ig, y0 + r, x0) : make_uint2(0, 0);
		}
		uint32_t vv[CPL] = {};
		if (live) {  // V = W of this band + S of every group above
			add_u16x8(vv, __ldcg(reinterpret_cast<const uint4*>(g.wsum + (size_t)b * g.wpad + x0)));
			const int gb = b / GB;
#pragma unroll 8
			for (int q = 0; q < gb; ++q) add_u16x8(vv, __ldcg(reinterpret_cast<const uint4*>(g.gsum + (size_t)q * g.wpad + x0)));
		}
		// thread totals of each row and of the V row, scanned over the block
		uint32_t tsum[RB + 1];
#pragma unroll
		for (int r = 0; r < RB; ++r) {
			uint32_t v[CPL];
			unpack8(raw[r], v);
			uint32_t t = 0;
#pragma unroll
			for (int k = 0; k < CPL; ++k) t += v[k];
			tsum[r] = t;
		}
		{
			uint32_t t = 0;
#pragma unroll
			for (int k = 0; k < CPL; ++k) t += vv[k];
			tsum[RB] = t;
		}
		uint32_t ex[RB + 1];
#pragma unroll
		for (int r = 0; r <= RB; ++r) {
			const uint32_t inc = warp_incl_scan(tsum[r], lane);
			ex[r] = inc - tsum[r];
			if (lane == 31) wtot[wp][r] = inc;
		}
		__syncthreads();
		uint32_t segtot[RB + 1];
#pragma unroll
		for (int r = 0; r <= RB; ++r) {
			uint32_t before = 0, all = 0;
#pragma unroll
			for (int k = 0; k < NW; ++k) {
				const uint32_t t = wtot[k][r];
				before += k < wp ? t : 0u;
				all += t;
			}
			ex[r] += before + carry[r];
			segtot[r] = all;
		}
		__syncthreads();  // wtot is rewritten by the next segment
		// outputs: T(x) = V-row prefix, plus the running column sum of the row prefixes
		uint32_t T[CPL], colacc[CPL];
		{
			uint32_t tp = ex[RB];
#pragma unroll
			for (int k = 0; k < CPL; ++k) {
				tp += vv[k];
				T[k] = tp;
				colacc[k] = 0;
			}
		}
#pragma unroll
		for (int r = 0; r < RB; ++r) {
			uint32_t rp = ex[r], o[CPL];
#pragma unroll
			for (int k = 0; k < CPL; ++k) {
				rp += (k < 4 ? (raw[r].x >> (8 * k)) : (raw[r].y >> (8 * (k - 4)))) & 0xffu;
				colacc[k] += rp;
				o[k] = T[k] + colacc[k];
			}
			const int y = y0 + r;
			if (live && y < g.h) {
				int32_t* op = out + (size_t)y * g.w + x0;
				if (g.vec_out && x0 + 7 < g.w) {
					reinterpret_cast<int4*>(op)[0] = make_int4(o[0], o[1], o[2], o[3]);
					reinterpret_cast<int4*>(op)[1] = make_int4(o[4], o[5], o[6], o[7]);
				} else {
#pragma unroll
					for (int k = 0; k < CPL; ++k)
						if (x0 + k < g.w) op[k] = (int32_t)o[k];
				}
			}
		}
#pragma unroll
		for (int r = 0; r <= RB; ++r) carry[r] += segtot[r];
	}
}

cudaLaunchAttribute pdl_attr() {
	cudaLaunchAttribute a;
	a.id = cudaLaunchAttributeProgrammaticStreamSerialization;
	a.val.programmaticStreamSerializationAllowed = 1;
	return a;
}

}  // namespace

extern "C" size_t umi_iimg_u8_i32_workspace_bytes(int32_t h, int32_t w) {
	if (h <= 0 || w <= 0) return 0;
	return band_ws_bytes(h, w);
}

extern "C" umi_status umi_iimg_u8_i32(const uint8_t* in, int32_t* out, int32_t h, int32_t w, void* workspace,
                                      size_t workspace_bytes, void* stream) {
	if (h < 0 || w < 0) return umi::fail(UMI_ERR_INVALID_ARG, "iimg: negative size %dx%d", h, w);
	if (h == 0 || w == 0) return umi::ok();
	if (!in || !out || !workspace) return umi::fail(UMI_ERR_INVALID_ARG, "iimg: null pointer");
	if (!umi::aligned(workspace, 16)) return umi::fail(UMI_ERR_INVALID_ARG, "iimg: workspace not 16-byte aligned");
	if (workspace_bytes < band_ws_bytes(h, w))
		return umi::fail(UMI_ERR_NO_MEMORY, "iimg: workspace of %zu bytes, need %zu", workspace_bytes,
		                 band_ws_bytes(h, w));
	if ((int64_t)h * w > ((int64_t)1 << 31) / 255)
		return umi::fail(UMI_ERR_UNSUPPORTED, "iimg: %dx%d frame: sums could exceed int32", h, w);
	BandGeom g{};
	g.h = h; g.w = w;
	g.nb = umi::ceil_div(h, RB);
	g.ng = umi::ceil_div(g.nb, GB);
	g.wpad = umi::ceil_div(w, CPL) * CPL;
	g.nseg = umi::ceil_div(w, SEG);
	g.vec_in = umi::aligned(in, 8) && (w % 8) == 0;
	g.vec_out = umi::aligned(out, 16) && (w % 4) == 0;
	auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
	char* ws = static_cast<char*>(workspace);
	g.wsum = reinterpret_cast<uint16_t*>(ws);
	g.gsum = reinterpret_cast<uint16_t*>(ws + al((size_t)g.ng * GB * g.wpad * 2));
	const cudaStream_t st = umi::as_stream(stream);
	// kernel 1 follows whatever the stream ran before: plain launch
	iimg_group_sums<<<dim3(umi::ceil_div(w, GCT * CPL), g.ng), NT, 0, st>>>(in, g);
	UMI_TRY(umi::launch_status("iimg_group_sums"));
	cudaLaunchAttribute attr[1] = {pdl_attr()};
	cudaLaunchConfig_t cfg{};
	cfg.gridDim = dim3(g.nb);
	cfg.blockDim = dim3(NT);
	cfg.stream = st;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	UMI_TRY(umi::cuda_status(cudaLaunchKernelEx(&cfg, iimg_band_out, in, out, g), "iimg_band_out"));
	return umi::ok();
}

// ---------------------------------------------------------------------------
// Allocation-free integral image.
//
// Some callers of this library cannot allocate device memory at all: a plugin
// inside a host application that owns the GPU memory budget, code that runs
// where cudaMalloc is not allowed (a real-time loop with a no-allocation
// rule, a host callback), or a caller that simply has no allocator to hand a
// workspace from.  umi_iimg_u8_i32_noalloc serves them: the tile sums go to
// a scratch array compiled into this library, so the caller passes only the
// frame and the output.
//
// The scratch is a file-scope __device__ array of kNoAllocScratchBytes
// (1 MiB: the tile sums of every frame the int32 limit accepts, up to 4096
// rows; the largest accepted frame has h*w*255 < 2^31, about 8.42 Mpx, so
// 3840x2160 is served and 4096x2160 is refused by that limit); every GPU that
// loads the library holds it until the process exits.  Host code cannot use
// the array's name as a device address, so the first call in each CUDA
// context (with that context current) looks the address up with
// cudaGetSymbolAddress and caches it under the context handle; make that
// first call before any stream capture.  A context destroyed and re-created
// while the library stays loaded (cudaDeviceReset) can come back with the
// same handle: such a caller calls umi_iimg_noalloc_forget() after the reset.
// All calls share the one array: calls that overlap on the GPU (different
// streams, different host threads) race on it and must be serialised by the
// caller.  Nothing in the scratch needs to start at zero: kernel 1 writes
// every entry kernel 2 reads.
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;
static_assert(kNoAllocScratchBytes == UMI_IIMG_NOALLOC_SCRATCH_BYTES, "header and library disagree");
static __device__ __align__(256) unsigned char g_iimg_scratch[kNoAllocScratchBytes];

// Scratch address per CUDA context (the module, and so the array, is loaded
// once per context: the primary context of each device, or a context the
// caller made current through the driver API).
constexpr int kMaxContexts = 64;
std::mutex g_scratch_mu;
struct ScratchEntry { void* ctx; void* addr; };
ScratchEntry g_scratch[kMaxContexts] = {};
int g_scratch_n = 0;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
CtxGetCurrentFn ctx_get_current_fn() {
	static CtxGetCurrentFn fn = nullptr;
	static std::once_flag once;
	std::call_once(once, [] {
		cudaDriverEntryPointQueryResult q;
		void* p = nullptr;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<CtxGetCurrentFn>(p);
	});
	return fn;
}

umi_status scratch_address(void** out) {
	int dev = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	// the runtime makes the device's primary context current if none is yet
	UMI_TRY(umi::cuda_status(cudaFree(nullptr), "cudaFree(0) (context initialisation)"));
	auto get = ctx_get_current_fn();
	if (!get) return umi::fail(UMI_ERR_CUDA, "iimg_noalloc: cuCtxGetCurrent unavailable");
	CUcontext ctx = nullptr;
	if (get(&ctx) != CUDA_SUCCESS || !ctx) return umi::fail(UMI_ERR_CUDA, "iimg_noalloc: no current CUDA context");
	std::lock_guard<std::mutex> lock(g_scratch_mu);
	for (int i = 0; i < g_scratch_n; ++i)
		if (g_scratch[i].ctx == ctx) {
			*out = g_scratch[i].addr;
			return UMI_OK;
		}
	if (g_scratch_n == kMaxContexts) return umi::fail(UMI_ERR_UNSUPPORTED, "iimg_noalloc: more than %d contexts", kMaxContexts);
	void* p = nullptr;
	UMI_TRY(umi::cuda_status(cudaGetSymbolAddress(&p, g_iimg_scratch), "cudaGetSymbolAddress"));
	g_scratch[g_scratch_n++] = {reinterpret_cast<void*>(ctx), p};
	*out = p;
	return UMI_OK;
}

}  // namespace

extern "C" umi_status umi_iimg_u8_i32_noalloc(const uint8_t* in, int32_t* out, int32_t h, int32_t w, void* stream) {
	if (h < 0 || w < 0) return umi::fail(UMI_ERR_INVALID_ARG, "iimg_noalloc: negative size %dx%d", h, w);
	if (h == 0 || w == 0) return umi::ok();
	if (!in || !out) return umi::fail(UMI_ERR_INVALID_ARG, "iimg_noalloc: null pointer");
	if (ws_bytes(h, w) > kNoAllocScratchBytes)
		return umi::fail(UMI_ERR_NO_MEMORY, "iimg_noalloc: a %dx%d frame needs %zu scratch bytes, the built-in scratch holds %zu",
		                 h, w, ws_bytes(h, w), kNoAllocScratchBytes);
	if (umi::ceil_div(h, TH) > MAXNTY)
		return umi::fail(UMI_ERR_UNSUPPORTED, "iimg_noalloc: %d rows (max %d)", h, MAXNTY * TH);
	if ((int64_t)h * w > ((int64_t)1 << 31) / 255)
		return umi::fail(UMI_ERR_UNSUPPORTED, "iimg_noalloc: %dx%d frame: sums could exceed int32", h, w);
	void* scratch = nullptr;
	UMI_TRY(scratch_address(&scratch));
	IimgGeom g{};
	g.h = h; g.w = w;
	g.ntx = umi::ceil_div(w, TW);
	g.nty = umi::ceil_div(h, TH);
	g.vec_in = umi::aligned(in, 8) && (w % 8) == 0;
	g.vec_out = umi::aligned(out, 16) && (w % 4) == 0;
	auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
	char* ws = static_cast<char*>(scratch);
	g.rowsum = reinterpret_cast<int32_t*>(ws);
	g.colsum = reinterpret_cast<int32_t*>(ws + al((size_t)h * g.ntx * 4));
	g.tilesum = reinterpret_cast<int32_t*>(ws + al((size_t)h * g.ntx * 4) + al((size_t)g.nty * w * 4));
	cudaLaunchConfig_t cfg{};
	cfg.gridDim = dim3(g.ntx, g.nty);
	cfg.blockDim = dim3(NT);
	cfg.stream = umi::as_stream(stream);
	cudaLaunchAttribute attr[1] = {pdl_attr()};
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	UMI_TRY(umi::cuda_status(cudaLaunchKernelEx(&cfg, iimg_tile_sums, in, g), "iimg_tile_sums"));
	UMI_TRY(umi::cuda_status(cudaLaunchKernelEx(&cfg, iimg_tiles, in, out, g), "iimg_tiles"));
	return umi::ok();
}

extern "C" void umi_iimg_noalloc_forget(void) {
	std::lock_guard<std::mutex> lock(g_scratch_mu);
	g_scratch_n = 0;
}
