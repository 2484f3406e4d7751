// Image operators for batches of uneven images, sm_103a: bilateral filter,
// per-pixel-weight 3x3 filter, dot-product cost volume.
//
// One persistent launch serves a whole batch: the image table (pointers and
// sizes, up to UMI_BATCH_MAX_IMAGES) and the exclusive prefix of per-image
// tile counts are kernel parameters (no allocation); CTA b takes tiles b,
// b + grid, ... and finds each tile's image by binary search in the prefix.
// The single-image entry points are batches of one.  Each operator has
// several tile shapes ("variants") for the autotuner.
//
// Reference counterparts: the Bilateral strategy (main/bilateral.cu:9-24),
// the WFilter3x3 strategy with a per-pixel weight memory
// (main/wfilter3x3.cu:8-15), and the horizontal cost volume
// (main/cost_volume.cu:8-65) with a dot-product cost.  The reference launches
// one Execute per image.
#include <algorithm>
#include <cmath>
#include <new>

#include "common.h"
#include "tc_common.cuh"

namespace {

constexpr int MAXIMG = UMI_BATCH_MAX_IMAGES;
constexpr int NT = 256;  // threads per CTA for every operator

struct Img {
	const float* in;
	const float* aux;
	float* out;
	int h, w, tiles_x;
	int vec;   // all pointers 16-byte aligned and w % 4 == 0
	int kind;  // batch_fused_kernel's filter phase: which operator variant serves this image
};

struct Table {
	int n;
	int start[MAXIMG + 1];
	Img img[MAXIMG];
};

__device__ __forceinline__ int find_image(const Table& t, int tile) {
	int lo = 0, hi = t.n;
	while (hi - lo > 1) {
		const int mid = (lo + hi) >> 1;
		if (t.start[mid] <= tile) lo = mid;
		else hi = mid;
	}
	return lo;
}

// 2^x on the special-function unit (PTX ex2.approx, relative error ~2^-22).
__device__ __forceinline__ float ex2(float x) {
	float y;
	asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}

// ------------------------------------------------------------------ bilateral
// Weight of neighbour n around centre c: 2^(fma((n-c)^2, k, lsw[dy][dx]))
// with k = -log2(e) / (2 sigma_r^2) and lsw = log2(ws[dy] * ws[dx]): one
// SFU instruction per neighbour.  Accumulation order (dy, dx) row-major as
// main/bilateral.cu:111-117.
struct BilParams {
	float k;
	float lsw[7][7];
};

template <int R, int TW, int TH, int PPT, int NTH = NT>
struct Bilateral {
	static constexpr int SW = TW + 2 * R, SH = TH + 2 * R;
	static_assert(TW * TH / PPT == NTH && TH % PPT == 0, "one pixel column of PPT per thread");
	static constexpr size_t smem = sizeof(float) * SW * SH;
	static int tiles_x(int w) { return umi::ceil_div(w, TW); }
	static int tiles(int h, int w) { return tiles_x(w) * umi::ceil_div(h, TH); }
	__device__ static void tile(const Img& im, int t, const BilParams& p, float* sm) {
		const int ty = t / im.tiles_x, tx = t - ty * im.tiles_x;
		const int X0 = tx * TW, Y0 = ty * TH;
		for (int i = threadIdx.x; i < SW * SH; i += NTH) {
			const int sy = i / SW, sx = i - sy * SW;
			const int gy = Y0 + sy - R, gx = X0 + sx - R;
			sm[i] = (gy >= 0 && gy < im.h && gx >= 0 && gx < im.w) ? __ldg(im.in + (size_t)gy * im.w + gx) : 0.0f;
		}
		__syncthreads();
		compute(im, t, p, sm);
		__syncthreads();
	}
	// The halo tile of tile t by 4-byte cp.async (zero fill outside the image),
	// committed as one group of this thread: lets the next tile's loads run
	// while the current one is computed (batch_fused_kernel).
	__device__ static void stage_async(const Img& im, int t, float* sm) {
		const int ty = t / im.tiles_x, tx = t - ty * im.tiles_x;
		const int X0 = tx * TW, Y0 = ty * TH;
		for (int i = threadIdx.x; i < SW * SH; i += NTH) {
			const int sy = i / SW, sx = i - sy * SW;
			const int gy = Y0 + sy - R, gx = X0 + sx - R;
			const bool in = gy >= 0 && gy < im.h && gx >= 0 && gx < im.w;
			const unsigned d = (unsigned)__cvta_generic_to_shared(sm + i);
			const float* src = in ? im.in + (size_t)gy * im.w + gx : im.in;
			asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(in ? 4 : 0) : "memory");
		}
		asm volatile("cp.async.commit_group;" ::: "memory");
	}
	// Outputs of tile t from its staged halo tile.
	__device__ static void compute(const Img& im, int t, const BilParams& p, const float* sm) {
		const int ty = t / im.tiles_x, tx = t - ty * im.tiles_x;
		const int X0 = tx * TW, Y0 = ty * TH;
		const int lx = threadIdx.x % TW, ly0 = (threadIdx.x / TW) * PPT;
#pragma unroll
		for (int q = 0; q < PPT; ++q) {
			const int ly = ly0 + q;
			const float c = sm[(ly + R) * SW + lx + R];
			float ws = 0.0f, wx = 0.0f;
#pragma unroll
			for (int dy = 0; dy <= 2 * R; ++dy)
#pragma unroll
				for (int dx = 0; dx <= 2 * R; ++dx) {
					const float n = sm[(ly + dy) * SW + lx + dx];
					const float d = n - c;
					const float wt = ex2(fmaf(d * d, p.k, p.lsw[dy][dx]));
					ws += wt;
					wx = fmaf(wt, n, wx);
				}
			const int gy = Y0 + ly, gx = X0 + lx;
			if (gy < im.h && gx < im.w) im.out[(size_t)gy * im.w + gx] = wx / ws;
		}
	}
};

// ------------------------------------------------------------------ wfilter
// A warp owns a 128-column strip and RY rows (4 pixels per lane, halo
// columns by shuffle, every input row loaded once); the 9 weights of 4
// pixels are 9 float4 loads.
struct NoParams {};

__device__ __forceinline__ float4 row4(const Img& im, int y, int x) {
	if (y < 0 || y >= im.h) return make_float4(0.f, 0.f, 0.f, 0.f);
	const float* r = im.in + (size_t)y * im.w;
	if (im.vec && x + 3 < im.w) return __ldg(reinterpret_cast<const float4*>(r + x));
	float4 v;
	v.x = x < im.w ? __ldg(r + x) : 0.f;
	v.y = x + 1 < im.w ? __ldg(r + x + 1) : 0.f;
	v.z = x + 2 < im.w ? __ldg(r + x + 2) : 0.f;
	v.w = x + 3 < im.w ? __ldg(r + x + 3) : 0.f;
	return v;
}

template <int RY, int NTH = NT>
struct WFilter {
	static constexpr int WARPS = NTH / 32;
	static constexpr int TH = WARPS * RY;
	static constexpr size_t smem = 0;
	static int tiles_x(int w) { return umi::ceil_div(w, 128); }
	static int tiles(int h, int w) { return tiles_x(w) * umi::ceil_div(h, TH); }
	__device__ static void tile(const Img& im, int t, const NoParams&, float*) {
		const int ty = t / im.tiles_x, tx = t - ty * im.tiles_x;
		const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
		const int x0 = tx * 128, x = x0 + 4 * lane;
		const int y0 = ty * TH + warp * RY;
		if (y0 >= im.h) return;  // no barrier in this operator
		float r[RY + 2][6];
#pragma unroll
		for (int i = 0; i < RY + 2; ++i) {
			const int y = y0 - 1 + i;
			const float4 v = row4(im, y, x);
			float left = __shfl_up_sync(0xffffffffu, v.w, 1);
			float right = __shfl_down_sync(0xffffffffu, v.x, 1);
			const bool rowok = y >= 0 && y < im.h;
			if (lane == 0) left = (rowok && x0 > 0) ? __ldg(im.in + (size_t)y * im.w + x0 - 1) : 0.f;
			if (lane == 31) right = (rowok && x0 + 128 < im.w) ? __ldg(im.in + (size_t)y * im.w + x0 + 128) : 0.f;
			r[i][0] = left; r[i][1] = v.x; r[i][2] = v.y; r[i][3] = v.z; r[i][4] = v.w; r[i][5] = right;
		}
#pragma unroll
		for (int i = 0; i < RY; ++i) {
			const int y = y0 + i;
			if (y >= im.h) break;
			float wv[36];
			const float* wp = im.aux + ((size_t)y * im.w + x) * 9;
			if (im.vec && x + 3 < im.w) {
#pragma unroll
				for (int k = 0; k < 9; ++k) {
					const float4 q = __ldg(reinterpret_cast<const float4*>(wp) + k);
					wv[4 * k] = q.x; wv[4 * k + 1] = q.y; wv[4 * k + 2] = q.z; wv[4 * k + 3] = q.w;
				}
			} else {
#pragma unroll
				for (int k = 0; k < 36; ++k) wv[k] = (x + k / 9 < im.w) ? __ldg(wp + k) : 0.f;
			}
			float o[4];
#pragma unroll
			for (int px = 0; px < 4; ++px) {
				float s = 0.0f;
#pragma unroll
				for (int dy = 0; dy < 3; ++dy)
#pragma unroll
					for (int dx = 0; dx < 3; ++dx) s = fmaf(wv[9 * px + 3 * dy + dx], r[i + dy][px + dx], s);
				o[px] = s;
			}
			float* dst = im.out + (size_t)y * im.w + x;
			if (im.vec && x + 3 < im.w) {
				*reinterpret_cast<float4*>(dst) = make_float4(o[0], o[1], o[2], o[3]);
			} else {
#pragma unroll
				for (int px = 0; px < 4; ++px)
					if (x + px < im.w) dst[px] = o[px];
			}
		}
	}
};

// ------------------------------------------------------------------ cost volume
// One CTA computes one image row segment of TX pixels x ND disparities.
// Lane (xb, db) of warp wv owns pixels x = wv*TXW + 8*xb + i and disparities
// d = 8*db + j (i, j < 8): 64 accumulators.  Per channel it reads its 8 left
// features (two 128-bit loads) and the 15 right features x + d it needs
// (four 128-bit loads) from shared memory.  Right rows are stored with 4
// floats of padding after every 32, which keeps 16-byte chunks whole and puts
// the 8 chunks one quarter-warp reads in 8 distinct bank groups.  Channels are
// staged CC at a time (one channel row per warp) with 16-byte cp.async,
// double-buffered; the image edge is zero-filled by partial copies.  Channel
// order 0..c-1 per output.
struct CvParams {
	int channels;
};

__device__ __forceinline__ void cp_async16(float* dst, const float* src, int bytes) {
	const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
	const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
	const int n = valid ? 4 : 0;  // src-size 0: zero fill
	asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_two() { asm volatile("cp.async.wait_group 2;" ::: "memory"); }

template <int DB>
struct CostVolume {
	static constexpr int ND = 8 * DB;
	static constexpr int XB = 32 / DB;
	static constexpr int TXW = 8 * XB;                  // pixels per warp
	static constexpr int TX = (NT / 32) * TXW;          // pixels per CTA
	static constexpr int CC = NT / 32;                  // channels per stage: one per warp
	static constexpr int RW = (TX + ND + 3) / 4 * 4;    // right columns staged (>= TX + ND - 1, whole chunks)
	static constexpr int RWP = RW + 4 * (RW / 32) + 4;  // padded row
	static constexpr int STAGE = CC * TX + CC * RWP;
	static constexpr int NBUF = 3;  // stages in flight: covers DRAM latency at two CTAs per SM
	static constexpr size_t smem = sizeof(float) * NBUF * STAGE;
	static_assert(TX % 4 == 0 && RWP % 4 == 0 && STAGE % 4 == 0, "16-byte aligned rows");
	static int tiles_x(int w) { return umi::ceil_div(w, TX); }
	static int tiles(int h, int w) { return tiles_x(w) * h; }
	__device__ static int pad(int e) { return e + 4 * (e >> 5); }

	__device__ static void stage(const Img& im, int y, int X0, int c0, int C, float* buf) {
		const int cc = threadIdx.x >> 5, lane = threadIdx.x & 31;
		const bool chan = c0 + cc < C;
		const size_t off = (size_t)(chan ? c0 + cc : 0) * im.h * im.w + (size_t)y * im.w + X0;
		const float* lsrc = im.in + off;
		const float* rsrc = im.aux + off;
		float* L = buf + cc * TX;
		float* Rr = buf + CC * TX + cc * RWP;
		const int lim = chan ? im.w - X0 : 0;  // valid columns from X0
		if (im.vec) {
			// rows are 16-byte aligned: whole chunks, partial (zero-filled) at the edge
			for (int q = lane; q < TX / 4; q += 32) {
				const int v = min(max(lim - 4 * q, 0), 4);
				cp_async16(L + 4 * q, v ? lsrc + 4 * q : im.in, 4 * v);
			}
			for (int q = lane; q < RW / 4; q += 32) {
				const int v = min(max(lim - 4 * q, 0), 4);
				cp_async16(Rr + pad(4 * q), v ? rsrc + 4 * q : im.aux, 4 * v);
			}
		} else {
			for (int x = lane; x < TX; x += 32) cp_async4(L + x, x < lim ? lsrc + x : im.in, x < lim);
			for (int x = lane; x < RW; x += 32) cp_async4(Rr + pad(x), x < lim ? rsrc + x : im.aux, x < lim);
		}
		cp_async_commit();
	}

	__device__ static void tile(const Img& im, int t, const CvParams& p, float* sm) {
		const int y = t / im.tiles_x, tx = t - y * im.tiles_x;
		const int X0 = tx * TX;
		const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
		const int xb = lane / DB, db = lane - xb * DB;
		const int xl = warp * TXW + 8 * xb;  // first local pixel of this thread
		const int e0 = xl + 8 * db;          // first right column it reads
		int roff[4];
#pragma unroll
		for (int q = 0; q < 4; ++q) roff[q] = pad(e0 + 4 * q);
		const int C = p.channels;
		float acc[8][8];
#pragma unroll
		for (int i = 0; i < 8; ++i)
#pragma unroll
			for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
		const int nst = (C + CC - 1) / CC;
		stage(im, y, X0, 0, C, sm);
		if (nst > 1) stage(im, y, X0, CC, C, sm + STAGE);
		for (int s = 0; s < nst; ++s) {
			const float* cur = sm + (s % NBUF) * STAGE;
			// keep up to NBUF stages in flight; wait until stage s has landed
			if (s + 2 < nst) {
				stage(im, y, X0, (s + 2) * CC, C, sm + ((s + 2) % NBUF) * STAGE);
				cp_async_wait_two();
			} else if (s + 1 < nst) {
				cp_async_wait_one();
			} else {
				cp_async_wait_all();
			}
			__syncthreads();
			const float* L = cur + xl;
			const float* Rr = cur + CC * TX;
#pragma unroll 1
			for (int cc = 0; cc < CC; ++cc) {
				float lv[8], rv[16];
				const float4 l0 = *reinterpret_cast<const float4*>(L + cc * TX);
				const float4 l1 = *reinterpret_cast<const float4*>(L + cc * TX + 4);
				lv[0] = l0.x; lv[1] = l0.y; lv[2] = l0.z; lv[3] = l0.w;
				lv[4] = l1.x; lv[5] = l1.y; lv[6] = l1.z; lv[7] = l1.w;
#pragma unroll
				for (int q = 0; q < 4; ++q) {
					const float4 r4 = *reinterpret_cast<const float4*>(Rr + cc * RWP + roff[q]);
					rv[4 * q] = r4.x; rv[4 * q + 1] = r4.y; rv[4 * q + 2] = r4.z; rv[4 * q + 3] = r4.w;
				}
#pragma unroll
				for (int i = 0; i < 8; ++i)
#pragma unroll
					for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(lv[i], rv[i + j], acc[i][j]);
			}
			__syncthreads();  // the next stage overwrites this buffer
		}
#pragma unroll
		for (int i = 0; i < 8; ++i) {
			const int x = X0 + xl + i;
			if (x >= im.w) break;
			float* dst = im.out + ((size_t)y * im.w + x) * ND + 8 * db;
			if (im.vec) {
				reinterpret_cast<float4*>(dst)[0] = make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
				reinterpret_cast<float4*>(dst)[1] = make_float4(acc[i][4], acc[i][5], acc[i][6], acc[i][7]);
			} else {
#pragma unroll
				for (int j = 0; j < 8; ++j) dst[j] = acc[i][j];
			}
		}
	}
};

// ------------------------------------------------------------------ cost volume on tcgen05
// cv[y, x, d] = sum_c L[c, y, x] R[c, y, x + d], d = 0..63, C <= 32, as a
// banded matrix product per image row: for the 128 pixels x0 .. x0 + 127 and
// the 192 right columns x0 .. x0 + 191 (zero past the row end),
//   P = A B^T,  A[p][c] = L[c, y, x0 + p],  B[n][c] = R[c, y, x0 + n],
//   cv[y, x0 + p, d] = P[p][p + d].
// Each fp32 operand is split into tf32 parts x = hi + lo (hi = x rounded to
// tf32, lo = x - hi exactly, then rounded to tf32), and
// P = Ahi Bhi + Ahi Blo + Alo Bhi (the dropped lo*lo term is ~2^-22 of the
// product) on tcgen05.mma kind::tf32 with fp32 accumulation in TMEM: three
// M=128 N=192 MMAs per 8 channels.  A pixel's 32 channels are one 128-byte
// row of the K-major, 128-byte-swizzled operand tiles (the layout of the
// bf16 GEMM in gemm_tc.cu; a K step of 8 tf32 is 32 bytes).
//
// Roles (480 threads): warps 0-4 and 5-9 are two producer groups taking
// alternate tiles, each filling its own operand stage (plain loads of two
// operand rows per thread, split, swizzled 16-byte stores, then a proxy fence
// and an mbarrier arrive), so two tiles' loads are in flight per SM; warp 10
// allocates TMEM (two accumulators of 192 columns) and one lane issues the
// MMAs; warps 11-14 drain an accumulator while the next tile computes: lane p
// of a warp holds TMEM row p (one pixel), loads the 96 columns its warp's band
// touches (32 at a time), stores its 64 with predicated conflict-free shared
// stores (word 63 p + j) into one of two staging buffers, and the warp writes
// its 32 pixels x 64 disparities (8 KB, contiguous in cv) with one bulk copy.
// Every wait is bounded (tc_common.cuh).
namespace cvtc {
constexpr int BM = 128, ND = 64, BNN = BM + ND, KC = 32;
constexpr uint32_t A_BYTES = BM * 128, B_BYTES = BNN * 128;
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // Ahi, Alo, Bhi, Blo
constexpr uint32_t OUT_WARP_BYTES = 32 * ND * 4;
constexpr int PG = 160;          // threads per producer group: 320 operand rows, two per thread
constexpr int NTH = 15 * 32;    // warps 0-4, 5-9 producers; 10 MMA; 11-14 epilogue
constexpr size_t SMEM = 2 * (size_t)STAGE_BYTES + 8 * OUT_WARP_BYTES + 1024 + 256;  // two staging buffers per epilogue warp
constexpr uint32_t TMEM_COLS = 512;  // 2 x 192, rounded to a power of two
// kind::tf32 instruction descriptor: fp32 accumulator (bits 4-5 = 1), A and
// B tf32 (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BNN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
static_assert(SMEM <= 227 * 1024, "one CTA per SM");

struct Params { int channels; };

__device__ __forceinline__ uint32_t to_tf32(float x) {
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return r;
}
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool acc) {
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"setp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
		"l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)acc)
		: "memory");
}
// shared -> global bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
	asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(umi_tc::smem_u32(src)),
	             "r"(bytes)
	             : "memory");
}

// Row `row` (pixel or right column) of the operand tiles: 32 channels of
// column x of image row y, split into tf32 hi / lo and stored as 8 swizzled
// 16-byte chunks (chunk j of row r at j ^ (r & 7)).
__device__ __forceinline__ void load_row(const float* __restrict__ src, size_t plane, int C, bool valid, float (&v)[KC]) {
#pragma unroll
	for (int c = 0; c < KC; ++c) v[c] = (valid && c < C) ? __ldg(src + (size_t)c * plane) : 0.0f;
}
__device__ __forceinline__ void store_row(uint8_t* hi, uint8_t* lo, int row, const float (&v)[KC]) {
#pragma unroll
	for (int j = 0; j < 8; ++j) {
		uint32_t h[4], l[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			h[k] = to_tf32(v[4 * j + k]);
			l[k] = to_tf32(v[4 * j + k] - __uint_as_float(h[k]));
		}
		const uint32_t off = (uint32_t)row * 128u + ((uint32_t)(j ^ (row & 7)) << 4);
		*reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
		*reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
	}
}
}  // namespace cvtc

struct CostVolumeTc {  // tiles of 128 pixels of one row
	static int tiles_x(int w) { return umi::ceil_div(w, cvtc::BM); }
	static int tiles(int h, int w) { return tiles_x(w) * h; }
};

// The whole cost-volume pass of one CTA (every role), used by
// cost_volume_tc_kernel and as the first phase of batch_fused_kernel.
// Returns after every role has finished and TMEM is freed (ends with a CTA
// barrier), so the caller may reuse the shared memory.
__device__ __forceinline__ void cv_tc_phase(const Table& t, const cvtc::Params& prm, int* err, uint8_t* smem_raw) {
	using namespace umi_tc;
	using namespace cvtc;
	// 1024-byte aligned start (128-byte swizzled operand tiles), formed by
	// indexing the shared array so that the compiler keeps shared-memory accesses
	uint8_t* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
	uint8_t* outbuf = base + 2 * STAGE_BYTES;
	uint64_t* full = reinterpret_cast<uint64_t*>(outbuf + 8 * OUT_WARP_BYTES);  // [2]
	uint64_t* empty = full + 2;     // [2]
	uint64_t* accfull = empty + 2;  // [2]
	uint64_t* accempty = accfull + 2;
	uint64_t* drain = accempty + 2;
	uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
	volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int total = t.start[t.n];
	if (threadIdx.x == 0) {
		for (int s = 0; s < 2; ++s) {
			mbar_init(&full[s], PG);  // the threads of a producer group
			mbar_init(&empty[s], 1);
			mbar_init(&accfull[s], 1);
			mbar_init(&accempty[s], 4);  // one arrive per epilogue warp
		}
		mbar_init(drain, 1);
		*abort_flag = 0;
		fence_mbar_init();
	}
	if (warp == 10) {
		tmem_alloc(tmem_slot, TMEM_COLS);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *tmem_slot;

	if (warp < 10) {
		// ---- producers: group G takes tiles G, G + 2, ... of this CTA into stage G
		const int G = warp / 5, tg = threadIdx.x - G * PG;
		uint8_t* st_base = base + G * STAGE_BYTES;
		int u = 0;
		for (int tile = blockIdx.x + G * gridDim.x; tile < total && !*abort_flag; tile += 2 * gridDim.x, ++u) {
			const int i = find_image(t, tile);
			const Img& im = t.img[i];
			const int lt = tile - t.start[i], y = lt / im.tiles_x, x0 = (lt - y * im.tiles_x) * BM;
			const size_t plane = (size_t)im.h * im.w, row0 = (size_t)y * im.w;
			// operand rows r = tg and tg + 160 of 320: r < 128 is pixel r of A (L), else column r - 128 of B (R)
			float va[KC], vb[KC];
			const int r0 = tg, r1 = tg + PG;  // r1 >= 160: always a B row
			const int xa = r0 < BM ? r0 : r0 - BM, xb = r1 - BM;
			load_row((r0 < BM ? im.in : im.aux) + row0 + x0 + xa, plane, prm.channels, x0 + xa < im.w, va);
			load_row(im.aux + row0 + x0 + xb, plane, prm.channels, x0 + xb < im.w, vb);
			// the loads are in flight while the stage's previous MMAs finish
			if (!mbar_wait(&empty[G], (uint32_t)(u & 1) ^ 1u, abort_flag, err, kErrTimeoutEmpty)) break;
			uint8_t* bhi = st_base + 2 * A_BYTES;
			if (r0 < BM) store_row(st_base, st_base + A_BYTES, r0, va);
			else store_row(bhi, bhi + B_BYTES, xa, va);
			store_row(bhi, bhi + B_BYTES, xb, vb);
			fence_proxy_async_smem();  // generic-proxy stores visible to the MMA
			mbar_arrive(&full[G]);
		}
	} else if (warp == 10) {
		if (lane == 0) {
			// ---- MMA issuer
			int i = 0;
			for (int tile = blockIdx.x; tile < total && !*abort_flag; tile += gridDim.x, ++i) {
				const int s = i & 1;
				const uint32_t use = (uint32_t)(i >> 1);
				if (!mbar_wait(&accempty[s], (use & 1) ^ 1u, abort_flag, err, kErrTimeoutAccEmpty)) break;
				if (!mbar_wait(&full[s], use & 1, abort_flag, err, kErrTimeoutFull)) break;
				tc_fence_after();
				const uint32_t acc = tmem + (uint32_t)(s * BNN);
				const uint32_t sb = smem_u32(base + s * STAGE_BYTES);
				const uint64_t ahi = desc_kmajor_sw128(sb), alo = desc_kmajor_sw128(sb + A_BYTES);
				const uint64_t bhi = desc_kmajor_sw128(sb + 2 * A_BYTES), blo = desc_kmajor_sw128(sb + 2 * A_BYTES + B_BYTES);
#pragma unroll
				for (int kk = 0; kk < KC / 8; ++kk) {  // 8 tf32 = 32 bytes per K step
					mma_tf32(acc, ahi + 2 * kk, bhi + 2 * kk, IDESC, kk > 0);
					mma_tf32(acc, ahi + 2 * kk, blo + 2 * kk, IDESC, true);
					mma_tf32(acc, alo + 2 * kk, bhi + 2 * kk, IDESC, true);
				}
				mma_commit(&empty[s]);
				mma_commit(&accfull[s]);
			}
			mma_commit(drain);  // every MMA issued above finishes before TMEM is freed
			volatile int own = 0;
			mbar_wait(drain, 0, &own, err, kErrTimeoutAccum);
		}
		__syncwarp();
	} else {
		// ---- epilogue: warp w drains TMEM lanes 32 (w % 4) .. + 31 (pixels of the tile)
		const int qd = warp & 3;
		int i = 0;
		for (int tile = blockIdx.x; tile < total; tile += gridDim.x, ++i) {
			const int s = i & 1;
			const uint32_t use = (uint32_t)(i >> 1);
			if (!mbar_wait(&accfull[s], use & 1, abort_flag, err, kErrTimeoutAccum)) break;
			tc_fence_after();
			const int idx = find_image(t, tile);
			const Img& im = t.img[idx];
			const int lt = tile - t.start[idx], y = lt / im.tiles_x, x0 = (lt - y * im.tiles_x) * BM;
			const int px0 = x0 + 32 * qd, nvalid = min(32, im.w - px0);
			float* ob = reinterpret_cast<float*>(outbuf + (2 * qd + (i & 1)) * OUT_WARP_BYTES);
			if (lane == 0) bulk_wait_read_1();  // the store that last used ob (two tiles ago) has read it
			__syncwarp();
			// lane p keeps columns p .. p + 63 of the 96 its warp's band touches, at word
			// 64 p + (j - p) = 63 p + j (conflict-free); one 32-column load at a time
			const uint32_t ta = tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(s * BNN + 32 * qd);
#pragma unroll
			for (int k = 0; k < 3; ++k) {
				float v[32];
				tmem_ld32(ta + 32 * k, v);
#pragma unroll
				for (int j = 0; j < 32; ++j) {
					const int d = 32 * k + j - lane;
					if (d >= 0 && d < ND) ob[63 * lane + 32 * k + j] = v[j];
				}
			}
			tc_fence_before();
			__syncwarp();
			if (lane == 0) mbar_arrive(&accempty[s]);
			fence_proxy_async_smem();
			__syncwarp();
			if (lane == 0 && nvalid > 0) {
				bulk_store(im.out + ((size_t)y * im.w + px0) * ND, ob, (uint32_t)nvalid * ND * 4);
				bulk_commit();
			}
		}
		if (lane == 0) bulk_wait_all();
		__syncwarp();
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 10) {
		tc_fence_after();
		tmem_dealloc(tmem, TMEM_COLS);
	}
	__syncthreads();
}

__global__ void __launch_bounds__(cvtc::NTH, 1) cost_volume_tc_kernel(const Table t, const cvtc::Params prm, int* err) {
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	cv_tc_phase(t, prm, err, smem_raw);
}

// ------------------------------------------------------------------ launcher
template <class Op, class P>
__global__ void __launch_bounds__(NT, 2) batch_kernel(const Table t, const P p) {
	extern __shared__ __align__(16) float sm[];
	const int total = t.start[t.n];
	for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
		const int i = find_image(t, tile);
		Op::tile(t.img[i], tile - t.start[i], p, sm);
	}
}

template <class Op>
umi_status make_table(const umi_batch_image* images, int n, bool need_aux, Table& t) {
	t.n = n;
	t.start[0] = 0;
	for (int i = 0; i < n; ++i) {
		const umi_batch_image& b = images[i];
		if (b.h < 0 || b.w < 0) return umi::fail(UMI_ERR_INVALID_ARG, "batch image %d: negative size", i);
		const bool empty = b.h == 0 || b.w == 0;
		if (!empty && (!b.in || !b.out || (need_aux && !b.aux)))
			return umi::fail(UMI_ERR_INVALID_ARG, "batch image %d: null pointer", i);
		Img& m = t.img[i];
		m.in = b.in; m.aux = b.aux; m.out = b.out; m.h = b.h; m.w = b.w;
		m.tiles_x = empty ? 1 : Op::tiles_x(b.w);
		m.vec = umi::aligned(b.in, 16) && umi::aligned(b.out, 16) && (!b.aux || umi::aligned(b.aux, 16)) &&
		        (b.w % 4) == 0;
		const int64_t nt = empty ? 0 : (int64_t)Op::tiles(b.h, b.w);
		if (t.start[i] + nt > INT32_MAX) return umi::fail(UMI_ERR_UNSUPPORTED, "batch too large");
		t.start[i + 1] = t.start[i] + (int)nt;
	}
	return UMI_OK;
}

template <class Op, class P>
umi_status launch(const umi_batch_image* images, int n, const P& p, bool need_aux, cudaStream_t st) {
	Table t;
	UMI_TRY(make_table<Op>(images, n, need_aux, t));
	if (t.start[n] == 0) return UMI_OK;
	auto kern = batch_kernel<Op, P>;
	const size_t smem = Op::smem;
	if (smem > 48 * 1024)
		UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
		                         "cudaFuncSetAttribute"));
	int dev = 0, sms = 0, per_sm = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	UMI_TRY(umi::cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem),
	                         "cudaOccupancyMaxActiveBlocksPerMultiprocessor"));
	const int grid = std::max(1, std::min(t.start[n], sms * std::max(per_sm, 1)));
	kern<<<grid, NT, smem, st>>>(t, p);
	return umi::launch_status("batch_kernel");
}

// The tensor-core cost volume: nd = 64, channels <= 32 and a 16-byte aligned
// output for every image (its bulk stores start at multiples of 256 bytes
// from it); inputs are read with scalar loads, any width (else the FP32
// kernel serves).
bool cv_tc_eligible(const umi_batch_image* images, int n, const umi_batch_params& bp) {
	if (bp.nd != cvtc::ND || bp.channels < 1 || bp.channels > cvtc::KC) return false;
	for (int i = 0; i < n; ++i) {
		const umi_batch_image& b = images[i];
		if (b.h == 0 || b.w == 0) continue;
		if (!umi::aligned(b.out, 16)) return false;
	}
	return true;
}

umi_status launch_cv_tc(const umi_batch_image* images, int n, int channels, cudaStream_t st) {
	Table t;
	UMI_TRY(make_table<CostVolumeTc>(images, n, true, t));
	if (t.start[n] == 0) return UMI_OK;
	auto kern = cost_volume_tc_kernel;
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cvtc::SMEM),
	                         "cudaFuncSetAttribute"));
	int dev = 0, sms = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	const int grid = std::max(1, std::min(t.start[n], sms));  // one CTA per SM (shared memory, TMEM)
	kern<<<grid, cvtc::NTH, cvtc::SMEM, st>>>(t, cvtc::Params{channels}, nullptr);
	return umi::launch_status("cost_volume_tc_kernel");
}

// ------------------------------------------------------------------ one launch for a whole batch step
// batch_fused_kernel serves the three operators of a batch step in one
// persistent launch (one CTA per SM, the 480 threads of the tensor-core cost
// volume): every CTA first takes its share of the cost-volume tiles (the
// warp-specialised pass of cost_volume_tc_kernel, static round robin), then,
// with all 15 warps, its share of one queue that holds the per-pixel-weight
// filter's and the bilateral filter's tiles of every image.  Each image of
// that queue carries its own variant (tile shape = P block, pixels per
// thread = Expand), chosen per operator and size class by the autotuner.
constexpr int FNT = cvtc::NTH;
enum : int { kKindBil = 0, kKindWf = 8 };
constexpr int kFusedBilVariants = 4, kFusedWfVariants = 3;
template <int R> using FBil0 = Bilateral<R, 32, 30, 2, FNT>;
template <int R> using FBil1 = Bilateral<R, 32, 60, 4, FNT>;
template <int R> using FBil2 = Bilateral<R, 96, 20, 4, FNT>;
template <int R> using FBil3 = Bilateral<R, 32, 15, 1, FNT>;
using FWf0 = WFilter<4, FNT>;
using FWf1 = WFilter<2, FNT>;
using FWf2 = WFilter<1, FNT>;
constexpr size_t kFusedSimtSmem = sizeof(float) * (96 + 6) * (60 + 6);  // one halo buffer, any bilateral variant at r <= 3

template <int R>
__global__ void __launch_bounds__(FNT, 1)
batch_fused_kernel(const Table cv, const cvtc::Params cvp, const Table q, const BilParams bp, int* err) {
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	if (cv.start[cv.n] > 0) cv_tc_phase(cv, cvp, err, smem_raw);  // uniform over the CTA
	// Filter phase.  Bilateral halo tiles are double-buffered: the next
	// bilateral tile's cp.async loads run while the current one is computed.
	float* sm = reinterpret_cast<float*>(smem_raw);
	constexpr int BUFW = (int)(kFusedSimtSmem / sizeof(float));
	const int total = q.start[q.n];
	auto stage = [&](const Img& im, int lt, float* b) {
		switch (im.kind) {
			case kKindBil + 0: FBil0<R>::stage_async(im, lt, b); break;
			case kKindBil + 1: FBil1<R>::stage_async(im, lt, b); break;
			case kKindBil + 2: FBil2<R>::stage_async(im, lt, b); break;
			default: FBil3<R>::stage_async(im, lt, b); break;
		}
	};
	int buf = 0;
	bool staged = false;  // the current tile's halo is already in sm[buf]
	for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
		const int i = find_image(q, tile);
		const Img& im = q.img[i];
		const int lt = tile - q.start[i];
		if (im.kind >= kKindWf) {  // uniform over the CTA: every thread serves the same tile
			switch (im.kind) {
				case kKindWf + 0: FWf0::tile(im, lt, NoParams{}, sm); break;
				case kKindWf + 1: FWf1::tile(im, lt, NoParams{}, sm); break;
				default: FWf2::tile(im, lt, NoParams{}, sm); break;
			}
			staged = false;
			continue;
		}
		float* cur = sm + buf * BUFW;
		if (!staged) stage(im, lt, cur);
		const int next = tile + (int)gridDim.x;
		bool prefetched = false;
		if (next < total) {
			const int ni = find_image(q, next);
			if (q.img[ni].kind < kKindWf) {
				stage(q.img[ni], next - q.start[ni], sm + (buf ^ 1) * BUFW);
				prefetched = true;
			}
		}
		if (prefetched) asm volatile("cp.async.wait_group 1;" ::: "memory");
		else asm volatile("cp.async.wait_group 0;" ::: "memory");
		__syncthreads();  // the current halo tile is complete for every thread
		switch (im.kind) {
			case kKindBil + 0: FBil0<R>::compute(im, lt, bp, cur); break;
			case kKindBil + 1: FBil1<R>::compute(im, lt, bp, cur); break;
			case kKindBil + 2: FBil2<R>::compute(im, lt, bp, cur); break;
			default: FBil3<R>::compute(im, lt, bp, cur); break;
		}
		__syncthreads();  // sm[buf] is free for the tile after next
		buf ^= 1;
		staged = prefetched;
	}
	asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// tiles_x and tile count of an image under a fused kind
void fused_tiles(int kind, int h, int w, int* tx, int64_t* nt) {
	switch (kind) {
		case kKindBil + 0: *tx = FBil0<1>::tiles_x(w); *nt = FBil0<1>::tiles(h, w); return;
		case kKindBil + 1: *tx = FBil1<1>::tiles_x(w); *nt = FBil1<1>::tiles(h, w); return;
		case kKindBil + 2: *tx = FBil2<1>::tiles_x(w); *nt = FBil2<1>::tiles(h, w); return;
		case kKindBil + 3: *tx = FBil3<1>::tiles_x(w); *nt = FBil3<1>::tiles(h, w); return;
		case kKindWf + 0: *tx = FWf0::tiles_x(w); *nt = FWf0::tiles(h, w); return;
		case kKindWf + 1: *tx = FWf1::tiles_x(w); *nt = FWf1::tiles(h, w); return;
		default: *tx = FWf2::tiles_x(w); *nt = FWf2::tiles(h, w); return;
	}
}

umi_status fused_queue(const umi_batch_job* const jobs[2], Table& t) {
	t.n = 0;
	t.start[0] = 0;
	for (int jb = 0; jb < 2; ++jb) {
		const umi_batch_job* j = jobs[jb];
		if (!j) continue;
		const bool wf = j->op == UMI_OP_WFILTER_PP;
		const int nvar = wf ? kFusedWfVariants : kFusedBilVariants;
		for (int i = 0; i < j->n_images; ++i) {
			const umi_batch_image& b = j->images[i];
			if (b.h < 0 || b.w < 0) return umi::fail(UMI_ERR_INVALID_ARG, "fused batch: negative size");
			if (b.h == 0 || b.w == 0) continue;
			if (!b.in || !b.out || (wf && !b.aux)) return umi::fail(UMI_ERR_INVALID_ARG, "fused batch: null pointer");
			if (t.n == MAXIMG) return umi::fail(UMI_ERR_UNSUPPORTED, "fused batch: more than %d filter images", MAXIMG);
			const int v = j->variants ? j->variants[i] : 0;
			if (v < 0 || v >= nvar) return umi::fail(UMI_ERR_INVALID_ARG, "fused batch: variant %d (0..%d)", v, nvar - 1);
			Img& m = t.img[t.n];
			m.in = b.in; m.aux = b.aux; m.out = b.out; m.h = b.h; m.w = b.w;
			m.vec = umi::aligned(b.in, 16) && umi::aligned(b.out, 16) && (!b.aux || umi::aligned(b.aux, 16)) &&
			        (b.w % 4) == 0;
			m.kind = (wf ? kKindWf : kKindBil) + v;
			int64_t nt = 0;
			fused_tiles(m.kind, b.h, b.w, &m.tiles_x, &nt);
			if (t.start[t.n] + nt > INT32_MAX) return umi::fail(UMI_ERR_UNSUPPORTED, "fused batch too large");
			t.start[t.n + 1] = t.start[t.n] + (int)nt;
			++t.n;
		}
	}
	return UMI_OK;
}

template <int R>
umi_status launch_fused_r(const Table& cv, const cvtc::Params& cvp, const Table& q, const BilParams& bp, cudaStream_t st) {
	auto kern = batch_fused_kernel<R>;
	const bool has_cv = cv.start[cv.n] > 0;
	const size_t smem = has_cv ? cvtc::SMEM : 2 * kFusedSimtSmem;
	static_assert(2 * kFusedSimtSmem <= cvtc::SMEM, "two halo buffers fit the cost volume's shared memory");
	UMI_TRY(umi::cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cvtc::SMEM),
	                         "cudaFuncSetAttribute"));
	int dev = 0, sms = 0;
	UMI_TRY(umi::cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(umi::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	const int tiles = std::max(cv.start[cv.n], q.start[q.n]);
	const int grid = std::max(1, std::min(tiles, sms));  // 480 threads x 128 registers: one CTA per SM
	kern<<<grid, FNT, smem, st>>>(cv, cvp, q, bp, nullptr);
	return umi::launch_status("batch_fused_kernel");
}

umi_status bil_params(const umi_batch_params& bp, BilParams& p) {
	if (bp.radius < 1 || bp.radius > 3) return umi::fail(UMI_ERR_UNSUPPORTED, "bilateral: radius %d (1..3)", bp.radius);
	if (!(bp.sigma_s > 0.0f) || !(bp.sigma_r > 0.0f)) return umi::fail(UMI_ERR_INVALID_ARG, "bilateral: sigmas must be > 0");
	const double log2e = 1.4426950408889634;
	p.k = (float)(-log2e / (2.0 * (double)bp.sigma_r * (double)bp.sigma_r));
	const int r = bp.radius;
	for (int dy = 0; dy <= 2 * r; ++dy)
		for (int dx = 0; dx <= 2 * r; ++dx) {
			const double a = (double)((dy - r) * (dy - r) + (dx - r) * (dx - r));
			p.lsw[dy][dx] = (float)(-a / (2.0 * (double)bp.sigma_s * (double)bp.sigma_s) * log2e);
		}
	return UMI_OK;
}

umi_status run_fused(const umi_batch_job* jobs, int n_jobs, cudaStream_t st) {
	if (n_jobs < 0 || (n_jobs > 0 && !jobs)) return umi::fail(UMI_ERR_INVALID_ARG, "fused batch: bad job list");
	const umi_batch_job* by_op[3] = {nullptr, nullptr, nullptr};
	for (int k = 0; k < n_jobs; ++k) {
		const int op = jobs[k].op;
		if (op < 0 || op > 2) return umi::fail(UMI_ERR_INVALID_ARG, "fused batch: unknown op %d", op);
		if (by_op[op]) return umi::fail(UMI_ERR_INVALID_ARG, "fused batch: two jobs of op %d", op);
		if (jobs[k].n_images < 0 || jobs[k].n_images > MAXIMG || (jobs[k].n_images > 0 && !jobs[k].images))
			return umi::fail(UMI_ERR_INVALID_ARG, "fused batch: job of op %d has a bad image list", op);
		by_op[op] = &jobs[k];
	}
	Table cv;
	cv.n = 0;
	cv.start[0] = 0;
	cvtc::Params cvp{0};
	if (const umi_batch_job* j = by_op[UMI_OP_COST_VOLUME]) {
		if (!cv_tc_eligible(j->images, j->n_images, j->params))
			return umi::fail(UMI_ERR_UNSUPPORTED,
			                 "fused batch: the cost volume needs nd = 64, 1..32 channels and 16-byte aligned outputs");
		UMI_TRY(make_table<CostVolumeTc>(j->images, j->n_images, true, cv));
		cvp.channels = j->params.channels;
	}
	Table q;
	const umi_batch_job* const simt[2] = {by_op[UMI_OP_WFILTER_PP], by_op[UMI_OP_BILATERAL]};
	UMI_TRY(fused_queue(simt, q));
	BilParams bp{};
	int r = 1;
	if (const umi_batch_job* j = by_op[UMI_OP_BILATERAL]) {
		UMI_TRY(bil_params(j->params, bp));
		r = j->params.radius;
	}
	if (cv.start[cv.n] == 0 && q.start[q.n] == 0) return UMI_OK;
	switch (r) {
		case 1: return launch_fused_r<1>(cv, cvp, q, bp, st);
		case 2: return launch_fused_r<2>(cv, cvp, q, bp, st);
		default: return launch_fused_r<3>(cv, cvp, q, bp, st);
	}
}

// Variant tables.
constexpr int kBilVariants = 4;
template <int R>
umi_status run_bilateral_r(const umi_batch_image* im, int n, const BilParams& p, int v, cudaStream_t st) {
	switch (v) {
		case 1: return launch<Bilateral<R, 32, 32, 4>>(im, n, p, false, st);
		case 2: return launch<Bilateral<R, 64, 16, 4>>(im, n, p, false, st);
		case 3: return launch<Bilateral<R, 32, 8, 1>>(im, n, p, false, st);
		default: return launch<Bilateral<R, 32, 16, 2>>(im, n, p, false, st);
	}
}
constexpr int kWfVariants = 3;
constexpr int kCvVariants = 2;  // tensor cores (where eligible), FP32

umi_status run_bilateral(const umi_batch_image* im, int n, const umi_batch_params& bp, int v, cudaStream_t st) {
	BilParams p{};
	UMI_TRY(bil_params(bp, p));
	switch (bp.radius) {
		case 1: return run_bilateral_r<1>(im, n, p, v, st);
		case 2: return run_bilateral_r<2>(im, n, p, v, st);
		default: return run_bilateral_r<3>(im, n, p, v, st);
	}
}

umi_status run_wfilter(const umi_batch_image* im, int n, int v, cudaStream_t st) {
	switch (v) {
		case 1: return launch<WFilter<2>>(im, n, NoParams{}, true, st);
		case 2: return launch<WFilter<1>>(im, n, NoParams{}, true, st);
		default: return launch<WFilter<4>>(im, n, NoParams{}, true, st);
	}
}

umi_status run_cost_volume(const umi_batch_image* im, int n, const umi_batch_params& bp, int v, cudaStream_t st) {
	if (bp.channels < 1) return umi::fail(UMI_ERR_INVALID_ARG, "cost volume: %d channels", bp.channels);
	// variant 0 (default): the tensor-core kernel where it applies; variant 1: the FP32 kernel
	if (v != 1 && cv_tc_eligible(im, n, bp)) return launch_cv_tc(im, n, bp.channels, st);
	const CvParams p{bp.channels};
	switch (bp.nd) {
		case 16: return launch<CostVolume<2>>(im, n, p, true, st);
		case 32: return launch<CostVolume<4>>(im, n, p, true, st);
		case 64: return launch<CostVolume<8>>(im, n, p, true, st);
		default: return umi::fail(UMI_ERR_UNSUPPORTED, "cost volume: nd %d (16, 32 or 64)", bp.nd);
	}
}

umi_status run(int op, const umi_batch_image* im, int n, const umi_batch_params* bp, int v, cudaStream_t st) {
	if (n < 0 || n > MAXIMG) return umi::fail(UMI_ERR_INVALID_ARG, "batch of %d images (max %d)", n, MAXIMG);
	if (n > 0 && !im) return umi::fail(UMI_ERR_INVALID_ARG, "null image table");
	if (!bp && op != UMI_OP_WFILTER_PP) return umi::fail(UMI_ERR_INVALID_ARG, "null params");
	switch (op) {
		case UMI_OP_BILATERAL: return run_bilateral(im, n, *bp, v, st);
		case UMI_OP_WFILTER_PP: return run_wfilter(im, n, v, st);
		case UMI_OP_COST_VOLUME: return run_cost_volume(im, n, *bp, v, st);
		default: return umi::fail(UMI_ERR_INVALID_ARG, "unknown batch op %d", op);
	}
}

}  // namespace

extern "C" int32_t umi_batch_variants(int32_t op) {
	switch (op) {
		case UMI_OP_BILATERAL: return kBilVariants;
		case UMI_OP_WFILTER_PP: return kWfVariants;
		case UMI_OP_COST_VOLUME: return kCvVariants;
		default: return 0;
	}
}

extern "C" umi_status umi_batch_run(int32_t op, const umi_batch_image* images, int32_t n_images,
                                    const umi_batch_params* params, int32_t variant, void* stream) {
	const umi_status st = run(op, images, n_images, params, variant, umi::as_stream(stream));
	return st == UMI_OK ? umi::ok() : st;
}

extern "C" umi_status umi_bilateral_f32(const float* in, float* out, int32_t h, int32_t w, int32_t radius, float sigma_s,
                                        float sigma_r, void* stream) {
	const umi_batch_image im{in, nullptr, out, h, w};
	umi_batch_params p{};
	p.radius = radius; p.sigma_s = sigma_s; p.sigma_r = sigma_r;
	return umi_batch_run(UMI_OP_BILATERAL, &im, 1, &p, -1, stream);
}

extern "C" umi_status umi_wfilter3x3_pp_f32(const float* in, const float* wts, float* out, int32_t h, int32_t w,
                                            void* stream) {
	const umi_batch_image im{in, wts, out, h, w};
	return umi_batch_run(UMI_OP_WFILTER_PP, &im, 1, nullptr, -1, stream);
}

extern "C" umi_status umi_cost_volume_dot_f32(const float* left, const float* right, float* cv, int32_t c, int32_t h,
                                              int32_t w, int32_t nd, void* stream) {
	const umi_batch_image im{left, right, cv, h, w};
	umi_batch_params p{};
	p.channels = c; p.nd = nd;
	return umi_batch_run(UMI_OP_COST_VOLUME, &im, 1, &p, -1, stream);
}

extern "C" umi_status umi_autotune_batch(int32_t op, const umi_batch_image* images, int32_t n_images,
                                         const umi_batch_params* params, int32_t reps, int32_t* best_variant,
                                         float* best_ms, void* stream) {
	if (!best_variant || !best_ms || reps < 1) return umi::fail(UMI_ERR_INVALID_ARG, "autotune: bad arguments");
	const int nv = umi_batch_variants(op);
	if (nv == 0) return umi::fail(UMI_ERR_INVALID_ARG, "autotune: unknown op %d", op);
	const cudaStream_t st = umi::as_stream(stream);
	cudaEvent_t a, b;
	UMI_TRY(umi::cuda_status(cudaEventCreate(&a), "cudaEventCreate"));
	UMI_TRY(umi::cuda_status(cudaEventCreate(&b), "cudaEventCreate"));
	int best = 0;
	float best_t = 0.0f;
	umi_status rc = UMI_OK;
	for (int v = 0; v < nv && rc == UMI_OK; ++v) {
		rc = run(op, images, n_images, params, v, st);  // warm-up
		if (rc != UMI_OK) break;
		cudaEventRecord(a, st);
		for (int r = 0; r < reps && rc == UMI_OK; ++r) rc = run(op, images, n_images, params, v, st);
		cudaEventRecord(b, st);
		if (rc != UMI_OK) break;
		rc = umi::cuda_status(cudaEventSynchronize(b), "cudaEventSynchronize");
		float ms = 0.0f;
		cudaEventElapsedTime(&ms, a, b);
		ms /= reps;
		if (v == 0 || ms < best_t) { best_t = ms; best = v; }
	}
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	if (rc != UMI_OK) return rc;
	*best_variant = best;
	*best_ms = best_t;
	return umi::ok();
}

extern "C" int32_t umi_batch_fused_variants(int32_t op) {
	switch (op) {
		case UMI_OP_BILATERAL: return kFusedBilVariants;
		case UMI_OP_WFILTER_PP: return kFusedWfVariants;
		case UMI_OP_COST_VOLUME: return 1;
		default: return 0;
	}
}

extern "C" umi_status umi_batch_run_fused(const umi_batch_job* jobs, int32_t n_jobs, void* stream) {
	const umi_status st = run_fused(jobs, n_jobs, umi::as_stream(stream));
	return st == UMI_OK ? umi::ok() : st;
}

// ---- batch graphs: a sequence of persistent batched launches recorded once
// into a CUDA graph and replayed with one cudaGraphLaunch.
struct umi_batch_graph {
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	cudaGraphNode_t last = nullptr;
	cudaStream_t capture = nullptr;
	int n_ops = 0;
};

extern "C" umi_status umi_batch_graph_create(umi_batch_graph** out) {
	if (!out) return umi::fail(UMI_ERR_INVALID_ARG, "batch graph: null pointer");
	*out = nullptr;
	umi_batch_graph* g = new (std::nothrow) umi_batch_graph();
	if (!g) return umi::fail(UMI_ERR_NO_MEMORY, "batch graph: host allocation failed");
	umi_status rc = umi::cuda_status(cudaGraphCreate(&g->graph, 0), "cudaGraphCreate");
	if (rc == UMI_OK)
		rc = umi::cuda_status(cudaStreamCreateWithFlags(&g->capture, cudaStreamNonBlocking), "cudaStreamCreate");
	if (rc != UMI_OK) {
		umi_batch_graph_destroy(g);
		return rc;
	}
	*out = g;
	return umi::ok();
}

extern "C" umi_status umi_batch_graph_add(umi_batch_graph* g, int32_t op, const umi_batch_image* images,
                                          int32_t n_images, const umi_batch_params* params, int32_t variant) {
	if (!g) return umi::fail(UMI_ERR_INVALID_ARG, "batch graph: null graph");
	UMI_TRY(umi::cuda_status(cudaStreamBeginCapture(g->capture, cudaStreamCaptureModeThreadLocal),
	                         "cudaStreamBeginCapture"));
	const umi_status rc = run(op, images, n_images, params, variant, g->capture);
	cudaGraph_t sub = nullptr;
	const umi_status ec = umi::cuda_status(cudaStreamEndCapture(g->capture, &sub), "cudaStreamEndCapture");
	if (rc != UMI_OK || ec != UMI_OK) {
		if (sub) cudaGraphDestroy(sub);
		return rc != UMI_OK ? rc : ec;
	}
	cudaGraphNode_t node = nullptr;
	const umi_status ac = umi::cuda_status(
		cudaGraphAddChildGraphNode(&node, g->graph, g->last ? &g->last : nullptr, g->last ? 1 : 0, sub),
		"cudaGraphAddChildGraphNode");
	cudaGraphDestroy(sub);  // the child node holds its own copy
	UMI_TRY(ac);
	g->last = node;
	++g->n_ops;
	if (g->exec) {
		cudaGraphExecDestroy(g->exec);
		g->exec = nullptr;
	}
	return umi::ok();
}

extern "C" umi_status umi_batch_graph_add_fused(umi_batch_graph* g, const umi_batch_job* jobs, int32_t n_jobs) {
	if (!g) return umi::fail(UMI_ERR_INVALID_ARG, "batch graph: null graph");
	UMI_TRY(umi::cuda_status(cudaStreamBeginCapture(g->capture, cudaStreamCaptureModeThreadLocal),
	                         "cudaStreamBeginCapture"));
	const umi_status rc = run_fused(jobs, n_jobs, g->capture);
	cudaGraph_t sub = nullptr;
	const umi_status ec = umi::cuda_status(cudaStreamEndCapture(g->capture, &sub), "cudaStreamEndCapture");
	if (rc != UMI_OK || ec != UMI_OK) {
		if (sub) cudaGraphDestroy(sub);
		return rc != UMI_OK ? rc : ec;
	}
	cudaGraphNode_t node = nullptr;
	const umi_status ac = umi::cuda_status(
		cudaGraphAddChildGraphNode(&node, g->graph, g->last ? &g->last : nullptr, g->last ? 1 : 0, sub),
		"cudaGraphAddChildGraphNode");
	cudaGraphDestroy(sub);
	UMI_TRY(ac);
	g->last = node;
	++g->n_ops;
	if (g->exec) {
		cudaGraphExecDestroy(g->exec);
		g->exec = nullptr;
	}
	return umi::ok();
}

extern "C" umi_status umi_batch_graph_launch(umi_batch_graph* g, void* stream) {
	if (!g) return umi::fail(UMI_ERR_INVALID_ARG, "batch graph: null graph");
	if (g->n_ops == 0) return umi::ok();
	if (!g->exec) UMI_TRY(umi::cuda_status(cudaGraphInstantiate(&g->exec, g->graph, 0), "cudaGraphInstantiate"));
	UMI_TRY(umi::cuda_status(cudaGraphLaunch(g->exec, umi::as_stream(stream)), "cudaGraphLaunch"));
	return umi::ok();
}

extern "C" void umi_batch_graph_destroy(umi_batch_graph* g) {
	if (!g) return;
	if (g->exec) cudaGraphExecDestroy(g->exec);
	if (g->graph) cudaGraphDestroy(g->graph);
	if (g->capture) cudaStreamDestroy(g->capture);
	delete g;
}
