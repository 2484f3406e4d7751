// Integral image uint8 -> int32, sm_103a.
//
// Replaces the two Execute calls of main/iimg.cu:37-82 (a Loop-output prefix
// scan along x written transposed, applied twice) with one read of the uint8
// frame from HBM and one write of the int32 result.
//
// The frame is cut into TH x TW tiles.  With the inclusive integral image
// ii[y][x] and a tile at (Y0, X0):
//   ii[y][x] = corner + sum_{X0<=x'<=x} top[x'] + sum_{Y0<=y'<=y} left[y'] + local[y][x]
//   top[x]   = sum over all rows above the tile of column x,
//   left[y]  = sum over all columns left of the tile of row y,
//   corner   = sum over the whole rectangle above-left of the tile,
//   local    = the 2-D prefix inside the tile.
// Kernel 1 (iimg_tile_sums) writes per-tile row sums, column sums and tile
// totals to a small workspace (about 4% of the output).  Kernel 2
// (iimg_tiles) loads its tile and computes the local prefix with warp-shuffle
// scans, then waits on kernel 1 (programmatic dependent launch: the wait is
// griddepcontrol.wait, so everything before it overlaps kernel 1), adds the
// carries from the workspace and writes the tile with 16-byte stores.
#include "common.h"

namespace {

constexpr int TH = 32;   // tile rows: 8 warps x 4 rows
constexpr int TW = 128;  // tile columns: 32 lanes x 4 columns
constexpr int RPW = 4;   // rows per warp
constexpr int NT = 256;

struct IimgGeom {
	int h, w, ntx, nty;
	int vec_in;   // in is 4-byte aligned and w % 4 == 0
	int vec_out;  // out is 16-byte aligned and w % 4 == 0
	int32_t* rowsum;   // [h][ntx]
	int32_t* colsum;   // [nty][w]
	int32_t* tilesum;  // [nty][ntx]
};

// Four consecutive pixels of row y starting at column x (zeros past the edge).
__device__ __forceinline__ void load4(const uint8_t* __restrict__ in, const IimgGeom& g, int y, int x, uint32_t v[4]) {
	const uint8_t* row = in + (size_t)y * g.w;
	if (g.vec_in && x + 3 < g.w) {
		const uint32_t p = __ldg(reinterpret_cast<const uint32_t*>(row + x));
		v[0] = p & 0xff; v[1] = (p >> 8) & 0xff; v[2] = (p >> 16) & 0xff; v[3] = p >> 24;
	} else {
#pragma unroll
		for (int k = 0; k < 4; ++k) v[k] = (x + k < g.w) ? __ldg(row + x + k) : 0u;
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
	__shared__ uint32_t colpart[NT / 32][TW];
	__shared__ uint32_t warptot[TW / 32];
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
	// Let the dependent tile kernel get scheduled as soon as SMs free up; it
	// waits for this grid's results with griddepcontrol.wait.
	asm volatile("griddepcontrol.launch_dependents;");
#endif
	const int tx = blockIdx.x, ty = blockIdx.y;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int X0 = tx * TW, Y0 = ty * TH;
	uint32_t col[4] = {0, 0, 0, 0};
#pragma unroll
	for (int r = 0; r < RPW; ++r) {
		const int y = Y0 + warp * RPW + r;
		uint32_t v[4] = {0, 0, 0, 0};
		if (y < g.h) load4(in, g, y, X0 + 4 * lane, v);
		uint32_t s = v[0] + v[1] + v[2] + v[3];
		s = __reduce_add_sync(0xffffffffu, s);
		if (lane == 0 && y < g.h) g.rowsum[(size_t)y * g.ntx + tx] = (int32_t)s;
#pragma unroll
		for (int k = 0; k < 4; ++k) col[k] += v[k];
	}
#pragma unroll
	for (int k = 0; k < 4; ++k) colpart[warp][4 * lane + k] = col[k];
	__syncthreads();
	if (threadIdx.x < TW) {
		uint32_t s = 0;
#pragma unroll
		for (int i = 0; i < NT / 32; ++i) s += colpart[i][threadIdx.x];
		const int x = X0 + threadIdx.x;
		if (x < g.w) g.colsum[(size_t)ty * g.w + x] = (int32_t)s;
		s = __reduce_add_sync(0xffffffffu, s);
		if ((threadIdx.x & 31) == 0) warptot[threadIdx.x >> 5] = s;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		const uint32_t t = warptot[0] + warptot[1] + warptot[2] + warptot[3];
		g.tilesum[(size_t)ty * g.ntx + tx] = (int32_t)t;
	}
}

__global__ void __launch_bounds__(NT) iimg_tiles(const uint8_t* __restrict__ in, int32_t* __restrict__ out,
                                                 const IimgGeom g) {
	__shared__ uint32_t wtot[NT / 32][TW];  // per-warp column totals, then their exclusive prefix
	__shared__ uint32_t topx[TW];           // inclusive x-prefix of the top carries
	__shared__ uint32_t lefty[TH];          // inclusive y-prefix of the left carries
	__shared__ uint32_t cornerp[NT / 32];
	const int tx = blockIdx.x, ty = blockIdx.y;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int X0 = tx * TW, Y0 = ty * TH;

	// Local 2-D prefix (needs only the input: runs before the dependency wait).
	uint32_t loc[RPW][4];
	uint32_t col[4] = {0, 0, 0, 0};
#pragma unroll
	for (int r = 0; r < RPW; ++r) {
		const int y = Y0 + warp * RPW + r;
		uint32_t v[4] = {0, 0, 0, 0};
		if (y < g.h) load4(in, g, y, X0 + 4 * lane, v);
		v[1] += v[0]; v[2] += v[1]; v[3] += v[2];
		const uint32_t excl = warp_incl_scan(v[3], lane) - v[3];
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			col[k] += v[k] + excl;
			loc[r][k] = col[k];
		}
	}
#pragma unroll
	for (int k = 0; k < 4; ++k) wtot[warp][4 * lane + k] = col[k];
	__syncthreads();
	if (threadIdx.x < TW) {
		uint32_t run = 0;
#pragma unroll
		for (int i = 0; i < NT / 32; ++i) {
			const uint32_t t = wtot[i][threadIdx.x];
			wtot[i][threadIdx.x] = run;
			run += t;
		}
	}

	// Carries from kernel 1.
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
	asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
	if (threadIdx.x < TW) {
		const int x = X0 + threadIdx.x;
		uint32_t s = 0;
		if (x < g.w)
			for (int t = 0; t < ty; ++t) s += (uint32_t)__ldcg(g.colsum + (size_t)t * g.w + x);
		s = warp_incl_scan(s, lane);
		topx[threadIdx.x] = s;
	} else if (threadIdx.x < TW + TH) {
		const int r = threadIdx.x - TW;
		const int y = Y0 + r;
		uint32_t s = 0;
		if (y < g.h)
			for (int t = 0; t < tx; ++t) s += (uint32_t)__ldcg(g.rowsum + (size_t)y * g.ntx + t);
		lefty[r] = warp_incl_scan(s, lane);
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
	// Stitch the four warps' x-prefix pieces of topx (each warp scanned 32 columns).
	uint32_t corner = 0;
#pragma unroll
	for (int i = 0; i < NT / 32; ++i) corner += cornerp[i];
	uint32_t topv[4];
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		const int c = 4 * lane + k;
		uint32_t t = topx[c];
		for (int seg = 0; seg < (c >> 5); ++seg) t += topx[seg * 32 + 31];
		topv[k] = t + corner + wtot[warp][c];
	}
#pragma unroll
	for (int r = 0; r < RPW; ++r) {
		const int y = Y0 + warp * RPW + r;
		if (y >= g.h) break;
		const uint32_t lv = lefty[warp * RPW + r];
		int32_t o[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) o[k] = (int32_t)(loc[r][k] + topv[k] + lv);
		const int x = X0 + 4 * lane;
		int32_t* dst = out + (size_t)y * g.w + x;
		if (g.vec_out && x + 3 < g.w) {
			*reinterpret_cast<int4*>(dst) = make_int4(o[0], o[1], o[2], o[3]);
		} else {
#pragma unroll
			for (int k = 0; k < 4; ++k)
				if (x + k < g.w) dst[k] = o[k];
		}
	}
}

size_t ws_bytes(int h, int w) {
	const size_t ntx = umi::ceil_div(w, TW), nty = umi::ceil_div(h, TH);
	auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
	return al((size_t)h * ntx * 4) + al(nty * (size_t)w * 4) + al(nty * ntx * 4);
}

}  // namespace

extern "C" size_t umi_iimg_u8_i32_workspace_bytes(int32_t h, int32_t w) {
	if (h <= 0 || w <= 0) return 0;
	return ws_bytes(h, w);
}

extern "C" umi_status umi_iimg_u8_i32(const uint8_t* in, int32_t* out, int32_t h, int32_t w, void* workspace,
                                      size_t workspace_bytes, void* stream) {
	if (h < 0 || w < 0) return umi::fail(UMI_ERR_INVALID_ARG, "iimg: negative size %dx%d", h, w);
	if (h == 0 || w == 0) return umi::ok();
	if (!in || !out || !workspace) return umi::fail(UMI_ERR_INVALID_ARG, "iimg: null pointer");
	if (!umi::aligned(workspace, 16)) return umi::fail(UMI_ERR_INVALID_ARG, "iimg: workspace not 16-byte aligned");
	if (workspace_bytes < ws_bytes(h, w))
		return umi::fail(UMI_ERR_NO_MEMORY, "iimg: workspace of %zu bytes, need %zu", workspace_bytes, ws_bytes(h, w));
	if ((int64_t)h * w > (int64_t)1 << 31) return umi::fail(UMI_ERR_UNSUPPORTED, "iimg: frame larger than 2^31 pixels");
	IimgGeom g{};
	g.h = h; g.w = w;
	g.ntx = umi::ceil_div(w, TW);
	g.nty = umi::ceil_div(h, TH);
	g.vec_in = umi::aligned(in, 4) && (w % 4) == 0;
	g.vec_out = umi::aligned(out, 16) && (w % 4) == 0;
	auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
	char* ws = static_cast<char*>(workspace);
	g.rowsum = reinterpret_cast<int32_t*>(ws);
	g.colsum = reinterpret_cast<int32_t*>(ws + al((size_t)h * g.ntx * 4));
	g.tilesum = reinterpret_cast<int32_t*>(ws + al((size_t)h * g.ntx * 4) + al((size_t)g.nty * w * 4));
	const cudaStream_t st = umi::as_stream(stream);
	const dim3 grid(g.ntx, g.nty);
	iimg_tile_sums<<<grid, NT, 0, st>>>(in, g);
	UMI_TRY(umi::launch_status("iimg_tile_sums"));
	cudaLaunchConfig_t cfg{};
	cfg.gridDim = grid;
	cfg.blockDim = dim3(NT);
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	UMI_TRY(umi::cuda_status(cudaLaunchKernelEx(&cfg, iimg_tiles, in, out, g), "iimg_tiles"));
	return umi::ok();
}
