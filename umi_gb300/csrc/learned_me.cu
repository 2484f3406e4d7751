// Learned motion proposal for block motion estimation (sm_103a).
//
// No counterpart in the reference: a small CNN proposes one motion vector
// per 16x16 block from the 1/4-downsampled frame pair, the UMI SAD kernel
// (full_me.cu) refines it in a small window, and blocks whose refined SAD is
// above a threshold fall back to exhaustive search.
//
// Network (all hand-written kernels below; fp32 master parameters, bf16
// weights in the forward/backward arithmetic, fp32 accumulation):
//   x0  = ((cur, ref) box-averaged 4x4 - 128) / 32                  (2, H4, W4)
//   a_l = ReLU(conv3x3_dil(a_{l-1}; W_l, b_l)), dilations 1, 2, 4, 8 (32, H4, W4)
//   mv  = Wh . a4[:, 4 cells x 4 cells of the block] + bh          (nblk, 2)
// The dilations give a receptive field of +-15 cells (+-60 pixels at full
// resolution).  mv is in units of 16 pixels.  Training minimises the smooth-L1
// distance to full-search vectors / 16 with Adam.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "common.h"
#include "me_pipeline.h"

namespace umi {
umi_status menet_conv_tc(const void* in, void* out, const void* wpack, const float* bias, int h, int w, int dil,
                         int* err, cudaStream_t st);
}

namespace {

constexpr int CH = 32;       // channels of every hidden layer
constexpr int NL = 4;        // conv layers
constexpr int HEADF = CH * 16;  // head features per block (32 channels x 4 x 4 cells)
constexpr int DIL[NL] = {1, 2, 4, 8};
constexpr int CIN[NL] = {2, CH, CH, CH};
constexpr int NT = 256;

// ---- parameter layout (fp32 master copy; bf16 copies are derived from it)
struct Layout {
	int w[NL], b[NL], wh, bh, total;
	Layout() {
		int o = 0;
		for (int l = 0; l < NL; ++l) {
			w[l] = o; o += CH * CIN[l] * 9;
			b[l] = o; o += CH;
		}
		wh = o; o += 2 * HEADF;
		bh = o; o += 2;
		total = o;
	}
};

// ---- workspace layout for a frame of h x w pixels
struct Work {
	int H4, W4, P, nbx, nby, nblk, tiles_wg;
	size_t x0, act[NL], dA[2], wb[NL], wt[NL], pred, centers, list, count, alist, amv, wpart, hpart, lpart;
	size_t nhwc[2], wtc[NL], err;  // tensor-core inference: bf16 (H4, W4, 32) activations, packed weights
	size_t bytes;
	Work(int h, int w) {
		H4 = h / 4; W4 = w / 4; P = H4 * W4;
		nbx = w / 16; nby = h / 16; nblk = nbx * nby;
		tiles_wg = umi::ceil_div(W4, 32) * umi::ceil_div(H4, 4);
		size_t o = 0;
		auto take = [&](size_t n) { size_t r = o; o += (n + 255) & ~size_t(255); return r; };
		x0 = take(sizeof(float) * 2 * P);
		for (int l = 0; l < NL; ++l) act[l] = take(sizeof(float) * CH * P);
		for (int i = 0; i < 2; ++i) dA[i] = take(sizeof(float) * CH * P);
		for (int l = 0; l < NL; ++l) wb[l] = take(2 * CH * CIN[l] * 9);
		for (int l = 0; l < NL; ++l) wt[l] = take(2 * CH * CIN[l] * 9);
		pred = take(sizeof(float) * 2 * nblk);
		centers = take(sizeof(int32_t) * 2 * nblk);
		list = take(sizeof(int32_t) * nblk);
		count = take(sizeof(int32_t) * 4);  // [0] fallback blocks, [2] audited blocks
		alist = take(sizeof(int32_t) * nblk);
		amv = take(sizeof(int32_t) * 3 * nblk);
		wpart = take(sizeof(float) * (size_t)tiles_wg * (CH * CH * 9 + CH));
		hpart = take(sizeof(float) * (size_t)umi::ceil_div(nblk, 8) * (2 * HEADF + 2));
		lpart = take(sizeof(float) * (size_t)umi::ceil_div(nblk, 8));
		for (int i = 0; i < 2; ++i) nhwc[i] = take((size_t)P * 64);
		for (int l = 0; l < NL; ++l) wtc[l] = take(2 * CH * 9 * CH);
		err = take(sizeof(int32_t));
		bytes = o;
	}
	template <class T> T* at(void* ws, size_t off) const { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }
};

// ------------------------------------------------------------------ kernels
__global__ void downsample4_kernel(const uint8_t* __restrict__ cur, const uint8_t* __restrict__ ref,
                                   float* __restrict__ x0, int w, int H4, int W4) {
	const int P = H4 * W4;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * P; i += gridDim.x * blockDim.x) {
		const int c = i / P, p = i - c * P, y = p / W4, x = p - y * W4;
		const uint8_t* src = (c == 0 ? cur : ref) + (size_t)(4 * y) * w + 4 * x;
		int s = 0;
#pragma unroll
		for (int dy = 0; dy < 4; ++dy)
#pragma unroll
			for (int dx = 0; dx < 4; ++dx) s += src[(size_t)dy * w + dx];
		x0[i] = (float)s * (1.0f / 512.0f) - 4.0f;  // (box mean - 128) / 32, exact in fp32
	}
}

// bf16 copies of the conv weights: forward [cout][cin][tap] and, for the
// data gradient, transposed and flipped [cin][cout][8 - tap].
__global__ void pack_weights_kernel(const float* __restrict__ params, __nv_bfloat16* __restrict__ wb,
                                    __nv_bfloat16* __restrict__ wt, int cin) {
	const int n = CH * cin * 9;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const int co = i / (cin * 9), r = i - co * cin * 9, ci = r / 9, tap = r - ci * 9;
		const __nv_bfloat16 v = __float2bfloat16_rn(params[i]);
		wb[i] = v;
		if (wt) wt[((size_t)ci * CH + co) * 9 + (8 - tap)] = v;
	}
}

// out[co][p] = act( bias[co] + sum_{ci,tap} w[co][ci][tap] * in[ci][p + dil*(tap - center)] ),
// zero outside the image; act = ReLU when relu, then zeroed where mask <= 0
// when mask is given.  CTA: 16 x 32 output pixels, thread: 2 pixels (rows r0,
// r0+1 of column lane) x 32 output channels.  Used for the forward pass
// (cin = 2 or 32) and for the data gradient (transposed, flipped weights).
template <int CI>
__global__ void __launch_bounds__(NT) conv3x3_kernel(const float* __restrict__ in, const __nv_bfloat16* __restrict__ w,
                                                     const float* __restrict__ bias, float* __restrict__ out,
                                                     const float* __restrict__ mask, int H, int W, int dil, int relu) {
	__shared__ __align__(16) float ws[CI * 9 * CH];  // [ci][tap][co]
	__shared__ float tin[32 * 48];                    // (16 + 2 dil) x (32 + 2 dil), dil <= 8
	const int tid = threadIdx.x, col = tid & 31, r0 = (tid >> 5) * 2;
	const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 16;
	const int P = H * W;
	for (int i = tid; i < CH * CI * 9; i += NT) {
		const int co = i / (CI * 9), r = i - co * CI * 9;
		ws[r * CH + co] = __bfloat162float(w[i]);
	}
	float acc0[CH], acc1[CH];
#pragma unroll
	for (int c = 0; c < CH; ++c) acc0[c] = acc1[c] = bias ? bias[c] : 0.0f;
	const int TW = 32 + 2 * dil, TH = 16 + 2 * dil;
	for (int ci = 0; ci < CI; ++ci) {
		__syncthreads();
		const float* src = in + (size_t)ci * P;
		for (int i = tid; i < TH * TW; i += NT) {
			const int sy = i / TW, sx = i - sy * TW;
			const int gy = y0 - dil + sy, gx = x0 - dil + sx;
			tin[i] = (gy >= 0 && gy < H && gx >= 0 && gx < W) ? src[(size_t)gy * W + gx] : 0.0f;
		}
		__syncthreads();
#pragma unroll
		for (int tap = 0; tap < 9; ++tap) {
			const int ty = tap / 3, tx = tap - ty * 3;
			const float v0 = tin[(r0 + ty * dil) * TW + col + tx * dil];
			const float v1 = tin[(r0 + 1 + ty * dil) * TW + col + tx * dil];
			const float4* wv = reinterpret_cast<const float4*>(ws + (ci * 9 + tap) * CH);
#pragma unroll
			for (int q = 0; q < CH / 4; ++q) {
				const float4 k = wv[q];
				acc0[4 * q] = fmaf(k.x, v0, acc0[4 * q]);
				acc0[4 * q + 1] = fmaf(k.y, v0, acc0[4 * q + 1]);
				acc0[4 * q + 2] = fmaf(k.z, v0, acc0[4 * q + 2]);
				acc0[4 * q + 3] = fmaf(k.w, v0, acc0[4 * q + 3]);
				acc1[4 * q] = fmaf(k.x, v1, acc1[4 * q]);
				acc1[4 * q + 1] = fmaf(k.y, v1, acc1[4 * q + 1]);
				acc1[4 * q + 2] = fmaf(k.z, v1, acc1[4 * q + 2]);
				acc1[4 * q + 3] = fmaf(k.w, v1, acc1[4 * q + 3]);
			}
		}
	}
	const int x = x0 + col;
#pragma unroll
	for (int rr = 0; rr < 2; ++rr) {
		const int y = y0 + r0 + rr;
		if (y >= H || x >= W) continue;
		const size_t p = (size_t)y * W + x;
#pragma unroll
		for (int c = 0; c < CH; ++c) {
			float v = rr ? acc1[c] : acc0[c];
			if (relu) v = fmaxf(v, 0.0f);
			if (mask && !(mask[(size_t)c * P + p] > 0.0f)) v = 0.0f;
			out[(size_t)c * P + p] = v;
		}
	}
}

// Weight gradient partials: for a 4 x 32 pixel tile and 4 input channels
// (blockIdx.z), part[tile][co][ci][tap] = sum_p dpre[co][p] * in[ci][p + off(tap)];
// the z = 0 slice also writes the bias partial sum_p dpre[co][p].  Thread:
// co = tid / 8, pixels pg, pg + 8, ... (pg = tid % 8); the 8 threads of one
// co reduce with shuffles.
template <int CI>
__global__ void __launch_bounds__(NT) wgrad_kernel(const float* __restrict__ in, const float* __restrict__ dpre,
                                                   float* __restrict__ part, int H, int W, int dil, int tiles_x) {
	__shared__ float sd[CH * 128];
	__shared__ float tin[4 * 20 * 48];  // 4 channels x (4 + 2 dil) x (32 + 2 dil), dil <= 8
	constexpr int CPB = CI < 4 ? CI : 4;  // input channels per CTA
	const int tid = threadIdx.x, co = tid >> 3, pg = tid & 7;
	const int tile = blockIdx.y * tiles_x + blockIdx.x;
	const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 4, c0 = blockIdx.z * CPB;
	const int P = H * W;
	const int TW = 32 + 2 * dil, TH = 4 + 2 * dil;
	for (int i = tid; i < CH * 128; i += NT) {
		const int c = i >> 7, p = i & 127, y = y0 + (p >> 5), x = x0 + (p & 31);
		sd[i] = (y < H && x < W) ? dpre[(size_t)c * P + (size_t)y * W + x] : 0.0f;
	}
	for (int i = tid; i < CPB * TH * TW; i += NT) {
		const int c = i / (TH * TW), r = i - c * TH * TW, sy = r / TW, sx = r - sy * TW;
		const int gy = y0 - dil + sy, gx = x0 - dil + sx;
		tin[c * TH * TW + r] =
			(gy >= 0 && gy < H && gx >= 0 && gx < W) ? in[(size_t)(c0 + c) * P + (size_t)gy * W + gx] : 0.0f;
	}
	__syncthreads();
	float acc[CPB][9];
	float bacc = 0.0f;
#pragma unroll
	for (int c = 0; c < CPB; ++c)
#pragma unroll
		for (int t = 0; t < 9; ++t) acc[c][t] = 0.0f;
	for (int p = pg; p < 128; p += 8) {
		const float d = sd[co * 128 + p];
		const int py = p >> 5, px = p & 31;
		bacc += d;
#pragma unroll
		for (int c = 0; c < CPB; ++c)
#pragma unroll
			for (int t = 0; t < 9; ++t) {
				const int ty = t / 3, tx = t - ty * 3;
				acc[c][t] = fmaf(d, tin[c * TH * TW + (py + ty * dil) * TW + px + tx * dil], acc[c][t]);
			}
	}
#pragma unroll
	for (int o = 1; o < 8; o <<= 1) {
		bacc += __shfl_xor_sync(0xffffffffu, bacc, o);
#pragma unroll
		for (int c = 0; c < CPB; ++c)
#pragma unroll
			for (int t = 0; t < 9; ++t) acc[c][t] += __shfl_xor_sync(0xffffffffu, acc[c][t], o);
	}
	if (pg == 0) {
		float* dst = part + (size_t)tile * (CH * CI * 9 + CH);
#pragma unroll
		for (int c = 0; c < CPB; ++c)
#pragma unroll
			for (int t = 0; t < 9; ++t) dst[(co * CI + c0 + c) * 9 + t] = acc[c][t];
		if (blockIdx.z == 0) dst[CH * CI * 9 + co] = bacc;
	}
}

// sum over the first n rows of a row-major (n, m) array -> out[m] (fixed order).
__global__ void reduce_rows_kernel(const float* __restrict__ part, float* __restrict__ out, int n, int m) {
	for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
		float s = 0.0f;
		for (int i = 0; i < n; ++i) s += part[(size_t)i * m + j];
		out[j] = s;
	}
}

__device__ __forceinline__ float head_feature(const float* a4, int P, int W4, int by, int bx, int f) {
	const int c = f >> 4, i = (f >> 2) & 3, k = f & 3;
	return a4[(size_t)c * P + (size_t)(4 * by + i) * W4 + 4 * bx + k];
}

// One warp per block: pred[blk][j] = bh[j] + sum_f wh[j][f] * feature_f.
__global__ void head_fwd_kernel(const float* __restrict__ a4, const float* __restrict__ params, int wh_off, int bh_off,
                                float* __restrict__ pred, int H4, int W4, int nbx, int nblk) {
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if (warp >= nblk) return;
	const int by = warp / nbx, bx = warp - by * nbx, P = H4 * W4;
	float s0 = 0.0f, s1 = 0.0f;
	for (int f = lane; f < HEADF; f += 32) {
		const float v = head_feature(a4, P, W4, by, bx, f);
		s0 = fmaf(__bfloat162float(__float2bfloat16_rn(params[wh_off + f])), v, s0);
		s1 = fmaf(__bfloat162float(__float2bfloat16_rn(params[wh_off + HEADF + f])), v, s1);
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		s0 += __shfl_xor_sync(0xffffffffu, s0, o);
		s1 += __shfl_xor_sync(0xffffffffu, s1, o);
	}
	if (lane == 0) {
		pred[2 * warp] = s0 + params[bh_off];
		pred[2 * warp + 1] = s1 + params[bh_off + 1];
	}
}

// Smooth-L1 loss against target/16 and the head backward pass.  One warp per
// block, 8 blocks per CTA: dA4 (masked by a4 > 0, i.e. through the ReLU) and
// per-CTA partials of dWh, dbh and the loss.
__global__ void __launch_bounds__(NT) head_bwd_kernel(const float* __restrict__ a4, const float* __restrict__ params,
                                                      int wh_off, const float* __restrict__ pred,
                                                      const int32_t* __restrict__ target, int tstride,
                                                      float* __restrict__ dpre4, float* __restrict__ hpart,
                                                      float* __restrict__ lpart, int H4, int W4, int nbx, int nblk) {
	__shared__ float sg[8][2];
	__shared__ float sl[8];
	const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int blk = blockIdx.x * 8 + wl;
	const int P = H4 * W4;
	float g0 = 0.0f, g1 = 0.0f, l = 0.0f;
	if (blk < nblk) {
		const float inv = 1.0f / (float)nblk;
		const float e0 = pred[2 * blk] - (float)target[tstride * blk] * (1.0f / 16.0f);
		const float e1 = pred[2 * blk + 1] - (float)target[tstride * blk + 1] * (1.0f / 16.0f);
		l = (fabsf(e0) < 1.0f ? 0.5f * e0 * e0 : fabsf(e0) - 0.5f) + (fabsf(e1) < 1.0f ? 0.5f * e1 * e1 : fabsf(e1) - 0.5f);
		g0 = fminf(fmaxf(e0, -1.0f), 1.0f) * inv;
		g1 = fminf(fmaxf(e1, -1.0f), 1.0f) * inv;
		const int by = blk / nbx, bx = blk - by * nbx;
		for (int f = lane; f < HEADF; f += 32) {
			const int c = f >> 4, i = (f >> 2) & 3, k = f & 3;
			const size_t p = (size_t)c * P + (size_t)(4 * by + i) * W4 + 4 * bx + k;
			const float w0 = __bfloat162float(__float2bfloat16_rn(params[wh_off + f]));
			const float w1 = __bfloat162float(__float2bfloat16_rn(params[wh_off + HEADF + f]));
			dpre4[p] = a4[p] > 0.0f ? w0 * g0 + w1 * g1 : 0.0f;
		}
	}
	if (lane == 0) {
		sg[wl][0] = g0;
		sg[wl][1] = g1;
		sl[wl] = l * (1.0f / (float)nblk);
	}
	__syncthreads();
	float* dst = hpart + (size_t)blockIdx.x * (2 * HEADF + 2);
	for (int f = threadIdx.x; f < HEADF; f += NT) {
		float s0 = 0.0f, s1 = 0.0f;
		for (int b = 0; b < 8; ++b) {
			const int bb = blockIdx.x * 8 + b;
			if (bb >= nblk) break;
			const int by = bb / nbx, bx = bb - by * nbx;
			const float v = head_feature(a4, P, W4, by, bx, f);
			s0 = fmaf(sg[b][0], v, s0);
			s1 = fmaf(sg[b][1], v, s1);
		}
		dst[f] = s0;
		dst[HEADF + f] = s1;
	}
	if (threadIdx.x == 0) {
		float b0 = 0.0f, b1 = 0.0f, ls = 0.0f;
		for (int b = 0; b < 8; ++b) { b0 += sg[b][0]; b1 += sg[b][1]; ls += sl[b]; }
		dst[2 * HEADF] = b0;
		dst[2 * HEADF + 1] = b1;
		lpart[blockIdx.x] = ls;
	}
}

// Adam (Kingma & Ba, 2015) on the fp32 master parameters.
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float gi = g[i];
		const float mi = b1 * m[i] + (1.0f - b1) * gi;
		const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
	}
}

// Search centres from the predictions: round(pred * 16), clamped to +-range.
__global__ void centers_kernel(const float* __restrict__ pred, int32_t* __restrict__ centers, int n, int range) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * n; i += gridDim.x * blockDim.x) {
		const float v = rintf(pred[i] * 16.0f);
		centers[i] = (int32_t)fminf(fmaxf(v, (float)-range), (float)range);
	}
}

// List for the exhaustive search: every block other than the audited ones
// (0, stride, 2 stride, ...) whose refined SAD exceeds the threshold
// (counted in count[1]), and, when `with_audit`, the audited blocks too
// (their refined SAD goes to audit_sums[0]).  count[0] is the list length.
// List order is the order of discovery; the search is per block, so the
// order changes no result.
__global__ void flag_kernel(const int32_t* __restrict__ mv, int n, int stride, int32_t thr, bool with_audit,
                            int32_t* __restrict__ list, int32_t* __restrict__ count,
                            unsigned long long* __restrict__ audit_sums) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		if (stride > 0 && i % stride == 0) {
			if (with_audit) {
				if (audit_sums) atomicAdd(audit_sums, (unsigned long long)mv[3 * i + 2]);
				list[atomicAdd(count, 1)] = i;
			}
		} else if (mv[3 * i + 2] > thr) {
			list[atomicAdd(count, 1)] = i;
			atomicAdd(count + 1, 1);
		}
	}
}

// audit_sums[1] += exhaustive SAD of the audited blocks, searched in the
// same list as the fallback blocks.
__global__ void audit_sum_kernel(const int32_t* __restrict__ mv, int n, int stride,
                                 unsigned long long* __restrict__ audit_sums) {
	const int na = (n + stride - 1) / stride;
	unsigned long long s = 0;
	for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < na; a += gridDim.x * blockDim.x)
		s += (unsigned long long)mv[3 * (size_t)a * stride + 2];
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	if ((threadIdx.x & 31) == 0 && s) atomicAdd(audit_sums + 1, s);
}

// alist = 0, stride, 2 stride, ... (*acount = their number).
__global__ void audit_list_kernel(int32_t* __restrict__ alist, int32_t* __restrict__ acount, int n, int stride) {
	const int na = (n + stride - 1) / stride;
	for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < na; a += gridDim.x * blockDim.x) alist[a] = a * stride;
	if (blockIdx.x == 0 && threadIdx.x == 0) *acount = na;
}

// The audited blocks take their exhaustive result (amv) in place of the
// refined one (mv); audit_sums (if non-null) += (refined SAD, exhaustive SAD).
__global__ void audit_merge_kernel(int32_t* __restrict__ mv, const int32_t* __restrict__ amv, int n, int stride,
                                   unsigned long long* __restrict__ audit_sums) {
	const int na = (n + stride - 1) / stride;
	unsigned long long s0 = 0, s1 = 0;
	for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < na; a += gridDim.x * blockDim.x) {
		const size_t j = 3 * (size_t)a * stride;
		s0 += (unsigned long long)mv[j + 2];
		s1 += (unsigned long long)amv[j + 2];
		mv[j] = amv[j];
		mv[j + 1] = amv[j + 1];
		mv[j + 2] = amv[j + 2];
	}
	if (!audit_sums) return;
	for (int o = 16; o > 0; o >>= 1) {
		s0 += __shfl_xor_sync(0xffffffffu, s0, o);
		s1 += __shfl_xor_sync(0xffffffffu, s1, o);
	}
	if ((threadIdx.x & 31) == 0) {
		if (s0) atomicAdd(audit_sums, s0);
		if (s1) atomicAdd(audit_sums + 1, s1);
	}
}

// ---- tensor-core inference path: bf16 NHWC activations, 32 channels (64
// bytes) per pixel, layers 2-4 on tcgen05 (umi::menet_conv_tc).

// Weights of layers 1..3 as (32, 9*32) bf16 K-major matrices (column
// tap*32 + ci), all three in one launch: blockIdx.y = layer - 1.
static_assert(NL == 4, "pack_tc_weights_kernel selects among three layers");
struct TcWeights {
	const float* w[NL - 1];
	__nv_bfloat16* out[NL - 1];
};
__global__ void pack_tc_weights_kernel(TcWeights p) {
	const int l = blockIdx.y;
	const float* w = l == 0 ? p.w[0] : l == 1 ? p.w[1] : p.w[2];
	__nv_bfloat16* out = l == 0 ? p.out[0] : l == 1 ? p.out[1] : p.out[2];
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < CH * 9 * CH; i += gridDim.x * blockDim.x) {
		const int co = i / (9 * CH), r = i - co * 9 * CH, tap = r / CH, ci = r - tap * CH;
		out[i] = __float2bfloat16_rn(w[(co * CH + ci) * 9 + tap]);
	}
}

// Layer 1 (2 -> 32 channels, dilation 1) on the FP32 pipe: + bias, ReLU,
// bf16, 64-byte NHWC pixels.  Weights come straight from the parameters
// ([co][ci][tap], rounded to bf16 here).  A thread computes one 16-byte
// quarter of the output pixel (8 channels, q = thread & 3) for four adjacent
// pixels x .. x+3 (x a multiple of 4, W a multiple of 4), from a 3 x 6 window
// per input channel: one 16-byte load and two edge loads per window row.
// Each accumulator sums bias, then the 18 products in (ci, tap) order.
__global__ void __launch_bounds__(NT) conv1_nhwc_kernel(const float* __restrict__ x0, const float* __restrict__ w,
                                                        const float* __restrict__ bias, __nv_bfloat16* __restrict__ out,
                                                        int H, int W) {
	__shared__ float4 ws[18][CH / 4];  // [ci * 9 + tap][co / 4]
	__shared__ float4 bs[CH / 4];
	for (int i = threadIdx.x; i < CH * 18; i += NT) {
		const int co = i / 18, k = i - co * 18;
		reinterpret_cast<float*>(ws)[k * CH + co] = __bfloat162float(__float2bfloat16_rn(w[i]));
	}
	if (threadIdx.x < CH) reinterpret_cast<float*>(bs)[threadIdx.x] = bias[threadIdx.x];
	__syncthreads();
	const int P = H * W, groups_x = W >> 2;
	const int t = blockIdx.x * NT + threadIdx.x, q = t & 3, pg = t >> 2;
	if (pg >= H * groups_x) return;
	const int y = pg / groups_x, x = (pg - y * groups_x) * 4;
	float in[2][3][6];
#pragma unroll
	for (int ci = 0; ci < 2; ++ci)
#pragma unroll
		for (int r = 0; r < 3; ++r) {
			const int yy = y + r - 1;
			if (yy >= 0 && yy < H) {
				const float* row = x0 + (size_t)ci * P + (size_t)yy * W + x;
				const float4 m = *reinterpret_cast<const float4*>(row);
				in[ci][r][0] = x > 0 ? row[-1] : 0.0f;
				in[ci][r][1] = m.x; in[ci][r][2] = m.y; in[ci][r][3] = m.z; in[ci][r][4] = m.w;
				in[ci][r][5] = x + 4 < W ? row[4] : 0.0f;
			} else {
#pragma unroll
				for (int c = 0; c < 6; ++c) in[ci][r][c] = 0.0f;
			}
		}
	float acc[4][8];
	{
		const float4 b0 = bs[2 * q], b1 = bs[2 * q + 1];
#pragma unroll
		for (int px = 0; px < 4; ++px) {
			acc[px][0] = b0.x; acc[px][1] = b0.y; acc[px][2] = b0.z; acc[px][3] = b0.w;
			acc[px][4] = b1.x; acc[px][5] = b1.y; acc[px][6] = b1.z; acc[px][7] = b1.w;
		}
	}
#pragma unroll
	for (int ci = 0; ci < 2; ++ci)
#pragma unroll
		for (int tap = 0; tap < 9; ++tap) {
			const float4 wa = ws[ci * 9 + tap][2 * q], wb = ws[ci * 9 + tap][2 * q + 1];
			const float wv[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
			for (int px = 0; px < 4; ++px) {
				const float v = in[ci][tap / 3][px + tap % 3];
#pragma unroll
				for (int c = 0; c < 8; ++c) acc[px][c] = fmaf(wv[c], v, acc[px][c]);
			}
		}
#pragma unroll
	for (int px = 0; px < 4; ++px) {
		uint32_t pk[4];
#pragma unroll
		for (int c2 = 0; c2 < 4; ++c2) {
			const __nv_bfloat162 b2 =
				__floats2bfloat162_rn(fmaxf(acc[px][2 * c2], 0.0f), fmaxf(acc[px][2 * c2 + 1], 0.0f));
			pk[c2] = *reinterpret_cast<const uint32_t*>(&b2);
		}
		*reinterpret_cast<uint4*>(out + ((size_t)y * W + x + px) * CH + q * 8) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
	}
}

// Head on the bf16 NHWC layer-4 activations.  A block's 16 cells are four
// rows of 256 contiguous bytes; a warp reads them as two 16-byte pieces per
// lane (piece j = lane + 32 s: row j >> 4, cell (j >> 2) & 3, channels
// 8 (j & 3) .. +7), so each lane keeps the 32 head weights of its pieces in
// registers for every block it serves.  HEAD_BPW blocks per warp, all their
// loads issued before the first product.
constexpr int HEAD_WARPS = 8, HEAD_BPW = 4;
__global__ void __launch_bounds__(HEAD_WARPS * 32)
	head_nhwc_kernel(const __nv_bfloat16* __restrict__ a4, const float* __restrict__ params, int wh_off, int bh_off,
                     float* __restrict__ pred, int W4, int nbx, int nblk) {
	__shared__ float4 wsm[2][64][2];  // [output][piece][channels 0-3, 4-7 of the piece], bf16-rounded
	for (int t = threadIdx.x; t < 2 * HEADF; t += blockDim.x) {
		const int o = t / HEADF, f = t - o * HEADF, c = f >> 4, cell = f & 15;
		const int j = (cell >> 2) * 16 + (cell & 3) * 4 + (c >> 3);
		reinterpret_cast<float*>(&wsm[o][j][0])[c & 7] = __bfloat162float(__float2bfloat16_rn(params[wh_off + t]));
	}
	__syncthreads();
	const int lane = threadIdx.x & 31;
	const int first = (blockIdx.x * HEAD_WARPS + (threadIdx.x >> 5)) * HEAD_BPW;
	if (first >= nblk) return;
	float wt[2][2][8];  // [output][piece s][channel in the piece]
#pragma unroll
	for (int o = 0; o < 2; ++o)
#pragma unroll
		for (int s = 0; s < 2; ++s) {
			const float4 a = wsm[o][lane + 32 * s][0], b = wsm[o][lane + 32 * s][1];
			wt[o][s][0] = a.x; wt[o][s][1] = a.y; wt[o][s][2] = a.z; wt[o][s][3] = a.w;
			wt[o][s][4] = b.x; wt[o][s][5] = b.y; wt[o][s][6] = b.z; wt[o][s][7] = b.w;
		}
	const size_t row_pieces = (size_t)W4 * CH * sizeof(__nv_bfloat16) / 16;
	uint4 v[HEAD_BPW][2];
#pragma unroll
	for (int u = 0; u < HEAD_BPW; ++u) {
		const int blk = min(first + u, nblk - 1);  // past the end: reload the last block, store nothing
		const int by = blk / nbx, bx = blk - by * nbx;
		const uint4* base = reinterpret_cast<const uint4*>(a4 + ((size_t)(4 * by) * W4 + 4 * bx) * CH) + (lane & 15);
#pragma unroll
		for (int s = 0; s < 2; ++s) v[u][s] = __ldg(base + ((lane >> 4) + 2 * s) * row_pieces);
	}
	const float b0 = params[bh_off], b1 = params[bh_off + 1];
#pragma unroll
	for (int u = 0; u < HEAD_BPW; ++u) {
		float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
		for (int s = 0; s < 2; ++s) {
			const uint32_t word[4] = {v[u][s].x, v[u][s].y, v[u][s].z, v[u][s].w};
#pragma unroll
			for (int e = 0; e < 8; ++e) {
				const float a = __uint_as_float(e & 1 ? word[e >> 1] & 0xffff0000u : word[e >> 1] << 16);
				s0 = fmaf(wt[0][s][e], a, s0);
				s1 = fmaf(wt[1][s][e], a, s1);
			}
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			s0 += __shfl_xor_sync(0xffffffffu, s0, o);
			s1 += __shfl_xor_sync(0xffffffffu, s1, o);
		}
		if (lane == 0 && first + u < nblk)
			*reinterpret_cast<float2*>(pred + 2 * (size_t)(first + u)) = make_float2(s0 + b0, s1 + b1);
	}
}

// ------------------------------------------------------------------ host side
const Layout& layout() {
	static const Layout L;
	return L;
}

umi_status check_frame(int h, int w) {
	if (h < 16 || w < 16) return umi::fail(UMI_ERR_INVALID_ARG, "learned ME: frame %dx%d smaller than one block", h, w);
	if (h % 16 || w % 16) return umi::fail(UMI_ERR_UNSUPPORTED, "learned ME: frame %dx%d not a multiple of 16", h, w);
	return UMI_OK;
}

int grid_for(size_t n) { return (int)std::min<size_t>((n + NT - 1) / NT, 4096); }

umi_status forward(const uint8_t* cur, const uint8_t* ref, int h, int w, const float* params, void* ws,
                   cudaStream_t st) {
	const Layout& L = layout();
	const Work K(h, w);
	downsample4_kernel<<<grid_for(2 * (size_t)K.P), NT, 0, st>>>(cur, ref, K.at<float>(ws, K.x0), w, K.H4, K.W4);
	UMI_TRY(umi::launch_status("downsample4_kernel"));
	for (int l = 0; l < NL; ++l) {
		pack_weights_kernel<<<grid_for(CH * CIN[l] * 9), NT, 0, st>>>(
			params + L.w[l], K.at<__nv_bfloat16>(ws, K.wb[l]), l > 0 ? K.at<__nv_bfloat16>(ws, K.wt[l]) : nullptr, CIN[l]);
		UMI_TRY(umi::launch_status("pack_weights_kernel"));
	}
	const dim3 grid(umi::ceil_div(K.W4, 32), umi::ceil_div(K.H4, 16));
	const float* in = K.at<float>(ws, K.x0);
	for (int l = 0; l < NL; ++l) {
		float* out = K.at<float>(ws, K.act[l]);
		if (l == 0)
			conv3x3_kernel<2><<<grid, NT, 0, st>>>(in, K.at<__nv_bfloat16>(ws, K.wb[0]), params + L.b[0], out, nullptr,
			                                        K.H4, K.W4, DIL[0], 1);
		else
			conv3x3_kernel<CH><<<grid, NT, 0, st>>>(in, K.at<__nv_bfloat16>(ws, K.wb[l]), params + L.b[l], out, nullptr,
			                                         K.H4, K.W4, DIL[l], 1);
		UMI_TRY(umi::launch_status("conv3x3_kernel"));
		in = out;
	}
	head_fwd_kernel<<<umi::ceil_div(K.nblk * 32, NT), NT, 0, st>>>(in, params, L.wh, L.bh, K.at<float>(ws, K.pred),
	                                                                K.H4, K.W4, K.nbx, K.nblk);
	return umi::launch_status("head_fwd_kernel");
}

// Inference forward pass with layers 2-4 on the tensor cores; prediction to K.pred.
umi_status infer(const uint8_t* cur, const uint8_t* ref, int h, int w, const float* params, void* ws, int32_t* err,
                 cudaStream_t st) {
	const Layout& L = layout();
	const Work K(h, w);
	downsample4_kernel<<<grid_for(2 * (size_t)K.P), NT, 0, st>>>(cur, ref, K.at<float>(ws, K.x0), w, K.H4, K.W4);
	UMI_TRY(umi::launch_status("downsample4_kernel"));
	TcWeights tw;
	for (int l = 1; l < NL; ++l) {
		tw.w[l - 1] = params + L.w[l];
		tw.out[l - 1] = K.at<__nv_bfloat16>(ws, K.wtc[l]);
	}
	pack_tc_weights_kernel<<<dim3(grid_for(CH * 9 * CH), NL - 1), NT, 0, st>>>(tw);
	UMI_TRY(umi::launch_status("pack_tc_weights_kernel"));
	__nv_bfloat16* a = K.at<__nv_bfloat16>(ws, K.nhwc[0]);
	__nv_bfloat16* b = K.at<__nv_bfloat16>(ws, K.nhwc[1]);
	conv1_nhwc_kernel<<<umi::ceil_div(K.P, NT), NT, 0, st>>>(K.at<float>(ws, K.x0), params + L.w[0], params + L.b[0], a,
	                                                         K.H4, K.W4);
	UMI_TRY(umi::launch_status("conv1_nhwc_kernel"));
	for (int l = 1; l < NL; ++l) {
		UMI_TRY(umi::menet_conv_tc(a, b, K.at<__nv_bfloat16>(ws, K.wtc[l]), params + L.b[l], K.H4, K.W4, DIL[l], err, st));
		std::swap(a, b);
	}
	head_nhwc_kernel<<<umi::ceil_div(K.nblk, HEAD_WARPS * HEAD_BPW), HEAD_WARPS * 32, 0, st>>>(
		a, params, L.wh, L.bh, K.at<float>(ws, K.pred), K.W4, K.nbx, K.nblk);
	return umi::launch_status("head_nhwc_kernel");
}

}  // namespace

extern "C" umi_status umi_menet_infer(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, const float* params,
                                      float* pred, int32_t* err, void* workspace, size_t workspace_bytes, void* stream) {
	UMI_TRY(check_frame(h, w));
	if (!cur || !ref || !params || !workspace) return umi::fail(UMI_ERR_INVALID_ARG, "menet_infer: null pointer");
	const Work K(h, w);
	if (workspace_bytes < K.bytes) return umi::fail(UMI_ERR_NO_MEMORY, "menet_infer: workspace too small");
	if (!umi::aligned(workspace, 256)) return umi::fail(UMI_ERR_INVALID_ARG, "menet_infer: workspace alignment");
	const cudaStream_t st = umi::as_stream(stream);
	UMI_TRY(infer(cur, ref, h, w, params, workspace, err, st));
	if (pred)
		UMI_TRY(umi::cuda_status(cudaMemcpyAsync(pred, K.at<float>(workspace, K.pred), sizeof(float) * 2 * K.nblk,
		                                         cudaMemcpyDeviceToDevice, st),
		                         "cudaMemcpyAsync"));
	return umi::ok();
}

extern "C" int32_t umi_menet_param_count(void) { return layout().total; }

extern "C" size_t umi_menet_workspace_bytes(int32_t h, int32_t w) {
	if (check_frame(h, w) != UMI_OK) return 0;
	return Work(h, w).bytes;
}

extern "C" umi_status umi_menet_forward(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, const float* params,
                                        float* pred, void* workspace, size_t workspace_bytes, void* stream) {
	UMI_TRY(check_frame(h, w));
	if (!cur || !ref || !params || !workspace) return umi::fail(UMI_ERR_INVALID_ARG, "menet_forward: null pointer");
	const Work K(h, w);
	if (workspace_bytes < K.bytes) return umi::fail(UMI_ERR_NO_MEMORY, "menet_forward: workspace too small");
	if (!umi::aligned(workspace, 256)) return umi::fail(UMI_ERR_INVALID_ARG, "menet_forward: workspace alignment");
	const cudaStream_t st = umi::as_stream(stream);
	UMI_TRY(forward(cur, ref, h, w, params, workspace, st));
	if (pred)
		UMI_TRY(umi::cuda_status(cudaMemcpyAsync(pred, K.at<float>(workspace, K.pred), sizeof(float) * 2 * K.nblk,
		                                         cudaMemcpyDeviceToDevice, st),
		                         "cudaMemcpyAsync"));
	return umi::ok();
}

extern "C" umi_status umi_menet_backward(const int32_t* target, int32_t target_stride, int32_t h, int32_t w,
                                         const float* params, float* grads, float* loss, void* workspace,
                                         size_t workspace_bytes, void* stream) {
	UMI_TRY(check_frame(h, w));
	if (!target || !params || !grads || !workspace) return umi::fail(UMI_ERR_INVALID_ARG, "menet_backward: null pointer");
	const Work K(h, w);
	if (workspace_bytes < K.bytes) return umi::fail(UMI_ERR_NO_MEMORY, "menet_backward: workspace too small");
	const Layout& L = layout();
	const cudaStream_t st = umi::as_stream(stream);
	void* ws = workspace;
	const int nhc = umi::ceil_div(K.nblk, 8);
	float* dcur = K.at<float>(ws, K.dA[0]);
	float* dnext = K.at<float>(ws, K.dA[1]);
	head_bwd_kernel<<<nhc, NT, 0, st>>>(K.at<float>(ws, K.act[NL - 1]), params, L.wh, K.at<float>(ws, K.pred), target,
	                                    target_stride, dcur, K.at<float>(ws, K.hpart), K.at<float>(ws, K.lpart), K.H4,
	                                    K.W4, K.nbx, K.nblk);
	UMI_TRY(umi::launch_status("head_bwd_kernel"));
	reduce_rows_kernel<<<grid_for(2 * HEADF + 2), NT, 0, st>>>(K.at<float>(ws, K.hpart), grads + L.wh, nhc, 2 * HEADF + 2);
	UMI_TRY(umi::launch_status("reduce_rows_kernel"));
	if (loss) {
		reduce_rows_kernel<<<1, 32, 0, st>>>(K.at<float>(ws, K.lpart), loss, nhc, 1);
		UMI_TRY(umi::launch_status("reduce_rows_kernel"));
	}
	const int tx = umi::ceil_div(K.W4, 32), ty = umi::ceil_div(K.H4, 4);
	const dim3 fgrid(umi::ceil_div(K.W4, 32), umi::ceil_div(K.H4, 16));
	for (int l = NL - 1; l >= 0; --l) {
		const float* in = l == 0 ? K.at<float>(ws, K.x0) : K.at<float>(ws, K.act[l - 1]);
		float* part = K.at<float>(ws, K.wpart);
		const int m = CH * CIN[l] * 9 + CH;
		if (l == 0) wgrad_kernel<2><<<dim3(tx, ty, 1), NT, 0, st>>>(in, dcur, part, K.H4, K.W4, DIL[l], tx);
		else wgrad_kernel<CH><<<dim3(tx, ty, CH / 4), NT, 0, st>>>(in, dcur, part, K.H4, K.W4, DIL[l], tx);
		UMI_TRY(umi::launch_status("wgrad_kernel"));
		// grads[w_l], then grads[b_l] right after it (same layout as the partial rows)
		reduce_rows_kernel<<<grid_for(m), NT, 0, st>>>(part, grads + L.w[l], tx * ty, m);
		UMI_TRY(umi::launch_status("reduce_rows_kernel"));
		if (l > 0) {
			// data gradient through the transposed, flipped weights, masked by ReLU(a_{l-1})
			conv3x3_kernel<CH><<<fgrid, NT, 0, st>>>(dcur, K.at<__nv_bfloat16>(ws, K.wt[l]), nullptr, dnext,
			                                          K.at<float>(ws, K.act[l - 1]), K.H4, K.W4, DIL[l], 0);
			UMI_TRY(umi::launch_status("conv3x3_kernel"));
			std::swap(dcur, dnext);
		}
	}
	return umi::ok();
}

extern "C" umi_status umi_menet_adam(float* params, const float* grads, float* m, float* v, int32_t step, float lr,
                                     void* stream) {
	if (!params || !grads || !m || !v || step < 1) return umi::fail(UMI_ERR_INVALID_ARG, "menet_adam: bad arguments");
	const int n = layout().total;
	const float b1 = 0.9f, b2 = 0.999f;
	const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
	adam_kernel<<<grid_for(n), NT, 0, umi::as_stream(stream)>>>(params, grads, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
	UMI_TRY(umi::launch_status("adam_kernel"));
	return umi::ok();
}

extern "C" umi_status umi_me_learned_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, const float* params,
                                        int32_t refine_r, int32_t full_r, int32_t sad_threshold, int32_t audit_stride,
                                        int32_t* mv, unsigned long long* audit_sums, int32_t* n_fallback,
                                        void* workspace, size_t workspace_bytes, void* stream) {
	UMI_TRY(check_frame(h, w));
	if (!cur || !ref || !params || !mv || !workspace) return umi::fail(UMI_ERR_INVALID_ARG, "me_learned: null pointer");
	const Work K(h, w);
	if (workspace_bytes < K.bytes) return umi::fail(UMI_ERR_NO_MEMORY, "me_learned: workspace too small");
	if (!umi::aligned(workspace, 256)) return umi::fail(UMI_ERR_INVALID_ARG, "me_learned: workspace alignment");
	if (refine_r < 1 || full_r < refine_r || full_r > 64)
		return umi::fail(UMI_ERR_UNSUPPORTED, "me_learned: refine %d / full %d ranges", refine_r, full_r);
	if (audit_stride < 0) return umi::fail(UMI_ERR_INVALID_ARG, "me_learned: negative audit stride");
	const cudaStream_t st = umi::as_stream(stream);
	void* ws = workspace;
	const umi::MeFinishBuffers fb{K.at<int32_t>(ws, K.list), K.at<int32_t>(ws, K.count), K.at<int32_t>(ws, K.alist),
	                              K.at<int32_t>(ws, K.amv)};
	umi::MeAudit audit;
	UMI_TRY(umi::me_audit_begin(cur, ref, h, w, full_r, audit_stride, fb, st, &audit));
	UMI_TRY(infer(cur, ref, h, w, params, ws, K.at<int32_t>(ws, K.err), st));
	int32_t* centers = K.at<int32_t>(ws, K.centers);
	centers_kernel<<<grid_for(2 * (size_t)K.nblk), NT, 0, st>>>(K.at<float>(ws, K.pred), centers, K.nblk,
	                                                             full_r - refine_r);
	UMI_TRY(umi::launch_status("centers_kernel"));
	return umi::me_refine_fallback_finish(cur, ref, h, w, centers, refine_r, full_r, sad_threshold, audit_stride, mv,
	                                      audit_sums, n_fallback, fb, audit, st);
}

namespace umi {

namespace {

// The calling thread's second stream on one device, with its fork and join
// events: made on first use outside a stream capture, destroyed at thread exit.
struct AuxStream {
	cudaStream_t s = nullptr;
	cudaEvent_t fork = nullptr, join = nullptr;
	~AuxStream() {
		if (join) cudaEventDestroy(join);
		if (fork) cudaEventDestroy(fork);
		if (s) cudaStreamDestroy(s);
	}
};

AuxStream* aux_stream(cudaStream_t st) {
	constexpr int kMaxDevices = 64;
	thread_local AuxStream aux[kMaxDevices];
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
	AuxStream& a = aux[dev];
	if (a.s && a.fork && a.join) return &a;
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
		cudaGetLastError();  // not an error of this call: the stage runs in order on st
		return nullptr;
	}
	if (cs != cudaStreamCaptureStatusNone) return nullptr;
	if (!a.s && cudaStreamCreateWithFlags(&a.s, cudaStreamNonBlocking) != cudaSuccess) a.s = nullptr;
	if (!a.fork && cudaEventCreateWithFlags(&a.fork, cudaEventDisableTiming) != cudaSuccess) a.fork = nullptr;
	if (!a.join && cudaEventCreateWithFlags(&a.join, cudaEventDisableTiming) != cudaSuccess) a.join = nullptr;
	cudaGetLastError();  // a failure here only means no second stream
	return a.s && a.fork && a.join ? &a : nullptr;
}

}  // namespace

umi_status me_audit_begin(const uint8_t* cur, const uint8_t* ref, int h, int w, int full_r, int audit_stride,
                          const MeFinishBuffers& b, cudaStream_t st, MeAudit* audit) {
	audit->active = audit->combined = audit->forked = audit->joined = false;
	audit->done = nullptr;
	audit->st = st;
	const int nblk = (h / 16) * (w / 16);
	if (audit_stride <= 0 || nblk == 0) return UMI_OK;
	audit->active = true;
	// A +-64 list search runs one block per SM at a time.  An audit of fewer
	// blocks than SMs leaves room in the fallback search's round, so it joins
	// that list; a larger one runs apart, beside the proposal.
	const int na = ceil_div(nblk, audit_stride);
	int dev = 0, sms = 0;
	UMI_TRY(cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
	UMI_TRY(cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
	if (na < sms) {
		audit->combined = true;
		return UMI_OK;
	}
	AuxStream* aux = aux_stream(st);
	cudaStream_t as = st;
	if (aux) {
		UMI_TRY(cuda_status(cudaEventRecord(aux->fork, st), "cudaEventRecord"));
		UMI_TRY(cuda_status(cudaStreamWaitEvent(aux->s, aux->fork, 0), "cudaStreamWaitEvent"));
		as = aux->s;
	}
	audit_list_kernel<<<grid_for(na), NT, 0, as>>>(b.alist, b.count + 2, nblk, audit_stride);
	umi_status rc = launch_status("audit_list_kernel");
	if (rc == UMI_OK)
		rc = umi_full_me_u8_list(cur, ref, h, w, 16, full_r, nullptr, b.alist, b.count + 2, na, b.amv, as);
	if (aux) {
		// recorded on every path once the fork happened: whatever was issued on
		// the second stream is joined back into the caller's stream
		const umi_status jr = cuda_status(cudaEventRecord(aux->join, aux->s), "cudaEventRecord");
		if (jr == UMI_OK) {
			audit->forked = true;
			audit->done = aux->join;
		} else {
			cudaStreamSynchronize(aux->s);  // no join event: the second stream's work ends here
			if (rc == UMI_OK) rc = jr;
		}
	}
	return rc;
}

// Refine around the proposal's centres, exhaustive search for every
// non-audited block whose refined SAD exceeds sad_threshold, then the
// audited blocks' exhaustive results (begun by me_audit_begin) replace the
// refined ones.  Shared by the learned and the coarse proposal.
umi_status me_refine_fallback_finish(const uint8_t* cur, const uint8_t* ref, int h, int w, const int32_t* centers,
                                     int refine_r, int full_r, int32_t sad_threshold, int audit_stride, int32_t* mv,
                                     unsigned long long* audit_sums, int32_t* n_fallback, const MeFinishBuffers& b,
                                     const MeAudit& audit, cudaStream_t st) {
	const int nblk = (h / 16) * (w / 16);
	void* stream = st;
	UMI_TRY(umi_full_me_u8(cur, ref, h, w, 16, refine_r, centers, mv, stream));
	UMI_TRY(cuda_status(cudaMemsetAsync(b.count, 0, 2 * sizeof(int32_t), st), "cudaMemsetAsync"));
	if (audit_sums)
		UMI_TRY(cuda_status(cudaMemsetAsync(audit_sums, 0, 2 * sizeof(unsigned long long), st), "cudaMemsetAsync"));
	flag_kernel<<<grid_for(nblk), NT, 0, st>>>(mv, nblk, audit.active ? audit_stride : 0, sad_threshold, audit.combined,
	                                           b.list, b.count, audit_sums);
	UMI_TRY(launch_status("flag_kernel"));
	UMI_TRY(umi_full_me_u8_list(cur, ref, h, w, 16, full_r, nullptr, b.list, b.count, nblk, mv, stream));
	if (audit.combined && audit_sums) {
		audit_sum_kernel<<<grid_for(ceil_div(nblk, audit_stride)), NT, 0, st>>>(mv, nblk, audit_stride, audit_sums);
		UMI_TRY(launch_status("audit_sum_kernel"));
	} else if (audit.active && !audit.combined) {
		if (audit.forked) {
			UMI_TRY(cuda_status(cudaStreamWaitEvent(st, audit.done, 0), "cudaStreamWaitEvent"));
			audit.joined = true;
		}
		audit_merge_kernel<<<grid_for(ceil_div(nblk, audit_stride)), NT, 0, st>>>(mv, b.amv, nblk, audit_stride,
		                                                                          audit_sums);
		UMI_TRY(launch_status("audit_merge_kernel"));
	}
	if (n_fallback)
		UMI_TRY(cuda_status(cudaMemcpyAsync(n_fallback, b.count + 1, sizeof(int32_t), cudaMemcpyDeviceToDevice, st),
		                    "cudaMemcpyAsync"));
	return ok();
}

}  // namespace umi
