// UMI operator, generic path: UMI::Execute for arbitrary strategies on sm_103a.
//
// Drop-in for the reference's templated launcher (johnjohnlin/UMI
// src/UMI_gpu.h:409-623): same template parameters, same descriptor
// arguments, so applications written against the reference compile
// unchanged.  Strategy callbacks are device code of the application, so the
// kernel is a template instantiated in the caller's translation unit; the
// descriptor validation and address maps come from the library's C ABI
// (umi_plan_build in libumi_gb300.so, link with -lumi_gb300).
//
// Differences from the reference launcher:
//  * no index tables, no cudaMalloc/cudaMemcpy/__constant__ LUT per call:
//    every address is a closed-form affine map of (p, a) passed by value;
//  * returns umi_status (the reference returns void and aborts on bad
//    descriptors); an extra trailing argument selects the CUDA stream;
//  * asynchronous on that stream (the reference synchronises by freeing its
//    tables);
//  * inputs are read through the read-only data path with the same
//    clamp/pad rule instead of a 64-thread shared-memory fill; ZeroStrideOpt
//    is accepted and has no effect on results (the cache deduplicates the
//    loads it would have saved);
//  * a Loop input whose whole accumulation window stays inside its extent at
//    a point (no clamp, no padding) is addressed linearly: base + a . stride,
//    precomputed per point; points near the edges take the clamped map.
//
// Checked builds: compiled with -DUMI_CHECKED, every output write whose
// physical coordinate falls outside [0, size) of its dimension (size 0 counts
// as 1) is skipped and sets bit 0 of a device flag word instead (no trap);
// UMI::checked_flags() synchronises the device and returns (and clears) it.
// Inputs need no check: their coordinates are clamped into the extent.
#pragma once
#include <cuda_runtime.h>

#include <cstring>

#include "umi/UMI.h"
#include "umi_gb300.h"

namespace UMI {
namespace gpu_detail {

#ifdef UMI_CHECKED
static __device__ unsigned int checked_flags_word = 0;
#endif

template <class EType, int NI, int NO>
struct Pointers {
	const EType* in[SafeArrayLength(NI) * MAX_PTR];
	EType pad[SafeArrayLength(NI) * MAX_PTR];
	EType* out[SafeArrayLength(NO) * MAX_PTR];
};

// Physical coordinates of memory `m` at point p (and accumulation index a
// when `with_a`), folded into a linear element index; `outside` reports a
// clamped PAD coordinate (inputs only).
// I is the index type of the launch: int32_t when the host has shown that
// every coordinate and every linear index of the call fits 32 bits
// (LinearMaps::fit32 and ::idx32), else int64_t.
template <bool CLAMP, class I>
__device__ __forceinline__ I address(const umi_mem_plan& m, const int (&p)[4], const int (&a)[4], bool with_a,
                                     bool& outside) {
	I addr = 0;
	outside = false;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		I c = m.base[k];
#pragma unroll
		for (int d = 0; d < 4; ++d) {
			c += (I)m.pcoef[k][d] * p[d];
			if (with_a) c += (I)m.acoef[k][d] * a[d];
		}
		if (CLAMP) {
			const I hi = (I)m.size[k] - 1;
			const I cl = c < 0 ? 0 : (c > hi ? hi : c);
			outside |= (cl != c) && ((m.pad_mask >> k) & 1);
			c = cl;
		}
#ifdef UMI_CHECKED
		if (!CLAMP) outside |= c < 0 || c >= (m.size[k] > 0 ? m.size[k] : 1);  // output outside its extent
#endif
		addr += c * (I)m.rowstride[k];
	}
	return addr;
}

template <class Umi, uint64_t PtrNum, int OFS, int N, class EType, class I, class P, class Arr>
__device__ __forceinline__ void gather(const umi_plan& plan, const P& ptrs, const int (&p)[4], const int (&a)[4],
                                       bool with_a, Arr& in) {
#pragma unroll
	for (int i = 0; i < N; ++i) {
		const int mem = OFS + i;
		bool outside;
		const I addr = address<true, I>(plan.mem[mem], p, a, with_a, outside);
#pragma unroll
		for (int j = 0; j < MAX_PTR; ++j) {
			if (j < (int)Slice(PtrNum, 4, mem)) {
				in[i * MAX_PTR + j] = outside ? ptrs.pad[mem * MAX_PTR + j] : ptrs.in[mem * MAX_PTR + j][addr];
			}
		}
	}
}

// Linear forms of the address maps, computed once on the host per launch:
// without clamping, memory m's element for point p and step a is
//   lin[m] + sum_d p[d] * pstr[m][d] + sum_d a[d] * astr[m][d],
// and its coordinate k spans [c_k + alo[m][k], c_k + ahi[m][k]] over the
// accumulation range (c_k its coordinate at a = 0).  fit32: every
// coordinate of every point and step fits comfortably in 32 bits; idx32:
// every linear index (clamped maps and linear forms over the launched points,
// one expanded block past P included) and every row stride fits 31 bits.
// gdiv / bdiv: q = (n * mul) >> shift equals n / grid[d] (n / block[d]) for
// every n < 2^31 (Granlund & Montgomery 1994, the round-up multiplier
// mul = ceil(2^(31 + l) / d) with l = ceil(log2 d), shift = 31 + l).
struct FastDiv {
	uint32_t mul;
	int32_t shift;
};
struct LinearMaps {
	int64_t lin[UMI_MAX_MEMS];
	int64_t pstr[UMI_MAX_MEMS][4];
	int64_t astr[UMI_MAX_MEMS][4];
	int64_t alo[UMI_MAX_MEMS][4];
	int64_t ahi[UMI_MAX_MEMS][4];
	int32_t fit32;
	int32_t idx32;
	int32_t bshift[4];  // log2 of the CTA block along each P dimension, -1 if not a power of two
	FastDiv gdiv[4], bdiv[4];
};

inline FastDiv fast_div(int32_t d) {
	FastDiv f{1u << 31, 31};  // d <= 1: n * 2^31 >> 31 = n
	if (d > 1) {
		int l = 0;
		while (((int64_t)1 << l) < d) ++l;
		const uint64_t num = (uint64_t)1 << (31 + l);
		f.mul = (uint32_t)((num + (uint64_t)d - 1) / (uint64_t)d);
		f.shift = 31 + l;
	}
	return f;
}

__device__ __forceinline__ uint32_t div_by(uint32_t n, FastDiv f) {
	return (uint32_t)(((uint64_t)n * f.mul) >> f.shift);
}

inline LinearMaps linear_maps(const umi_plan& plan) {
	LinearMaps L;
	std::memset(&L, 0, sizeof(L));
	bool fit = true;
	for (int m = 0; m < plan.n_in + plan.n_out && m < UMI_MAX_MEMS; ++m) {
		const umi_mem_plan& mp = plan.mem[m];
		for (int k = 0; k < 4; ++k) {
			L.lin[m] += (int64_t)mp.base[k] * mp.rowstride[k];
			int64_t bound = mp.base[k] < 0 ? -(int64_t)mp.base[k] : mp.base[k];
			for (int d = 0; d < 4; ++d) {
				L.pstr[m][d] += (int64_t)mp.pcoef[k][d] * mp.rowstride[k];
				L.astr[m][d] += (int64_t)mp.acoef[k][d] * mp.rowstride[k];
				const int64_t span = (int64_t)mp.acoef[k][d] * (plan.atotal[d] > 0 ? plan.atotal[d] - 1 : 0);
				if (span < 0) L.alo[m][k] += span;
				else L.ahi[m][k] += span;
				const int64_t pc = mp.pcoef[k][d] < 0 ? -(int64_t)mp.pcoef[k][d] : mp.pcoef[k][d];
				bound += pc * (plan.ptotal[d] > 0 ? plan.ptotal[d] : 0);
			}
			bound += L.ahi[m][k] - L.alo[m][k];
			fit &= bound < ((int64_t)1 << 30);
		}
	}
	L.fit32 = fit;
	bool idx = true;
	const int64_t lim = (int64_t)1 << 31;
	auto mag = [](int64_t v) { return v < 0 ? -v : v; };
	for (int m = 0; m < plan.n_in + plan.n_out && m < UMI_MAX_MEMS; ++m) {
		const umi_mem_plan& mp = plan.mem[m];
		int64_t span = 0, lb = mag(L.lin[m]);
		for (int k = 0; k < 4; ++k) {
			idx &= mag(mp.rowstride[k]) < lim;
			span += (int64_t)(mp.size[k] > 0 ? mp.size[k] - 1 : 0) * mag(mp.rowstride[k]);
		}
		for (int d = 0; d < 4; ++d) {
			const int64_t preach = (int64_t)plan.ptotal[d] + (int64_t)plan.block[d] * plan.expand[d];
			lb += mag(L.pstr[m][d]) * preach + mag(L.astr[m][d]) * (plan.atotal[d] > 0 ? plan.atotal[d] - 1 : 0);
		}
		idx &= span < lim && lb < lim;
	}
	L.idx32 = fit && idx;
	for (int d = 0; d < 4; ++d) {
		const int b = plan.block[d];
		L.bshift[d] = -1;
		for (int sh = 0; sh < 31; ++sh)
			if (b == (1 << sh)) L.bshift[d] = sh;
		L.gdiv[d] = fast_div(plan.grid[d]);
		L.bdiv[d] = fast_div(plan.block[d]);
	}
	return L;
}

// A Pre / Post input at point p: the linear form when every coordinate is
// inside the extent (no clamp, no padding), else the clamped map.
template <class Umi, uint64_t PtrNum, int OFS, int N, class EType, class I, class P, class Arr>
__device__ __forceinline__ void gather_point(const umi_plan& plan, const LinearMaps& lm, const P& ptrs,
                                             const int (&p)[4], Arr& in) {
#pragma unroll
	for (int i = 0; i < N; ++i) {
		const int mem = OFS + i;
		const umi_mem_plan& m = plan.mem[mem];
		bool inside = true;
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			I c = m.base[k];
#pragma unroll
			for (int d = 0; d < 4; ++d) c += (I)m.pcoef[k][d] * p[d];
			inside &= c >= 0 && c <= (I)m.size[k] - 1;
		}
		I addr;
		bool outside = false;
		if (inside) {
			addr = (I)lm.lin[mem] + p[0] * (I)lm.pstr[mem][0] + p[1] * (I)lm.pstr[mem][1] + p[2] * (I)lm.pstr[mem][2] +
			       p[3] * (I)lm.pstr[mem][3];
		} else {
			const int zero[4] = {0, 0, 0, 0};
			addr = address<true, I>(m, p, zero, false, outside);
		}
#pragma unroll
		for (int j = 0; j < MAX_PTR; ++j)
			if (j < (int)Slice(PtrNum, 4, mem))
				in[i * MAX_PTR + j] = outside ? ptrs.pad[mem * MAX_PTR + j] : ptrs.in[mem * MAX_PTR + j][addr];
	}
}

// Fast addressing of a Loop input at one point: when every accumulation step
// of the point keeps every physical coordinate inside [0, size-1] (no clamp,
// no padding), the element of step a sits at base + sum_d a[d] * astr[d]:
// the same element the clamped map reads, without recomputing it per step.
template <class I>
struct LinearAddr {
	I base;
	bool inside;
};

template <typename I>
__device__ __forceinline__ bool window_inside(const umi_mem_plan& m, const LinearMaps& L, int mi, const int (&p)[4]) {
	bool in = true;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		I c = (I)m.base[k];
#pragma unroll
		for (int d = 0; d < 4; ++d) c += (I)m.pcoef[k][d] * (I)p[d];
		in &= c + (I)L.alo[mi][k] >= 0 && c + (I)L.ahi[mi][k] <= (I)m.size[k] - 1;
	}
	return in;
}

template <class I>
__device__ __forceinline__ LinearAddr<I> linear_addr(const umi_mem_plan& m, const LinearMaps& L, int mi, const int (&p)[4]) {
	LinearAddr<I> f;
	f.base = (I)L.lin[mi] + p[0] * (I)L.pstr[mi][0] + p[1] * (I)L.pstr[mi][1] + p[2] * (I)L.pstr[mi][2] +
	         p[3] * (I)L.pstr[mi][3];
	f.inside = L.fit32 ? window_inside<int32_t>(m, L, mi, p) : window_inside<int64_t>(m, L, mi, p);
	return f;
}

template <class Umi, uint64_t PtrNum, int OFS, int N, class EType, class I, class P, class Arr>
__device__ __forceinline__ void scatter(const umi_plan& plan, const LinearMaps& lm, const P& ptrs, const int (&p)[4],
                                        const int (&a)[4], bool with_a, const Arr& out) {
#pragma unroll
	for (int i = 0; i < N; ++i) {
		const int mem = OFS + i;
#ifdef UMI_CHECKED
		bool outside;
		const I addr = address<false, I>(plan.mem[Umi::TOTAL_IN + mem], p, a, with_a, outside);
		if (outside) {
			atomicOr(&checked_flags_word, 1u);
			continue;
		}
#else
		// outputs are not clamped: the linear form is the map
		const int mi = Umi::TOTAL_IN + mem;
		I addr = (I)lm.lin[mi] + p[0] * (I)lm.pstr[mi][0] + p[1] * (I)lm.pstr[mi][1] + p[2] * (I)lm.pstr[mi][2] +
		         p[3] * (I)lm.pstr[mi][3];
		if (with_a)
			addr += a[0] * (I)lm.astr[mi][0] + a[1] * (I)lm.astr[mi][1] + a[2] * (I)lm.astr[mi][2] +
			        a[3] * (I)lm.astr[mi][3];
#endif
#pragma unroll
		for (int j = 0; j < MAX_PTR; ++j) {
			if (j < (int)Slice(PtrNum, 4, Umi::TOTAL_IN + mem)) ptrs.out[mem * MAX_PTR + j][addr] = out[i * MAX_PTR + j];
		}
	}
}

// One thread runs E0*E1*E2*E3 output points: p = cta_origin + e*block + t
// (the reference's expand layout, src/UMI.cpp:153-155).  Each point runs Pre,
// the Loop over A in blocked row-major order (src/UMI_gpu.h:287-346), then
// Post; points outside P are skipped (the reference runs them and drops the
// writes).
template <class Umi, uint64_t PtrNum, uint64_t Expand, class EType, class CType, int MAXT = 1024, class I = int64_t>
__global__ void __launch_bounds__(MAXT, MAXT <= 256 ? 3 : 1) generic_kernel(const umi_plan plan, const CType uc,
                                                        const Pointers<EType, Umi::TOTAL_IN, Umi::TOTAL_OUT> ptrs,
                                                        const LinearMaps lm) {
	constexpr int E0 = (int)Slice(Expand, 4, 3), E1 = (int)Slice(Expand, 4, 2);
	constexpr int E2 = (int)Slice(Expand, 4, 1), E3 = (int)Slice(Expand, 4, 0);
	constexpr int ES = E0 * E1 * E2 * E3;
	constexpr int PRE_I = 0, LOOP_I = Umi::N_PRE_IN, POST_I = Umi::N_PRE_IN + Umi::N_LOOP_IN;
	constexpr int PRE_O = 0, LOOP_O = Umi::N_PRE_OUT, POST_O = Umi::N_PRE_OUT + Umi::N_LOOP_OUT;
	const int zero[4] = {0, 0, 0, 0};
	for (int64_t cta = blockIdx.x; cta < plan.n_cta; cta += gridDim.x) {
		int g[4], t[4];
		{
			if (cta <= 0x7fffffff) {  // 32-bit index arithmetic (every CTA of plans below 2^31 CTAs)
				uint32_t r = (uint32_t)cta;
#pragma unroll
				for (int d = 3; d >= 0; --d) {
					const uint32_t q = div_by(r, lm.gdiv[d]);
					g[d] = (int)(r - q * (uint32_t)plan.grid[d]);
					r = q;
				}
			} else {
				int64_t r = cta;
#pragma unroll
				for (int d = 3; d >= 0; --d) {
					g[d] = (int)(r % plan.grid[d]);
					r /= plan.grid[d];
				}
			}
			int s = threadIdx.x;
			const bool pow2 = lm.bshift[0] >= 0 && lm.bshift[1] >= 0 && lm.bshift[2] >= 0 && lm.bshift[3] >= 0;
#pragma unroll
			for (int d = 3; d >= 0; --d) {
				if (pow2) {
					t[d] = s & ((1 << lm.bshift[d]) - 1);
					s >>= lm.bshift[d];
				} else {
					const int q = (int)div_by((uint32_t)s, lm.bdiv[d]);
					t[d] = s - q * plan.block[d];
					s = q;
				}
			}
		}
		int pts[ES][4];
		bool valid[ES];
#pragma unroll
		for (int e = 0; e < ES; ++e) {
			const int ex[4] = {e / (E1 * E2 * E3), (e / (E2 * E3)) % E1, (e / E3) % E2, e % E3};
			bool v = true;
#pragma unroll
			for (int d = 0; d < 4; ++d) {
				pts[e][d] = g[d] * plan.expand[d] * plan.block[d] + ex[d] * plan.block[d] + t[d];
				v &= pts[e][d] < plan.ptotal[d];
			}
			valid[e] = v;
		}
		Umi ctx[ES];
		// Pre
#pragma unroll
		for (int e = 0; e < ES; ++e) {
			if (!valid[e]) continue;
			simple_array<EType, Umi::N_PRE_IN * MAX_PTR> in;
			simple_array<EType, Umi::N_PRE_OUT * MAX_PTR> out;
			gather_point<Umi, PtrNum, PRE_I, Umi::N_PRE_IN, EType, I>(plan, lm, ptrs, pts[e], in);
			ctx[e].Pre(uc, in, out);
			scatter<Umi, PtrNum, PRE_O, Umi::N_PRE_OUT, EType, I>(plan, lm, ptrs, pts[e], zero, false, out);
		}
		// Loop inputs: linear addressing for points whose whole window is inside.
		constexpr int NLI = SafeArrayLength(Umi::N_LOOP_IN);
		I lbase[ES][NLI];
		I astr[NLI][4];
		bool fast[ES];
#pragma unroll
		for (int i = 0; i < Umi::N_LOOP_IN; ++i)
#pragma unroll
			for (int d = 0; d < 4; ++d) astr[i][d] = (I)lm.astr[LOOP_I + i][d];
#pragma unroll
		for (int e = 0; e < ES; ++e) {
			bool f = Umi::N_LOOP_IN > 0;
#pragma unroll
			for (int i = 0; i < Umi::N_LOOP_IN; ++i) {
				const LinearAddr<I> la = linear_addr<I>(plan.mem[LOOP_I + i], lm, LOOP_I + i, pts[e]);
				lbase[e][i] = la.base;
				f &= la.inside;
			}
			fast[e] = f;
		}
		bool all_fast = true;
#pragma unroll
		for (int e = 0; e < ES; ++e) all_fast &= fast[e] || !valid[e];
		// Loop: accumulation blocks row-major, steps row-major inside a block
		// (dimension 3 fastest), as four nested loops clipped to the A extent.
		if (plan.n_ablock > 0) {
			int ab[4] = {0, 0, 0, 0};
			for (int bi = 0; bi < plan.n_ablock; ++bi) {
				int a0[4], lim[4];
#pragma unroll
				for (int d = 0; d < 4; ++d) {
					a0[d] = ab[d] * plan.ablock[d];
					lim[d] = min(plan.ablock[d], plan.atotal[d] - a0[d]);
				}
				if (ES == 1 && all_fast) {
					// every point of the thread reads inside its extents: linear rows, one stride per step
					// (one point per thread only: with several, the optimiser's time grows steeply)
					for (int s0 = 0; s0 < lim[0]; ++s0)
						for (int s1 = 0; s1 < lim[1]; ++s1)
							for (int s2 = 0; s2 < lim[2]; ++s2) {
								I row[ES][NLI];
								const int ar[4] = {a0[0] + s0, a0[1] + s1, a0[2] + s2, a0[3]};
#pragma unroll
								for (int e = 0; e < ES; ++e)
#pragma unroll
									for (int i = 0; i < NLI; ++i)
										row[e][i] = lbase[e][i] + ar[0] * astr[i][0] + ar[1] * astr[i][1] +
										            ar[2] * astr[i][2] + ar[3] * astr[i][3];
								// four steps per trip: a quarter of the loop control per step
#pragma unroll 4
								for (int s3 = 0; s3 < lim[3]; ++s3) {
									const int a[4] = {a0[0] + s0, a0[1] + s1, a0[2] + s2, a0[3] + s3};
#pragma unroll
									for (int e = 0; e < ES; ++e) {
										if (!valid[e]) continue;
										simple_array<EType, Umi::N_LOOP_IN * MAX_PTR> in;
										simple_array<EType, Umi::N_LOOP_OUT * MAX_PTR> out;
#pragma unroll
										for (int i = 0; i < Umi::N_LOOP_IN; ++i) {
											const int mem = LOOP_I + i;
#pragma unroll
											for (int j = 0; j < MAX_PTR; ++j)
												if (j < (int)Slice(PtrNum, 4, mem))
													in[i * MAX_PTR + j] = ptrs.in[mem * MAX_PTR + j][row[e][i]];
											row[e][i] += astr[i][3];
										}
										ctx[e].Loop(uc, in, out);
										scatter<Umi, PtrNum, LOOP_O, Umi::N_LOOP_OUT, EType, I>(plan, lm, ptrs, pts[e], a, true, out);
									}
								}
							}
				} else {
					// points near the edges: the clamped map for every step
					for (int s0 = 0; s0 < lim[0]; ++s0)
						for (int s1 = 0; s1 < lim[1]; ++s1)
							for (int s2 = 0; s2 < lim[2]; ++s2)
								for (int s3 = 0; s3 < lim[3]; ++s3) {
									const int a[4] = {a0[0] + s0, a0[1] + s1, a0[2] + s2, a0[3] + s3};
#pragma unroll
									for (int e = 0; e < ES; ++e) {
										if (!valid[e]) continue;
										simple_array<EType, Umi::N_LOOP_IN * MAX_PTR> in;
										simple_array<EType, Umi::N_LOOP_OUT * MAX_PTR> out;
										gather<Umi, PtrNum, LOOP_I, Umi::N_LOOP_IN, EType, I>(plan, ptrs, pts[e], a, true, in);
										ctx[e].Loop(uc, in, out);
										scatter<Umi, PtrNum, LOOP_O, Umi::N_LOOP_OUT, EType, I>(plan, lm, ptrs, pts[e], a, true, out);
									}
								}
				}
#pragma unroll
				for (int d = 3; d >= 0; --d) {
					if (++ab[d] < plan.agrid[d]) break;
					ab[d] = 0;
				}
			}
		}
		// Post
#pragma unroll
		for (int e = 0; e < ES; ++e) {
			if (!valid[e]) continue;
			simple_array<EType, Umi::N_POST_IN * MAX_PTR> in;
			simple_array<EType, Umi::N_POST_OUT * MAX_PTR> out;
			gather_point<Umi, PtrNum, POST_I, Umi::N_POST_IN, EType, I>(plan, lm, ptrs, pts[e], in);
			ctx[e].Post(uc, in, out);
			scatter<Umi, PtrNum, POST_O, Umi::N_POST_OUT, EType, I>(plan, lm, ptrs, pts[e], zero, false, out);
		}
	}
}

// Plans of at most 256 threads (the common case) get the variant with a
// larger register budget; calls whose indices fit 32 bits the int32_t one.
template <class Umi, uint64_t PtrNum, uint64_t Expand, class EType, class CType>
void launch_generic(const umi_plan& plan, const CType& c, const Pointers<EType, Umi::TOTAL_IN, Umi::TOTAL_OUT>& ptrs,
                    const LinearMaps& lm, unsigned grid, cudaStream_t stream) {
	if (plan.n_threads <= 256) {
		if (lm.idx32)
			generic_kernel<Umi, PtrNum, Expand, EType, CType, 256, int32_t><<<grid, plan.n_threads, 0, stream>>>(plan, c, ptrs, lm);
		else
			generic_kernel<Umi, PtrNum, Expand, EType, CType, 256, int64_t><<<grid, plan.n_threads, 0, stream>>>(plan, c, ptrs, lm);
	} else {
		if (lm.idx32)
			generic_kernel<Umi, PtrNum, Expand, EType, CType, 1024, int32_t><<<grid, plan.n_threads, 0, stream>>>(plan, c, ptrs, lm);
		else
			generic_kernel<Umi, PtrNum, Expand, EType, CType, 1024, int64_t><<<grid, plan.n_threads, 0, stream>>>(plan, c, ptrs, lm);
	}
}

inline umi_vdim lower(const ViewDim& v) { return umi_vdim{v.physical_dim_id, v.ofs, v.stride}; }
inline umi_phydim lower(const PhysicalDim& p) { return umi_phydim{p.size, (int32_t)p.mode}; }

}  // namespace gpu_detail

#ifdef UMI_CHECKED
// Flags raised by checked kernels of this translation unit since the last call
// (bit 0: an output write outside its extent was skipped); synchronises the device.
inline unsigned int checked_flags(bool reset = true) {
	unsigned int v = 0;
	cudaDeviceSynchronize();
	cudaMemcpyFromSymbol(&v, gpu_detail::checked_flags_word, sizeof(v));
	if (reset) {
		const unsigned int z = 0;
		cudaMemcpyToSymbol(gpu_detail::checked_flags_word, &z, sizeof(z));
	}
	return v;
}
#endif

// Generic UMI operator (reference interface: src/UMI_gpu.h:409-422).
template <
	class Umi,
	uint64_t PtrNum = 0x1111111111111111ull,
	uint64_t Expand = 0x1111,
	uint64_t ZeroStrideOpt = 0,
	class EType = typename std::remove_cv<typename Umi::ElementType>::type,
	class CType = typename std::remove_cv<typename Umi::UserConstantType>::type>
umi_status Execute(
	const NDTuple<ParallelDim>& p_dims,
	const NDTuple<AccumulationDim>& a_dims,
	const std::array<UnrolledI<EType>, Umi::TOTAL_IN>& imems,
	const std::array<UnrolledO<EType>, Umi::TOTAL_OUT>& omems,
	const CType& c = CType(),
	cudaStream_t stream = 0) {
	static_assert(Umi::TOTAL_IN + Umi::TOTAL_OUT <= UMI_MAX_MEMS, "at most 16 memories per call");
	static_assert(((Expand >> 12) & 0xf) * ((Expand >> 8) & 0xf) * ((Expand >> 4) & 0xf) * (Expand & 0xf) > 0,
	              "every Expand nibble must be >= 1");
	(void)ZeroStrideOpt;
	umi_desc d;
	std::memset(&d, 0, sizeof(d));
	for (int i = 0; i < DIM; ++i) {
		d.p[i] = umi_pdim{p_dims[i].total_size, p_dims[i].block_size, p_dims[i].warp_size, p_dims[i].warp_shuf};
		d.a[i] = umi_adim{a_dims[i].total_size, a_dims[i].block_size};
	}
	d.expand = (uint32_t)(Expand & 0xffff);
	d.n_in = Umi::TOTAL_IN;
	d.n_out = Umi::TOTAL_OUT;
	auto stage_in = [](int i) { return i < Umi::N_PRE_IN ? 0 : (i < Umi::N_PRE_IN + Umi::N_LOOP_IN ? 1 : 2); };
	auto stage_out = [](int i) { return i < Umi::N_PRE_OUT ? 0 : (i < Umi::N_PRE_OUT + Umi::N_LOOP_OUT ? 1 : 2); };
	gpu_detail::Pointers<EType, Umi::TOTAL_IN, Umi::TOTAL_OUT> ptrs;
	std::memset(&ptrs, 0, sizeof(ptrs));
	for (int i = 0; i < Umi::TOTAL_IN; ++i) {
		umi_mem_desc& m = d.mem[i];
		for (int k = 0; k < DIM; ++k) {
			m.p_view[k] = gpu_detail::lower(imems[i].p_view_dims[k]);
			m.a_view[k] = gpu_detail::lower(imems[i].a_view_dims[k]);
			m.phys[k] = gpu_detail::lower(imems[i].physical_dims[k]);
		}
		m.stage = stage_in(i);
		m.n_ptr = (int32_t)Slice(PtrNum, 4, i);
		for (int j = 0; j < MAX_PTR; ++j) {
			ptrs.in[i * MAX_PTR + j] = imems[i].ptr[j];
			ptrs.pad[i * MAX_PTR + j] = imems[i].padding[j];
		}
	}
	for (int i = 0; i < Umi::TOTAL_OUT; ++i) {
		umi_mem_desc& m = d.mem[Umi::TOTAL_IN + i];
		for (int k = 0; k < DIM; ++k) {
			m.p_view[k] = gpu_detail::lower(omems[i].p_view_dims[k]);
			m.a_view[k] = gpu_detail::lower(omems[i].a_view_dims[k]);
			m.phys[k] = gpu_detail::lower(omems[i].physical_dims[k]);
		}
		m.stage = stage_out(i);
		m.n_ptr = (int32_t)Slice(PtrNum, 4, Umi::TOTAL_IN + i);
		for (int j = 0; j < MAX_PTR; ++j) ptrs.out[i * MAX_PTR + j] = omems[i].ptr[j];
	}
	umi_plan plan;
	const umi_status st = umi_plan_build(&d, &plan);
	if (st != UMI_OK) return st;
	for (int i = 0; i < Umi::TOTAL_IN + Umi::TOTAL_OUT; ++i)
		for (int j = 0; j < d.mem[i].n_ptr; ++j)
			if (i < Umi::TOTAL_IN ? ptrs.in[i * MAX_PTR + j] == nullptr
			                      : ptrs.out[(i - Umi::TOTAL_IN) * MAX_PTR + j] == nullptr)
				return UMI_ERR_INVALID_ARG;
	if (plan.n_cta == 0) return UMI_OK;
	const unsigned grid = (unsigned)(plan.n_cta < 0x7fffffff ? plan.n_cta : 0x7fffffff);
	const gpu_detail::LinearMaps lm = gpu_detail::linear_maps(plan);
	gpu_detail::launch_generic<Umi, PtrNum, Expand, EType, CType>(plan, c, ptrs, lm, grid, stream);
	return cudaGetLastError() == cudaSuccess ? UMI_OK : UMI_ERR_CUDA;
}

}  // namespace UMI
