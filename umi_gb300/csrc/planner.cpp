// Descriptor validation and closed-form address maps for the generic UMI
// kernel (include/umi/UMI_gpu.h).
//
// The reference builds six host index tables per call, uploads them with
// cudaMalloc/cudaMemcpy and a __constant__ LUT, and aborts on bad geometry
// (src/UMI.cpp:39-226, src/UMI_gpu.h:423-609).  Here the same information is
// an affine map per memory (a few dozen integers), computed once on the host,
// passed by value to the kernel, with no allocation and no global state.
#include <cstring>

#include "common.h"

namespace {

bool is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

// Fill one memory's address map.  The a-view offsets always enter the base
// (src/UMI_gpu.h:492-494, :535-537); the a-view index term only for
// Loop-stage memories (src/UMI_gpu.h:54-57, :145-147, :176-179).
umi_status map_mem(const umi_mem_desc& m, bool is_output, bool reads, umi_mem_plan& out) {
	std::memset(&out, 0, sizeof(out));
	if (m.stage < 0 || m.stage > 2)
		return umi::fail(UMI_ERR_INVALID_DESC, "memory stage %d is not 0 (Pre), 1 (Loop) or 2 (Post)", m.stage);
	if (m.n_ptr < 0 || m.n_ptr > UMI_MAX_PTR)
		return umi::fail(UMI_ERR_INVALID_DESC, "a memory carries %d pointers (max %d)", m.n_ptr, UMI_MAX_PTR);
	for (int d = 0; d < UMI_DIM; ++d) {
		const umi_vdim& pv = m.p_view[d];
		const umi_vdim& av = m.a_view[d];
		if (pv.physical_dim_id < 0 || pv.physical_dim_id >= UMI_DIM || av.physical_dim_id < 0 ||
		    av.physical_dim_id >= UMI_DIM)
			return umi::fail(UMI_ERR_INVALID_DESC, "view dimension maps to physical dimension outside 0..3");
		out.base[pv.physical_dim_id] += pv.ofs;
		out.base[av.physical_dim_id] += av.ofs;
		out.pcoef[pv.physical_dim_id][d] += pv.stride;
		if (m.stage == 1) out.acoef[av.physical_dim_id][d] += av.stride;
	}
	int64_t stride = 1;
	for (int k = UMI_DIM - 1; k >= 0; --k) {
		const int32_t sz = m.phys[k].size;
		if (sz < 0) return umi::fail(UMI_ERR_INVALID_DESC, "negative physical size");
		if (!is_output && reads && sz == 0) {
			// An input read through a 0-sized dimension has no element to clamp to.
			bool used = out.base[k] != 0;
			for (int d = 0; d < UMI_DIM; ++d) used |= out.pcoef[k][d] != 0 || out.acoef[k][d] != 0;
			if (used) return umi::fail(UMI_ERR_INVALID_DESC, "input physical dimension %d has size 0", k);
		}
		out.size[k] = sz;
		out.rowstride[k] = stride;
		stride *= sz;
		if (m.phys[k].mode == 0) out.pad_mask |= 1 << k;
		else if (m.phys[k].mode != 1)
			return umi::fail(UMI_ERR_INVALID_DESC, "boundary mode %d is neither PAD (0) nor WRAP (1)", m.phys[k].mode);
	}
	out.stage = m.stage;
	out.n_ptr = m.n_ptr;
	out.is_output = is_output ? 1 : 0;
	return UMI_OK;
}

}  // namespace

extern "C" umi_status umi_plan_build(const umi_desc* desc, umi_plan* plan) {
	if (!desc || !plan) return umi::fail(UMI_ERR_INVALID_ARG, "umi_plan_build: null argument");
	std::memset(plan, 0, sizeof(*plan));
	const umi_desc& d = *desc;
	if (d.n_in < 0 || d.n_out < 0 || d.n_in + d.n_out > UMI_MAX_MEMS)
		return umi::fail(UMI_ERR_INVALID_DESC, "%d inputs + %d outputs (max %d memories)", d.n_in, d.n_out,
		                 UMI_MAX_MEMS);
	// Parallel dims: src/UMI.cpp:39-66.
	int64_t warp = 1, threads = 1, cta = 1;
	bool empty = false;
	for (int i = 0; i < UMI_DIM; ++i) {
		const umi_pdim& p = d.p[i];
		const int32_t shuf = p.warp_shuf == 0 ? 1 : p.warp_shuf;
		const int32_t e = (int32_t)((d.expand >> (4 * (UMI_DIM - 1 - i))) & 0xf);
		if (p.block_size <= 0 || p.warp_size <= 0)
			return umi::fail(UMI_ERR_INVALID_DESC, "parallel dim %d: block_size %d, warp_size %d must be positive", i,
			                 p.block_size, p.warp_size);
		if (!is_pow2(shuf))
			return umi::fail(UMI_ERR_INVALID_DESC, "parallel dim %d: warp_shuf %d is not a power of two", i, shuf);
		if (p.block_size % ((int64_t)p.warp_size * shuf) != 0)
			return umi::fail(UMI_ERR_INVALID_DESC, "parallel dim %d: block_size %d not divisible by warp_size*warp_shuf %d",
			                 i, p.block_size, p.warp_size * shuf);
		if (e <= 0) return umi::fail(UMI_ERR_INVALID_DESC, "Expand nibble for dim %d is 0", i);
		if (p.total_size < 0) return umi::fail(UMI_ERR_INVALID_DESC, "parallel dim %d: negative total", i);
		if (p.total_size == 0) empty = true;
		warp *= p.warp_size;
		threads *= p.block_size;
		plan->ptotal[i] = p.total_size;
		plan->block[i] = p.block_size;
		plan->expand[i] = e;
		plan->grid[i] = p.total_size == 0 ? 0 : (int32_t)umi::ceil_div<int64_t>(p.total_size, (int64_t)e * p.block_size);
		cta *= plan->grid[i];
	}
	if (warp != 32)
		return umi::fail(UMI_ERR_INVALID_DESC, "product of warp sizes is %lld, must be 32", (long long)warp);
	if (threads > 1024)
		return umi::fail(UMI_ERR_INVALID_DESC, "product of block sizes is %lld threads (max 1024)", (long long)threads);
	plan->n_threads = (int32_t)threads;
	plan->n_cta = empty ? 0 : cta;
	// Accumulation dims: src/UMI.cpp:68-76.
	int64_t nab = 1, abs = 1;
	for (int i = 0; i < UMI_DIM; ++i) {
		const umi_adim& a = d.a[i];
		if (a.block_size <= 0)
			return umi::fail(UMI_ERR_INVALID_DESC, "accumulation dim %d: block_size %d must be positive", i, a.block_size);
		if (a.total_size < 0) return umi::fail(UMI_ERR_INVALID_DESC, "accumulation dim %d: negative total", i);
		plan->atotal[i] = a.total_size;
		plan->ablock[i] = a.block_size;
		plan->agrid[i] = a.total_size == 0 ? 0 : (int32_t)umi::ceil_div<int64_t>(a.total_size, a.block_size);
		nab *= plan->agrid[i];
		abs *= a.block_size;
	}
	if (nab > INT32_MAX || abs > INT32_MAX) return umi::fail(UMI_ERR_INVALID_DESC, "accumulation space too large");
	plan->n_ablock = (int32_t)nab;
	plan->ablock_size = (int32_t)abs;
	plan->n_in = d.n_in;
	plan->n_out = d.n_out;
	// With an empty parallel space nothing is read, so 0-sized inputs are fine.
	for (int i = 0; i < d.n_in + d.n_out; ++i)
		UMI_TRY(map_mem(d.mem[i], i >= d.n_in, plan->n_cta > 0, plan->mem[i]));
	return umi::ok();
}
