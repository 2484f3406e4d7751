// Generic UMI operator behind the C ABI: umi_plan_create / umi_launch / umi_plan_destroy.
//
// The reference's Execute (src/UMI_gpu.h:409-623) is a C++ template over a
// user strategy, so a C caller cannot pass its own functor.  This entry
// point serves the strategies of the reference's example applications,
// compiled into the library, on any descriptor the planner accepts:
//   UMI_STRATEGY_NEIGHBOUR_SUM_I32  main/filter3x3.cu:10-17   (constants: int init, mul)
//   UMI_STRATEGY_WEIGHTED_SUM_I32   main/wfilter3x3.cu:8-15   (constant: int init)
//   UMI_STRATEGY_RANGE_WEIGHTED_F32 main/bilateral.cu:9-24    (constant: float norm)
//   UMI_STRATEGY_ABS_DIFF_SUM_I32   main/cost_volume.cu:8-15, main/full_me.cu (same strategy)
//   UMI_STRATEGY_RUNNING_SUM_I32    main/iimg.cu:11-18
//   UMI_STRATEGY_DOT_I32            main/gemm.cu:8-15, main/fprop.cu (same strategy)
//   UMI_STRATEGY_DOT_F32            the gemm strategy on float
// and four more window operators of the same family (no reference example):
//   UMI_STRATEGY_CENSUS_I32         Pre(1 in) centre; Loop(1 in) bits = bits << 1 | (x < centre); Post out = bits
//   UMI_STRATEGY_WEIGHTED_SUM_F32   the wfilter3x3 strategy on float (constant: float init)
//   UMI_STRATEGY_MAX_I32            Loop t = max(t, x) (grey-level dilation; constant: int init)
//   UMI_STRATEGY_MIN_I32            Loop t = min(t, x) (grey-level erosion; constant: int init)
// The kernel is the same closed-form generic kernel as the header-only
// drop-in (include/umi/UMI_gpu.h); tiling never changes results, so the
// launch runs the plan with one point per thread.
#include <cstdlib>
#include <cstring>

#include "common.h"
#include "umi/UMI_gpu.h"

using namespace UMI;

namespace {

struct NeighbourSumI32 {
	int total;
	struct Constant { int init, mul; };
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = c.init; }
	STRATEGY_LOOP_STUB(1, 0) { total += IMEM(0, 0); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = total * c.mul; }
};

struct WeightedSumI32 {
	int total;
	struct Constant { int init; };
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = c.init; }
	STRATEGY_LOOP_STUB(2, 0) { total += IMEM(0, 0) * IMEM(1, 0); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = total; }
};

struct RangeWeightedF32 {
	float wsum, wxsum, centre;
	struct Constant { float norm; };
	STRATEGY_TYPEDEF_STUB(float, Constant)
	STRATEGY_PRE_STUB(1, 0) {
		wsum = 0.0f;
		wxsum = 0.0f;
		centre = IMEM(0, 0);
	}
	STRATEGY_LOOP_STUB(3, 0) {
		const float v = IMEM(0, 0), diff = v - centre;
		const float wgt = expf(diff * diff * c.norm) * IMEM(1, 0) * IMEM(2, 0);
		wsum += wgt;
		wxsum += wgt * v;
	}
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = wxsum / wsum; }
};

struct AbsDiffSumI32 {
	int sad;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { sad = 0; }
	STRATEGY_LOOP_STUB(2, 0) { sad += abs(IMEM(0, 0) - IMEM(1, 0)); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = sad; }
};

struct RunningSumI32 {
	int total;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = 0; }
	STRATEGY_LOOP_STUB(1, 1) { OMEM(0, 0) = total += IMEM(0, 0); }
	STRATEGY_POST_STUB_
};

template <class T>
struct DotT {
	T total;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(T, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = T(0); }
	STRATEGY_LOOP_STUB(2, 0) { total += IMEM(0, 0) * IMEM(1, 0); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = total; }
};

// Census transform: one bit per window element in the A loop order, set
// where the element is below the centre (the last 32 elements for larger
// windows; the centre itself contributes a 0).
struct CensusI32 {
	uint32_t bits;
	int centre;
	struct Constant {};
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(1, 0) {
		bits = 0u;
		centre = IMEM(0, 0);
	}
	STRATEGY_LOOP_STUB(1, 0) { bits = (bits << 1) | (IMEM(0, 0) < centre ? 1u : 0u); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = (int)bits; }
};

struct WeightedSumF32 {
	float total;
	struct Constant { float init; };
	STRATEGY_TYPEDEF_STUB(float, Constant)
	STRATEGY_PRE_STUB(0, 0) { total = c.init; }
	STRATEGY_LOOP_STUB(2, 0) { total = fmaf(IMEM(0, 0), IMEM(1, 0), total); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = total; }
};

template <bool MAX>
struct ExtremumI32 {
	int t;
	struct Constant { int init; };
	STRATEGY_TYPEDEF_STUB(int, Constant)
	STRATEGY_PRE_STUB(0, 0) { t = c.init; }
	STRATEGY_LOOP_STUB(1, 0) { t = MAX ? max(t, IMEM(0, 0)) : min(t, IMEM(0, 0)); }
	STRATEGY_POST_STUB(0, 1) { OMEM(0, 0) = t; }
};

constexpr uint64_t kOnePtr = 0x1111111111111111ull;

// The memories of `plan` must be the strategy's, in its stage order, one pointer each.
template <class Umi>
umi_status check_shape(const umi_plan& plan) {
	if (plan.n_in != Umi::TOTAL_IN || plan.n_out != Umi::TOTAL_OUT)
		return umi::fail(UMI_ERR_INVALID_DESC, "umi_launch: %d inputs / %d outputs, strategy needs %d / %d",
		                 plan.n_in, plan.n_out, (int)Umi::TOTAL_IN, (int)Umi::TOTAL_OUT);
	for (int i = 0; i < Umi::TOTAL_IN; ++i) {
		const int want = i < Umi::N_PRE_IN ? 0 : (i < Umi::N_PRE_IN + Umi::N_LOOP_IN ? 1 : 2);
		if (plan.mem[i].stage != want)
			return umi::fail(UMI_ERR_INVALID_DESC, "umi_launch: input %d has stage %d, strategy needs %d", i,
			                 plan.mem[i].stage, want);
	}
	for (int i = 0; i < Umi::TOTAL_OUT; ++i) {
		const int want = i < Umi::N_PRE_OUT ? 0 : (i < Umi::N_PRE_OUT + Umi::N_LOOP_OUT ? 1 : 2);
		if (plan.mem[Umi::TOTAL_IN + i].stage != want)
			return umi::fail(UMI_ERR_INVALID_DESC, "umi_launch: output %d has stage %d, strategy needs %d", i,
			                 plan.mem[Umi::TOTAL_IN + i].stage, want);
	}
	for (int i = 0; i < Umi::TOTAL_IN + Umi::TOTAL_OUT; ++i)
		if (plan.mem[i].n_ptr != 1)
			return umi::fail(UMI_ERR_UNSUPPORTED, "umi_launch: memory %d has %d pointers (built-in strategies take 1)",
			                 i, plan.mem[i].n_ptr);
	return UMI_OK;
}

template <class Umi>
umi_status launch_as(const umi_plan& plan0, const void* const* in, const void* pad, void* const* out,
                     const void* user_const, size_t uc_bytes, cudaStream_t st) {
	using E = typename Umi::ElementType;
	using C = typename Umi::UserConstantType;
	UMI_TRY(check_shape<Umi>(plan0));
	C c{};
	if (std::is_empty<C>::value == false) {
		if (!user_const || uc_bytes < sizeof(C))
			return umi::fail(UMI_ERR_INVALID_ARG, "umi_launch: strategy needs %zu bytes of constants, got %zu",
			                 sizeof(C), user_const ? uc_bytes : (size_t)0);
		std::memcpy(&c, user_const, sizeof(C));
	}
	gpu_detail::Pointers<E, Umi::TOTAL_IN, Umi::TOTAL_OUT> ptrs;
	std::memset(&ptrs, 0, sizeof(ptrs));
	for (int i = 0; i < Umi::TOTAL_IN; ++i) {
		if (!in[i]) return umi::fail(UMI_ERR_INVALID_ARG, "umi_launch: input %d is null", i);
		ptrs.in[i * MAX_PTR] = static_cast<const E*>(in[i]);
		if (pad) std::memcpy(&ptrs.pad[i * MAX_PTR], static_cast<const char*>(pad) + 4 * i, sizeof(E));
	}
	for (int i = 0; i < Umi::TOTAL_OUT; ++i) {
		if (!out[i]) return umi::fail(UMI_ERR_INVALID_ARG, "umi_launch: output %d is null", i);
		ptrs.out[i * MAX_PTR] = static_cast<E*>(out[i]);
	}
	// One point per thread (results do not depend on the tiling).
	umi_plan plan = plan0;
	int64_t n_cta = 1;
	for (int d = 0; d < UMI_DIM; ++d) {
		plan.expand[d] = 1;
		plan.grid[d] = plan.block[d] > 0 ? (int32_t)umi::ceil_div(plan.ptotal[d], plan.block[d]) : 0;
		n_cta *= plan.grid[d];
	}
	plan.n_cta = n_cta;
	if (n_cta == 0) return umi::ok();
	const unsigned grid = (unsigned)(n_cta < 0x7fffffff ? n_cta : 0x7fffffff);
	const gpu_detail::LinearMaps lm = gpu_detail::linear_maps(plan);
	gpu_detail::launch_generic<Umi, kOnePtr, 0x1111, E, C>(plan, c, ptrs, lm, grid, st);
	return umi::launch_status("generic_kernel");
}

}  // namespace

extern "C" umi_status umi_plan_create(const umi_desc* desc, umi_plan** out) {
	if (!desc || !out) return umi::fail(UMI_ERR_INVALID_ARG, "umi_plan_create: null pointer");
	*out = nullptr;
	umi_plan* p = static_cast<umi_plan*>(std::malloc(sizeof(umi_plan)));
	if (!p) return umi::fail(UMI_ERR_NO_MEMORY, "umi_plan_create: host allocation failed");
	const umi_status st = umi_plan_build(desc, p);
	if (st != UMI_OK) {
		std::free(p);
		return st;
	}
	*out = p;
	return UMI_OK;
}

extern "C" void umi_plan_destroy(umi_plan* plan) { std::free(plan); }

extern "C" umi_status umi_launch(const umi_plan* plan, int32_t op, const void* const* in, const void* pad,
                                 void* const* out, const void* user_const, size_t uc_bytes, void* stream) {
	if (!plan || (plan->n_in > 0 && !in) || (plan->n_out > 0 && !out))
		return umi::fail(UMI_ERR_INVALID_ARG, "umi_launch: null pointer");
	const cudaStream_t st = umi::as_stream(stream);
	switch (op) {
		case UMI_STRATEGY_NEIGHBOUR_SUM_I32: return launch_as<NeighbourSumI32>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_WEIGHTED_SUM_I32: return launch_as<WeightedSumI32>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_RANGE_WEIGHTED_F32: return launch_as<RangeWeightedF32>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_ABS_DIFF_SUM_I32: return launch_as<AbsDiffSumI32>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_RUNNING_SUM_I32: return launch_as<RunningSumI32>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_DOT_I32: return launch_as<DotT<int>>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_DOT_F32: return launch_as<DotT<float>>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_CENSUS_I32: return launch_as<CensusI32>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_WEIGHTED_SUM_F32: return launch_as<WeightedSumF32>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_MAX_I32: return launch_as<ExtremumI32<true>>(*plan, in, pad, out, user_const, uc_bytes, st);
		case UMI_STRATEGY_MIN_I32: return launch_as<ExtremumI32<false>>(*plan, in, pad, out, user_const, uc_bytes, st);
		default: return umi::fail(UMI_ERR_UNSUPPORTED, "umi_launch: unknown strategy %d", op);
	}
}
