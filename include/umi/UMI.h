// UMI operator API: descriptor types and strategy macros.
//
// Source-compatible front end for the templated operator interface of
// johnjohnlin/UMI (src/UMI.h:77-137).  The struct names, member order and
// macro names are kept identical so that application code written against the
// reference (aggregate-initialised descriptors, STRATEGY_* functors, IMEM/OMEM)
// compiles unchanged.  Everything else (packing, index tables, Int4 helpers)
// is not part of the interface and is not reproduced: the GB300 kernels use
// closed-form index arithmetic.
//
// This header is usable from plain C++ (host-only, e.g. the CPU oracle) and
// from nvcc translation units (strategy callbacks become __host__ __device__).
#pragma once
#include <algorithm>
#include <array>
#include <cassert>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <tuple>
#include <type_traits>
#include <vector>

#if defined(__CUDACC__)
#  define DHFunc __host__ __device__
#  define DFunc __device__
#else
#  define DHFunc
#  define DFunc
#endif

namespace UMI {

// Interface constants (src/UMI.h:42-49).  MAX_PTR is the number of pointers a
// single memory descriptor may carry; DIM is the fixed rank of every index
// space; WARP_SIZE is the product every ParallelDim.warp_size set must reach.
static constexpr int MAX_PTR = 4;
static constexpr int DIM = 4;
static constexpr int MAX_WARP = 32;
static constexpr int WARP_SIZE = 32;
static constexpr int WORD_SIZE = 4;
static constexpr int MAX_BLOCK_SIZE = MAX_WARP * WARP_SIZE;

template <class Int> inline constexpr bool IsPowOf2(const Int i) { return i > 0 && (i & (i - 1)) == 0; }
template <class Int> inline constexpr Int CeilDiv(const Int a, const Int b) { return (a + b - 1) / b; }

// A fixed-size array usable in device code; the strategy callbacks receive
// their inputs and outputs as simple_array<ElementType, n*MAX_PTR>
// (src/UMI.h:55-65).  N == 0 still reserves one slot so the type is complete.
constexpr DHFunc int SafeArrayLength(int i) { return i >= 1 ? i : 1; }
template <class T, size_t N>
struct simple_array {
	DHFunc T& operator[](size_t i) { return data_[i]; }
	DHFunc const T& operator[](size_t i) const { return data_[i]; }
	DHFunc simple_array() {}
	simple_array(const std::array<T, N>& a) { std::copy(a.begin(), a.end(), data_); }
	T data_[SafeArrayLength(N)];
};

template <class T> using NDTuple = std::array<T, DIM>;

// Nibble/bit extraction used by the PtrNum / Expand / ZeroStrideOpt template
// words: bits [n*b, (n+1)*b) of i.
constexpr DHFunc uint64_t Slice(const uint64_t i, int b, int nth) {
	return (i >> (nth * b)) & ((b >= 64) ? ~0ull : ((1ull << b) - 1ull));
}

// Accumulation index space A: total extent and the block used to order the
// accumulation (blocked row-major, see UMI_gpu.h).
struct AccumulationDim {
	int32_t total_size, block_size;
};

// Parallel index space P.  block_size / warp_size / warp_shuf are tiling hints;
// they are validated exactly as the reference validates them but do not change
// results.  warp_shuf == 0 (left out of a brace initialiser) means 1.
struct ParallelDim {
	int32_t total_size, block_size, warp_size, warp_shuf;
};

// One view dimension: index d of P (or A) moves physical dimension
// physical_dim_id by `stride` per step, starting at `ofs`.
struct ViewDim {
	int32_t physical_dim_id, ofs, stride;
};

// Physical array dimension.  Out-of-range coordinates are clamped to
// [0, size-1]; PAD additionally replaces the value by the pointer's padding
// value, WRAP keeps the clamped (edge-replicated) element.
struct PhysicalDim {
	enum BoundaryMode : int32_t { PAD, WRAP };
	int32_t size;
	BoundaryMode mode;
};

// Input memory descriptor (src/UMI.h:95-103).  shm_dims is accepted and
// ignored, as in the reference (the tile shape is derived from the views).
template <typename T>
struct UnrolledI {
	NDTuple<ViewDim> p_view_dims;
	NDTuple<ViewDim> a_view_dims;
	NDTuple<PhysicalDim> physical_dims;
	NDTuple<int32_t> shm_dims;
	const T* ptr[MAX_PTR];
	const T padding[MAX_PTR];
};

// Output memory descriptor (src/UMI.h:105-111).  Outputs are never clamped.
template <typename T>
struct UnrolledO {
	NDTuple<ViewDim> p_view_dims;
	NDTuple<ViewDim> a_view_dims;
	NDTuple<PhysicalDim> physical_dims;
	T* ptr[MAX_PTR];
};

// Strategy protocol (src/UMI.h:113-137).  A strategy is a struct with an
// ElementType, a UserConstantType and three callbacks.  Inputs/outputs of a
// stage are numbered memory-major: IMEM(i, j) is pointer j of the stage's
// i-th input memory.
#define STRATEGY_TYPEDEF_STUB(e, c)\
	typedef e ElementType;\
	typedef c UserConstantType;\
	template <int s> using A = UMI::simple_array<ElementType, s>;
#define STRATEGY_PRE_STUB(ni, no)\
	static constexpr int N_PRE_IN = ni;\
	static constexpr int N_PRE_OUT = no;\
	DHFunc void Pre(const UserConstantType &c, const A<N_PRE_IN*UMI::MAX_PTR> &in, A<N_PRE_OUT*UMI::MAX_PTR> &out)
#define STRATEGY_LOOP_STUB(ni, no)\
	static constexpr int N_LOOP_IN = ni;\
	static constexpr int N_LOOP_OUT = no;\
	DHFunc void Loop(const UserConstantType &c, const A<N_LOOP_IN*UMI::MAX_PTR> &in, A<N_LOOP_OUT*UMI::MAX_PTR> &out)
#define STRATEGY_POST_STUB(ni, no)\
	static constexpr int N_POST_IN = ni;\
	static constexpr int N_POST_OUT = no;\
	static constexpr int TOTAL_IN = N_PRE_IN + N_LOOP_IN + N_POST_IN;\
	static constexpr int TOTAL_OUT = N_PRE_OUT + N_LOOP_OUT + N_POST_OUT;\
	static constexpr int TOTAL = TOTAL_IN + TOTAL_OUT;\
	DHFunc void Post(const UserConstantType &c, const A<N_POST_IN*UMI::MAX_PTR> &in, A<N_POST_OUT*UMI::MAX_PTR> &out)
#define STRATEGY_POST_PRE_ STRATEGY_PRE_STUB(0, 0){}
#define STRATEGY_LOOP_STUB_ STRATEGY_LOOP_STUB(0, 0){}
#define STRATEGY_POST_STUB_ STRATEGY_POST_STUB(0, 0){}
#define IMEM(i, j) in[(i)*UMI::MAX_PTR+(j)]
#define OMEM(i, j) out[(i)*UMI::MAX_PTR+(j)]
#define DEFAULT_SHM {-1,-1,-1,-1}

}  // namespace UMI
