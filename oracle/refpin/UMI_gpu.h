// Oracle pinning shim: stands in for the reference's GPU header so that the
// reference's own example programs (main/*.cu of johnjohnlin/UMI) can be
// compiled as plain C++ and run on the CPU with every UMI::Execute call served
// by the oracle interpreter (../umi_interp.hpp).
//
// TEST INFRASTRUCTURE ONLY.  Each example program ends with its own scalar
// CPU loop and asserts equality with what Execute produced; an example that
// exits 0 therefore certifies the oracle against the reference's checks on
// the reference's own inputs and sizes.
//
// When UMI_REFPIN_DUMP names a directory, every output memory of every call is
// written there as raw little-endian bytes (<app>.<call>.out<i>.bin) so that
// golden vectors can be derived from them.
#pragma once
#include "umi/UMI.h"
#include "../umi_interp.hpp"
#include <cstdlib>
#include <string>

namespace UMI {

namespace refpin_detail {
inline int& CallCounter() { static int n = 0; return n; }
template <class T>
inline void Dump(const UnrolledO<T>& o, int call, int i, int j) {
	const char* dir = std::getenv("UMI_REFPIN_DUMP");
	const char* app = std::getenv("UMI_REFPIN_APP");
	if (!dir || !o.ptr[j]) return;
	// Leading physical sizes left at 0 by a brace initialiser address like 1.
	size_t n = 1;
	for (int k = 0; k < DIM; ++k) n *= (size_t)std::max(o.physical_dims[k].size, 1);
	std::string path = std::string(dir) + "/" + (app ? app : "app") + "." + std::to_string(call) +
	                   ".out" + std::to_string(i) + (j ? "_" + std::to_string(j) : "") + ".bin";
	FILE* f = std::fopen(path.c_str(), "wb");
	if (!f) return;
	std::fwrite(o.ptr[j], sizeof(T), n, f);
	std::fclose(f);
}
}  // namespace refpin_detail

template <
	class Umi,
	uint64_t PtrNum = 0x1111111111111111ull,
	uint64_t Expand = 0x1111,
	uint64_t ZeroStrideOpt = 0,
	class EType = typename std::remove_cv<typename Umi::ElementType>::type,
	class CType = typename std::remove_cv<typename Umi::UserConstantType>::type>
void Execute(
	const NDTuple<ParallelDim>& p_dims,
	const NDTuple<AccumulationDim>& a_dims,
	const std::array<UnrolledI<EType>, Umi::TOTAL_IN>& imems,
	const std::array<UnrolledO<EType>, Umi::TOTAL_OUT>& omems,
	const CType& c = CType()) {
	const int rc = umi_oracle::Interpret<Umi, PtrNum, Expand, ZeroStrideOpt, EType, CType>(
		p_dims, a_dims, imems, omems, c);
	const int call = refpin_detail::CallCounter()++;
	if (rc != 0) {
		std::fprintf(stderr, "oracle: descriptor rejected (call %d)\n", call);
		std::exit(3);
	}
	for (int i = 0; i < Umi::TOTAL_OUT; ++i)
		for (int j = 0; j < (int)Slice(PtrNum, 4, Umi::TOTAL_IN + i); ++j)
			refpin_detail::Dump(omems[i], call, i, j);
}

}  // namespace UMI
