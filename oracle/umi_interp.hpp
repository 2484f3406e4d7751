// CPU oracle: scalar interpreter of the UMI operator semantics.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU path: only
// tests, the smoke entry and the bench's CPU-baseline leg may use it.  The
// product path never includes it.
//
// It restates, one output point at a time, what the reference kernel computes
// (johnjohnlin/UMI src/UMI_gpu.h:189-358 with the tables of src/UMI.cpp:97-226):
//
//   * input address (src/UMI_gpu.h:450-522, FillShm :33-83): per physical
//     dimension k, coord_k = sum of the p-view and a-view offsets mapped to k
//     + sum_d p[d]*pstride[d] (p-view dims mapped to k)
//     + sum_d a[d]*astride[d] (a-view dims mapped to k, Loop-stage inputs only);
//   * boundary (Int4::ClampedSum, src/UMI.h:205-218): every coord is clamped to
//     [0, size-1]; if a clamped coord belongs to a PAD dimension the value is
//     the pointer's padding value, otherwise the clamped element is read;
//   * outputs (src/UMI_gpu.h:523-552, :170-185): same affine map without
//     clamping, row-major over physical sizes, written only when p < P;
//   * stage order per point (src/UMI_gpu.h:272-357): Pre, then Loop over A in
//     blocked row-major order (accumulation blocks row-major, steps row-major
//     inside a block, steps with a >= A skipped), then Post;
//   * descriptor validation (src/UMI.cpp:39-66): product of warp sizes == 32,
//     warp_shuf a power of two, block divisible by warp*shuf.  The reference
//     aborts; the oracle returns a non-zero code.  warp_shuf == 0 is taken as 1
//     (see the GPU planner, which does the same).
#pragma once
#include "umi/UMI.h"
#include <cstring>

namespace umi_oracle {

using namespace UMI;

enum { ORACLE_OK = 0, ORACLE_BAD_DESC = 1 };

struct MemMap {
	int64_t base[DIM];
	int64_t pstr[DIM][DIM];  // [physical k][p dim d]
	int64_t astr[DIM][DIM];  // [physical k][a dim d]
	int64_t size[DIM];
	bool pad[DIM];
};

inline MemMap BuildMap(const NDTuple<ViewDim>& pv, const NDTuple<ViewDim>& av,
                       const NDTuple<PhysicalDim>& phys, bool use_a_index) {
	MemMap m;
	std::memset(&m, 0, sizeof(m));
	for (int d = 0; d < DIM; ++d) {
		m.base[pv[d].physical_dim_id] += pv[d].ofs;
		m.base[av[d].physical_dim_id] += av[d].ofs;
		m.pstr[pv[d].physical_dim_id][d] += pv[d].stride;
		if (use_a_index) m.astr[av[d].physical_dim_id][d] += av[d].stride;
	}
	for (int k = 0; k < DIM; ++k) {
		m.size[k] = phys[k].size;
		m.pad[k] = phys[k].mode == PhysicalDim::PAD;
	}
	return m;
}

inline void Coords(const MemMap& m, const int64_t* p, const int64_t* a, int64_t* c) {
	for (int k = 0; k < DIM; ++k) {
		int64_t v = m.base[k];
		for (int d = 0; d < DIM; ++d) v += m.pstr[k][d] * p[d] + m.astr[k][d] * a[d];
		c[k] = v;
	}
}

// Input read with clamp / pad.
template <class T>
inline T Load(const MemMap& m, const T* ptr, T padv, const int64_t* p, const int64_t* a) {
	int64_t c[DIM];
	Coords(m, p, a, c);
	bool outside = false;
	int64_t addr = 0;
	for (int k = 0; k < DIM; ++k) {
		int64_t v = c[k] < 0 ? 0 : (c[k] > m.size[k] - 1 ? m.size[k] - 1 : c[k]);
		outside |= (v != c[k]) && m.pad[k];
		addr = addr * m.size[k] + v;
	}
	return outside ? padv : ptr[addr];
}

// Output address: row-major, no clamp.
inline int64_t OutAddr(const MemMap& m, const int64_t* p, const int64_t* a) {
	int64_t c[DIM];
	Coords(m, p, a, c);
	int64_t addr = 0;
	for (int k = 0; k < DIM; ++k) addr = addr * m.size[k] + c[k];
	return addr;
}

inline int ValidatePDims(const NDTuple<ParallelDim>& p) {
	int64_t warp = 1;
	for (int d = 0; d < DIM; ++d) {
		const int32_t shuf = p[d].warp_shuf == 0 ? 1 : p[d].warp_shuf;
		if (!IsPowOf2(shuf)) return ORACLE_BAD_DESC;
		if (p[d].warp_size <= 0 || p[d].block_size <= 0) return ORACLE_BAD_DESC;
		if (p[d].block_size % (p[d].warp_size * shuf) != 0) return ORACLE_BAD_DESC;
		warp *= p[d].warp_size;
	}
	return warp == WARP_SIZE ? ORACLE_OK : ORACLE_BAD_DESC;
}

// Advance a row-major odometer; returns false after the last element.
inline bool Next(int64_t* idx, const int64_t* ext) {
	for (int d = DIM - 1; d >= 0; --d) {
		if (++idx[d] < ext[d]) return true;
		idx[d] = 0;
	}
	return false;
}

template <
	class Umi,
	uint64_t PtrNum = 0x1111111111111111ull,
	uint64_t Expand = 0x1111,
	uint64_t ZeroStrideOpt = 0,
	class EType = typename std::remove_cv<typename Umi::ElementType>::type,
	class CType = typename std::remove_cv<typename Umi::UserConstantType>::type>
int Interpret(
	const NDTuple<ParallelDim>& pdims,
	const NDTuple<AccumulationDim>& adims,
	const std::array<UnrolledI<EType>, Umi::TOTAL_IN>& imems,
	const std::array<UnrolledO<EType>, Umi::TOTAL_OUT>& omems,
	const CType& uc = CType()) {
	if (ValidatePDims(pdims) != ORACLE_OK) return ORACLE_BAD_DESC;
	for (int d = 0; d < DIM; ++d)
		if (adims[d].block_size <= 0) return ORACLE_BAD_DESC;
	constexpr int NI = Umi::TOTAL_IN, NO = Umi::TOTAL_OUT;
	constexpr int PRE_I = 0, LOOP_I = Umi::N_PRE_IN, POST_I = Umi::N_PRE_IN + Umi::N_LOOP_IN;
	constexpr int PRE_O = 0, LOOP_O = Umi::N_PRE_OUT, POST_O = Umi::N_PRE_OUT + Umi::N_LOOP_OUT;
	MemMap im[SafeArrayLength(NI)], om[SafeArrayLength(NO)];
	for (int i = 0; i < NI; ++i)
		im[i] = BuildMap(imems[i].p_view_dims, imems[i].a_view_dims, imems[i].physical_dims,
		                 LOOP_I <= i && i < POST_I);
	for (int i = 0; i < NO; ++i)
		om[i] = BuildMap(omems[i].p_view_dims, omems[i].a_view_dims, omems[i].physical_dims,
		                 LOOP_O <= i && i < POST_O);
	int64_t P[DIM], At[DIM], Ab[DIM], Ag[DIM];
	for (int d = 0; d < DIM; ++d) {
		P[d] = pdims[d].total_size;
		At[d] = adims[d].total_size;
		Ab[d] = adims[d].block_size;
		Ag[d] = At[d] <= 0 ? 0 : CeilDiv<int64_t>(At[d], Ab[d]);
		if (P[d] <= 0) return ORACLE_OK;  // empty parallel space: nothing to do
	}
	const int64_t zero[DIM] = {0, 0, 0, 0};
	auto n_ptr = [](int mem) { return (int)Slice(PtrNum, 4, mem); };

	// One stage call: gather inputs [ofs_i, ofs_i+ni) at (p, a), run the
	// callback, scatter outputs [ofs_o, ofs_o+no).
	auto stage = [&](Umi& u, int st, int ofs_i, int ni, int ofs_o, int no, const int64_t* p, const int64_t* a) {
		simple_array<EType, 16 * MAX_PTR> inbuf;
		simple_array<EType, 16 * MAX_PTR> outbuf;
		for (int k = 0; k < 16 * MAX_PTR; ++k) inbuf[k] = outbuf[k] = EType();
		for (int i = 0; i < ni; ++i)
			for (int j = 0; j < n_ptr(ofs_i + i); ++j)
				inbuf[i * MAX_PTR + j] = Load<EType>(im[ofs_i + i], imems[ofs_i + i].ptr[j],
				                                     imems[ofs_i + i].padding[j], p, a);
		// The callbacks take simple_array<E, n*MAX_PTR> of the exact size; copy
		// through correctly sized arrays.
		if (st == 0) {
			simple_array<EType, Umi::N_PRE_IN * MAX_PTR> in;
			simple_array<EType, Umi::N_PRE_OUT * MAX_PTR> out;
			for (int k = 0; k < Umi::N_PRE_IN * MAX_PTR; ++k) in[k] = inbuf[k];
			u.Pre(uc, in, out);
			for (int k = 0; k < Umi::N_PRE_OUT * MAX_PTR; ++k) outbuf[k] = out[k];
		} else if (st == 1) {
			simple_array<EType, Umi::N_LOOP_IN * MAX_PTR> in;
			simple_array<EType, Umi::N_LOOP_OUT * MAX_PTR> out;
			for (int k = 0; k < Umi::N_LOOP_IN * MAX_PTR; ++k) in[k] = inbuf[k];
			u.Loop(uc, in, out);
			for (int k = 0; k < Umi::N_LOOP_OUT * MAX_PTR; ++k) outbuf[k] = out[k];
		} else {
			simple_array<EType, Umi::N_POST_IN * MAX_PTR> in;
			simple_array<EType, Umi::N_POST_OUT * MAX_PTR> out;
			for (int k = 0; k < Umi::N_POST_IN * MAX_PTR; ++k) in[k] = inbuf[k];
			u.Post(uc, in, out);
			for (int k = 0; k < Umi::N_POST_OUT * MAX_PTR; ++k) outbuf[k] = out[k];
		}
		for (int i = 0; i < no; ++i)
			for (int j = 0; j < n_ptr(NI + ofs_o + i); ++j)
				omems[ofs_o + i].ptr[j][OutAddr(om[ofs_o + i], p, a)] = outbuf[i * MAX_PTR + j];
	};
	static_assert(Umi::TOTAL_IN <= 16 && Umi::TOTAL_OUT <= 16, "at most 16 memories per stage");

	int64_t p[DIM] = {0, 0, 0, 0};
	do {
		Umi u;
		stage(u, 0, PRE_I, Umi::N_PRE_IN, PRE_O, Umi::N_PRE_OUT, p, zero);
		bool any_a = true;
		for (int d = 0; d < DIM; ++d) any_a &= Ag[d] > 0;
		if (any_a) {
			int64_t ab[DIM] = {0, 0, 0, 0};
			do {
				int64_t as[DIM] = {0, 0, 0, 0};
				do {
					int64_t a[DIM];
					bool ok = true;
					for (int d = 0; d < DIM; ++d) {
						a[d] = ab[d] * Ab[d] + as[d];
						ok &= a[d] < At[d];
					}
					if (ok) stage(u, 1, LOOP_I, Umi::N_LOOP_IN, LOOP_O, Umi::N_LOOP_OUT, p, a);
				} while (Next(as, Ab));
			} while (Next(ab, Ag));
		}
		stage(u, 2, POST_I, Umi::N_POST_IN, POST_O, Umi::N_POST_OUT, p, zero);
	} while (Next(p, P));
	return ORACLE_OK;
}

}  // namespace umi_oracle
