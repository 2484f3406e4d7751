// Schedule of the rolling-accumulator form of the motion-proposal layers
// (menet_rows_kernel in gemm_tc.cu), kept free of device code so that the
// host tests compile it too.
//
// A CTA walks runs of output rows (rows y, y + d, y + 2d, ... of one
// dilation class and one 128-pixel block).  In a run of `rows` output rows
// whose first is the CTA's row r0, strip m (input row m - 1 of the run,
// m = 0 .. rows + 1) is read by output rows m - dy for the filter rows dy in
// [lo, hi].  The sixteen 32-column accumulators take the CTA's rows in
// descending column order, row r at block roll_slot(r), so the rows
// m - lo, m - lo - 1, ... sit in adjacent blocks from roll_slot(r0 + m - lo)
// up, except where the ring wraps to block 0: the first c1 of the cnt blocks
// come before the wrap, the other cnt - c1 start at block 0.
#pragma once

#ifndef __CUDACC__
#define UMI_ROLL_HD inline
#else
#define UMI_ROLL_HD __host__ __device__ __forceinline__
#endif

namespace umi_roll {

constexpr int kSlots = 16;  // 32-column accumulators: all 512 TMEM columns

UMI_ROLL_HD int slot(int r) { return kSlots - 1 - (r & (kSlots - 1)); }

struct Step {
	int lo, hi;  // filter rows reading strip m
	int first;   // accumulator block of output row r0 + m - lo
	int c1;      // blocks before the ring wraps (cnt = hi - lo + 1 in all)
};

UMI_ROLL_HD Step step(int m, int rows, int r0) {
	Step s;
	s.lo = m - rows + 1 > 0 ? m - rows + 1 : 0;
	s.hi = m < 2 ? m : 2;
	s.first = slot(r0 + m - s.lo);
	const int cnt = s.hi - s.lo + 1;
	s.c1 = cnt < kSlots - s.first ? cnt : kSlots - s.first;
	return s;
}

}  // namespace umi_roll
