"""Host check of the rolling-accumulator schedule of the motion-proposal
layers (umi_gb300/csrc/menet_roll.h, the code the layer kernel runs): for
every way a CTA's rows can split into runs, each output row receives the
three filter rows exactly once, in its own accumulator, after its first
strip; it completes at the strip that commits it; and an accumulator is
started again only after the row that held it completed (otherwise the
MMA thread would wait for an epilogue that waits for it)."""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "umi_gb300", "csrc")

CHECKER = r"""
#include "menet_roll.h"
#include <cstdio>
#include <cstdint>
#include <vector>
using namespace umi_roll;

static int fail(const char* what, const std::vector<int>& runs) {
	std::printf("FAIL %s; runs:", what);
	for (int r : runs) std::printf(" %d", r);
	std::printf("\n");
	return 1;
}

// One CTA's walk over its runs, as the MMA thread issues it.
static int check(const std::vector<int>& runs) {
	int total = 0;
	for (int n : runs) total += n;
	std::vector<int> got(total, 0), first_at(total, -1), done_at(total, -1);
	int r0 = 0, q = 0;
	for (int rows : runs) {
		for (int m = 0; m < rows + 2; ++m, ++q) {
			const Step s = step(m, rows, r0);
			const int cnt = s.hi - s.lo + 1;
			if (cnt < 1 || cnt > 3 || s.c1 < 1 || s.c1 > cnt) return fail("block count", runs);
			if (s.first < 0 || s.first >= kSlots) return fail("first block", runs);
			if (s.lo == 0) {  // output row r0 + m starts here
				if (m >= rows || first_at[r0 + m] != -1) return fail("start", runs);
				first_at[r0 + m] = q;
			}
			for (int j = 0; j < cnt; ++j) {
				const int block = j < s.c1 ? s.first + j : j - s.c1;  // D block of this part
				const int dy = s.lo + j;                                // B block: filter row
				const int r = r0 + m - dy;                              // output row fed
				if (r < r0 || r >= r0 + rows) return fail("row outside the run", runs);
				if (block < 0 || block >= kSlots || block != slot(r)) return fail("accumulator", runs);
				if (got[r] >> dy & 1) return fail("filter row twice", runs);
				if (first_at[r] < 0) return fail("fed before its first strip", runs);
				got[r] |= 1 << dy;
			}
			if (m >= 2) {  // the commit of row r0 + m - 2
				const int r = r0 + m - 2;
				if (got[r] != 7) return fail("committed before all nine taps", runs);
				done_at[r] = q;
			}
		}
		r0 += rows;
	}
	for (int r = 0; r < total; ++r)
		if (got[r] != 7 || done_at[r] < 0) return fail("row incomplete", runs);
	for (int r = kSlots; r < total; ++r)
		if (first_at[r] <= done_at[r - kSlots]) return fail("accumulator reused before its row completed", runs);
	return 0;
}

int main() {
	long cases = 0;
	// every composition of 1 .. 14 rows into runs
	for (int n = 1; n <= 14; ++n)
		for (uint32_t cut = 0; cut < (1u << (n - 1)); ++cut) {
			std::vector<int> runs;
			int len = 1;
			for (int i = 0; i < n - 1; ++i) {
				if (cut >> i & 1) { runs.push_back(len); len = 1; } else ++len;
			}
			runs.push_back(len);
			if (check(runs)) return 1;
			++cases;
		}
	// longer CTAs: runs of 1 .. 70 rows (a 4K layer has runs of up to 68)
	uint64_t x = 88172645463325252ull;
	for (int t = 0; t < 20000; ++t) {
		std::vector<int> runs;
		int total = 0;
		const int want = 15 + (int)(t % 120);
		while (total < want) {
			x ^= x << 13; x ^= x >> 7; x ^= x << 17;
			const int len = 1 + (int)(x % 70);
			runs.push_back(len);
			total += len;
		}
		if (check(runs)) return 1;
		++cases;
	}
	std::printf("%ld cases ok\n", cases);
	return 0;
}
"""


def test_menet_roll_schedule(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "roll.cpp"
    src.write_text(CHECKER)
    exe = tmp_path / "roll"
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip().endswith("cases ok"), out.stdout + out.stderr
