// The stage shared by the motion proposals (learned_me.cu, coarse_me.cu):
// refine around the proposed centres, audit, exhaustive fallback.
#pragma once
#include "common.h"

extern "C" umi_status umi_full_me_u8(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b, int32_t r,
                                     const int32_t* centers, int32_t* mv, void* stream);
extern "C" umi_status umi_full_me_u8_list(const uint8_t* cur, const uint8_t* ref, int32_t h, int32_t w, int32_t b,
                                          int32_t r, const int32_t* centers, const int32_t* blocks,
                                          const int32_t* n_blocks, int32_t max_blocks, int32_t* mv, void* stream);

namespace umi {

// Device scratch of the shared stage, nblk = (h/16)(w/16) blocks.
struct MeFinishBuffers {
	int32_t* list;   // nblk: fallback blocks (and audited blocks when the audit is combined)
	int32_t* count;  // 4: [0] list length, [1] fallback blocks, [2] audited blocks (audit apart)
	int32_t* alist;  // nblk: audited blocks 0, stride, 2 stride, ...
	int32_t* amv;    // 3 nblk: exhaustive results, written at the audited blocks' rows only
};

// The audit's exhaustive search.  An audit of fewer blocks than SMs is
// `combined`: its blocks join the fallback blocks' list search after the
// refine (one round holds both).  A larger one is started before the
// proposal, so that it can run beside it: `forked` when it went to the
// calling thread's second stream on this device (joined by `done`), else
// in order on the caller's stream.
// Once forked, the caller's stream waits for `done` on every return path:
// me_refine_fallback_finish joins it before the merge, and the destructor
// joins it if an error returned earlier, so that no audit kernel can still be
// writing the caller's workspace after the entry point has returned.
struct MeAudit {
	bool active = false;
	bool combined = false;
	bool forked = false;
	cudaEvent_t done = nullptr;
	cudaStream_t st = nullptr;    // the caller's stream (joined to `done`)
	mutable bool joined = false;
	MeAudit() = default;
	MeAudit(const MeAudit&) = delete;
	MeAudit& operator=(const MeAudit&) = delete;
	void join() const {
		if (forked && !joined) {
			cudaStreamWaitEvent(st, done, 0);
			joined = true;
		}
	}
	~MeAudit() { join(); }
};

// Audit: every audit_stride-th block (0: none) is searched exhaustively in
// +-full_r (into b.amv when not combined).  Call before the proposal, on
// the proposal's stream.
umi_status me_audit_begin(const uint8_t* cur, const uint8_t* ref, int h, int w, int full_r, int audit_stride,
                          const MeFinishBuffers& b, cudaStream_t st, MeAudit* audit);

// mv (nblk, 3) <- refine +-refine_r around centers (nblk, 2); every other
// block than the audited ones whose refined SAD exceeds sad_threshold is
// searched exhaustively (n_fallback, if non-null, receives their count);
// then the audited blocks take their exhaustive result and add (refined
// SAD, exhaustive SAD) to audit_sums[0..1] (if non-null).  The centres must
// lie within +-(full_r - refine_r).
umi_status me_refine_fallback_finish(const uint8_t* cur, const uint8_t* ref, int h, int w, const int32_t* centers,
                                     int refine_r, int full_r, int32_t sad_threshold, int audit_stride, int32_t* mv,
                                     unsigned long long* audit_sums, int32_t* n_fallback, const MeFinishBuffers& b,
                                     const MeAudit& audit, cudaStream_t st);

}  // namespace umi
