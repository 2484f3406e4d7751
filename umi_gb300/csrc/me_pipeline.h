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
	int32_t* list;   // nblk: blocks searched exhaustively (audited and fallback)
	int32_t* count;  // 2: [0] listed blocks, [1] fallback blocks
};

// mv (nblk, 3) <- refine +-refine_r around centers (nblk, 2); every
// audit_stride-th block (0: none) takes its +-full_r exhaustive result and
// adds (refined SAD, exhaustive SAD) to audit_sums[0..1] (if non-null); every
// other block whose refined SAD exceeds sad_threshold is searched
// exhaustively; n_fallback (if non-null) receives their count.  Audited and
// fallback blocks go through one exhaustive list search.  The centres must
// lie within +-(full_r - refine_r).
umi_status me_refine_audit_fallback(const uint8_t* cur, const uint8_t* ref, int h, int w, const int32_t* centers,
                                    int refine_r, int full_r, int32_t sad_threshold, int audit_stride, int32_t* mv,
                                    unsigned long long* audit_sums, int32_t* n_fallback, const MeFinishBuffers& b,
                                    cudaStream_t st);

}  // namespace umi
