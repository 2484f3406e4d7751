// Blackwell (sm_103a) building blocks for the tensor-core kernels: mbarriers
// with bounded waits, TMA tensor loads, tcgen05 MMA / TMEM, shared-memory
// matrix descriptors.  All inline PTX, written from the PTX ISA.
//
// Every wait is bounded: after kWaitNs nanoseconds of %globaltimer the waiter
// records an error code (global word, when given) and raises the CTA's abort
// flag; all roles poll the abort flag and return, TMEM is freed on every exit
// path.  No wait can hang the GPU.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace umi_tc {

constexpr unsigned long long kWaitNs = 1000ull * 1000ull * 1000ull;  // 1 s
enum : int { kErrTimeoutFull = 1, kErrTimeoutEmpty = 2, kErrTimeoutAccum = 4, kErrTimeoutAccEmpty = 8 };

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
	uint32_t ok;
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(ok)
		: "r"(smem_u32(bar)), "r"(parity)
		: "memory");
	return ok != 0;
}

// The same test with a suspend-time hint: a thread whose phase is not yet
// complete sleeps until it completes or about hint_ns nanoseconds pass,
// instead of spinning on the issue slots of the warps that do the work.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
	uint32_t ok;
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(ok)
		: "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
		: "memory");
	return ok != 0;
}

// mbar_wait that sleeps between tests (for waits that can last a whole
// work unit, e.g. a producer that ran ahead of its consumers).
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, volatile int* abort, int* err, int code,
                                                uint32_t hint_ns = 20000, unsigned long long limit_ns = kWaitNs) {
	if (mbar_try_wait(bar, parity)) return true;
	const unsigned long long t0 = gtimer();
	while (!mbar_try_wait_sleep(bar, parity, hint_ns)) {
		if (*abort) return false;
		if (gtimer() - t0 > limit_ns) {
			*abort = 1;
			if (err) atomicOr(err, code);
			return false;
		}
	}
	return true;
}

// Waits for the phase with the given parity.  Returns false (after raising
// *abort and recording `code` in *err) when the limit passes or another role
// has aborted.  A phase that has already completed costs one test: the clock
// is read only when the first test fails.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort, int* err, int code,
                                          unsigned long long limit_ns = kWaitNs) {
	if (mbar_try_wait(bar, parity)) return true;
	const unsigned long long t0 = gtimer();
	while (!mbar_try_wait(bar, parity)) {
		if (*abort) return false;
		if (gtimer() - t0 > limit_ns) {
			*abort = 1;
			if (err) atomicOr(err, code);
			return false;
		}
	}
	return true;
}

// ---- TMA (tiled tensor loads into shared memory, completion on an mbarrier)
__device__ __forceinline__ void tma_prefetch(const CUtensorMap* m) {
	asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* m, uint64_t* bar, int x, int y) {
	asm volatile(
		"cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
			smem_u32(dst)),
		"l"(reinterpret_cast<uint64_t>(m)), "r"(smem_u32(bar)), "r"(x), "r"(y)
		: "memory");
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* m, uint64_t* bar, int x, int y, int z, int w) {
	asm volatile(
		"cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(
			smem_u32(dst)),
		"l"(reinterpret_cast<uint64_t>(m)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z), "r"(w)
		: "memory");
}

// TMA tile store from shared memory (bulk-group completion), and its waits.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* m, const void* src, int x, int y) {
	asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
	                 reinterpret_cast<uint64_t>(m)),
	             "r"(smem_u32(src)), "r"(x), "r"(y)
	             : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// at most one bulk group of this thread still reading its shared-memory source
__device__ __forceinline__ void bulk_wait_read_1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
// every bulk group of this thread complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// generic-proxy shared-memory writes visible to the async proxy (TMA)
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- tcgen05 / TMEM
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {  // whole warp
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
	             : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {  // whole warp
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {  // whole warp
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (bf16 or f16 inputs, fp32 accumulate).
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"setp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
		"l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
		: "memory");
}
// Arrive on `bar` once every tcgen05 operation issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
	             : "memory");
}

// Zero into 32 consecutive columns of the warp's 32 TMEM lanes, and the wait
// for this thread's TMEM stores.
__device__ __forceinline__ void tmem_zero32(uint32_t taddr) {
	asm volatile(
		"tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
		"{%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr),
		"r"(0u)
		: "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// 32 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
	uint32_t r[32];
	asm volatile(
		"tcgen05.ld.sync.aligned.32x32b.x32.b32 "
		"{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
		"%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
		: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
		  "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
		  "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
		  "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
		: "r"(taddr)
		: "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor for a K-major operand tile written by TMA
// with 128-byte swizzling: rows of 128 bytes, 8-row groups 1024 bytes apart
// (stride byte offset), leading byte offset unused, descriptor version 1
// (bits 46-47), layout SWIZZLE_128B (2, bits 61-63).  The tile base must be
// 1024-byte aligned; the K sub-block kk of 16 two-byte elements starts 32*kk
// bytes further (low address field + 2*kk).
__device__ __forceinline__ uint64_t desc_kmajor_sw128(uint32_t saddr) {
	uint64_t d = 0;
	d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
	d |= (uint64_t)1 << 16;             // leading byte offset (unused for this layout)
	d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
	d |= (uint64_t)1 << 46;             // descriptor version
	d |= (uint64_t)2 << 61;             // 128-byte swizzle
	return d;
}

// The same layout for an operand that starts `row` 128-byte rows into a
// 1024-byte-aligned swizzled tile (row need not be a multiple of 8): only
// the start address moves.  The 128-byte swizzle is a function of the
// absolute shared-memory address (bits 7-9 select the XOR of the 16-byte
// chunk), for the TMA that wrote the tile and for the MMA that reads it, so
// the matrix base offset field stays 0 (checked on the GPU against an FP64
// convolution for row = 1, 2).
__device__ __forceinline__ uint64_t desc_kmajor_sw128_rows(uint32_t tile_saddr, int row) {
	return desc_kmajor_sw128(tile_saddr + 128u * (uint32_t)row);
}

// The same for K-major tiles written by TMA with 64-byte swizzling: rows of
// 64 bytes (32 two-byte elements, one K slice of a 3x3 tap over 32
// channels), 8-row groups 512 bytes apart, layout SWIZZLE_64B (4, bits
// 61-63).  The tile base must be 512-byte aligned; the K sub-block kk of 16
// elements starts 32*kk bytes further.  An operand that starts `row` rows
// into such a tile moves only the start address (64 bytes per row), as for
// the 128-byte swizzle.
__device__ __forceinline__ uint64_t desc_kmajor_sw64(uint32_t saddr) {
	uint64_t d = 0;
	d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
	d |= (uint64_t)1 << 16;            // leading byte offset (unused for this layout)
	d |= (uint64_t)(512 >> 4) << 32;   // stride byte offset
	d |= (uint64_t)1 << 46;            // descriptor version
	d |= (uint64_t)4 << 61;            // 64-byte swizzle
	return d;
}

// Instruction descriptor, kind::f16: fp32 accumulator, A and B of one type
// (0 = f16, 1 = bf16), both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t ab_type, int m, int n) {
	return (1u << 4) | (ab_type << 7) | (ab_type << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

}  // namespace umi_tc
