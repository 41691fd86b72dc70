// tc05.cuh — the Blackwell (sm_100 family) primitives the guiding network's
// inference kernel is built from, as inline PTX:
//
//   tensor memory    tcgen05.alloc / relinquish_alloc_permit / dealloc, and
//                    tcgen05.ld (32 lanes x 32 bit, 16 columns per thread)
//   tensor core      tcgen05.mma.cta_group::1.kind::f16 (FP16 x FP16 -> FP32
//                    accumulators in tensor memory), issued by one thread, its
//                    completion signalled on an mbarrier by tcgen05.commit
//   bulk copy        cp.async.bulk global -> shared, completing on an mbarrier
//   mbarrier         init / arrive.expect_tx / bounded try_wait
//   descriptors      shared-memory matrix descriptor (no swizzle) and the
//                    instruction descriptor of kind::f16
//
// Operands are kept in shared memory in the canonical no-swizzle K-major
// layout: the matrix is cut into core matrices of 8 rows x 16 bytes (8 FP16),
// each stored as 128 contiguous bytes (row r at 16 r); the descriptor's
// leading byte offset is the distance between core matrices adjacent in K,
// the stride byte offset the distance between core matrices adjacent in the
// row (M or N) dimension.
#pragma once

#include <cstdint>

namespace are_core {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// 64-bit shared-memory matrix descriptor: start address, leading and stride
// byte offsets (all in 16-byte units), descriptor version 1 (bit 46), no
// swizzle (bits 61-63 = 0), base offset 0.
__device__ __forceinline__ uint64_t umma_sdesc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
	return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16) |
		((uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1),
// A and B FP16 (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_f16(uint32_t m, uint32_t n) {
	return (1u << 4) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
				 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[sdesc] x B[sdesc]^T, one instruction (K = 16)
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
	uint32_t accumulate) {
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"setp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
		"l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
		: "memory");
}
// the mbarrier receives one arrival when all tcgen05 work this thread issued is complete
__device__ __forceinline__ void umma_commit(uint64_t *mbar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
				 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 lanes x 32 bit, 16 consecutive columns: thread t of the warp gets lane
// (taddr lane + t), columns taddr .. taddr + 15
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
	asm volatile(
		"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
		: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
		"=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
		: "r"(taddr)
		: "memory");
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *mbar, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(bytes) : "memory");
}
// waits for the phase of parity `parity` to complete, at most `limit` polls
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t limit) {
	const uint32_t a = smem_addr(mbar);
	for (uint32_t i = 0; i < limit; ++i) {
		uint32_t done;
		asm volatile(
			"{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}\n"
			: "=r"(done)
			: "r"(a), "r"(parity)
			: "memory");
		if (done) return true;
	}
	return false;
}

// bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned)
// global -> shared, counted on the mbarrier's transaction count
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
					 smem_addr(dst)),
		"l"(src), "r"(bytes), "r"(smem_addr(mbar))
		: "memory");
}

__device__ __forceinline__ void named_bar(uint32_t id, uint32_t threads) {
	asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

}  // namespace are_core
