// umma.cuh -- Blackwell (sm_100 family) tensor-core building blocks in inline
// PTX: tcgen05 MMA with its accumulator in tensor memory (TMEM), TMEM
// allocation and loads, shared-memory matrix descriptors, mbarriers with
// bounded waits, and the proxy / tcgen05 fences that order them.
//
// Operand layout used throughout (K-major, no swizzle): an R x K tile of
// 16-bit elements is stored as 8-row x 16-byte "core matrices",
//     byte(r, k) = (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2,
// with LBO = 128 (core matrices adjacent along K are contiguous) and
// SBO = 128 * K / 8 (the next 8 rows follow all K core matrices of the
// previous 8).  One kind::f16 MMA consumes K = 16, i.e. two core matrices
// along K; the next K step starts 2 * LBO = 256 bytes further.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace bm4dof {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading (K) and
// stride (M/N) byte offsets, all in 16-byte units; bits 46-47 hold the
// descriptor version 1; no swizzle (bits 61-63 = 0), base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
	return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
	       ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: F32 accumulator (bits 4-5 = 1),
// A and B F16 (bits 7-9, 10-12 = 0) or BF16 (= 1), both K-major (bits 15, 16
// = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, bool bf16)
{
	return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | ((uint32_t)(N >> 3) << 17) |
	       ((uint32_t)(M >> 4) << 24);
}

// ---- TMEM ----------------------------------------------------------------
// Allocation by one whole warp; the column base is written to *dst (shared).
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
	             "r"(ncols)
	             : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync()
{
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync()
{
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes made visible to the async proxy (the
// tensor cores read their operands through it).
__device__ __forceinline__ void fence_proxy_async()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate)
{
	asm volatile(
		"{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
		"l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
		: "memory");
}
// The mbarrier receives one arrival when every MMA this thread issued before
// has completed.
__device__ __forceinline__ void mma_commit(uint64_t *mbar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
		             smem_u32(mbar))
	             : "memory");
}

// 32 consecutive TMEM columns of this warp's 32 lanes (lane i of the warp
// reads TMEM lane (warp % 4) * 32 + i); taddr carries that lane base in
// bits 16-31.  Complete with tmem_wait_ld before reading v.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32])
{
	asm volatile(
		"tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
		"%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
		: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
		  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
		  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
		  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
		  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
		: "r"(taddr)
		: "memory");
}
__device__ __forceinline__ void tmem_wait_ld()
{
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- mbarriers -------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile(
		"{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(ok)
		: "r"(smem_u32(bar)), "r"(parity)
		: "memory");
	return ok != 0;
}
// Waits for the phase of the given parity to complete, at most `limit`
// polls (each try_wait also suspends for a hardware-chosen while); false when
// it gave up.  No wait in this library spins without a bound.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit)
{
	for (uint32_t i = 0; i < limit; i++)
		if (mbar_try_wait(bar, parity)) return true;
	return false;
}

}  // namespace umma
}  // namespace bm4dof
