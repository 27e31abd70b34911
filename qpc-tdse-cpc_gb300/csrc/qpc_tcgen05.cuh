// Inline-PTX building blocks of the tcgen05 kernels (sm_103a): shared-memory matrix descriptors,
// bounded mbarrier waits, the bf16 x bf16 -> fp32 MMA with its accumulator in tensor memory, the MMA
// completion commit and tensor-memory loads.  Used by the slice-product GEMM (qpc_ozaki.cu) and the
// length-gauge l-space transform (qpc_ltrans.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace qpc {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// instruction descriptor, kind::f16: D fp32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1), both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// shared-memory matrix descriptor of a 128-byte-swizzled K-major tile at byte address saddr: start
// address >> 4 (bits 0-13), leading byte offset 16 (encoded 1, unused for this layout), stride byte
// offset 1024 between 8-row groups (bits 32-45), descriptor version 1 (bits 46-47), swizzle mode
// 128B (2 at bits 61-63).  Row r of the tile holds 64 bf16 (128 bytes) at r * 128, its 16-byte chunk c
// stored at chunk c ^ (r & 7); the tile starts at a 1024-byte boundary.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
	return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
		((uint64_t)2 << 61);
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}

// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity)
{
	for (long it = 0; it < (1L << 22); ++it) {
		uint32_t ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
			: "=r"(ok) : "r"(a), "r"(parity) : "memory");
		if (ok) return true;
	}
	return false;
}

// D (tensor memory) = A B^T (+ D when accumulate != 0), A and B from shared-memory descriptors
__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
		::"r"(tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// the mbarrier's phase completes when every tcgen05 operation this thread has issued so far is done
__device__ __forceinline__ void commit(uint32_t mbar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar) : "memory");
}

// 32 consecutive fp32 columns of this thread's tensor-memory lane (waits for the load)
__device__ __forceinline__ void ld32(uint32_t taddr, uint32_t (&v)[32])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
		"%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
		: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
		  "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
		  "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]),
		  "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
		: "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// 8 consecutive fp32 columns of this thread's lane; the caller waits (wait_ld) before using them
__device__ __forceinline__ void ld8(uint32_t taddr, uint32_t (&v)[8])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
		: "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
		: "r"(taddr));
}

__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// generic-proxy shared-memory writes of this thread -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

} // namespace tc
} // namespace qpc
