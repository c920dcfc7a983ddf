// Fifth-generation tensor-core (tcgen05) building blocks for sm_100-family
// GPUs (sm_103a here), written as inline PTX: TMEM allocation, shared-memory
// matrix descriptors, BF16 MMA with FP32 accumulation in TMEM, commit to an
// mbarrier with a bounded wait, and TMEM -> register loads.
//
// Operand layout: "K-major, no swizzle" canonical layout.  A matrix of R rows
// and K columns (BF16) is stored as 8-row x 16-byte core matrices: element
// (r, k) lives at byte ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so the leading-dimension byte offset (next core matrix along K) is 128 and
// the stride byte offset (next 8-row group) is K / 8 * 128.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>

namespace gbrt {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__host__ __device__ constexpr uint32_t kmajor_offset(uint32_t r, uint32_t k, uint32_t K)
{
	return ((r >> 3) * (K >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// tcgen05 shared-memory matrix descriptor: start >> 4 [0,14), LBO >> 4
// [16,30), SBO >> 4 [32,46), fixed 0b001 at [46,49), no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
	uint64_t d = 0;
	d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
	d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
	d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
	d |= static_cast<uint64_t>(1u) << 46;
	return d;
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// One warp allocates ncols TMEM columns (power of two >= 32); the base
// address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_addr(slot)), "r"(ncols) : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}

// D (TMEM) [+]= A (smem) * B (smem)^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate)
{
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"setp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
		:: "r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// Arrive on the mbarrier once all previously issued MMAs of this thread complete.
__device__ __forceinline__ void mma_commit(uint64_t *mbar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(smem_addr(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(mbar)), "r"(count) : "memory");
}

// Bounded wait for the mbarrier phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t max_iter)
{
	const uint32_t a = smem_addr(mbar);
	for(uint32_t i = 0; i < max_iter; ++i)
	{
		uint32_t done;
		asm volatile(
			"{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.b32 %0, 1, 0, p;\n\t}\n"
			: "=r"(done) : "r"(a), "r"(parity) : "memory");
		if(done) return true;
	}
	return false;
}

// Make an mbarrier initialisation visible to the async proxy (tcgen05.commit).
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Make generic-proxy shared-memory writes visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
	uint32_t r[16];
	asm volatile(
		"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
		: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
		  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
		: "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
	for(int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void store_bf16_row(uint8_t *base, uint32_t row, uint32_t K, const float *v, uint32_t k0, uint32_t n)
{
	for(uint32_t k = 0; k < n; k += 2)
	{
		const __nv_bfloat162 p = __floats2bfloat162_rn(v[k], v[k + 1]);
		*reinterpret_cast<__nv_bfloat162 *>(base + kmajor_offset(row, k0 + k, K)) = p;
	}
}

} // namespace tc
} // namespace gbrt
