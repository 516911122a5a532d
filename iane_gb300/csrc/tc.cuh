// tcgen05 (5th-generation tensor core) helpers for sm_103a: TMEM allocation, shared-memory
// matrix descriptors, the kind::f16 MMA with FP32 accumulation, commit to an mbarrier and
// TMEM loads. Inline PTX written from the public PTX ISA description of tcgen05.
#pragma once

#include "common.cuh"

namespace iane_gb {
namespace tc {

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout: the operand is
// tiled into core matrices of 8 rows x 16 bytes (8 bf16) stored as 128 contiguous bytes;
// `lbo` is the byte distance between core matrices adjacent along K, `sbo` along M (or N).
__device__ __forceinline__ uint64_t smem_desc(uint32_t smem_byte_addr, uint32_t lbo, uint32_t sbo)
{
	uint64_t d = 0;
	d |= static_cast<uint64_t>((smem_byte_addr >> 4) & 0x3FFFu);
	d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
	d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
	d |= 1ull << 46; // descriptor version for sm_100-family tcgen05
	// base offset 0, absolute LBO mode 0, layout type 0 (no swizzle)
	return d;
}

// Instruction descriptor for kind::f16: D = F32, A = B = BF16, both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int m, int n)
{
	return (1u << 4)                                    // D format F32
		| (1u << 7)                                     // A format BF16
		| (1u << 10)                                    // B format BF16
		| (static_cast<uint32_t>(n >> 3) << 17)         // N / 8
		| (static_cast<uint32_t>(m >> 4) << 24);        // M / 16
}

// Allocate `cols` TMEM columns (power of two >= 32) for this CTA; one full warp executes
// it and the base address lands in *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t cols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(cols)
		: "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem], issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
	bool accumulate)
{
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"setp.ne.b32 p, %4, 0;\n\t"
		"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
		::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
		: "memory");
}

// Arrive once on `bar` when every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint64_t* bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
		: "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Each lane of the warp reads 16 consecutive 32-bit columns of its own TMEM lane.
__device__ __forceinline__ void ld_32x32b_x8(uint32_t taddr, float (&v)[8])
{
	uint32_t r[8];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
		: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
		: "r"(taddr)
		: "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void ld_32x32b_x16(uint32_t taddr, float (&v)[16])
{
	uint32_t r[16];
	asm volatile(
		"tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
		: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
		  "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
		: "r"(taddr)
		: "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 1-D bulk copy global -> shared completing on `bar` (16-byte aligned, size multiple of 16).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
		::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
		: "memory");
}

}  // namespace tc
}  // namespace iane_gb
