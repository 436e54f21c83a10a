// Inline-PTX wrappers for the Blackwell tensor-core path (sm_100a / sm_103a): tensor memory
// allocation, tcgen05.mma with shared-memory operand descriptors, tcgen05.commit to an mbarrier,
// tensor-memory loads, and cp.async tile copies.
//
// Operand layout used throughout: K-major, no swizzle.  A core matrix is 8 rows x 16 bytes (four
// 32-bit elements of one row stored contiguously, rows 16 bytes apart, 128 contiguous bytes); core
// matrices adjacent along K are `lbo` bytes apart (128, or 144 to spread a row's core matrices over
// the shared-memory banks), groups of 8 rows sbo = (kdim / 4) * lbo bytes apart.
#pragma once

#include <cstdint>

namespace qcs {
namespace tc {

// byte offset of element (row, k) of a K-major operand whose rows hold `kdim` 32-bit elements
__host__ __device__ inline uint32_t kmajor_offset(uint32_t row, uint32_t k, uint32_t kdim, uint32_t lbo = 128) {
	return (row >> 3) * (kdim / 4) * lbo + (k >> 2) * lbo + (row & 7) * 16 + (k & 3) * 4;
}

// shared-memory matrix descriptor (no swizzle, version 1 in bits 46-48)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
	return static_cast<uint64_t>((saddr >> 4) & 0x3FFF) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16) |
	       (static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32) | (1ULL << 46);
}

// instruction descriptor: D F32, A and B TF32, both K-major, N and M as given
__host__ __device__ constexpr uint32_t idesc_tf32(uint32_t m, uint32_t n) {
	return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// x rounded to TF32 (10 mantissa bits), to nearest with ties away from zero: half a TF32 unit added to the
// magnitude bits, the 13 low bits cleared.  For finite x of magnitude below 2^128 - 2^116 the same value as
// cvt.rna.tf32.f32 (tests/tf32_rounding_check.cu compares the two on every such input), in two integer
// instructions instead of a conversion, whose lower throughput bounded the tensor-core operand gather.
__device__ __forceinline__ float tf32_rna(float x) { return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u); }

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// whole warp: allocate `ncols` tensor-memory columns, address written to *slot
template <uint32_t NCOLS> __device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "n"(NCOLS));
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
template <uint32_t NCOLS> __device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "n"(NCOLS));
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the async proxy (tensor cores, bulk copies)
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// one thread: D (+)= A * B, kind::tf32
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
	asm volatile(
	    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
	    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
	    : "memory");
}
// one thread: D (+)= A * B, kind::tf32, with A (M rows = tensor-memory lanes, K = columns) in tensor memory
__device__ __forceinline__ void mma_tf32_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
	asm volatile(
	    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d_tmem),
	    "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
	    : "memory");
}
// one thread: the mbarrier gets one arrival when every MMA this thread issued so far has completed
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar)) : "memory");
}

// 32 lanes x 16 columns of 32-bit values: thread i of the warp gets lane (base lane + i), columns c..c+15
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
	uint32_t r[16];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
	      "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}
// two loads of 32 lanes x 16 columns, one wait for both
__device__ __forceinline__ void tmem_ld16x2(uint32_t ta, uint32_t tb, float (&va)[16], float (&vb)[16]) {
	uint32_t r[16], q[16];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
	      "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(ta));
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
	    : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]), "=r"(q[4]), "=r"(q[5]), "=r"(q[6]), "=r"(q[7]), "=r"(q[8]), "=r"(q[9]),
	      "=r"(q[10]), "=r"(q[11]), "=r"(q[12]), "=r"(q[13]), "=r"(q[14]), "=r"(q[15])
	    : "r"(tb));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int j = 0; j < 16; ++j) {
		va[j] = __uint_as_float(r[j]);
		vb[j] = __uint_as_float(q[j]);
	}
}

// 32 lanes x 16 columns of 32-bit values: thread i of the warp writes lane (base lane + i), columns c..c+15;
// completed (for this thread) by tmem_wait_st.  It touches no generic memory, so shared-memory loads may be
// scheduled across it; volatile keeps it in order with the other tensor-memory instructions.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
	asm volatile(
	    "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
	    "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
	    "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
	    "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
	    "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15])));
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count));
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// bounded wait for the phase with the given parity to complete; false when the bound ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_tries) {
	const uint32_t a = smem_addr(mbar);
	for (uint32_t it = 0; it < max_tries; ++it) {
		uint32_t done;
		asm volatile(
		    "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
		    : "=r"(done)
		    : "r"(a), "r"(parity)
		    : "memory");
		if (done) return true;
	}
	return false;
}

// 16-byte asynchronous copy global -> shared, completed by cp_async_wait_all (per thread)
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
	asm volatile("cp.async.commit_group;" ::: "memory");
	asm volatile("cp.async.wait_group 0;" ::: "memory");
}

}  // namespace tc
}  // namespace qcs
