// Inline-PTX helpers for the 5th-generation tensor cores (tcgen05) and
// mbarriers, shared by the learned frame's kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sphgb {
namespace tc {

constexpr uint32_t kWaitPolls = 1u << 22;
constexpr uint64_t kWaitNs = 200000000ull;  // 0.2 s

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, canonical K-major layout without swizzle:
// start address, leading byte offset (between K-adjacent 8-row x 16-byte
// core matrices), stride byte offset (between 8-row groups), version 1.
__device__ __forceinline__ uint64_t desc_noswizzle(uint32_t addr, uint32_t lbo, uint32_t sbo) {
	uint64_t d = 0;
	d |= (uint64_t)((addr >> 4) & 0x3fff);
	d |= (uint64_t)((lbo >> 4) & 0x3fff) << 16;
	d |= (uint64_t)((sbo >> 4) & 0x3fff) << 32;
	d |= (uint64_t)1 << 46;
	return d;
}

// Instruction descriptor of kind::tf32: FP32 accumulator (bits 4-5 = 1),
// A and B TF32 (bits 7-9 and 10-12 = 2), both K-major, N/8 at bit 17,
// M/16 at bit 24.
__device__ __forceinline__ uint32_t idesc_tf32(int m, int n) {
	return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Bounded wait for the phase with the given parity: try_wait (which may
// suspend the thread for a while in hardware), after 8 tries a 64 ns sleep
// between tries; gives up after kWaitNs nanoseconds or kWaitPolls tries.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity) {
	const uint32_t addr = smem_u32(bar);
	uint64_t start = 0;
	for (uint32_t i = 0; i < kWaitPolls; ++i) {
		uint32_t ok;
		asm volatile(
		    "{\n\t.reg .pred p;\n\t"
		    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		    "selp.u32 %0, 1, 0, p;\n\t}"
		    : "=r"(ok)
		    : "r"(addr), "r"(parity)
		    : "memory");
		if (ok) return true;
		if (i == 8) start = globaltimer_ns();
		if (i >= 8) {
			__nanosleep(64);
			if ((i & 255) == 0 && globaltimer_ns() - start > kWaitNs) return false;
		}
	}
	return false;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "setp.ne.u32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
	    "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)acc)
	    : "memory");
}

__device__ __forceinline__ void commit(unsigned long long *bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
	             : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Whole-warp allocation of `cols` tensor-memory columns (a power of two,
// >= 32); the base address is written to shared memory.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols) {
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
	             : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t tmem, uint32_t cols) {
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols) : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns: thread t of the warp receives
// lane (base lane + t), columns [col, col + 32).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
	    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
	    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
	      "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
	      "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
	      "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
	    : "r"(taddr)
	    : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Round to TF32 (10 explicit mantissa bits), to nearest with ties away from
// zero; the low 13 bits of the result are zero.
__device__ __forceinline__ float to_tf32(float x) {
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return __uint_as_float(r);
}

}  // namespace tc
}  // namespace sphgb
