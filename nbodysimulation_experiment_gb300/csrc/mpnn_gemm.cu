// BF16 tensor-core GEMM for the message-passing network (5th-generation
// tensor cores: tcgen05.mma with the accumulator in tensor memory).
//
//   C[M x N] (+)= A[M x K] * B[N x K]^T      A, B bf16 row-major (K-major),
//                                            FP32 accumulation in TMEM.
//
// One CTA of four warps computes a 128-row tile of C for all N <= 256
// columns: operands are staged in shared memory in the canonical no-swizzle
// K-major layout (8-row x 16-byte core matrices), thread 0 issues
// tcgen05.mma (M=128, N, K=16) per 16-wide K step and commits to an
// mbarrier; two stages let the next K chunk load while the tensor core works
// on the current one.  The epilogue reads the accumulator with tcgen05.ld
// (warp w owns TMEM lanes 32w..32w+31, one row per thread) and applies the
// requested bias, row-scaled bias and ReLU before storing FP32 and/or BF16
// (row-major or transposed).  Split-K over gridDim.y accumulates FP32 with
// atomics.  Every mbarrier wait is bounded; a timeout sets an error flag and
// the CTA still frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "mpnn_internal.cuh"

namespace sphgb {

namespace {

constexpr int kGemmThreads = 128;
constexpr int kTileM = 128;
constexpr int kChunkK = 64;                  // K per stage
constexpr int kCoreBytes = 128;              // 8 rows x 16 bytes
constexpr int kLbo = kCoreBytes;             // K-adjacent core matrices
constexpr int kSbo = kCoreBytes * (kChunkK / 8);  // 8-row groups: 1 KiB
constexpr int kStageABytes = kTileM * kChunkK * 2;
constexpr int kMaxN = 256;
constexpr int kStageBBytes = kMaxN * kChunkK * 2;
constexpr uint32_t kWaitPolls = 1u << 22;

struct __align__(1024) GemmSmem {
	unsigned char a[2][kStageABytes];
	unsigned char b[2][kStageBBytes];
	unsigned long long bar[2];  // MMA-done barrier per stage
	unsigned long long done;    // all MMAs done
	uint32_t tmem;
	int fail;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
	return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets of core matrices, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
	uint64_t d = 0;
	d |= (uint64_t)((addr >> 4) & 0x3fff);
	d |= (uint64_t)((kLbo >> 4) & 0x3fff) << 16;
	d |= (uint64_t)((kSbo >> 4) & 0x3fff) << 32;
	d |= (uint64_t)1 << 46;
	return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M.
__device__ __forceinline__ uint32_t instr_desc(int n) {
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Bounded wait for the phase with the given parity to complete: a
// non-blocking test with a short sleep between polls, at most 2^22 polls
// (well under a second) before giving up.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity) {
	const uint32_t addr = smem_u32(bar);
	for (uint32_t i = 0; i < kWaitPolls; ++i) {
		uint32_t ok;
		asm volatile(
		    "{\n\t.reg .pred p;\n\t"
		    "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		    "selp.u32 %0, 1, 0, p;\n\t}"
		    : "=r"(ok)
		    : "r"(addr), "r"(parity)
		    : "memory");
		if (ok) return true;
		if (i > 64) __nanosleep(64);
	}
	return false;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "setp.ne.u32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
	    "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)acc)
	    : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned long long *bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
	             : "memory");
}

// Stage rows [row0, row0+rows) x K [k0, k0+kc) of a row-major bf16 matrix
// (leading dimension ld) into the core-matrix layout; rows past `valid` and
// K past kc are zero.  Four 16-byte loads per thread are issued before their
// shared-memory stores, so several loads are in flight per thread.
__device__ __forceinline__ void stage_tile(unsigned char *dst, const __nv_bfloat16 *__restrict__ src, int ld, int row0,
                                           int rows, int valid, int k0, int kc) {
	const int chunks = rows * (kChunkK / 8);
	for (int q0 = threadIdx.x; q0 < chunks; q0 += 4 * kGemmThreads) {
		uint4 v[4];
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const int q = q0 + u * kGemmThreads;
			const int r = q / (kChunkK / 8), c8 = q % (kChunkK / 8);
			v[u] = make_uint4(0, 0, 0, 0);
			if (q < chunks && row0 + r < valid && c8 * 8 < kc)
				v[u] = __ldg(reinterpret_cast<const uint4 *>(src + (size_t)(row0 + r) * ld + k0 + c8 * 8));
		}
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const int q = q0 + u * kGemmThreads;
			if (q >= chunks) break;
			const int r = q / (kChunkK / 8), c8 = q % (kChunkK / 8);
			*reinterpret_cast<uint4 *>(dst + (r / 8) * kSbo + c8 * kLbo + (r % 8) * 16) = v[u];
		}
	}
}

// Epilogue: thread = row (warp w reads TMEM lanes 32w..32w+31); 16 columns
// per tensor-memory load; bias, row-scaled bias, ReLU, then the requested
// stores.
__device__ __forceinline__ void epilogue(const GemmArgs &g, uint32_t tmem, int row0, int warp, int lane) {
	const int row = row0 + warp * 32 + lane;
	for (int c0 = 0; c0 < g.N; c0 += 16) {
		uint32_t v[16];
		const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
		asm volatile(
		    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
		    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
		      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
		    : "r"(taddr)
		    : "memory");
		asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
		if (row >= g.M) continue;
		// N is a multiple of 16, so all 16 columns exist.
		float x[16];
		const float rs = g.rowScale ? g.rowScale[row] : 0.0f;
#pragma unroll
		for (int u = 0; u < 16; ++u) {
			const int col = c0 + u;
			x[u] = __uint_as_float(v[u]);
			if (g.bias) x[u] += g.bias[col];
			if (g.rowScale) x[u] += rs * g.bias2[col];
			if (g.relu) x[u] = fmaxf(x[u], 0.0f);
		}
		if (g.C) {
			float *dst = g.C + (size_t)row * g.ldc + c0;
			if (g.accumulate) {
#pragma unroll
				for (int u = 0; u < 16; ++u) atomicAdd(dst + u, x[u]);
			} else if ((g.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(g.C) & 15) == 0) {
#pragma unroll
				for (int u = 0; u < 16; u += 4)
					*reinterpret_cast<float4 *>(dst + u) = make_float4(x[u], x[u + 1], x[u + 2], x[u + 3]);
			} else {
#pragma unroll
				for (int u = 0; u < 16; ++u) dst[u] = x[u];
			}
		}
		if (g.Cb) {
			__nv_bfloat16 *dst = g.Cb + (size_t)row * g.ldcb + c0;
			if ((g.ldcb & 7) == 0 && (reinterpret_cast<uintptr_t>(g.Cb) & 15) == 0) {
#pragma unroll
				for (int u = 0; u < 16; u += 8) {
					uint4 pk;
					__nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&pk);
#pragma unroll
					for (int w = 0; w < 4; ++w) h[w] = __floats2bfloat162_rn(x[u + 2 * w], x[u + 2 * w + 1]);
					*reinterpret_cast<uint4 *>(dst + u) = pk;
				}
			} else {
#pragma unroll
				for (int u = 0; u < 16; ++u) dst[u] = __float2bfloat16_rn(x[u]);
			}
		}
		if (g.CbT) {
#pragma unroll
			for (int u = 0; u < 16; ++u) g.CbT[(size_t)(c0 + u) * g.ldcbT + row] = __float2bfloat16_rn(x[u]);
		}
	}
}

}  // namespace

size_t gemm_smem_bytes() { return sizeof(GemmSmem) + 1024; }

__global__ void __launch_bounds__(kGemmThreads, 1) k_gemm_bf16(GemmArgs g) {
	extern __shared__ unsigned char smem_raw[];
	GemmSmem &S = *reinterpret_cast<GemmSmem *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
	const int tid = threadIdx.x, warp = tid / 32, lane = tid & 31;
	const int row0 = blockIdx.x * kTileM;
	// K range of this split.
	const int kPer = ((g.K + gridDim.y - 1) / gridDim.y + kChunkK - 1) / kChunkK * kChunkK;
	const int kBegin = blockIdx.y * kPer;
	const int kEnd = min(g.K, kBegin + kPer);
	const int ncols = g.N <= 32 ? 32 : (g.N <= 64 ? 64 : (g.N <= 128 ? 128 : 256));

	if (tid == 0) {
		mbar_init(&S.bar[0], 1);
		mbar_init(&S.bar[1], 1);
		mbar_init(&S.done, 1);
		S.fail = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
		             "r"(ncols)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = S.tmem;
	const uint32_t idesc = instr_desc(g.N);

	const int nChunks = kEnd > kBegin ? (kEnd - kBegin + kChunkK - 1) / kChunkK : 0;
	uint32_t phase[2] = {0, 0};
	bool ok = true;
	for (int c = 0; c < nChunks; ++c) {
		const int st = c & 1;
		if (c >= 2) {
			// The MMAs that read this stage two chunks ago must be done; if
			// the bounded wait runs out, no further MMA is issued.
			const bool w = mbar_wait(&S.bar[st], phase[st]);
			phase[st] ^= 1;
			if (__syncthreads_or(!w)) {
				ok = false;
				break;
			}
		}
		const int k0 = kBegin + c * kChunkK;
		const int kc = min(kChunkK, kEnd - k0);
		stage_tile(S.a[st], g.A, g.lda, row0, kTileM, g.M, k0, kc);
		stage_tile(S.b[st], g.B, g.ldb, 0, (g.N + 7) / 8 * 8, g.N, k0, kc);
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		__syncthreads();
		if (tid == 0) {
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			const uint32_t a0 = smem_u32(S.a[st]), b0 = smem_u32(S.b[st]);
			for (int s = 0; s < kc / 16; ++s) {
				mma_bf16(tmem, smem_desc(a0 + s * 2 * kLbo), smem_desc(b0 + s * 2 * kLbo), idesc, c > 0 || s > 0);
			}
			mma_commit(&S.bar[st]);
		}
	}
	if (tid == 0) mma_commit(&S.done);  // arrives when every MMA issued above is complete
	// Always wait (bounded) for the issued MMAs before reading or freeing
	// tensor memory.
	const bool d = mbar_wait(&S.done, 0);
	if (!ok || !d) atomicOr(&S.fail, 1);
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	__syncthreads();
	const bool good = S.fail == 0;
	if (!good && tid == 0) atomicOr(g.error, 1u);

	// Epilogue: thread = row; 16 columns per tensor-memory load.
	if (good && nChunks > 0) epilogue(g, tmem, row0, warp, lane);
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	if (warp == 0) {
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
	}
}

// ---------------------------------------------------------------------------
// TMA-fed variant: each operand tile (128 or N rows x 64 K) is one
// cp.async.bulk.tensor load with 128-byte swizzle into a 1 KiB-aligned stage,
// completing on the stage's "full" mbarrier; the MMAs read it through
// SWIZZLE_128B K-major descriptors (8-row groups 1 KiB apart; the 16-wide K
// steps advance the start address by 32 bytes inside the swizzle atom) and
// release it through tcgen05.commit on the stage's "empty" mbarrier.  One
// thread drives the three-stage pipeline; the others wait for the final
// commit and run the epilogue.  Rows and K beyond the matrices read as zero.

namespace {

constexpr int kTmaStages = 3;
constexpr int kTmaABytes = kTileM * kChunkK * 2;  // 16 KiB

__host__ __device__ inline size_t tma_stage_bytes(int n) { return (size_t)kTmaABytes + (size_t)n * kChunkK * 2; }

__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
	uint64_t d = 0;
	d |= (uint64_t)((addr >> 4) & 0x3fff);
	d |= (uint64_t)1 << 16;                  // leading byte offset (unused for swizzled K-major)
	d |= (uint64_t)(1024 >> 4) << 32;        // 8-row groups 1 KiB apart
	d |= (uint64_t)1 << 46;                  // descriptor version
	d |= (uint64_t)2 << 61;                  // SWIZZLE_128B
	return d;
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
	             : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            unsigned long long *bar) {
	asm volatile(
	    "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
	    "[%4];" ::"r"(smem_u32(dst)),
	    "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
	    : "memory");
}

}  // namespace

size_t gemm_tma_smem_bytes(int n) { return kTmaStages * tma_stage_bytes(n) + 2048; }

__global__ void __launch_bounds__(kGemmThreads, 1) k_gemm_bf16_tma(GemmArgs g, const __grid_constant__ CUtensorMap mapA,
                                                                   const __grid_constant__ CUtensorMap mapB) {
	extern __shared__ unsigned char smem_raw[];
	unsigned char *base =
	    reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
	const size_t stage = tma_stage_bytes(g.N);
	unsigned long long *full = reinterpret_cast<unsigned long long *>(base + kTmaStages * stage);
	unsigned long long *empty = full + kTmaStages;
	unsigned long long *done = empty + kTmaStages;
	uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(done + 1);
	int *fail = reinterpret_cast<int *>(tmemSlot + 1);
	const int tid = threadIdx.x, warp = tid / 32, lane = tid & 31;
	const int row0 = blockIdx.x * kTileM;
	const int kPer = ((g.K + gridDim.y - 1) / gridDim.y + kChunkK - 1) / kChunkK * kChunkK;
	const int kBegin = blockIdx.y * kPer;
	const int kEnd = min(g.K, kBegin + kPer);
	const int ncols = g.N <= 32 ? 32 : (g.N <= 64 ? 64 : (g.N <= 128 ? 128 : 256));
	const int nChunks = kEnd > kBegin ? (kEnd - kBegin + kChunkK - 1) / kChunkK : 0;

	if (tid == 0) {
		for (int s = 0; s < kTmaStages; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], 1);
		}
		mbar_init(done, 1);
		*fail = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
		asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmemSlot)),
		             "r"(ncols)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = *tmemSlot;

	if (tid == 0) {
		const uint32_t idesc = instr_desc(g.N);
		const uint32_t bytes = (uint32_t)stage;
		bool ok = true;
		for (int c = 0; c < nChunks && c < kTmaStages; ++c) {
			unsigned char *st = base + c * stage;
			mbar_expect_tx(&full[c], bytes);
			tma_load_2d(st, &mapA, kBegin + c * kChunkK, row0, &full[c]);
			tma_load_2d(st + kTmaABytes, &mapB, kBegin + c * kChunkK, 0, &full[c]);
		}
		for (int c = 0; c < nChunks && ok; ++c) {
			const int s = c % kTmaStages;
			const uint32_t parity = (uint32_t)(c / kTmaStages) & 1u;
			if (!mbar_wait(&full[s], parity)) {
				ok = false;
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			const uint32_t a0 = smem_u32(base + s * stage), b0 = a0 + kTmaABytes;
			const int kc = min(kChunkK, kEnd - (kBegin + c * kChunkK));
			for (int k = 0; k < kc / 16; ++k)
				mma_bf16(tmem, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), idesc, c > 0 || k > 0);
			mma_commit(&empty[s]);
			const int next = c + kTmaStages;
			if (next < nChunks) {
				// The stage is reloaded once the MMAs reading it are done.
				if (!mbar_wait(&empty[s], parity)) {
					ok = false;
					break;
				}
				unsigned char *st = base + s * stage;
				mbar_expect_tx(&full[s], bytes);
				tma_load_2d(st, &mapA, kBegin + next * kChunkK, row0, &full[s]);
				tma_load_2d(st + kTmaABytes, &mapB, kBegin + next * kChunkK, 0, &full[s]);
			}
		}
		mma_commit(done);
		if (!ok) *fail = 1;
	}
	__syncwarp();
	// Always wait (bounded) for the issued MMAs before reading or freeing
	// tensor memory.  A load still in flight after a failed wait completes
	// into this CTA's own shared memory.
	const bool d = mbar_wait(done, 0);
	if (!d) atomicOr(fail, 1);
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	__syncthreads();
	const bool good = *fail == 0;
	if (!good && tid == 0) atomicOr(g.error, 1u);
	if (good && nChunks > 0) epilogue(g, tmem, row0, warp, lane);
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	if (warp == 0) {
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
	}
}

// ---------------------------------------------------------------------------
// Persistent TMA-fed variant for one K split: each CTA loops over row tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...  B (all of N x K) is loaded once
// per CTA and stays in shared memory; A arrives in 128 x 64 chunks through a
// kPersistStages-deep ring (full/empty mbarriers); the accumulator is
// double-buffered in tensor memory (tfull/tempty mbarriers), so one tile's
// epilogue overlaps the next tile's loads and MMAs.  Warps 0-3 run the
// epilogue (warp w owns TMEM lanes 32w..32w+31), lane 0 of warp 4 drives
// TMA, lane 0 of warp 5 issues the MMAs.  Every wait is bounded; a wait that
// runs out raises the CTA's abort flag and the error word, every role then
// leaves its loop (collectively within a warp), and the MMA thread waits
// (bounded) for its last MMAs before tensor memory is freed.

namespace {

constexpr int kPersistStages = 4;
constexpr int kPersistThreads = 192;
constexpr int kPersistMaxBBytes = 96 * 1024;

struct PersistCtl {
	unsigned long long full[kPersistStages], empty[kPersistStages];
	unsigned long long bfull, tfull[2], tempty[2], fin;
	uint32_t tmem;
	volatile int abort;
};

__host__ __device__ inline int k_chunks(int K) { return (K + kChunkK - 1) / kChunkK; }
__host__ __device__ inline size_t persist_b_bytes(int n, int K) { return (size_t)k_chunks(K) * n * kChunkK * 2; }

}  // namespace

size_t gemm_persist_smem_bytes(int n, int K) {
	// More than half of an SM's shared memory: one CTA per SM, which then
	// owns up to all 512 tensor-memory columns.
	const size_t need = persist_b_bytes(n, K) + (size_t)kPersistStages * kTmaABytes + sizeof(PersistCtl) + 1024;
	const size_t minimum = 116 * 1024;
	return need > minimum ? need : minimum;
}

__global__ void __launch_bounds__(kPersistThreads, 1) k_gemm_bf16_persist(GemmArgs g,
                                                                          const __grid_constant__ CUtensorMap mapA,
                                                                          const __grid_constant__ CUtensorMap mapB) {
	extern __shared__ unsigned char smem_raw[];
	unsigned char *base =
	    reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
	const int nk = k_chunks(g.K);
	const size_t bBytes = persist_b_bytes(g.N, g.K);
	unsigned char *bRes = base;                         // chunk c at c * N * 128 bytes
	unsigned char *aRing = base + bBytes;               // 1 KiB-aligned: bBytes is a multiple of 1 KiB
	PersistCtl &C = *reinterpret_cast<PersistCtl *>(aRing + kPersistStages * kTmaABytes);
	const int tid = threadIdx.x, warp = tid / 32, lane = tid & 31;
	const int ncols = g.N <= 32 ? 32 : (g.N <= 64 ? 64 : (g.N <= 128 ? 128 : 256));
	const int tiles = (g.M + kTileM - 1) / kTileM;

	if (tid == 0) {
		for (int s = 0; s < kPersistStages; ++s) {
			mbar_init(&C.full[s], 1);
			mbar_init(&C.empty[s], 1);
		}
		mbar_init(&C.bfull, 1);
		for (int b = 0; b < 2; ++b) {
			mbar_init(&C.tfull[b], 1);
			mbar_init(&C.tempty[b], 128);
		}
		mbar_init(&C.fin, 1);
		C.abort = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
		asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
	}
	if (warp == 5) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&C.tmem)),
		             "r"(2 * ncols)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	const uint32_t tmem = C.tmem;

	if (warp == 4) {
		if (lane == 0) {
			// TMA: B once, then A chunk by chunk for every tile of this CTA.
			mbar_expect_tx(&C.bfull, (uint32_t)bBytes);
			for (int c = 0; c < nk; ++c) tma_load_2d(bRes + (size_t)c * g.N * kChunkK * 2, &mapB, c * kChunkK, 0, &C.bfull);
			int it = 0;
			for (int t = blockIdx.x; t < tiles && !C.abort; t += gridDim.x) {
				for (int c = 0; c < nk; ++c, ++it) {
					const int s = it % kPersistStages;
					if (it >= kPersistStages && !mbar_wait(&C.empty[s], ((it / kPersistStages) - 1) & 1)) {
						C.abort = 1;
						break;
					}
					mbar_expect_tx(&C.full[s], (uint32_t)kTmaABytes);
					tma_load_2d(aRing + s * kTmaABytes, &mapA, c * kChunkK, t * kTileM, &C.full[s]);
				}
			}
		}
		__syncwarp();
	} else if (warp == 5) {
		if (lane == 0) {
			const uint32_t idesc = instr_desc(g.N);
			bool ok = mbar_wait(&C.bfull, 0);
			int it = 0, i = 0;
			for (int t = blockIdx.x; ok && t < tiles && !C.abort; t += gridDim.x, ++i) {
				const int b = i & 1;
				// The epilogue has read this buffer's previous tile.
				if (i >= 2 && !mbar_wait(&C.tempty[b], ((i - 2) >> 1) & 1)) {
					ok = false;
					break;
				}
				asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
				for (int c = 0; c < nk; ++c, ++it) {
					const int s = it % kPersistStages;
					if (!mbar_wait(&C.full[s], (it / kPersistStages) & 1)) {
						ok = false;
						break;
					}
					asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
					const uint32_t a0 = smem_u32(aRing + s * kTmaABytes);
					const uint32_t b0 = smem_u32(bRes + (size_t)c * g.N * kChunkK * 2);
					const int kc = min(kChunkK, g.K - c * kChunkK);
					for (int k = 0; k < kc / 16; ++k)
						mma_bf16(tmem + (uint32_t)(b * ncols), sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), idesc,
						         c > 0 || k > 0);
					mma_commit(&C.empty[s]);
				}
				if (!ok) break;
				mma_commit(&C.tfull[b]);
			}
			if (!ok) {
				C.abort = 1;
				atomicOr(g.error, 1u);
			}
			// Every MMA issued above is complete before tensor memory is freed.
			mma_commit(&C.fin);
			if (!mbar_wait(&C.fin, 0)) atomicOr(g.error, 1u);
		}
		__syncwarp();
	} else {
		// Epilogue warps 0-3.
		int i = 0;
		for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++i) {
			const int b = i & 1;
			if (__any_sync(0xffffffffu, C.abort != 0)) break;
			const bool ok = mbar_wait(&C.tfull[b], (i >> 1) & 1);
			if (!__all_sync(0xffffffffu, ok)) {
				C.abort = 1;
				atomicOr(g.error, 1u);
				break;
			}
			asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
			epilogue(g, tmem + (uint32_t)(b * ncols), t * kTileM, warp, lane);
			asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
			asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&C.tempty[b])) : "memory");
		}
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	if (warp == 5) {
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * ncols) : "memory");
	}
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
	static std::once_flag once;
	static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
	std::call_once(once, [] {
		void *p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
		        cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
	});
	return fn;
}

// Row-major bf16 matrix [rows][K] (leading dimension ld) as 64 x boxRows
// tiles with 128-byte swizzle.
bool encode(CUtensorMap *map, const __nv_bfloat16 *ptr, int rows, int K, int ld, int boxRows) {
	PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
	if (!fn) return false;
	const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
	const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
	const cuuint32_t box[2] = {(cuuint32_t)kChunkK, (cuuint32_t)boxRows};
	const cuuint32_t estr[2] = {1, 1};
	return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(ptr), dims, strides, box, estr,
	          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
	          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int gemm_check(const GemmArgs &g, int splits) {
	if (g.M <= 0 || g.N <= 0 || g.K <= 0 || g.N > kMaxN || g.N % 16 != 0 || g.K % 16 != 0) return -1;
	if (g.lda % 8 != 0 || g.ldb % 8 != 0 || splits < 1) return -1;
	if ((reinterpret_cast<uintptr_t>(g.A) | reinterpret_cast<uintptr_t>(g.B)) & 15) return -1;
	if (splits > 1 && !(g.C && g.accumulate)) return -1;
	return 0;
}

cudaError_t gemm_launch(const GemmArgs &g, int splits, cudaStream_t stream) {
	// Kernel attributes are per device: set them once on each device used.
	static std::mutex mu;
	static bool done[64] = {};
	static int sms[64] = {};
	int device = 0;
	cudaError_t e = cudaGetDevice(&device);
	if (e != cudaSuccess) return e;
	{
		std::lock_guard<std::mutex> lock(mu);
		if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
		if (!done[device]) {
			e = cudaFuncSetAttribute(k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                         (int)gemm_smem_bytes());
			if (e == cudaSuccess)
				e = cudaFuncSetAttribute(k_gemm_bf16_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
				                         (int)gemm_tma_smem_bytes(kMaxN));
			if (e == cudaSuccess)
				e = cudaFuncSetAttribute(k_gemm_bf16_persist, cudaFuncAttributeMaxDynamicSharedMemorySize,
				                         (int)gemm_persist_smem_bytes(kMaxN, kPersistMaxBBytes / (kMaxN * 2)));
			if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms[device], cudaDevAttrMultiProcessorCount, device);
			if (e != cudaSuccess) return e;
			done[device] = true;
		}
	}
	const int tiles = (g.M + kTileM - 1) / kTileM;
	dim3 grid(tiles, splits);
	CUtensorMap mapA, mapB;
	if (g.noTma != 1 && encode(&mapA, g.A, g.M, g.K, g.lda, kTileM) && encode(&mapB, g.B, g.N, g.K, g.ldb, g.N)) {
		if (g.noTma == 0 && splits == 1 && persist_b_bytes(g.N, g.K) <= (size_t)kPersistMaxBBytes) {
			k_gemm_bf16_persist<<<std::min(tiles, sms[device]), kPersistThreads, gemm_persist_smem_bytes(g.N, g.K),
			                      stream>>>(g, mapA, mapB);
		} else {
			k_gemm_bf16_tma<<<grid, kGemmThreads, gemm_tma_smem_bytes(g.N), stream>>>(g, mapA, mapB);
		}
	} else {
		k_gemm_bf16<<<grid, kGemmThreads, gemm_smem_bytes(), stream>>>(g);
	}
	return cudaGetLastError();
}

}  // namespace sphgb
