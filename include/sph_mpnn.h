/*
 * sph_mpnn.h -- C ABI of the learned frame (no counterpart in the reference).
 *
 * A small message-passing network stands in for one frame of the plain
 * method (the reference's four Update(dt/4) substeps per frame,
 * kSPHSubsteps, sph.h:32-34 / app.cpp:231-233).  Its dense layers run on the
 * GB300's 5th-generation tensor cores (tcgen05, BF16 operands, FP32
 * accumulation); the plain step stays its judge and fallback.
 */
#ifndef SPH_MPNN_H
#define SPH_MPNN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* C[M x N] (+)= A[M x K] * B[N x K]^T on the tensor cores: A and B bf16
 * row-major device arrays (leading dimensions lda, ldb in elements, multiples
 * of 8, 16-byte aligned), C FP32 row-major (ldc).  N a multiple of 16 up to
 * 256, K a multiple of 16, any M.  Optional bias [N] and ReLU; accumulate = 1
 * adds into C atomically (required when splits > 1 divides K over CTAs).
 * Enqueued on `stream` (cudaStream_t) and waited for. */
int sph_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, int lda, int ldb, int ldc,
                  const float *bias, int relu, int accumulate, int splits, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SPH_MPNN_H */
