// Internal declarations of the message-passing network (learned frame).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sphgb {

// C[M x N] (+)= A[M x K] * B[N x K]^T with the epilogue below; A and B are
// bf16 row-major (leading dimensions in elements, multiples of 8, 16-byte
// aligned); N a multiple of 16 up to 256, K a multiple of 16.
struct GemmArgs {
	const __nv_bfloat16 *A;
	const __nv_bfloat16 *B;
	int M, N, K;
	int lda, ldb;
	const float *bias;      // [N] added to every row (nullable)
	const float *rowScale;  // [M] x bias2 [N] added (nullable)
	const float *bias2;
	int relu;
	float *C;               // FP32 [M][ldc] (nullable)
	int ldc;
	int accumulate;         // atomically add into C (required for split-K)
	__nv_bfloat16 *Cb;      // bf16 [M][ldcb] (nullable)
	int ldcb;
	__nv_bfloat16 *CbT;     // bf16 transposed [N][ldcbT] (nullable)
	int ldcbT;
	uint32_t *error;        // set to 1 if a bounded wait ran out
};

size_t gemm_smem_bytes();
int gemm_check(const GemmArgs &g, int splits);
cudaError_t gemm_launch(const GemmArgs &g, int splits, cudaStream_t stream);

}  // namespace sphgb
