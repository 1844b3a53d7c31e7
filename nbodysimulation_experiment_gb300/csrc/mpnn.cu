// Host side of the message-passing network: the C entry points of
// include/sph_mpnn.h.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sph_gb300.h"
#include "../../include/sph_mpnn.h"
#include "mpnn_internal.cuh"

using namespace sphgb;

namespace {

// Error word of the standalone GEMM entry point, one per device.
uint32_t *gemm_error_word(int device) {
	static std::mutex mu;
	static uint32_t *words[64] = {};
	std::lock_guard<std::mutex> lock(mu);
	if (device < 0 || device >= 64) return nullptr;
	if (!words[device]) {
		if (cudaMalloc(&words[device], sizeof(uint32_t)) != cudaSuccess) return nullptr;
		if (cudaMemset(words[device], 0, sizeof(uint32_t)) != cudaSuccess) return nullptr;
	}
	return words[device];
}

}  // namespace

extern "C" int sph_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, int lda, int ldb, int ldc,
                             const float *bias, int relu, int accumulate, int splits, void *stream) {
	int device = 0;
	if (cudaGetDevice(&device) != cudaSuccess) return SPH_ERR_NO_DEVICE;
	GemmArgs g{};
	g.A = static_cast<const __nv_bfloat16 *>(A);
	g.B = static_cast<const __nv_bfloat16 *>(B);
	g.M = M;
	g.N = N;
	g.K = K;
	g.lda = lda;
	g.ldb = ldb;
	g.bias = bias;
	g.relu = relu;
	g.C = C;
	g.ldc = ldc;
	g.accumulate = accumulate;
	g.error = gemm_error_word(device);
	if (!A || !B || !C || !g.error || ldc < N) return SPH_ERR_INVALID_ARGUMENT;
	if (gemm_check(g, splits) != 0) return SPH_ERR_INVALID_ARGUMENT;
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	if (gemm_launch(g, splits, st) != cudaSuccess) return SPH_ERR_CUDA;
	uint32_t err = 0;
	if (cudaStreamSynchronize(st) != cudaSuccess) return SPH_ERR_CUDA;
	if (cudaMemcpy(&err, g.error, sizeof(err), cudaMemcpyDeviceToHost) != cudaSuccess) return SPH_ERR_CUDA;
	if (err) {
		cudaMemset(g.error, 0, sizeof(uint32_t));
		return SPH_ERR_TIMEOUT;
	}
	return SPH_OK;
}
