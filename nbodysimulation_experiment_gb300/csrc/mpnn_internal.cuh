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
	int noTma;              // 0: TMA (persistent CTAs for one K split), 1: plain loads, 2: TMA, one tile per CTA
};

size_t gemm_smem_bytes();
int gemm_check(const GemmArgs &g, int splits);
cudaError_t gemm_launch(const GemmArgs &g, int splits, cudaStream_t stream);

}  // namespace sphgb

// ---------------------------------------------------------------------------
// The network (no counterpart in the reference).  Per round r (two rounds,
// separate weights), over the directed edges (i, j), j != i, |x_j - x_i| < h,
// j in the 3x3 cell block of i:
//   e_ij = [d/h (2), r/h, z_j - z_i (2), (1 - r/h)^2]
//   H_i  = (1/S) sum_j relu(W1 e_ij + b1)            edge MLP layer 1, summed
//   M_i  = W2 H_i + (deg_i/S) b2                      edge MLP layer 2 (linear, so applied after the sum)
//   c_i  = relu(W3 [M_i, z_i, 0..] + b3)              node MLP layer 1
//   z_i += W4 c_i + b4                                node MLP layer 2
// with z^0 = v dt / h and output u = z^2 - z^0, a correction of positions in
// units of h.

namespace sphgb {

constexpr int kHidden = 128;
constexpr int kEdgeIn = 6;
constexpr int kNodeIn = 130;
constexpr int kNodeInPad = 144;
constexpr int kRounds = 2;
constexpr float kAggScale = 1.0f / 32.0f;  // 1/S
// Parameter offsets within one round of the flat FP32 parameter vector.
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHidden * kEdgeIn;
constexpr int kOffW2 = kOffB1 + kHidden;
constexpr int kOffB2 = kOffW2 + kHidden * kHidden;
constexpr int kOffW3 = kOffB2 + kHidden;
constexpr int kOffB3 = kOffW3 + kHidden * kNodeInPad;
constexpr int kOffW4 = kOffB3 + kHidden;
constexpr int kOffB4 = kOffW4 + 2 * kHidden;
constexpr int kRoundParams = kOffB4 + 2;
constexpr int kParams = kRounds * kRoundParams;
constexpr int kMpnnStage = 1024;  // staged 3x3-block entries per warp

// One graph: particles numbered cell by cell (cellStart/cellCount), the
// positions the edges are built from and the initial node state.
struct MpnnGraph {
	const float2 *pos;
	const float2 *z0;
	const int *cellStart, *cellCount;
	int n, gx, gy;
	float h, invH;
};

constexpr int kEdgeWarps = 4;
size_t mpnn_edge_smem(bool backward);
size_t mpnn_edge_tc_smem();
int mpnn_edge_tc_blocks_per_sm();
int mpnn_edge_tc_threads();

__global__ void k_mpnn_edge_fwd(MpnnGraph G, const float *W1, const float *b1, const float2 *z, __nv_bfloat16 *Hb,
                                float *degS, int np, uint32_t *error);
__global__ void k_mpnn_edge_fwd_tc(MpnnGraph G, const float *W1, const float *b1, const float2 *z,
                                   __nv_bfloat16 *Hb, float *degS, int np, uint32_t *error);
__global__ void k_mpnn_edge_bwd(MpnnGraph G, const float *W1, const float *b1, const float2 *z, const float *dH,
                                float2 *dzEdge, float *gW1, float *gb1, int needDz, uint32_t *error);
__global__ void k_mpnn_x3_tail(const float2 *z, __nv_bfloat16 *X3b, __nv_bfloat16 *X3f, int np, int ldf);
__global__ void k_mpnn_node_out(const __nv_bfloat16 *cb, const float *W4, const float *b4, const float2 *zin,
                                float2 *zout, int np);
__global__ void k_mpnn_loss(const float2 *z2, const float2 *z0, const float2 *target, float2 *dz, int n, int np,
                            float *loss);
__global__ void k_mpnn_node_bwd(const float2 *dz, const float *W4, const __nv_bfloat16 *cb, __nv_bfloat16 *da3b,
                                int np);
__global__ void k_mpnn_dw4(const float2 *dz, const __nv_bfloat16 *cf, int ldf, int n, float *gW4, float *gb4);
__global__ void k_mpnn_rowsum(const __nv_bfloat16 *X, int ld, int n, const float *w, float *out);
__global__ void k_mpnn_combine(const float2 *dzNext, const float *dX, const float2 *dzEdge, float2 *dz, int n,
                               int np);
__global__ void k_mpnn_transpose(const __nv_bfloat16 *src, int rows, int cols, int lds, __nv_bfloat16 *dst, int ldd);
__global__ void k_mpnn_adam(float *p, const float *g, float *m, float *v, int count, float lr, float beta1,
                            float beta2, float eps, float bc1, float bc2, float clip);
__global__ void k_mpnn_refresh(const float *p, __nv_bfloat16 *W2b, __nv_bfloat16 *W2Tb, __nv_bfloat16 *W3b,
                               __nv_bfloat16 *W3Tb);
__global__ void k_mpnn_u(const float2 *z2, const float2 *z0, float2 *u, int n);

}  // namespace sphgb

struct sph_mpnn;

namespace sphgb {

// Inference on one graph: u (device, n entries) = z^2 - z^0.  The graph's z0
// must hold zeros on [n, round_up(n, 128)).  Runs on `stream`.
int mpnn_forward_dev(sph_mpnn *m, const MpnnGraph &g, float2 *u, cudaStream_t stream);
// Store a training sample: copies positions, z0 (with its zero padding) and
// the cell tables; returns device pointers to the sample's positions (n),
// and to its target (n) and id (n) arrays for the caller to fill.
int mpnn_add_sample(sph_mpnn *m, const MpnnGraph &g, cudaStream_t stream, float2 **pos, float2 **target, int **ids);
size_t mpnn_capacity(const sph_mpnn *m);
int mpnn_device(const sph_mpnn *m);

inline int round_up128(int n) { return (n + 127) / 128 * 128; }

}  // namespace sphgb
