// Kernels of the message-passing network other than the dense GEMM
// (mpnn_gemm.cu): the edge layer (built on the fly from the cell grid,
// summed per particle) on the tensor cores and, selectable, on the CUDA
// cores; its backward pass; elementwise node work, reductions, layout
// transposes and the optimizer.  In every form the edge layer's inputs
// (edge features, W1, b1) are rounded to TF32.  Arithmetic follows the FP64
// restatement in the oracle up to FP32/TF32/BF16 rounding.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mpnn_internal.cuh"
#include "sph_internal.cuh"
#include "tc_ptx.cuh"

namespace sphgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;

struct EdgeWarp {
	float2 pos[kMpnnStage];
	float2 z[kMpnnStage];
	float feat[kWarp][8];  // features of the in-range edges of one group of 32 candidates
	int nbr[kWarp];        // their neighbour numbers
};

struct EdgeWarpBwd {
	EdgeWarp core;
	float part[2][kWarp][kWarp + 1];  // per-edge partial sums, one per lane
};

// The 3x3 block of cells around cell c (y-major), as segments of the
// cell-ordered particle numbering.
struct Block {
	int start[9], off[9];
	int L, own;
};

__device__ __forceinline__ Block make_block(const MpnnGraph &G, int c) {
	Block b;
	const int cx = c % G.gx, cy = c / G.gx;
	b.L = 0;
	b.own = 0;
#pragma unroll
	for (int q = 0; q < 9; ++q) {
		const int x = cx + q % 3 - 1, y = cy + q / 3 - 1;
		int st = 0, nn = 0;
		if (x >= 0 && x < G.gx && y >= 0 && y < G.gy) {
			const int c2 = y * G.gx + x;
			st = G.cellStart[c2];
			nn = G.cellCount[c2];
		}
		b.start[q] = st;
		b.off[q] = b.L;
		if (q == 4) b.own = b.L;
		b.L += nn;
	}
	return b;
}

__device__ __forceinline__ int block_number(const Block &b, int e) {
	int src = b.start[0] + e;
#pragma unroll
	for (int q = 1; q < 9; ++q) src = (e >= b.off[q]) ? b.start[q] + (e - b.off[q]) : src;
	return src;
}

__device__ __forceinline__ void stage_block(EdgeWarp &S, const Block &b, const MpnnGraph &G, const float2 *z,
                                            int lane) {
	for (int e = lane; e < b.L; e += kWarp) {
		const int num = block_number(b, e);
		S.pos[e] = G.pos[num];
		S.z[e] = z[num];
	}
	__syncwarp();
}

__device__ __forceinline__ unsigned lanemask_lt() {
	unsigned m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

// The in-range edges among staged candidates [base, base+32) of the particle
// at staged slot `self`: each lane tests one candidate and writes its edge
// features (e_ij, see mpnn_internal.cuh) and neighbour number into the
// group's compacted list; returns the list length.
__device__ __forceinline__ int edge_group(EdgeWarp &S, const Block &b, int base, int self, float2 xi, float2 zi,
                                          float h2, float invH, int lane) {
	const int e = base + lane;
	bool in = false;
	float dx = 0.f, dy = 0.f, r2 = 0.f;
	if (e < b.L && e != self) {
		const float2 xj = S.pos[e];
		dx = xj.x - xi.x;
		dy = xj.y - xi.y;
		// Unfused, as the neighbour sets of the plain step are computed.
		r2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
		in = r2 < h2;
	}
	const unsigned mask = __ballot_sync(kFull, in);
	if (in) {
		const int slot = __popc(mask & lanemask_lt());
		const float r = sqrtf(r2);
		const float q = r * invH;
		const float2 zj = S.z[e];
		float *f = S.feat[slot];
		*reinterpret_cast<float4 *>(f) =
		    make_float4(tc::to_tf32(dx * invH), tc::to_tf32(dy * invH), tc::to_tf32(q), tc::to_tf32(zj.x - zi.x));
		*reinterpret_cast<float2 *>(f + 4) =
		    make_float2(tc::to_tf32(zj.y - zi.y), tc::to_tf32((1.0f - q) * (1.0f - q)));
		S.nbr[slot] = block_number(b, e);
	}
	__syncwarp();
	return __popc(mask);
}

__device__ __forceinline__ void load_feat(const EdgeWarp &S, int q, float (&f)[kEdgeIn]) {
	const float4 a = *reinterpret_cast<const float4 *>(S.feat[q]);
	const float2 c = *reinterpret_cast<const float2 *>(S.feat[q] + 4);
	f[0] = a.x;
	f[1] = a.y;
	f[2] = a.z;
	f[3] = a.w;
	f[4] = c.x;
	f[5] = c.y;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
	return v;
}

}  // namespace

// Edge layer 1 on the CUDA cores, summed per particle: one warp per cell
// stages the cell's 3x3 block; per group of 32 candidates the lanes compute
// the in-range edges' features once, then every lane applies its hidden
// features l, l+32, l+64, l+96 to each edge.
__global__ void __launch_bounds__(kEdgeWarps * kWarp) k_mpnn_edge_fwd(MpnnGraph G, const float *W1, const float *b1,
                                                                     const float2 *z, __nv_bfloat16 *Hb, float *degS,
                                                                     int np, uint32_t *error) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	EdgeWarp &S = reinterpret_cast<EdgeWarp *>(smem_raw)[threadIdx.x / kWarp];
	const int lane = threadIdx.x & (kWarp - 1);
	float w[4][kEdgeIn], bias[4];
#pragma unroll
	for (int q = 0; q < 4; ++q) {
		const int f = lane + 32 * q;
#pragma unroll
		for (int k = 0; k < kEdgeIn; ++k) w[q][k] = tc::to_tf32(W1[f * kEdgeIn + k]);
		bias[q] = tc::to_tf32(b1[f]);
	}
	const float h2 = __fmul_rn(G.h, G.h);
	const int ncell = G.gx * G.gy;
	const int warpsTotal = gridDim.x * kEdgeWarps;
	for (int c = blockIdx.x * kEdgeWarps + threadIdx.x / kWarp; c < ncell; c += warpsTotal) {
		const int cnt = G.cellCount[c];
		if (cnt == 0) continue;
		const Block b = make_block(G, c);
		const int st = G.cellStart[c];
		if (b.L > kMpnnStage) {
			if (lane == 0) atomicOr(error, 2u);
			for (int jj = 0; jj < cnt; ++jj) {
#pragma unroll
				for (int q = 0; q < 4; ++q) Hb[(size_t)(st + jj) * kHidden + lane + 32 * q] = __float2bfloat16_rn(0.f);
				if (lane == 0) degS[st + jj] = 0.f;
			}
			continue;
		}
		stage_block(S, b, G, z, lane);
		for (int jj = 0; jj < cnt; ++jj) {
			const int self = b.own + jj;
			const float2 xi = S.pos[self], zi = S.z[self];
			float acc[4] = {0.f, 0.f, 0.f, 0.f};
			int deg = 0;
			for (int base = 0; base < b.L; base += kWarp) {
				const int m = edge_group(S, b, base, self, xi, zi, h2, G.invH, lane);
				for (int q = 0; q < m; ++q) {
					float fe[kEdgeIn];
					load_feat(S, q, fe);
#pragma unroll
					for (int u = 0; u < 4; ++u) {
						float a = bias[u];
#pragma unroll
						for (int k = 0; k < kEdgeIn; ++k) a += w[u][k] * fe[k];
						acc[u] += fmaxf(a, 0.f);
					}
				}
				deg += m;
				__syncwarp();
			}
			const int i = st + jj;
#pragma unroll
			for (int q = 0; q < 4; ++q) Hb[(size_t)i * kHidden + lane + 32 * q] = __float2bfloat16_rn(acc[q] * kAggScale);
			if (lane == 0) degS[i] = (float)deg * kAggScale;
		}
		__syncwarp();
	}
	// Padding rows [n, np) are zero.
	const int tail = (np - G.n) * kHidden;
	for (int t = (blockIdx.x * blockDim.x + threadIdx.x); t < tail; t += gridDim.x * blockDim.x) {
		Hb[(size_t)G.n * kHidden + t] = __float2bfloat16_rn(0.f);
		if (t % kHidden == 0) degS[G.n + t / kHidden] = 0.f;
	}
}

// ---------------------------------------------------------------------------
// Edge layer 1 on the tensor cores (tcgen05.mma kind::tf32).
//
// A CTA of four warps takes cells in turn and stages each cell's 3x3 block;
// the cell's particles go in batches of up to kTcBatch.  A batch's in-range
// edges form a stream of columns, particle by particle in block order, each
// particle's run padded with zero columns to a multiple of 8 (at least 8).
// Per tile of up to kTcCols columns, thread t writes column t's operand row
// E = [e_ij, 1, 0] (TF32) into shared memory and one thread issues
//     D[f, e] = sum_k W1'[f, k] E[e, k]      M = 128 features, N = kTcCols,
//                                            K = 8, FP32 accumulator in TMEM
// with W1' = [W1 | b1 | 0] (TF32), so that D = W1 e + b1 and a zero column
// gives 0.  Thread f then reads TMEM lane f (warp w owns lanes
// 32w..32w+31), 32 columns per load, and sums relu(D) along the stream with
// packed FP32 adds, 8 columns at a time, writing H_i = sum / S where a run
// ends (a run may span tiles).  The per-particle sums stay on the CUDA
// cores: a second MMA would contract over edges, 16 per instruction, and a
// tcgen05.mma costs ~100 cycles whatever its N.  Four CTAs share an SM's
// 512 TMEM columns and overlap one another's phases.  Thread 0 waits for
// the MMA (bounded) while the other threads wait at the CTA barrier; if the
// wait runs out the CTA stops, flags the error, waits (bounded) once more
// for the tensor core and frees its tensor memory.

namespace {

constexpr int kTcThreads = 128;
constexpr int kTcCols = 128;       // columns per tile = TMEM columns per CTA
constexpr int kTcBatch = 8;        // particles per batch
constexpr int kTcRowBytes = 32;    // 8 TF32 values per operand row
constexpr int kTcGroupBytes = 8 * kTcRowBytes;  // one 8-row group of core matrices
constexpr int kTcChunks = kTcCols / 8;
constexpr int kTcMaxChunks = kTcBatch * (kMpnnStage / 8 + 1);  // of a batch
constexpr int kTcBlocksPerSm = 4;  // 4 x 128 TMEM columns = an SM's 512

struct __align__(128) EdgeTcSmem {
	unsigned char a[kHidden * kTcRowBytes];  // W1' rows, core-matrix layout
	unsigned char b[kTcCols * kTcRowBytes];  // the tile's edge rows, core-matrix layout
	float2 pos[kMpnnStage];
	float2 z[kMpnnStage];
	uint16_t list[kTcBatch][kMpnnStage];  // each batch particle's in-range block entries
	uint8_t owner[kTcMaxChunks];          // batch particle of each 8-column chunk
	int8_t endp[kTcMaxChunks];            // batch particle whose run ends with the chunk, or -1
	int deg[kTcBatch];
	int colStart[kTcBatch + 1];  // run starts; past the batch: the batch's column count
	unsigned long long bar;
	uint32_t tmem;
	int ok;                      // thread 0's verdict on the MMA wait
};

__device__ __forceinline__ unsigned char *tc_row(unsigned char *base, int r) {
	return base + (r >> 3) * kTcGroupBytes + (r & 7) * 16;
}

// Sum of relu over 8 columns, as two partial sums.
__device__ __forceinline__ float2 relu_sum8(const uint32_t *v) {
	float r[8];
#pragma unroll
	for (int q = 0; q < 8; ++q) r[q] = fmaxf(__uint_as_float(v[q]), 0.f);
	const float2 a = __fadd2_rn(make_float2(r[0], r[1]), make_float2(r[2], r[3]));
	const float2 b = __fadd2_rn(make_float2(r[4], r[5]), make_float2(r[6], r[7]));
	return __fadd2_rn(a, b);
}

}  // namespace

size_t mpnn_edge_tc_smem() {
	// At least 48 KiB, so that no more than four CTAs (all of the SM's
	// tensor memory) are resident on an SM.
	return sizeof(EdgeTcSmem) > 48 * 1024 ? sizeof(EdgeTcSmem) : 48 * 1024;
}

int mpnn_edge_tc_blocks_per_sm() { return kTcBlocksPerSm; }
int mpnn_edge_tc_threads() { return kTcThreads; }

__global__ void __launch_bounds__(kTcThreads, kTcBlocksPerSm)
    k_mpnn_edge_fwd_tc(MpnnGraph G, const float *W1, const float *b1, const float2 *z, __nv_bfloat16 *Hb,
                       float *degS, int np, uint32_t *error) {
	extern __shared__ __align__(1024) unsigned char smem_raw[];
	EdgeTcSmem &S = *reinterpret_cast<EdgeTcSmem *>(smem_raw);
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	{
		// W1' row f = tid.
		const int f = tid;
		float w[kEdgeIn];
#pragma unroll
		for (int k = 0; k < kEdgeIn; ++k) w[k] = tc::to_tf32(W1[f * kEdgeIn + k]);
		unsigned char *row = tc_row(S.a, f);
		*reinterpret_cast<float4 *>(row) = make_float4(w[0], w[1], w[2], w[3]);
		*reinterpret_cast<float4 *>(row + 128) = make_float4(w[4], w[5], tc::to_tf32(b1[f]), 0.f);
	}
	if (tid == 0) {
		tc::mbar_init(&S.bar, 1);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 0) tc::tmem_alloc(&S.tmem, kTcCols);
	tc::fence_async_smem();
	tc::fence_before();
	__syncthreads();
	tc::fence_after();
	const uint32_t tmem = S.tmem;
	const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);
	const uint64_t descA = tc::desc_noswizzle(tc::smem_u32(S.a), 128, kTcGroupBytes);
	const uint64_t descB = tc::desc_noswizzle(tc::smem_u32(S.b), 128, kTcGroupBytes);
	const uint32_t idesc = tc::idesc_tf32(kHidden, kTcCols);
	uint32_t phase = 0;
	bool good = true;
	const float h2 = __fmul_rn(G.h, G.h);
	const int ncell = G.gx * G.gy;
	for (int c = blockIdx.x; good && c < ncell; c += gridDim.x) {
		const int cnt = G.cellCount[c];
		if (cnt == 0) continue;
		const Block b = make_block(G, c);
		const int st = G.cellStart[c];
		if (b.L > kMpnnStage) {
			if (tid == 0) atomicOr(error, 2u);
			for (int t = tid; t < cnt * kHidden; t += kTcThreads)
				Hb[(size_t)st * kHidden + t] = __float2bfloat16_rn(0.f);
			for (int t = tid; t < cnt; t += kTcThreads) degS[st + t] = 0.f;
			continue;
		}
		for (int e = tid; e < b.L; e += kTcThreads) {
			const int num = block_number(b, e);
			S.pos[e] = G.pos[num];
			S.z[e] = z[num];
		}
		__syncthreads();
		for (int jb = 0; good && jb < cnt; jb += kTcBatch) {
			const int nb = min(kTcBatch, cnt - jb);
			// In-range block entries of each batch particle (warp w takes
			// particles w and w + 4), in block order, with the same unfused
			// distance test as the plain step's neighbour search.
			for (int p = warp; p < nb; p += kTcThreads / kWarp) {
				const int self = b.own + jb + p;
				const float2 xi = S.pos[self];
				int deg = 0;
				for (int base = 0; base < b.L; base += kWarp) {
					const int e = base + lane;
					bool in = false;
					if (e < b.L && e != self) {
						const float2 xj = S.pos[e];
						const float dx = xj.x - xi.x, dy = xj.y - xi.y;
						in = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) < h2;
					}
					const unsigned mask = __ballot_sync(kFull, in);
					if (in) S.list[p][deg + __popc(mask & lanemask_lt())] = (uint16_t)e;
					deg += __popc(mask);
				}
				if (lane == 0) {
					S.deg[p] = deg;
					degS[st + jb + p] = (float)deg * kAggScale;
				}
			}
			__syncthreads();
			if (tid == 0) {
				int acc = 0;
				for (int p = 0; p <= kTcBatch; ++p) {
					S.colStart[p] = acc;
					if (p < nb) acc += max(8, (S.deg[p] + 7) & ~7);
				}
			}
			__syncthreads();
			int cs[kTcBatch + 1];
#pragma unroll
			for (int p = 0; p <= kTcBatch; ++p) cs[p] = S.colStart[p];
			const int cols = cs[kTcBatch];
			for (int ch = tid; ch < cols / 8; ch += kTcThreads) {
				int p = 0;
#pragma unroll
				for (int q = 1; q < kTcBatch; ++q) p += ch * 8 >= cs[q] ? 1 : 0;
				S.owner[ch] = (uint8_t)p;
				S.endp[ch] = (int8_t)(ch * 8 + 8 == S.colStart[p + 1] ? p : -1);
			}
			__syncthreads();
			float2 acc = make_float2(0.f, 0.f);
			for (int t0 = 0; t0 < cols; t0 += kTcCols) {
				const int ncol = min(kTcCols, cols - t0);
				{
					const int col = t0 + tid;
					float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
					if (col < cols) {
						const int p = S.owner[col >> 3];
						const int k = col - S.colStart[p];
						if (k < S.deg[p]) {
							const int self = b.own + jb + p;
							const int j = S.list[p][k];
							const float2 xi = S.pos[self], zi = S.z[self], xj = S.pos[j], zj = S.z[j];
							const float dx = xj.x - xi.x, dy = xj.y - xi.y;
							const float r = sqrtf(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
							const float q = r * G.invH;
							lo = make_float4(tc::to_tf32(dx * G.invH), tc::to_tf32(dy * G.invH), tc::to_tf32(q),
							                 tc::to_tf32(zj.x - zi.x));
							hi = make_float4(tc::to_tf32(zj.y - zi.y), tc::to_tf32((1.0f - q) * (1.0f - q)), 1.0f, 0.f);
						}
					}
					unsigned char *row = tc_row(S.b, tid);
					*reinterpret_cast<float4 *>(row) = lo;
					*reinterpret_cast<float4 *>(row + 128) = hi;
				}
				tc::fence_async_smem();
				__syncthreads();
				if (tid == 0) {
					tc::fence_after();
					tc::mma_tf32(tmem, descA, descB, idesc, false);
					tc::commit(&S.bar);
					S.ok = tc::mbar_wait(&S.bar, phase);
				}
				phase ^= 1;
				__syncthreads();
				if (!S.ok) {
					good = false;
					break;
				}
				tc::fence_after();
#pragma unroll
				for (int half = 0; half < 2; ++half) {
					const int c0 = half * (kTcCols / 2);
					if (c0 < ncol) {
						uint32_t v[kTcCols / 2];
						tc::tmem_ld32(tlane + (uint32_t)c0, *reinterpret_cast<uint32_t(*)[32]>(v));
						tc::tmem_ld32(tlane + (uint32_t)(c0 + 32), *reinterpret_cast<uint32_t(*)[32]>(v + 32));
						tc::tmem_wait_ld();
#pragma unroll
						for (int q = 0; q < kTcChunks / 2; ++q) {
							acc = __fadd2_rn(acc, relu_sum8(v + 8 * q));
							const int ch = (t0 + c0) / 8 + q;
							if (ch < cols / 8) {
								const int pe = S.endp[ch];
								if (pe >= 0) {
									Hb[(size_t)(st + jb + pe) * kHidden + tid] =
									    __float2bfloat16_rn((acc.x + acc.y) * kAggScale);
									acc = make_float2(0.f, 0.f);
								}
							}
						}
					}
				}
				tc::fence_before();
				__syncthreads();
			}
		}
	}
	// Padding rows [n, np) are zero.
	const int tail = (np - G.n) * kHidden;
	for (int t = blockIdx.x * kTcThreads + tid; t < tail; t += gridDim.x * kTcThreads)
		Hb[(size_t)G.n * kHidden + t] = __float2bfloat16_rn(0.f);
	if (!good && tid == 0) {
		atomicOr(error, 1u);
		// The tensor core may still be working on the last tile: wait for
		// it (bounded) before the tensor memory is freed.
		tc::mbar_wait(&S.bar, phase ^ 1);
	}
	tc::fence_before();
	__syncthreads();
	if (warp == 0) tc::tmem_free(tmem, kTcCols);
}

// Backward of the edge layer: dW1, db1 from every edge (i aggregates j),
// and, if needDz, the node-state gradient through the z_j - z_i features.
// Per group of edges, each lane's share of the two node-state components is
// summed across lanes through shared memory (lane q then owns edge q and
// scatters its +share to the neighbour with atomics).
__global__ void __launch_bounds__(kEdgeWarps * kWarp) k_mpnn_edge_bwd(MpnnGraph G, const float *W1, const float *b1,
                                                                     const float2 *z, const float *dH, float2 *dzEdge,
                                                                     float *gW1, float *gb1, int needDz,
                                                                     uint32_t *error) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	EdgeWarpBwd &SB = reinterpret_cast<EdgeWarpBwd *>(smem_raw)[threadIdx.x / kWarp];
	EdgeWarp &S = SB.core;
	const int lane = threadIdx.x & (kWarp - 1);
	float w[4][kEdgeIn], bias[4];
	float gw[4][kEdgeIn], gb[4];
#pragma unroll
	for (int q = 0; q < 4; ++q) {
		const int f = lane + 32 * q;
#pragma unroll
		for (int k = 0; k < kEdgeIn; ++k) {
			w[q][k] = tc::to_tf32(W1[f * kEdgeIn + k]);
			gw[q][k] = 0.f;
		}
		bias[q] = tc::to_tf32(b1[f]);
		gb[q] = 0.f;
	}
	const float h2 = __fmul_rn(G.h, G.h);
	const int ncell = G.gx * G.gy;
	const int warpsTotal = gridDim.x * kEdgeWarps;
	for (int c = blockIdx.x * kEdgeWarps + threadIdx.x / kWarp; c < ncell; c += warpsTotal) {
		const int cnt = G.cellCount[c];
		if (cnt == 0) continue;
		const Block b = make_block(G, c);
		if (b.L > kMpnnStage) {
			if (lane == 0) atomicOr(error, 2u);
			continue;
		}
		stage_block(S, b, G, z, lane);
		const int st = G.cellStart[c];
		for (int jj = 0; jj < cnt; ++jj) {
			const int self = b.own + jj;
			const int i = st + jj;
			const float2 xi = S.pos[self], zi = S.z[self];
			float g[4];
#pragma unroll
			for (int q = 0; q < 4; ++q) g[q] = dH[(size_t)i * kHidden + lane + 32 * q] * kAggScale;
			float dzx = 0.f, dzy = 0.f;  // lane q: minus the shares of the edges it owned
			for (int base = 0; base < b.L; base += kWarp) {
				const int m = edge_group(S, b, base, self, xi, zi, h2, G.invH, lane);
				for (int q = 0; q < m; ++q) {
					float fe[kEdgeIn];
					load_feat(S, q, fe);
					float d3 = 0.f, d4 = 0.f;
#pragma unroll
					for (int u = 0; u < 4; ++u) {
						float a = bias[u];
#pragma unroll
						for (int k = 0; k < kEdgeIn; ++k) a += w[u][k] * fe[k];
						const float da = a > 0.f ? g[u] : 0.f;
#pragma unroll
						for (int k = 0; k < kEdgeIn; ++k) gw[u][k] += da * fe[k];
						gb[u] += da;
						d3 += w[u][3] * da;
						d4 += w[u][4] * da;
					}
					if (needDz) {
						SB.part[0][q][lane] = d3;
						SB.part[1][q][lane] = d4;
					}
				}
				if (needDz) {
					__syncwarp();
					if (lane < m) {
						float s3 = 0.f, s4 = 0.f;
						for (int t = 0; t < kWarp; ++t) {
							s3 += SB.part[0][lane][t];
							s4 += SB.part[1][lane][t];
						}
						const int j = S.nbr[lane];
						atomicAdd(&dzEdge[j].x, s3);
						atomicAdd(&dzEdge[j].y, s4);
						dzx -= s3;
						dzy -= s4;
					}
				}
				__syncwarp();
			}
			if (needDz) {
				dzx = warp_sum(dzx);
				dzy = warp_sum(dzy);
				if (lane == 0) {
					atomicAdd(&dzEdge[i].x, dzx);
					atomicAdd(&dzEdge[i].y, dzy);
				}
			}
		}
		__syncwarp();
	}
#pragma unroll
	for (int q = 0; q < 4; ++q) {
		const int f = lane + 32 * q;
#pragma unroll
		for (int k = 0; k < kEdgeIn; ++k)
			if (gw[q][k] != 0.f) atomicAdd(&gW1[f * kEdgeIn + k], gw[q][k]);
		if (gb[q] != 0.f) atomicAdd(&gb1[f], gb[q]);
	}
}

// Node-MLP input columns 128..143: z, then zeros (row-major and, if given,
// feature-major).
__global__ void k_mpnn_x3_tail(const float2 *z, __nv_bfloat16 *X3b, __nv_bfloat16 *X3f, int np, int ldf) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= np) return;
	const float2 zi = z[i];
	for (int k = kHidden; k < kNodeInPad; ++k) {
		const float v = k == kHidden ? zi.x : (k == kHidden + 1 ? zi.y : 0.f);
		const __nv_bfloat16 b = __float2bfloat16_rn(v);
		X3b[(size_t)i * kNodeInPad + k] = b;
		if (X3f) X3f[(size_t)k * ldf + i] = b;
	}
}

// z_out = z_in + W4 c + b4.
__global__ void k_mpnn_node_out(const __nv_bfloat16 *cb, const float *W4, const float *b4, const float2 *zin,
                                float2 *zout, int np) {
	__shared__ float w[2 * kHidden];
	for (int t = threadIdx.x; t < 2 * kHidden; t += blockDim.x) w[t] = W4[t];
	__syncthreads();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= np) return;
	const uint4 *row = reinterpret_cast<const uint4 *>(cb + (size_t)i * kHidden);
	float s0 = b4[0], s1 = b4[1];
	for (int v = 0; v < kHidden / 8; ++v) {
		const uint4 pk = row[v];
		const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&pk);
#pragma unroll
		for (int u = 0; u < 8; ++u) {
			const float c = __bfloat162float(e[u]);
			s0 += w[v * 8 + u] * c;
			s1 += w[kHidden + v * 8 + u] * c;
		}
	}
	const float2 z = zin[i];
	zout[i] = make_float2(z.x + s0, z.y + s1);
}

// Loss sum_i |u_i - t_i|^2 (accumulated; the mean is taken on the host) and
// its gradient 2 (u - t) / n on [0, n), zero on the padding.
__global__ void k_mpnn_loss(const float2 *z2, const float2 *z0, const float2 *target, float2 *dz, int n, int np,
                            float *loss) {
	__shared__ float part[256];
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	float l = 0.f;
	if (i < n) {
		const float ux = z2[i].x - z0[i].x, uy = z2[i].y - z0[i].y;
		const float ex = ux - target[i].x, ey = uy - target[i].y;
		dz[i] = make_float2(2.f * ex / (float)n, 2.f * ey / (float)n);
		l = ex * ex + ey * ey;
	} else if (i < np) {
		dz[i] = make_float2(0.f, 0.f);
	}
	part[threadIdx.x] = l;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0 && part[0] != 0.f) atomicAdd(loss, part[0]);
}

// da3 = (W4^T dz) * [c > 0], one warp per particle.
__global__ void k_mpnn_node_bwd(const float2 *dz, const float *W4, const __nv_bfloat16 *cb, __nv_bfloat16 *da3b,
                                int np) {
	const int i = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
	const int lane = threadIdx.x & (kWarp - 1);
	if (i >= np) return;
	const float2 g = dz[i];
#pragma unroll
	for (int q = 0; q < 4; ++q) {
		const int f = lane + 32 * q;
		const float dc = W4[f] * g.x + W4[kHidden + f] * g.y;
		const float c = __bfloat162float(cb[(size_t)i * kHidden + f]);
		da3b[(size_t)i * kHidden + f] = __float2bfloat16_rn(c > 0.f ? dc : 0.f);
	}
}

// gW4[o][f] += sum_i dz_i[o] c_i[f]; block f (one per hidden feature); block
// 0 also adds gb4 += sum_i dz_i.
__global__ void k_mpnn_dw4(const float2 *dz, const __nv_bfloat16 *cf, int ldf, int n, float *gW4, float *gb4) {
	__shared__ float p0[256], p1[256], q0[256], q1[256];
	const int f = blockIdx.x;
	float a0 = 0.f, a1 = 0.f, s0 = 0.f, s1 = 0.f;
	for (int i = threadIdx.x; i < n; i += blockDim.x) {
		const float2 g = dz[i];
		const float c = __bfloat162float(cf[(size_t)f * ldf + i]);
		a0 += g.x * c;
		a1 += g.y * c;
		s0 += g.x;
		s1 += g.y;
	}
	p0[threadIdx.x] = a0;
	p1[threadIdx.x] = a1;
	q0[threadIdx.x] = s0;
	q1[threadIdx.x] = s1;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) {
			p0[threadIdx.x] += p0[threadIdx.x + o];
			p1[threadIdx.x] += p1[threadIdx.x + o];
			q0[threadIdx.x] += q0[threadIdx.x + o];
			q1[threadIdx.x] += q1[threadIdx.x + o];
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		gW4[f] += p0[0];
		gW4[kHidden + f] += p1[0];
		if (f == 0) {
			gb4[0] += q0[0];
			gb4[1] += q1[0];
		}
	}
}

// out[r] += sum_{i<n} X[r][i] (* w[i]); one block per row.
__global__ void k_mpnn_rowsum(const __nv_bfloat16 *X, int ld, int n, const float *w, float *out) {
	__shared__ float part[256];
	const int r = blockIdx.x;
	float s = 0.f;
	for (int i = threadIdx.x; i < n; i += blockDim.x) {
		const float x = __bfloat162float(X[(size_t)r * ld + i]);
		s += w ? x * w[i] : x;
	}
	part[threadIdx.x] = s;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) out[r] += part[0];
}

// dz_r = dz_{r+1} + (dX3 columns of z) + edge term, zero on the padding.
__global__ void k_mpnn_combine(const float2 *dzNext, const float *dX, const float2 *dzEdge, float2 *dz, int n,
                               int np) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= np) return;
	if (i >= n) {
		dz[i] = make_float2(0.f, 0.f);
		return;
	}
	const float2 a = dzNext[i], e = dzEdge[i];
	const float *row = dX + (size_t)i * kNodeInPad;
	dz[i] = make_float2(a.x + row[kHidden] + e.x, a.y + row[kHidden + 1] + e.y);
}

// dst[c][r] = src[r][c] for a rows x cols bf16 matrix (32x32 tiles).
__global__ void k_mpnn_transpose(const __nv_bfloat16 *src, int rows, int cols, int lds, __nv_bfloat16 *dst, int ldd) {
	__shared__ __nv_bfloat16 tile[32][33];
	const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
	for (int y = threadIdx.y; y < 32; y += blockDim.y) {
		const int r = r0 + y, c = c0 + threadIdx.x;
		if (r < rows && c < cols) tile[y][threadIdx.x] = src[(size_t)r * lds + c];
	}
	__syncthreads();
	for (int y = threadIdx.y; y < 32; y += blockDim.y) {
		const int c = c0 + y, r = r0 + threadIdx.x;
		if (r < rows && c < cols) dst[(size_t)c * ldd + r] = tile[threadIdx.x][y];
	}
}

// Adam (Kingma & Ba 2015) with optional gradient clipping by value.
__global__ void k_mpnn_adam(float *p, const float *g, float *m, float *v, int count, float lr, float beta1,
                            float beta2, float eps, float bc1, float bc2, float clip) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= count) return;
	float gi = g[i];
	if (clip > 0.f) gi = fminf(fmaxf(gi, -clip), clip);
	const float mi = beta1 * m[i] + (1.f - beta1) * gi;
	const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
	m[i] = mi;
	v[i] = vi;
	p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// BF16 copies of the GEMM weights of round blockIdx.y: W2, W2^T, W3, W3^T.
__global__ void k_mpnn_refresh(const float *p, __nv_bfloat16 *W2b, __nv_bfloat16 *W2Tb, __nv_bfloat16 *W3b,
                               __nv_bfloat16 *W3Tb) {
	const int r = blockIdx.y;
	const float *P = p + (size_t)r * kRoundParams;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t < kHidden * kHidden) {
		const int a = t / kHidden, b = t % kHidden;
		const __nv_bfloat16 x = __float2bfloat16_rn(P[kOffW2 + t]);
		W2b[(size_t)r * kHidden * kHidden + t] = x;
		W2Tb[(size_t)r * kHidden * kHidden + b * kHidden + a] = x;
	}
	if (t < kHidden * kNodeInPad) {
		const int a = t / kNodeInPad, b = t % kNodeInPad;
		const __nv_bfloat16 x = __float2bfloat16_rn(P[kOffW3 + t]);
		W3b[(size_t)r * kHidden * kNodeInPad + t] = x;
		W3Tb[(size_t)r * kHidden * kNodeInPad + b * kHidden + a] = x;
	}
}

__global__ void k_mpnn_u(const float2 *z2, const float2 *z0, float2 *u, int n) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	u[i] = make_float2(z2[i].x - z0[i].x, z2[i].y - z0[i].y);
}

size_t mpnn_edge_smem(bool backward) {
	return (backward ? sizeof(EdgeWarpBwd) : sizeof(EdgeWarp)) * kEdgeWarps;
}

}  // namespace sphgb
