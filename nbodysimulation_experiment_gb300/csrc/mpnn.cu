// Host side of the message-passing network: the model object (parameters,
// Adam state, activations, training samples) and the C entry points of
// include/sph_mpnn.h.  One model serves one device; its calls are not
// reentrant (activations and scratch are shared).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/sph_gb300.h"
#include "../../include/sph_mpnn.h"
#include "mpnn_internal.cuh"
#include "sph_internal.cuh"

using namespace sphgb;

namespace {

struct Sample {
	int n = 0, np = 0, gx = 0, gy = 0;
	float h = 0.f, invH = 0.f;
	float2 *pos = nullptr, *z0 = nullptr, *target = nullptr;
	int *cellStart = nullptr, *cellCount = nullptr, *ids = nullptr;
	MpnnGraph graph() const {
		MpnnGraph g;
		g.pos = pos;
		g.z0 = z0;
		g.cellStart = cellStart;
		g.cellCount = cellCount;
		g.n = n;
		g.gx = gx;
		g.gy = gy;
		g.h = h;
		g.invH = invH;
		return g;
	}
	void release() {
		void *p[] = {pos, z0, target, cellStart, cellCount, ids};
		for (void *q : p)
			if (q) cudaFree(q);
	}
};

#define MPNN_CUDA(call)                                 \
	do {                                                \
		cudaError_t e_ = (call);                        \
		if (e_ != cudaSuccess) return SPH_ERR_CUDA;     \
	} while (0)

template <typename T>
int zalloc(T **p, size_t count) {
	if (cudaMalloc(reinterpret_cast<void **>(p), std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess)
		return SPH_ERR_CUDA;
	return cudaMemset(*p, 0, std::max<size_t>(count, 1) * sizeof(T)) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

// splitmix64: the seeded source of the initial weights.
uint64_t splitmix(uint64_t &s) {
	uint64_t z = (s += 0x9e3779b97f4a7c15ull);
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}

int blocks(size_t items, int threads) { return (int)std::max<size_t>(1, (items + threads - 1) / threads); }

}  // namespace

struct sph_mpnn {
	int device = 0;
	cudaStream_t stream = nullptr;
	size_t cap = 0;  // padded particle capacity
	float *params = nullptr, *grads = nullptr, *adamM = nullptr, *adamV = nullptr;
	int adamStep = 0;
	__nv_bfloat16 *W2b = nullptr, *W2Tb = nullptr, *W3b = nullptr, *W3Tb = nullptr;
	__nv_bfloat16 *Hb[kRounds] = {}, *Hf[kRounds] = {}, *X3b[kRounds] = {}, *X3f[kRounds] = {};
	__nv_bfloat16 *cb[kRounds] = {}, *cf[kRounds] = {};
	float *degS = nullptr;
	float2 *z[kRounds + 1] = {};  // z[0] unused (the graph's z0)
	float2 *dz[kRounds + 1] = {};
	float2 *dzEdge = nullptr, *u = nullptr;
	__nv_bfloat16 *da3b = nullptr, *da3f = nullptr, *dXb = nullptr, *dXf = nullptr;
	float *dX = nullptr, *dH = nullptr;
	float *loss = nullptr;
	uint32_t *error = nullptr;
	int edgePath = 0;  // 0: edge layer on the tensor cores, 1: on the CUDA cores
	int sms = 0;
	std::vector<Sample> samples;
};

namespace {

GemmArgs gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K, uint32_t *err) {
	GemmArgs g{};
	g.A = A;
	g.B = B;
	g.M = M;
	g.N = N;
	g.K = K;
	g.lda = lda;
	g.ldb = ldb;
	g.error = err;
	return g;
}

int run_gemm(const GemmArgs &g, int splits, cudaStream_t st) {
	if (gemm_check(g, splits) != 0) return SPH_ERR_INVALID_ARGUMENT;
	return gemm_launch(g, splits, st) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

int split_for(int k) { return std::max(1, std::min(64, k / 4096)); }

int refresh(sph_mpnn *m, cudaStream_t st) {
	dim3 grid(blocks(kHidden * kNodeInPad, 256), kRounds);
	k_mpnn_refresh<<<grid, 256, 0, st>>>(m->params, m->W2b, m->W2Tb, m->W3b, m->W3Tb);
	return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}


int edge_blocks(const MpnnGraph &g) { return blocks((size_t)g.gx * g.gy, kEdgeWarps); }

// Forward pass; `training` also writes the feature-major copies the
// backward pass needs.  Leaves z^1, z^2 in m->z.
int forward(sph_mpnn *m, const MpnnGraph &G, bool training, cudaStream_t st) {
	const int np = round_up128(G.n);
	if ((size_t)np > m->cap) return SPH_ERR_CAPACITY;
	const float2 *zin = G.z0;
	for (int r = 0; r < kRounds; ++r) {
		const float *P = m->params + (size_t)r * kRoundParams;
		if (m->edgePath == 0) {
			const int grid = std::max(1, std::min(G.gx * G.gy, mpnn_edge_tc_blocks_per_sm() * m->sms));
			k_mpnn_edge_fwd_tc<<<grid, mpnn_edge_tc_threads(), mpnn_edge_tc_smem(), st>>>(G, P + kOffW1, P + kOffB1, zin, m->Hb[r],
			                                                          m->degS, np, m->error);
		} else {
			k_mpnn_edge_fwd<<<edge_blocks(G), kEdgeWarps * kWarp, mpnn_edge_smem(false), st>>>(
			    G, P + kOffW1, P + kOffB1, zin, m->Hb[r], m->degS, np, m->error);
		}
		MPNN_CUDA(cudaGetLastError());
		if (training) {
			dim3 tg(blocks(kHidden, 32), blocks(np, 32));
			k_mpnn_transpose<<<tg, dim3(32, 8), 0, st>>>(m->Hb[r], np, kHidden, kHidden, m->Hf[r], np);
			MPNN_CUDA(cudaGetLastError());
		}
		// M = W2 H + (deg/S) b2, into the first 128 columns of X3.
		GemmArgs g1 = gemm(m->Hb[r], kHidden, m->W2b + (size_t)r * kHidden * kHidden, kHidden, np, kHidden, kHidden,
		                   m->error);
		g1.rowScale = m->degS;
		g1.bias2 = P + kOffB2;
		g1.Cb = m->X3b[r];
		g1.ldcb = kNodeInPad;
		if (training) {
			g1.CbT = m->X3f[r];
			g1.ldcbT = np;
		}
		int rc = run_gemm(g1, 1, st);
		if (rc) return rc;
		k_mpnn_x3_tail<<<blocks(np, 256), 256, 0, st>>>(zin, m->X3b[r], training ? m->X3f[r] : nullptr, np, np);
		MPNN_CUDA(cudaGetLastError());
		// c = relu(W3 [M, z] + b3).
		GemmArgs g2 = gemm(m->X3b[r], kNodeInPad, m->W3b + (size_t)r * kHidden * kNodeInPad, kNodeInPad, np, kHidden,
		                   kNodeInPad, m->error);
		g2.bias = P + kOffB3;
		g2.relu = 1;
		g2.Cb = m->cb[r];
		g2.ldcb = kHidden;
		if (training) {
			g2.CbT = m->cf[r];
			g2.ldcbT = np;
		}
		rc = run_gemm(g2, 1, st);
		if (rc) return rc;
		k_mpnn_node_out<<<blocks(np, 256), 256, 0, st>>>(m->cb[r], P + kOffW4, P + kOffB4, zin, m->z[r + 1], np);
		MPNN_CUDA(cudaGetLastError());
		zin = m->z[r + 1];
	}
	return SPH_OK;
}

// Loss against `target` and the gradient of every parameter into m->grads.
int backward(sph_mpnn *m, const MpnnGraph &G, const float2 *target, cudaStream_t st) {
	const int n = G.n, np = round_up128(n);
	MPNN_CUDA(cudaMemsetAsync(m->grads, 0, sizeof(float) * kParams, st));
	MPNN_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), st));
	k_mpnn_loss<<<blocks(np, 256), 256, 0, st>>>(m->z[kRounds], G.z0, target, m->dz[kRounds], n, np, m->loss);
	MPNN_CUDA(cudaGetLastError());
	const float2 *dzNext = m->dz[kRounds];
	const int splits = split_for(np);
	for (int r = kRounds - 1; r >= 0; --r) {
		const float *P = m->params + (size_t)r * kRoundParams;
		float *Gp = m->grads + (size_t)r * kRoundParams;
		const float2 *zr = r == 0 ? G.z0 : m->z[r];
		k_mpnn_node_bwd<<<blocks((size_t)np * kWarp, 256), 256, 0, st>>>(dzNext, P + kOffW4, m->cb[r], m->da3b, np);
		MPNN_CUDA(cudaGetLastError());
		dim3 tg(blocks(kHidden, 32), blocks(np, 32));
		k_mpnn_transpose<<<tg, dim3(32, 8), 0, st>>>(m->da3b, np, kHidden, kHidden, m->da3f, np);
		k_mpnn_dw4<<<kHidden, 256, 0, st>>>(dzNext, m->cf[r], np, n, Gp + kOffW4, Gp + kOffB4);
		k_mpnn_rowsum<<<kHidden, 256, 0, st>>>(m->da3f, np, n, nullptr, Gp + kOffB3);
		MPNN_CUDA(cudaGetLastError());
		// dW3 += da3^T X3 (reduction over particles).
		GemmArgs g3 = gemm(m->da3f, np, m->X3f[r], np, kHidden, kNodeInPad, np, m->error);
		g3.C = Gp + kOffW3;
		g3.ldc = kNodeInPad;
		g3.accumulate = 1;
		int rc = run_gemm(g3, splits, st);
		if (rc) return rc;
		// dX3 = da3 W3.
		GemmArgs g4 = gemm(m->da3b, kHidden, m->W3Tb + (size_t)r * kHidden * kNodeInPad, kHidden, np, kNodeInPad,
		                   kHidden, m->error);
		g4.C = m->dX;
		g4.ldc = kNodeInPad;
		g4.Cb = m->dXb;
		g4.ldcb = kNodeInPad;
		g4.CbT = m->dXf;
		g4.ldcbT = np;
		rc = run_gemm(g4, 1, st);
		if (rc) return rc;
		k_mpnn_rowsum<<<kHidden, 256, 0, st>>>(m->dXf, np, n, m->degS, Gp + kOffB2);
		MPNN_CUDA(cudaGetLastError());
		// dW2 += dM^T H.
		GemmArgs g5 = gemm(m->dXf, np, m->Hf[r], np, kHidden, kHidden, np, m->error);
		g5.C = Gp + kOffW2;
		g5.ldc = kHidden;
		g5.accumulate = 1;
		rc = run_gemm(g5, splits, st);
		if (rc) return rc;
		// dH = dM W2.
		GemmArgs g6 = gemm(m->dXb, kNodeInPad, m->W2Tb + (size_t)r * kHidden * kHidden, kHidden, np, kHidden,
		                   kHidden, m->error);
		g6.C = m->dH;
		g6.ldc = kHidden;
		rc = run_gemm(g6, 1, st);
		if (rc) return rc;
		MpnnGraph Gr = G;
		const int needDz = r > 0;
		if (needDz) MPNN_CUDA(cudaMemsetAsync(m->dzEdge, 0, sizeof(float2) * np, st));
		k_mpnn_edge_bwd<<<edge_blocks(G), kEdgeWarps * kWarp, mpnn_edge_smem(true), st>>>(
		    Gr, P + kOffW1, P + kOffB1, zr, m->dH, m->dzEdge, Gp + kOffW1, Gp + kOffB1, needDz, m->error);
		MPNN_CUDA(cudaGetLastError());
		if (needDz) {
			k_mpnn_combine<<<blocks(np, 256), 256, 0, st>>>(dzNext, m->dX, m->dzEdge, m->dz[r], n, np);
			MPNN_CUDA(cudaGetLastError());
			dzNext = m->dz[r];
		}
	}
	return SPH_OK;
}

int check_error(sph_mpnn *m, cudaStream_t st) {
	MPNN_CUDA(cudaStreamSynchronize(st));
	uint32_t err = 0;
	MPNN_CUDA(cudaMemcpy(&err, m->error, sizeof(err), cudaMemcpyDeviceToHost));
	if (err) {
		MPNN_CUDA(cudaMemset(m->error, 0, sizeof(err)));
		return (err & 1u) ? SPH_ERR_TIMEOUT : SPH_ERR_DEVICE_OVERFLOW;
	}
	return SPH_OK;
}

int read_loss(sph_mpnn *m, int n, float *loss) {
	float l = 0.f;
	MPNN_CUDA(cudaMemcpy(&l, m->loss, sizeof(l), cudaMemcpyDeviceToHost));
	if (loss) *loss = n > 0 ? l / (float)n : 0.f;
	return SPH_OK;
}

}  // namespace

namespace sphgb {

int mpnn_forward_dev(sph_mpnn *m, const MpnnGraph &g, float2 *u, cudaStream_t stream) {
	if (!m || !u) return SPH_ERR_INVALID_ARGUMENT;
	if (g.n == 0) return SPH_OK;
	int rc = forward(m, g, false, stream);
	if (rc) return rc;
	k_mpnn_u<<<blocks(g.n, 256), 256, 0, stream>>>(m->z[kRounds], g.z0, u, g.n);
	return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

int mpnn_add_sample(sph_mpnn *m, const MpnnGraph &g, cudaStream_t st, float2 **pos, float2 **target, int **ids) {
	if (!m || g.n <= 0) return SPH_ERR_INVALID_ARGUMENT;
	Sample s;
	s.n = g.n;
	s.np = round_up128(g.n);
	if ((size_t)s.np > m->cap) return SPH_ERR_CAPACITY;
	s.gx = g.gx;
	s.gy = g.gy;
	s.h = g.h;
	s.invH = g.invH;
	const size_t nc = (size_t)g.gx * g.gy;
	int rc;
	if ((rc = zalloc(&s.pos, s.np)) || (rc = zalloc(&s.z0, s.np)) || (rc = zalloc(&s.target, s.np)) ||
	    (rc = zalloc(&s.cellStart, nc)) || (rc = zalloc(&s.cellCount, nc)) || (rc = zalloc(&s.ids, s.n))) {
		s.release();
		return rc;
	}
	cudaError_t e = cudaMemcpyAsync(s.pos, g.pos, sizeof(float2) * s.n, cudaMemcpyDeviceToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(s.z0, g.z0, sizeof(float2) * s.np, cudaMemcpyDeviceToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(s.cellStart, g.cellStart, sizeof(int) * nc, cudaMemcpyDeviceToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(s.cellCount, g.cellCount, sizeof(int) * nc, cudaMemcpyDeviceToDevice, st);
	if (e != cudaSuccess) {
		s.release();
		return SPH_ERR_CUDA;
	}
	m->samples.push_back(s);
	*pos = s.pos;
	*target = s.target;
	*ids = s.ids;
	return SPH_OK;
}

size_t mpnn_capacity(const sph_mpnn *m) { return m ? m->cap : 0; }
int mpnn_device(const sph_mpnn *m) { return m ? m->device : -1; }

}  // namespace sphgb

extern "C" {

int sph_mpnn_param_count(size_t *out) {
	if (!out) return SPH_ERR_INVALID_ARGUMENT;
	*out = (size_t)kParams;
	return SPH_OK;
}

int sph_mpnn_destroy(sph_mpnn *m) {
	if (!m) return SPH_ERR_INVALID_ARGUMENT;
	cudaSetDevice(m->device);
	if (m->stream) cudaStreamSynchronize(m->stream);
	for (Sample &s : m->samples) s.release();
	std::vector<void *> ptrs = {m->params, m->grads, m->adamM, m->adamV, m->W2b, m->W2Tb, m->W3b, m->W3Tb,
	                            m->degS,   m->dzEdge, m->u,    m->da3b,  m->da3f, m->dXb, m->dXf, m->dX,
	                            m->dH,     m->loss,  m->error};
	for (int r = 0; r < kRounds; ++r) {
		ptrs.insert(ptrs.end(), {m->Hb[r], m->Hf[r], m->X3b[r], m->X3f[r], m->cb[r], m->cf[r]});
	}
	for (int r = 0; r <= kRounds; ++r) ptrs.insert(ptrs.end(), {m->z[r], m->dz[r]});
	for (void *p : ptrs)
		if (p) cudaFree(p);
	if (m->stream) cudaStreamDestroy(m->stream);
	delete m;
	return SPH_OK;
}

int sph_mpnn_create(int device, size_t max_particles, uint64_t seed, sph_mpnn **out) {
	if (!out || max_particles == 0 || max_particles > (1u << 26)) return SPH_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	int devices = 0;
	if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) return SPH_ERR_NO_DEVICE;
	if (device < 0 || device >= devices) return SPH_ERR_INVALID_ARGUMENT;
	if (cudaSetDevice(device) != cudaSuccess) return SPH_ERR_CUDA;
	sph_mpnn *m = new (std::nothrow) sph_mpnn();
	if (!m) return SPH_ERR_CAPACITY;
	m->device = device;
	m->cap = (size_t)round_up128((int)max_particles);
	const size_t C = m->cap;
	int rc = SPH_OK;
	auto fail = [&](int code) {
		sph_mpnn_destroy(m);
		return code;
	};
	if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(SPH_ERR_CUDA);
	if (cudaFuncSetAttribute(k_mpnn_edge_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                         (int)mpnn_edge_smem(false)) != cudaSuccess ||
	    cudaFuncSetAttribute(k_mpnn_edge_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                         (int)mpnn_edge_smem(true)) != cudaSuccess ||
	    cudaFuncSetAttribute(k_mpnn_edge_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                         (int)mpnn_edge_tc_smem()) != cudaSuccess ||
	    cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
		return fail(SPH_ERR_CUDA);
	if ((rc = zalloc(&m->params, kParams)) || (rc = zalloc(&m->grads, kParams)) || (rc = zalloc(&m->adamM, kParams)) ||
	    (rc = zalloc(&m->adamV, kParams)) || (rc = zalloc(&m->W2b, kRounds * kHidden * kHidden)) ||
	    (rc = zalloc(&m->W2Tb, kRounds * kHidden * kHidden)) || (rc = zalloc(&m->W3b, kRounds * kHidden * kNodeInPad)) ||
	    (rc = zalloc(&m->W3Tb, kRounds * kHidden * kNodeInPad)) || (rc = zalloc(&m->degS, C)) ||
	    (rc = zalloc(&m->dzEdge, C)) || (rc = zalloc(&m->u, C)) || (rc = zalloc(&m->da3b, C * kHidden)) ||
	    (rc = zalloc(&m->da3f, C * kHidden)) || (rc = zalloc(&m->dXb, C * kNodeInPad)) ||
	    (rc = zalloc(&m->dXf, C * kNodeInPad)) || (rc = zalloc(&m->dX, C * kNodeInPad)) ||
	    (rc = zalloc(&m->dH, C * kHidden)) || (rc = zalloc(&m->loss, 1)) || (rc = zalloc(&m->error, 1)))
		return fail(rc);
	for (int r = 0; r < kRounds; ++r) {
		if ((rc = zalloc(&m->Hb[r], C * kHidden)) || (rc = zalloc(&m->Hf[r], C * kHidden)) ||
		    (rc = zalloc(&m->X3b[r], C * kNodeInPad)) || (rc = zalloc(&m->X3f[r], C * kNodeInPad)) ||
		    (rc = zalloc(&m->cb[r], C * kHidden)) || (rc = zalloc(&m->cf[r], C * kHidden)))
			return fail(rc);
	}
	for (int r = 0; r <= kRounds; ++r)
		if ((rc = zalloc(&m->z[r], C)) || (rc = zalloc(&m->dz[r], C))) return fail(rc);
	// Uniform(+-1/sqrt(fan_in)) weights, zero biases, output layer scaled by
	// 0.1 so that an untrained network predicts small corrections.
	std::vector<float> p(kParams, 0.f);
	uint64_t st = seed;
	auto uni = [&](float lim) {
		const double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
		return (float)((2.0 * u - 1.0) * lim);
	};
	for (int r = 0; r < kRounds; ++r) {
		float *P = p.data() + (size_t)r * kRoundParams;
		for (int i = 0; i < kHidden * kEdgeIn; ++i) P[kOffW1 + i] = uni(1.0f / std::sqrt((float)kEdgeIn));
		for (int i = 0; i < kHidden * kHidden; ++i) P[kOffW2 + i] = uni(1.0f / std::sqrt((float)kHidden));
		for (int a = 0; a < kHidden; ++a)
			for (int b = 0; b < kNodeIn; ++b) P[kOffW3 + a * kNodeInPad + b] = uni(1.0f / std::sqrt((float)kNodeIn));
		for (int i = 0; i < 2 * kHidden; ++i) P[kOffW4 + i] = 0.1f * uni(1.0f / std::sqrt((float)kHidden));
	}
	if (cudaMemcpy(m->params, p.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice) != cudaSuccess)
		return fail(SPH_ERR_CUDA);
	if ((rc = refresh(m, m->stream)) || (rc = check_error(m, m->stream))) return fail(rc);
	*out = m;
	return SPH_OK;
}

int sph_mpnn_get_params(sph_mpnn *m, float *out) {
	if (!m || !out) return SPH_ERR_INVALID_ARGUMENT;
	MPNN_CUDA(cudaStreamSynchronize(m->stream));
	MPNN_CUDA(cudaMemcpy(out, m->params, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
	return SPH_OK;
}

int sph_mpnn_set_params(sph_mpnn *m, const float *in) {
	if (!m || !in) return SPH_ERR_INVALID_ARGUMENT;
	MPNN_CUDA(cudaStreamSynchronize(m->stream));
	std::vector<float> p(in, in + kParams);
	for (int r = 0; r < kRounds; ++r)  // the padding columns of W3 stay zero
		for (int a = 0; a < kHidden; ++a)
			for (int b = kNodeIn; b < kNodeInPad; ++b) p[(size_t)r * kRoundParams + kOffW3 + a * kNodeInPad + b] = 0.f;
	MPNN_CUDA(cudaMemcpy(m->params, p.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice));
	MPNN_CUDA(cudaMemset(m->adamM, 0, sizeof(float) * kParams));
	MPNN_CUDA(cudaMemset(m->adamV, 0, sizeof(float) * kParams));
	m->adamStep = 0;
	int rc = refresh(m, m->stream);
	return rc ? rc : check_error(m, m->stream);
}

int sph_mpnn_set_edge_path(sph_mpnn *m, int path) {
	if (!m || (path != 0 && path != 1)) return SPH_ERR_INVALID_ARGUMENT;
	MPNN_CUDA(cudaStreamSynchronize(m->stream));
	m->edgePath = path;
	return SPH_OK;
}

int sph_mpnn_get_edge_path(sph_mpnn *m, int *path) {
	if (!m || !path) return SPH_ERR_INVALID_ARGUMENT;
	*path = m->edgePath;
	return SPH_OK;
}

int sph_mpnn_sample_count(sph_mpnn *m, size_t *out) {
	if (!m || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = m->samples.size();
	return SPH_OK;
}

int sph_mpnn_clear_samples(sph_mpnn *m) {
	if (!m) return SPH_ERR_INVALID_ARGUMENT;
	MPNN_CUDA(cudaDeviceSynchronize());
	for (Sample &s : m->samples) s.release();
	m->samples.clear();
	return SPH_OK;
}

int sph_mpnn_sample_info(sph_mpnn *m, size_t index, size_t *n, int *gx, int *gy, float *h) {
	if (!m || index >= m->samples.size()) return SPH_ERR_INVALID_ARGUMENT;
	const Sample &s = m->samples[index];
	if (n) *n = (size_t)s.n;
	if (gx) *gx = s.gx;
	if (gy) *gy = s.gy;
	if (h) *h = s.h;
	return SPH_OK;
}

int sph_mpnn_read_sample(sph_mpnn *m, size_t index, void *pos, void *z0, void *target, int32_t *cell_start,
                         int32_t *cell_count) {
	if (!m || index >= m->samples.size()) return SPH_ERR_INVALID_ARGUMENT;
	const Sample &s = m->samples[index];
	MPNN_CUDA(cudaDeviceSynchronize());
	const size_t nc = (size_t)s.gx * s.gy;
	if (pos) MPNN_CUDA(cudaMemcpy(pos, s.pos, sizeof(float2) * s.n, cudaMemcpyDeviceToHost));
	if (z0) MPNN_CUDA(cudaMemcpy(z0, s.z0, sizeof(float2) * s.n, cudaMemcpyDeviceToHost));
	if (target) MPNN_CUDA(cudaMemcpy(target, s.target, sizeof(float2) * s.n, cudaMemcpyDeviceToHost));
	if (cell_start) MPNN_CUDA(cudaMemcpy(cell_start, s.cellStart, sizeof(int) * nc, cudaMemcpyDeviceToHost));
	if (cell_count) MPNN_CUDA(cudaMemcpy(cell_count, s.cellCount, sizeof(int) * nc, cudaMemcpyDeviceToHost));
	return SPH_OK;
}

int sph_mpnn_eval(sph_mpnn *m, size_t index, float *loss, void *u_host) {
	if (!m || index >= m->samples.size()) return SPH_ERR_INVALID_ARGUMENT;
	MPNN_CUDA(cudaSetDevice(m->device));
	const Sample &s = m->samples[index];
	const MpnnGraph g = s.graph();
	int rc = forward(m, g, false, m->stream);
	if (rc) return rc;
	MPNN_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream));
	k_mpnn_loss<<<blocks(s.np, 256), 256, 0, m->stream>>>(m->z[kRounds], g.z0, s.target, m->dz[kRounds], s.n, s.np,
	                                                       m->loss);
	MPNN_CUDA(cudaGetLastError());
	if (u_host) {
		k_mpnn_u<<<blocks(s.n, 256), 256, 0, m->stream>>>(m->z[kRounds], g.z0, m->u, s.n);
		MPNN_CUDA(cudaGetLastError());
		MPNN_CUDA(cudaMemcpyAsync(u_host, m->u, sizeof(float2) * s.n, cudaMemcpyDeviceToHost, m->stream));
	}
	rc = check_error(m, m->stream);
	if (rc) return rc;
	return read_loss(m, s.n, loss);
}

int sph_mpnn_gradient(sph_mpnn *m, size_t index, float *loss, float *grad_host) {
	if (!m || index >= m->samples.size()) return SPH_ERR_INVALID_ARGUMENT;
	MPNN_CUDA(cudaSetDevice(m->device));
	const Sample &s = m->samples[index];
	const MpnnGraph g = s.graph();
	int rc = forward(m, g, true, m->stream);
	if (!rc) rc = backward(m, g, s.target, m->stream);
	if (!rc) rc = check_error(m, m->stream);
	if (rc) return rc;
	if (grad_host) MPNN_CUDA(cudaMemcpy(grad_host, m->grads, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
	return read_loss(m, s.n, loss);
}

int sph_mpnn_train_step(sph_mpnn *m, size_t index, float lr, float *loss) {
	if (!m || index >= m->samples.size() || !(lr >= 0.f)) return SPH_ERR_INVALID_ARGUMENT;
	MPNN_CUDA(cudaSetDevice(m->device));
	const Sample &s = m->samples[index];
	const MpnnGraph g = s.graph();
	int rc = forward(m, g, true, m->stream);
	if (!rc) rc = backward(m, g, s.target, m->stream);
	if (rc) return rc;
	m->adamStep++;
	const float b1 = 0.9f, b2 = 0.999f;
	const float bc1 = 1.f - std::pow(b1, (float)m->adamStep), bc2 = 1.f - std::pow(b2, (float)m->adamStep);
	k_mpnn_adam<<<blocks(kParams, 256), 256, 0, m->stream>>>(m->params, m->grads, m->adamM, m->adamV, kParams, lr, b1,
	                                                          b2, 1e-8f, bc1, bc2, 1.0f);
	MPNN_CUDA(cudaGetLastError());
	rc = refresh(m, m->stream);
	if (!rc) rc = check_error(m, m->stream);
	if (rc) return rc;
	return read_loss(m, s.n, loss);
}

}  // extern "C"

// Standalone GEMM entry point (tests and other callers).
namespace {

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
                             const float *bias, int relu, int accumulate, int splits, int staging, void *stream) {
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
	g.noTma = staging;
	g.error = gemm_error_word(device);
	if (!A || !B || !C || !g.error || ldc < N || staging < 0 || staging > 2) return SPH_ERR_INVALID_ARGUMENT;
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
