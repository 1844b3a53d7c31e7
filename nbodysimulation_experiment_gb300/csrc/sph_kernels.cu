// CUDA kernels of the GB300-native Demo4 SPH step (sm_103a).
//
// One Update (NBodySimulation/demo4.cpp:286-451) runs as:
//   k_integrate     integrate forces (demo4.cpp:302-309) + per-step resets
//   k_viscosity     ordered viscosity sweep over the stale neighbour lists
//                   (demo4.cpp:223-237, sph.h:497-512)
//   k_predict       prev = x; x += v dt; new cell (demo4.cpp:329-347, sph.h:450-463)
//   k_scan          prefix sums of the grid update
//   k_scatter       appendix and mover lists per cell
//   k_grid_update   the reference's remove/insert grid update, event by event
//                   (demo4.cpp:341-356, 37-76)
//   k_density       density and pressure gather (demo4.cpp:208-221, sph.h:465-481)
//   k_delta         ordered double-density relaxation sweep (demo4.cpp:239-255,
//                   sph.h:483-495)
//   k_collide       body collisions + velocity + renumbering (demo4.cpp:411-450)
//
// Every kernel covers all scenes of the simulation at once (one launch per
// stage): particle numbers and cells carry their scene, whose step scalars,
// grid and bodies live in the scene table.
//
// The two pairwise passes of the reference are serial Gauss-Seidel sweeps in
// particle-number order: a particle's updates land in its neighbours
// immediately.  They are reproduced exactly by running them as dataflow
// "sweeps": a task is a run of consecutively numbered particles of one scene
// processed in order by one thread block, tasks are claimed in increasing
// order, and a task first waits (bounded) until every earlier task of its
// scene whose footprint can overlap its own has finished.  Two particles'
// footprints overlap only when their cells are at most two apart, so with
// particles numbered cell by cell in a 3x3-colour-major cell order most tasks
// are independent; tasks of different scenes never wait on each other.  All
// waits are bounded; a timeout raises kErrTimeout and an abort flag that
// releases every other wait, so a kernel always terminates.
//
// Arithmetic: the library is compiled with --fmad=false and IEEE division and
// square root, and every expression below follows the reference's operation
// order, so per-pair results are bit-identical to the reference.
#include "sph_internal.cuh"
#include "sph_kernels.cuh"

namespace sphgb {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kWaitLimitIter = 1u << 24;

__device__ __forceinline__ uint64_t global_ns() {
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
	uint32_t v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
	asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned lanemask_lt() {
	unsigned m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

// Diagnostics: %globaltimer stamps per task (coarse; for task ordering, not
// for sub-microsecond durations).
__device__ __forceinline__ void stamp(const SimTables &T, int sweep, int task, int slot, int lane) {
	if (T.prof != nullptr && lane == 0 && task < T.profStride)
		T.prof[((size_t)sweep * T.profStride + task) * 4 + slot] = global_ns();
}

// Converged bounded wait of a whole warp: each lane names one done flag (or
// none) and the warp polls until every named flag is set.  All lanes run the
// same loop, so a wait never leaves a warp diverged.  Gives up after
// `limitNs` (SimTables::waitLimitNs, 2 s by default) or 2^24 polls, raising
// kErrTimeout and the abort flag that ends every wait.
__device__ __forceinline__ void warp_wait(const uint32_t *flag, uint32_t *abortFlag, uint32_t *err,
                                          unsigned long long limitNs) {
	if (!__any_sync(kFull, flag != nullptr && ld_acquire(flag) == 0u)) return;
	const uint64_t t0 = global_ns();
	unsigned ns = 32;
	for (uint32_t it = 0; it < kWaitLimitIter; ++it) {
		const bool pending = flag != nullptr && ld_acquire(flag) == 0u;
		if (!__any_sync(kFull, pending)) return;
		if (__any_sync(kFull, ld_acquire(abortFlag) != 0u)) return;
		if (__any_sync(kFull, global_ns() - t0 > limitNs)) break;
		__nanosleep(ns);
		if (ns < 256) ns <<= 1;
	}
	if ((threadIdx.x & 31) == 0) {
		atomicOr(err, kErrTimeout);
		atomicExch(abortFlag, 1u);
	}
}

// Cell of a position within its scene's grid (SPHComputeCellPos + clamp,
// sph.h:450-463): IEEE divide, truncation.
__device__ __forceinline__ int cell_of(float2 p, const StepParams &s) {
	int x = (int)((p.x + s.halfW) / s.cellSize);
	int y = (int)((p.y + s.halfH) / s.cellSize);
	x = min(max(x, 0), s.gx - 1);
	y = min(max(y, 0), s.gy - 1);
	return y * s.gx + x;
}

__device__ __forceinline__ int rect_dist(int ax0, int ay0, int ax1, int ay1, int bx0, int by0, int bx1, int by1) {
	int dx = max(0, max(ax0 - bx1, bx0 - ax1));
	int dy = max(0, max(ay0 - by1, by0 - ay1));
	return max(dx, dy);
}

}  // namespace

// ---------------------------------------------------------------------------
// Integrate forces (demo4.cpp:302-309) and reset the per-step cell tables.
__global__ void k_integrate(Totals tt, Particles P, SimTables T) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < tt.n) {
		const StepParams &s = T.scenes[T.sceneOf[i]].p;
		float2 a = P.acc[i];
		float2 v = P.vel[i];
		a.x = s.extX + a.x;  // acceleration += gravity + externalForce
		a.y = s.extY + a.y;
		v.x = a.x * s.dt + v.x;  // velocity += acceleration * dt
		v.y = a.y * s.dt + v.y;
		P.vel[i] = v;
		P.acc[i] = make_float2(0.0f, 0.0f);
	}
	if (i < tt.ncell) {
		const SceneDev &sc = T.scenes[T.sceneOfCell[i]];
		const int local = i - sc.cellBase;
		T.enterCount[i] = 0;
		T.leaveCount[i] = 0;
		T.enterCursor[i] = 0;
		T.appCursor[i] = 0;
		const int cx = local % sc.p.gx, cy = local / sc.p.gx;
		T.bbox[4 * i + 0] = cx;
		T.bbox[4 * i + 1] = cy;
		T.bbox[4 * i + 2] = cx;
		T.bbox[4 * i + 3] = cy;
	}
	if (i == 0) {
		T.moverCount[0] = 0;
		T.moverCount[1] = 0;
	}
}

// ---------------------------------------------------------------------------
// Viscosity sweep.  Task t = canonical cell taskCell[t]; its particles share
// one stale neighbour list: the first (list-time) members of the 3x3 block of
// cells around it, y-major then x, each cell in array order (demo4.cpp:
// 188-201).  The block's positions and velocities are staged in shared
// memory, the task's particles are processed in number order, and the
// block's velocities are written back.  Two tasks conflict iff they belong to
// one scene and their cells are at most two apart; every task waits for the
// earlier conflicting ones.
// One task per block: lanes 0 and 1 of warp 0 run the ordered velocity
// chains while warps 1..3 compute the compacted pair geometry of the next
// particle (positions do not change during this pass, so the geometry of
// every particle of the task is known in advance).
// The task's particles k = 0, 1, ... sit at consecutive list slots own + k
// of one shared list.  Particle k's pairs before slot own + k - 1 (its head)
// need only what particles < k did at those slots, and particle k - 1 has
// passed them once it is past slot own + k + 1.  So the head of k runs in
// lockstep with the tail of k - 1 (its pairs after slot own + k), on the
// other lane: the two touch disjoint slots.  The middle of k (its pairs with
// k - 1, itself and k + 1) follows once k - 1 is finished, and k's tail runs
// beside the head of k + 1.  Each particle costs about the longer of its head
// and tail instead of its whole list, with every pair in the reference's
// order for each particle it touches.
// This is the wide shape (ViscWide); the lean one, k_viscosity_multi below,
// runs several tasks per block for throughput.  Both run the geometry inline
// in the chain for particles with more in-range pairs than their geometry
// buffer holds.
template <class C>
struct ViscSmemT {
	float2 pos[kStageCap];
	float2 vel[kStageCap + 2];  // + a scratch slot (kStageCap) for the chains' idle steps
	float4 geo[3][C::kGeom];  // in-range pairs of a particle, list order: slot, unit vector, 1 - q
	int m[3];
	int2 split[3];            // first pair of the middle, first pair of the tail
	int warpCnt[2][C::kWarps];
	int headCnt[C::kWarps], midCnt[C::kWarps];
	int task;
};

namespace {

// Source index of flat position e of NSEG consecutive segments (segment s
// starts at flat offset off[s] and at source index start[s]); selects only,
// so the arrays stay in registers.
template <int NSEG>
__device__ __forceinline__ int seg_src(int e, const int (&off)[NSEG], const int (&start)[NSEG]) {
	int src = start[0] + e;
#pragma unroll
	for (int q = 1; q < NSEG; ++q) src = (e >= off[q]) ? start[q] + (e - off[q]) : src;
	return src;
}

template <class C>
__device__ __forceinline__ void producers_sync() {
	asm volatile("bar.sync 1, %0;" ::"r"(C::kProducers) : "memory");
}

// Geometry of the particle at staged slot `slot` over the L staged entries
// (its whole list): in-range pairs in list order with their unit vectors
// and 1 - q (sph.h:497-505), and where its middle (slots slot-1..slot+1)
// and tail begin.  Run by the producer warps only, in two passes: the
// in-range entries are compacted first (slot, r, r^2), then the square roots
// and divisions run over the dense compacted list.
template <class C>
__device__ __forceinline__ void visc_geometry(ViscSmemT<C> &S, int buf, int slot, int L, const StepParams &s, int p) {
	const int lane = p & (kWarp - 1), w = p / kWarp;
	const float2 xi = S.pos[slot];
	int m = 0, parity = 0, nHead = 0, nToTail = 0;
	for (int base = 0; base < L; base += C::kProducers) {
		const int e = base + p;
		bool in = false;
		float rx = 0.f, ry = 0.f, r2 = 0.f;
		if (e < L) {
			const float2 xj = S.pos[e];
			rx = xj.x - xi.x;
			ry = xj.y - xi.y;
			r2 = rx * rx + ry * ry;
			in = r2 < s.h2;
		}
		nHead += (in && e < slot - 1) ? 1 : 0;
		nToTail += (in && e <= slot + 1) ? 1 : 0;
		const unsigned mask = __ballot_sync(kFull, in);
		int before = m, total = __popc(mask);
		if (C::kProducers > kWarp) {
			if (lane == 0) S.warpCnt[parity][w] = total;
			producers_sync<C>();
			total = 0;
#pragma unroll
			for (int q = 0; q < C::kWarps - 1; ++q) {
				const int c = S.warpCnt[parity][q];
				before += (q < w) ? c : 0;
				total += c;
			}
			parity ^= 1;
		}
		const int at = before + __popc(mask & lanemask_lt());
		if (in && at < C::kGeom) S.geo[buf][at] = make_float4(__int_as_float(e), rx, ry, r2);
		m += total;
	}
	nHead = __reduce_add_sync(kFull, nHead);
	nToTail = __reduce_add_sync(kFull, nToTail);
	if (lane == 0) {
		S.headCnt[w] = nHead;
		S.midCnt[w] = nToTail;
	}
	if (C::kProducers > kWarp) producers_sync<C>(); else __syncwarp();
	if (p == 0) {
		int h = 0, t = 0;
#pragma unroll
		for (int q = 0; q < C::kProducers / kWarp; ++q) {
			h += S.headCnt[q];
			t += S.midCnt[q];
		}
		S.split[buf] = make_int2(h, t);
	}
	const int mm = min(m, C::kGeom);
	for (int q = p; q < mm; q += C::kProducers) {
		const float4 g = S.geo[buf][q];
		const float r = sqrtf(g.w);
		const float qq = r * s.invH;
		float len = r;  // Vec2Length(Rij) == rij
		if (len == 0.0f) len = 1.0f;
		const float inv = 1.0f / len;
		S.geo[buf][q] = make_float4(g.x, g.y * inv, g.z * inv, 1.0f - qq);
	}
	if (p == 0) S.m[buf] = m;
}

// The serial part of the viscosity pass for one particle, in list order
// (sph.h:497-512, demo4.cpp:231-234): v_i carries from pair to pair.  Each
// slot occurs once per list, so the next pairs' velocities may be loaded
// before this pair's store.  The impulse (f n * 0.5) * dt is computed as
// (f n) * (0.5 dt): 0.5 dt is exact and halving is exact, so both round the
// same real product once (unless |f n| < 2^-125).
template <bool kBranchy>
__device__ __forceinline__ void visc_pair(float2 *vel, int j, float2 n, float o, float2 vj, float2 &vi, float sigma,
                                          float beta, float hdt) {
	// Only approaching pairs (u > 0) exchange an impulse: computed
	// unconditionally and selected, or (kBranchy) skipped.
	const float uu = (vi.x - vj.x) * n.x + (vi.y - vj.y) * n.y;
	if (kBranchy) {
		if (uu > 0.0f) {
			const float f = o * (sigma * uu + beta * (uu * uu));
			const float ix = (f * n.x) * hdt;
			const float iy = (f * n.y) * hdt;
			vi.x = vi.x - ix;
			vi.y = vi.y - iy;
			vel[j] = make_float2(ix + vj.x, iy + vj.y);
		}
		return;
	}
	const float f = o * (sigma * uu + beta * (uu * uu));
	const float ix = (f * n.x) * hdt;
	const float iy = (f * n.y) * hdt;
	const bool ap = uu > 0.0f;
	vi.x = ap ? vi.x - ix : vi.x;
	vi.y = ap ? vi.y - iy : vi.y;
	vel[j] = ap ? make_float2(ix + vj.x, iy + vj.y) : vj;
}

// The chain over m buffered pairs G (slot, unit vector, 1 - q) with the
// velocities vel.  Software pipeline: the geometry and partner velocities of
// the next kU pairs are loaded while the chain runs over the current kU.
template <bool kBranchy, int kU>
__device__ __forceinline__ void visc_run(float2 *vel, const float4 *G, int m, float2 &vi, float sigma, float beta,
                                         float hdt) {
	float4 g[kU];
	float2 vj[kU];
#pragma unroll
	for (int u = 0; u < kU; ++u) g[u] = u < m ? G[u] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
	for (int u = 0; u < kU; ++u) vj[u] = vel[__float_as_int(g[u].x)];
	int q = 0;
	for (; q + 2 * kU <= m; q += kU) {
		float4 gn[kU];
		float2 vn[kU];
#pragma unroll
		for (int u = 0; u < kU; ++u) gn[u] = G[q + kU + u];
#pragma unroll
		for (int u = 0; u < kU; ++u) vn[u] = vel[__float_as_int(gn[u].x)];
#pragma unroll
		for (int u = 0; u < kU; ++u)
			visc_pair<kBranchy>(vel, __float_as_int(g[u].x), make_float2(g[u].y, g[u].z), g[u].w, vj[u], vi, sigma,
			                    beta, hdt);
#pragma unroll
		for (int u = 0; u < kU; ++u) {
			g[u] = gn[u];
			vj[u] = vn[u];
		}
	}
	// At most 2 kU - 1 pairs left, the first kU of them loaded.
	if (q + kU <= m) {
		float4 gn[kU];
		float2 vn[kU];
#pragma unroll
		for (int u = 0; u < kU; ++u) gn[u] = q + kU + u < m ? G[q + kU + u] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
		for (int u = 0; u < kU; ++u) vn[u] = vel[__float_as_int(gn[u].x)];
#pragma unroll
		for (int u = 0; u < kU; ++u)
			visc_pair<kBranchy>(vel, __float_as_int(g[u].x), make_float2(g[u].y, g[u].z), g[u].w, vj[u], vi, sigma,
			                    beta, hdt);
#pragma unroll
		for (int u = 0; u < kU; ++u) {
			g[u] = gn[u];
			vj[u] = vn[u];
		}
		q += kU;
	}
#pragma unroll
	for (int u = 0; u < kU; ++u)
		if (q + u < m)
			visc_pair<kBranchy>(vel, __float_as_int(g[u].x), make_float2(g[u].y, g[u].z), g[u].w, vj[u], vi, sigma,
			                    beta, hdt);
}

// The chain over pairs [start, start + len) of G, in lockstep with the
// other chain lane: both run n >= len steps (the longer of the two).  This
// lane's steps past len take an idle pair: the scratch slot kStageCap with a
// zero unit vector, so u = 0 is not approaching and neither velocity
// changes; the steps stay branch-free.  Software pipeline: the next kU pairs'
// geometry and partner velocities load while the chain runs the current kU
// (two measured fastest: 1.32 ms for the 65,536-particle sweep against 1.51
// with four and 1.42 with eight).  The two lanes touch disjoint slots, so a
// prefetched velocity is never one the other lane changes.
template <bool kBranchy>
__device__ __forceinline__ void visc_run_range(float2 *vel, const float4 *G, int start, int len, int n, float2 &vi,
                                               float sigma, float beta, float hdt) {
	constexpr int kU = 2;
	const float4 idle = make_float4(__int_as_float(kStageCap), 0.f, 0.f, 0.f);
	float4 g[kU];
	float2 vj[kU];
#pragma unroll
	for (int u = 0; u < kU; ++u) g[u] = u < len ? G[start + u] : idle;
#pragma unroll
	for (int u = 0; u < kU; ++u) vj[u] = vel[__float_as_int(g[u].x)];
	for (int q = 0; q < n; q += kU) {
		float4 gn[kU];
		float2 vn[kU];
#pragma unroll
		for (int u = 0; u < kU; ++u) gn[u] = q + kU + u < len ? G[start + q + kU + u] : idle;
#pragma unroll
		for (int u = 0; u < kU; ++u) vn[u] = vel[__float_as_int(gn[u].x)];
#pragma unroll
		for (int u = 0; u < kU; ++u)
			visc_pair<kBranchy>(vel, __float_as_int(g[u].x), make_float2(g[u].y, g[u].z), g[u].w, vj[u], vi, sigma,
			                    beta, hdt);
#pragma unroll
		for (int u = 0; u < kU; ++u) {
			g[u] = gn[u];
			vj[u] = vn[u];
		}
	}
}

// Phase k of a task's chains (lanes 0 and 1 of warp 0; cnt particles at
// slots own..own+cnt-1, particle j's geometry in buffer j % 3).  Lane k & 1
// starts particle k: its head beside the tail of particle k - 1 on the other
// lane, then (once k - 1 is finished and stored) its middle.  vi is the
// lane's particle velocity, carried from the head to the tail.  A particle
// with more in-range pairs than the geometry buffer holds runs its whole
// chain in the middle, in list order, computing the geometry there.
template <class C>
__device__ __forceinline__ void visc_wave(ViscSmemT<C> &S, int k, int cnt, int own, int L, const StepParams &s,
                                          float2 &vi) {
	const int lane = threadIdx.x & (kWarp - 1);
	const float hdt = 0.5f * s.dt;
	const bool head = (k & 1) == lane;  // head and middle of particle k; else the tail of particle k - 1
	const bool has = head ? k < cnt : k >= 1;
	const int buf = has ? (head ? k : k - 1) % 3 : 0;
	int start = 0, len = 0, m = 0;
	int2 sp = make_int2(0, 0);
	if (has) {
		m = S.m[buf];
		sp = S.split[buf];
		const bool inl = m > C::kGeom;
		if (head) {
			vi = S.vel[own + k];
			len = inl ? 0 : sp.x;
		} else {
			start = sp.y;
			len = inl ? 0 : m - sp.y;
		}
	}
	const int n = max(len, __shfl_xor_sync(0x3u, len, 1));
	visc_run_range<C::kBranchy>(S.vel, S.geo[buf], start, len, n, vi, s.sigma, s.beta, hdt);
	if (has && !head) S.vel[own + k - 1] = vi;  // particle k - 1 is finished
	__syncwarp(0x3u);
	if (!(has && head)) return;
	if (m > C::kGeom) {
		const float2 xi = S.pos[own + k];
		for (int e = 0; e < L; ++e) {
			const float2 xj = S.pos[e];
			const float rx = xj.x - xi.x, ry = xj.y - xi.y;
			const float r2 = rx * rx + ry * ry;
			if (!(r2 < s.h2)) continue;
			const float r = sqrtf(r2);
			const float qq = r * s.invH;
			float lenr = r;
			if (lenr == 0.0f) lenr = 1.0f;
			const float inv = 1.0f / lenr;
			visc_pair<C::kBranchy>(S.vel, e, make_float2(rx * inv, ry * inv), 1.0f - qq, S.vel[e], vi, s.sigma,
			                       s.beta, hdt);
		}
		return;
	}
	const float4 *G = S.geo[buf];
	for (int q = sp.x; q < sp.y; ++q) {
		const float4 g = G[q];
		const int j = __float_as_int(g.x);
		visc_pair<C::kBranchy>(S.vel, j, make_float2(g.y, g.z), g.w, S.vel[j], vi, s.sigma, s.beta, hdt);
	}
}

}  // namespace

template <class C>
__global__ void __launch_bounds__(C::kWarps * kWarp, C::kMinBlocks) k_viscosity(Totals tt, Particles P, SimTables T) {
	constexpr int kVT = C::kWarps * kWarp;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	ViscSmemT<C> &S = *reinterpret_cast<ViscSmemT<C> *>(smem_raw);
	const int tid = threadIdx.x, warp = tid / kWarp;
	const int nLive = *T.nLive;
	for (;;) {
		if (tid == 0) S.task = atomicAdd(&T.taskCounter[0], 1);
		__syncthreads();
		const int i = S.task;
		__syncthreads();
		if (i >= nLive) break;
		const int t = T.liveTask[i];
		stamp(T, 0, t, 0, tid);
		const int c = T.taskCell[t];
		const int cnt = T.cellCount[c];
		if (cnt > 0) {
			const SceneDev &sc = T.scenes[T.sceneOfCell[c]];
			const StepParams s = sc.p;
			const int base = sc.cellBase, gx = s.gx, gy = s.gy;
			const int cx = (c - base) % gx, cy = (c - base) / gx;
			// Wait for earlier tasks of the scene within Chebyshev distance 2
			// (warp 0).
			if (warp == 0) {
				const uint32_t *flag = nullptr;
				const int x = cx + tid % 5 - 2, y = cy + tid / 5 - 2;
				if (tid < 25 && tid != 12 && x >= 0 && x < gx && y >= 0 && y < gy) {
					const int c2 = base + y * gx + x;
					const int r2 = T.taskOfCell[c2];
					if (r2 < t && T.cellCount[c2] > 0) flag = &T.done[r2];
				}
				warp_wait(flag, T.abort, T.error, T.waitLimitNs);
			}
			__syncthreads();
			stamp(T, 0, t, 1, tid);
			// Segments of the 3x3 block in list order.
			int segStart[9], segOff[9];
			int L = 0, own = 0;
#pragma unroll
			for (int q = 0; q < 9; ++q) {
				const int x = cx + q % 3 - 1, y = cy + q / 3 - 1;
				int st = 0, nn = 0;
				if (x >= 0 && x < gx && y >= 0 && y < gy) {
					const int c2 = base + y * gx + x;
					st = T.cellStart[c2];
					nn = T.cellCount[c2];
				}
				segStart[q] = st;
				segOff[q] = L;
				if (q == 4) own = L;
				L += nn;
			}
			if (L > kStageCap) {
				if (tid == 0) atomicOr(T.error, kErrStageOverflow);
			} else {
				for (int b0 = 0; b0 < L; b0 += 4 * kVT) {
					float2 xp[4], vp[4];
#pragma unroll
					for (int u = 0; u < 4; ++u) {
						const int e = b0 + u * kVT + tid;
						if (e < L) {
							const int src = seg_src<9>(e, segOff, segStart);
							xp[u] = __ldcg(&P.pos[src]);
							vp[u] = __ldcg(&P.vel[src]);
						}
					}
#pragma unroll
					for (int u = 0; u < 4; ++u) {
						const int e = b0 + u * kVT + tid;
						if (e < L) {
							S.pos[e] = xp[u];
							S.vel[e] = vp[u];
						}
					}
				}
				__syncthreads();
				stamp(T, 0, t, 2, tid);
				if (warp > 0) visc_geometry<C>(S, 0, own, L, s, tid - kWarp);
				__syncthreads();
				float2 vi = make_float2(0.0f, 0.0f);
				for (int k = 0; k <= cnt; ++k) {
					if (warp == 0) {
						if (tid < 2) visc_wave<C>(S, k, cnt, own, L, s, vi);
					} else if (k + 1 < cnt) {
						visc_geometry<C>(S, (k + 1) % 3, own + k + 1, L, s, tid - kWarp);
					}
					__syncthreads();
				}
				for (int e = tid; e < L; e += kVT) __stcg(&P.vel[seg_src<9>(e, segOff, segStart)], S.vel[e]);
			}
			__syncthreads();
			__threadfence();
		}
		__syncthreads();
		stamp(T, 0, t, 3, tid);
		if (tid == 0 && i != T.hold[0]) st_release(&T.done[t], 1u);
	}
}

// ---------------------------------------------------------------------------
// Viscosity sweep, many chains per block (the lean shape, ViscLean): the
// same tasks, waits and arithmetic as k_viscosity, laid out for throughput.
// A block holds kSlots tasks at once.  Lane s of warp 0 runs the ordered
// velocity chain of slot s's current particle (the slots' chains share one
// instruction stream), while producer warp 1 + (s % kProd) looks after slot
// s: it claims a task, polls the task's earlier conflicting tasks (without
// blocking), stages the velocities of its 3x3 block, computes the pair
// geometry of the slot's next particle (positions, which this pass does not
// change, are read through L1), and writes the velocities back and releases
// the task when its chain is done.  The block advances in phases: one
// particle per running slot per phase.
template <class C>
struct ViscSlotT {
	float2 vel[kStageCap];    // velocities of the 3x3 block, list order
	float4 geo[2][C::kGeom];  // per buffer: in-range pairs (slot, unit vector, 1 - q) of one particle
	float4 pad;               // consecutive slots start 16 bytes apart in the bank space
};
template <class C>
struct ViscMultiSmemT {
	ViscSlotT<C> slot[C::kSlots];
	int segStart[C::kSlots][9], segOff[C::kSlots][9];
	int state[C::kSlots], task[C::kSlots], first[C::kSlots], cnt[C::kSlots], own[C::kSlots], L[C::kSlots],
	    k[C::kSlots], cell[C::kSlots], claim[C::kSlots];
	int m[C::kSlots][2];
	float h2[C::kSlots], invH[C::kSlots], sigma[C::kSlots], beta[C::kSlots], hdt[C::kSlots];
	unsigned long long waitSince[C::kSlots];
	int exhausted;  // no tasks left to claim
	int aborted;    // the abort flag was seen set
};

namespace {

enum : int { kSlotFree = 0, kSlotWait = 1, kSlotStaged = 2, kSlotRun = 3, kSlotDone = 4 };

// Pair geometry of particle k of slot s (one warp): in-range pairs in list
// order (sph.h:497-505), compacted first, then the square roots and
// divisions over the dense list.
template <class C>
__device__ __forceinline__ void slot_geometry(ViscMultiSmemT<C> &S, int s, int k, const Particles &P, int lane) {
	const int buf = k & 1;
	float4 *G = S.slot[s].geo[buf];
	int segStart[9], segOff[9];
#pragma unroll
	for (int q = 0; q < 9; ++q) {
		segStart[q] = S.segStart[s][q];
		segOff[q] = S.segOff[s][q];
	}
	const int L = S.L[s];
	const float h2 = S.h2[s], invH = S.invH[s];
	const float2 xi = __ldg(&P.pos[S.first[s] + k]);
	int m = 0;
	for (int b0 = 0; b0 < L; b0 += 4 * kWarp) {
		float2 xj[4];
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const int e = b0 + u * kWarp + lane;
			xj[u] = e < L ? __ldg(&P.pos[seg_src<9>(e, segOff, segStart)]) : make_float2(0.f, 0.f);
		}
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const int e = b0 + u * kWarp + lane;
			const float rx = xj[u].x - xi.x, ry = xj[u].y - xi.y;
			const float r2 = rx * rx + ry * ry;
			const bool in = e < L && r2 < h2;
			const unsigned mask = __ballot_sync(kFull, in);
			const int at = m + __popc(mask & lanemask_lt());
			if (in && at < C::kGeom) G[at] = make_float4(__int_as_float(e), rx, ry, r2);
			m += __popc(mask);
		}
	}
	__syncwarp();
	const int mm = min(m, C::kGeom);
	for (int q = lane; q < mm; q += kWarp) {
		const float4 g = G[q];
		const float r = sqrtf(g.w);
		const float qq = r * invH;
		float len = r;  // Vec2Length(Rij) == rij
		if (len == 0.0f) len = 1.0f;
		const float inv = 1.0f / len;
		G[q] = make_float4(g.x, g.y * inv, g.z * inv, 1.0f - qq);
	}
	if (lane == 0) S.m[s][buf] = m;
}

// Claim the next task into slot s (one warp).  Returns false when none is
// left.
template <class C>
__device__ __forceinline__ bool slot_claim(ViscMultiSmemT<C> &S, int s, const SimTables &T, int nLive, int lane) {
	int i = 0;
	if (lane == 0) i = atomicAdd(&T.taskCounter[0], 1);
	i = __shfl_sync(kFull, i, 0);
	if (i >= nLive) return false;
	const int t = T.liveTask[i];
	const int c = T.taskCell[t];
	const SceneDev &sc = T.scenes[T.sceneOfCell[c]];
	const int base = sc.cellBase, gx = sc.p.gx, gy = sc.p.gy;
	const int cx = (c - base) % gx, cy = (c - base) / gx;
	// Segments of the 3x3 block in list order (lanes 0..8, then a scan).
	int st = 0, nn = 0;
	if (lane < 9) {
		const int x = cx + lane % 3 - 1, y = cy + lane / 3 - 1;
		if (x >= 0 && x < gx && y >= 0 && y < gy) {
			const int c2 = base + y * gx + x;
			st = T.cellStart[c2];
			nn = T.cellCount[c2];
		}
	}
	int incl = nn;
#pragma unroll
	for (int o = 1; o < 16; o <<= 1) {
		const int v = __shfl_up_sync(kFull, incl, o);
		if (lane >= o) incl += v;
	}
	if (lane < 9) {
		S.segStart[s][lane] = st;
		S.segOff[s][lane] = incl - nn;
	}
	const int L = __shfl_sync(kFull, incl, 8);
	const int own = __shfl_sync(kFull, incl - nn, 4);
	if (lane == 0) {
		S.task[s] = t;
		S.claim[s] = i;
		S.cell[s] = c;
		S.first[s] = T.cellStart[c];
		S.cnt[s] = T.cellCount[c];
		S.own[s] = own;
		S.L[s] = L;
		S.h2[s] = sc.p.h2;
		S.invH[s] = sc.p.invH;
		S.sigma[s] = sc.p.sigma;
		S.beta[s] = sc.p.beta;
		S.hdt[s] = 0.5f * sc.p.dt;
		S.state[s] = kSlotWait;
		S.waitSince[s] = global_ns();
	}
	stamp(T, 0, t, 0, lane);
	__syncwarp();
	return true;
}

// One non-blocking poll of slot s's earlier conflicting tasks (cells of the
// scene at most two apart, as k_viscosity).  True when all are done.
template <class C>
__device__ __forceinline__ bool slot_ready(ViscMultiSmemT<C> &S, int s, const SimTables &T, int lane) {
	const int t = S.task[s], c = S.cell[s];
	const SceneDev &sc = T.scenes[T.sceneOfCell[c]];
	const int base = sc.cellBase, gx = sc.p.gx, gy = sc.p.gy;
	const int cx = (c - base) % gx, cy = (c - base) / gx;
	bool pending = false;
	const int x = cx + lane % 5 - 2, y = cy + lane / 5 - 2;
	if (lane < 25 && lane != 12 && x >= 0 && x < gx && y >= 0 && y < gy) {
		const int c2 = base + y * gx + x;
		const int r2 = T.taskOfCell[c2];
		if (r2 < t && T.cellCount[c2] > 0) pending = ld_acquire(&T.done[r2]) == 0u;
	}
	return !__any_sync(kFull, pending);
}

template <class C>
__device__ __forceinline__ void slot_copy_vel(ViscMultiSmemT<C> &S, int s, const Particles &P, int lane, bool in) {
	int segStart[9], segOff[9];
#pragma unroll
	for (int q = 0; q < 9; ++q) {
		segStart[q] = S.segStart[s][q];
		segOff[q] = S.segOff[s][q];
	}
	const int L = S.L[s];
	float2 *V = S.slot[s].vel;
	for (int b0 = 0; b0 < L; b0 += 4 * kWarp) {
		if (in) {
			float2 v[4];
#pragma unroll
			for (int u = 0; u < 4; ++u) {
				const int e = b0 + u * kWarp + lane;
				if (e < L) v[u] = __ldcg(&P.vel[seg_src<9>(e, segOff, segStart)]);
			}
#pragma unroll
			for (int u = 0; u < 4; ++u) {
				const int e = b0 + u * kWarp + lane;
				if (e < L) V[e] = v[u];
			}
		} else {
#pragma unroll
			for (int u = 0; u < 4; ++u) {
				const int e = b0 + u * kWarp + lane;
				if (e < L) __stcg(&P.vel[seg_src<9>(e, segOff, segStart)], V[e]);
			}
		}
	}
}

// The producer warp's turn for slot s in one phase.
template <class C>
__device__ __forceinline__ void slot_produce(ViscMultiSmemT<C> &S, int s, const Particles &P, const SimTables &T,
                                             int nLive, int lane) {
	int state = S.state[s];
	if (state == kSlotDone) {
		// Chain finished: write the block's velocities back and release.
		slot_copy_vel<C>(S, s, P, lane, false);
		__threadfence();
		__syncwarp();
		stamp(T, 0, S.task[s], 3, lane);
		if (lane == 0) {
			if (S.claim[s] != T.hold[0]) st_release(&T.done[S.task[s]], 1u);
			S.state[s] = kSlotFree;
		}
		__syncwarp();
		state = kSlotFree;
	}
	if (state == kSlotFree) {
		if (__shfl_sync(kFull, S.exhausted, 0)) return;
		if (!slot_claim<C>(S, s, T, nLive, lane)) {
			if (lane == 0) S.exhausted = 1;
			return;
		}
		state = kSlotWait;
	}
	if (state == kSlotWait) {
		if (!slot_ready<C>(S, s, T, lane)) {
			if (lane == 0 && global_ns() - S.waitSince[s] > T.waitLimitNs) {
				atomicOr(T.error, kErrTimeout);
				atomicExch(T.abort, 1u);
			}
			return;
		}
		if (S.L[s] > kStageCap) {
			// The block does not fit: flag it and release the task untouched.
			if (lane == 0) {
				atomicOr(T.error, kErrStageOverflow);
				st_release(&T.done[S.task[s]], 1u);
				S.state[s] = kSlotFree;
			}
			__syncwarp();
			return;
		}
		stamp(T, 0, S.task[s], 1, lane);
		slot_copy_vel<C>(S, s, P, lane, true);
		slot_geometry<C>(S, s, 0, P, lane);
		if (lane == 0) S.state[s] = kSlotStaged;
		__syncwarp();
		return;
	}
	if (state == kSlotRun) {
		const int k = S.k[s];
		if (k + 1 < S.cnt[s]) slot_geometry<C>(S, s, k + 1, P, lane);
	}
}

// The chain of slot s's current particle (lane s of warp 0).
template <class C>
__device__ __forceinline__ void slot_chain(ViscMultiSmemT<C> &S, int s, const Particles &P) {
	const int k = S.k[s], buf = k & 1, m = S.m[s][buf];
	const int own = S.own[s] + k;
	float2 *V = S.slot[s].vel;
	const float sigma = S.sigma[s], beta = S.beta[s], hdt = S.hdt[s];
	float2 vi = V[own];
	if (m > C::kGeom) {
		// More in-range pairs than the geometry buffer holds: the same pair
		// geometry (sph.h:497-505), computed here in list order.
		int segStart[9], segOff[9];
#pragma unroll
		for (int q = 0; q < 9; ++q) {
			segStart[q] = S.segStart[s][q];
			segOff[q] = S.segOff[s][q];
		}
		const int L = S.L[s];
		const float h2 = S.h2[s], invH = S.invH[s];
		const float2 xi = __ldg(&P.pos[S.first[s] + k]);
		for (int e = 0; e < L; ++e) {
			const float2 xj = __ldg(&P.pos[seg_src<9>(e, segOff, segStart)]);
			const float rx = xj.x - xi.x, ry = xj.y - xi.y;
			const float r2 = rx * rx + ry * ry;
			if (!(r2 < h2)) continue;
			const float r = sqrtf(r2);
			const float qq = r * invH;
			float len = r;
			if (len == 0.0f) len = 1.0f;
			const float inv = 1.0f / len;
			visc_pair<false>(V, e, make_float2(rx * inv, ry * inv), 1.0f - qq, V[e], vi, sigma, beta, hdt);
		}
	} else {
		visc_run<false, 4>(V, S.slot[s].geo[buf], m, vi, sigma, beta, hdt);
	}
	V[own] = vi;
}

}  // namespace

template <class C>
__global__ void __launch_bounds__(C::kWarps * kWarp, C::kMinBlocks) k_viscosity_multi(Totals tt, Particles P,
                                                                                     SimTables T) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	ViscMultiSmemT<C> &S = *reinterpret_cast<ViscMultiSmemT<C> *>(smem_raw);
	const int tid = threadIdx.x, warp = tid / kWarp, lane = tid & (kWarp - 1);
	const int nLive = *T.nLive;
	if (tid < C::kSlots) {
		S.state[tid] = kSlotFree;
		S.k[tid] = 0;
	}
	if (tid == 0) {
		S.exhausted = 0;
		S.aborted = 0;
	}
	__syncthreads();
	for (;;) {
		// Bookkeeping of the phase just ended: thread s advances slot s.
		int busy = 0;
		if (tid < C::kSlots) {
			int st = S.state[tid];
			if (st == kSlotStaged) {
				st = kSlotRun;
				S.k[tid] = 0;
			} else if (st == kSlotRun) {
				const int k = S.k[tid] + 1;
				S.k[tid] = k;
				if (k == S.cnt[tid]) st = kSlotDone;
			}
			S.state[tid] = st;
			busy = st != kSlotFree;
		}
		const int anyBusy = __syncthreads_or(busy);
		if ((!anyBusy && S.exhausted) || S.aborted) break;
		if (warp == 0) {
			if (lane < C::kSlots && S.state[lane] == kSlotRun) slot_chain<C>(S, lane, P);
		} else {
			if (tid == kWarp && ld_acquire(T.abort) != 0u) S.aborted = 1;
			__syncwarp();
			for (int s = warp - 1; s < C::kSlots; s += C::kProd) slot_produce<C>(S, s, P, T, nLive, lane);
		}
		__syncthreads();
	}
}

// ---------------------------------------------------------------------------
// Reference order (single scene).  The reference's Update visits particles
// in its own index order, which is AddParticle order for a scene that was
// built and then stepped (demo4.cpp:223-255, 344-352).  In reference order
// the library does the same: refOrd lists the particles' numbers in
// AddParticle order; the viscosity sweep runs as tasks of kAppendixRun
// consecutive AddParticle indices (k_viscosity_ref), the delta sweep as the
// same runs over the whole scene (k_delta's run path), and the grid update
// applies each cell's events in AddParticle order.

__global__ void k_ref_order(Totals tt, Particles P, SimTables T) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= tt.n) return;
	const SceneDev &sc = T.scenes[T.sceneOf[i]];
	const int id = P.id[i];
	if (id < 0 || id >= sc.n) {
		atomicOr(T.error, kErrIndex);
		return;
	}
	T.refOrd[sc.pBase + id] = i;
}

// Bounding box (cell coordinates) of the old cells of each viscosity run:
// the cells whose canonical arrays made its particles' neighbour lists.  One
// warp per run.
__global__ void k_visc_boxes(Totals tt, Particles P, SimTables T) {
	const int a = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
	const int lane = threadIdx.x & (kWarp - 1);
	if (a >= tt.nViscRuns) return;
	const SceneDev &sc = T.scenes[0];
	const int gx = sc.p.gx;
	const int p0 = sc.pBase + a * kAppendixRun;
	const int p1 = min(sc.pBase + sc.n0, p0 + kAppendixRun);
	int bx0 = sc.p.gx, by0 = sc.p.gy, bx1 = -1, by1 = -1;
	for (int k = p0 + lane; k < p1; k += kWarp) {
		const int lc = P.cellOf[T.refOrd[k]] - sc.cellBase;
		bx0 = min(bx0, lc % gx);
		bx1 = max(bx1, lc % gx);
		by0 = min(by0, lc / gx);
		by1 = max(by1, lc / gx);
	}
	for (int o = 16; o > 0; o >>= 1) {
		bx0 = min(bx0, __shfl_xor_sync(kFull, bx0, o));
		by0 = min(by0, __shfl_xor_sync(kFull, by0, o));
		bx1 = max(bx1, __shfl_xor_sync(kFull, bx1, o));
		by1 = max(by1, __shfl_xor_sync(kFull, by1, o));
	}
	if (lane == 0) *reinterpret_cast<int4 *>(&T.viscBox[4 * a]) = make_int4(bx0, by0, bx1, by1);
}

// Viscosity sweep in reference order: one warp per task (run a: the
// canonical particles with AddParticle indices a*kAppendixRun onwards), each
// task waiting for the earlier runs whose old cells come within two cells of
// its own.  For each particle, in order, the warp walks its stale list (the
// 3x3 block of canonical cell arrays around its old cell, demo4.cpp:188-201)
// 32 entries at a time, computing the pair geometry of the in-range entries
// (sph.h:497-505), and lane 0 runs the ordered velocity chain over them
// (demo4.cpp:231-234), velocities in global memory.
__global__ void __launch_bounds__(kViscRefWarps * kWarp) k_viscosity_ref(Totals tt, Particles P, SimTables T) {
	__shared__ float4 geo[kViscRefWarps][kWarp];
	const int lane = threadIdx.x & (kWarp - 1), w = threadIdx.x / kWarp;
	const SceneDev &sc = T.scenes[0];
	const StepParams s = sc.p;
	const int base = sc.cellBase, gx = s.gx, gy = s.gy;
	const float hdt = 0.5f * s.dt;
	for (;;) {
		int a = 0;
		if (lane == 0) a = atomicAdd(&T.taskCounter[0], 1);
		a = __shfl_sync(kFull, a, 0);
		if (a >= tt.nViscRuns) break;
		const int4 box = *reinterpret_cast<const int4 *>(&T.viscBox[4 * a]);
		for (int q0 = 0; q0 < a; q0 += kWarp) {
			const int q = q0 + lane;
			const uint32_t *flag = nullptr;
			if (q < a) {
				const int4 o = *reinterpret_cast<const int4 *>(&T.viscBox[4 * q]);
				if (rect_dist(o.x, o.y, o.z, o.w, box.x, box.y, box.z, box.w) <= 2) flag = &T.done[q];
			}
			warp_wait(flag, T.abort, T.error, T.waitLimitNs);
		}
		const int p0 = sc.pBase + a * kAppendixRun;
		const int p1 = min(sc.pBase + sc.n0, p0 + kAppendixRun);
		for (int k = p0; k < p1; ++k) {
			const int i = T.refOrd[k];
			const int lc = P.cellOf[i] - base;
			const int cx = lc % gx, cy = lc / gx;
			const float2 xi = P.pos[i];
			float2 vi = __ldcg(&P.vel[i]);
			for (int q = 0; q < 9; ++q) {
				const int x = cx + q % 3 - 1, y = cy + q / 3 - 1;
				if (x < 0 || x >= gx || y < 0 || y >= gy) continue;
				const int c2 = base + y * gx + x;
				const int st = T.cellStart[c2], nn = T.cellCount[c2];
				for (int b0 = 0; b0 < nn; b0 += kWarp) {
					const int e = b0 + lane;
					bool in = false;
					if (e < nn) {
						const int j = st + e;
						const float2 xj = P.pos[j];
						const float rx = xj.x - xi.x, ry = xj.y - xi.y;
						const float r2 = rx * rx + ry * ry;
						in = r2 < s.h2;
						if (in) {
							const float r = sqrtf(r2);
							const float qq = r * s.invH;
							float len = r;  // Vec2Length(Rij) == rij
							if (len == 0.0f) len = 1.0f;
							const float inv = 1.0f / len;
							geo[w][lane] = make_float4(__int_as_float(j), rx * inv, ry * inv, 1.0f - qq);
						}
					}
					unsigned mask = __ballot_sync(kFull, in);
					__syncwarp();
					if (lane == 0) {
						while (mask) {
							const int t = __ffs(mask) - 1;
							mask &= mask - 1;
							const float4 g = geo[w][t];
							const int j = __float_as_int(g.x);
							const float2 vj = __ldcg(&P.vel[j]);
							const float2 n = make_float2(g.y, g.z);
							const float uu = (vi.x - vj.x) * n.x + (vi.y - vj.y) * n.y;
							if (uu > 0.0f) {
								const float f = g.w * (s.sigma * uu + s.beta * (uu * uu));
								const float ix = (f * n.x) * hdt;
								const float iy = (f * n.y) * hdt;
								vi.x = vi.x - ix;
								vi.y = vi.y - iy;
								__stcg(&P.vel[j], make_float2(ix + vj.x, iy + vj.y));
							}
						}
					}
					__syncwarp();
				}
			}
			if (lane == 0) __stcg(&P.vel[i], vi);
			__syncwarp();
		}
		__threadfence();
		__syncwarp();
		if (lane == 0 && a != T.hold[0]) st_release(&T.done[a], 1u);
	}
}

// ---------------------------------------------------------------------------
// Predict (demo4.cpp:329-337) and the new cell (demo4.cpp:347).  Movers
// extend the bounding box of new cells of their old cell, count as leaving
// their old cell and entering their new cell.
__global__ void k_predict(Totals tt, Particles P, SimTables T) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= tt.n) return;
	const SceneDev &sc = T.scenes[T.sceneOf[i]];
	const float2 x = P.pos[i];
	const float2 v = P.vel[i];
	P.prev[i] = x;
	const float2 xn = make_float2(v.x * sc.p.dt + x.x, v.y * sc.p.dt + x.y);
	P.pos[i] = xn;
	const int local = cell_of(xn, sc.p);
	const int nc = sc.cellBase + local;
	T.newCell[i] = nc;
	const int oc = P.cellOf[i];
	if (nc != oc) {
		atomicAdd(&T.enterCount[nc], 1);
		atomicAdd(&T.leaveCount[oc], 1);
		const int gx = sc.p.gx;
		const int nx = local % gx, ny = local / gx;
		const int ox = (oc - sc.cellBase) % gx, oy = (oc - sc.cellBase) / gx;
		atomicMin(&T.bbox[4 * oc + 0], nx);
		atomicMin(&T.bbox[4 * oc + 1], ny);
		atomicMax(&T.bbox[4 * oc + 2], nx);
		atomicMax(&T.bbox[4 * oc + 3], ny);
		atomicMax(&T.moverCount[1], max(abs(nx - ox), abs(ny - oy)));
		atomicAdd(&T.moverCount[0], 1);
	}
}

// ---------------------------------------------------------------------------
// The occupied canonical cells in task order (both sweeps skip empty cells):
// per-tile counts, a scan of the tile counts, then the compacted list.

__global__ void __launch_bounds__(kScanThreads) k_live_reduce(Totals tt, SimTables T) {
	__shared__ int part[kScanThreads / kWarp];
	const int tile = blockIdx.x;
	int cnt = 0;
	for (int k = 0; k < kScanTile / kScanThreads; ++k) {
		const int t = tile * kScanTile + k * kScanThreads + threadIdx.x;
		if (t < tt.ncell) cnt += T.cellCount[T.taskCell[t]] > 0;
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
	if ((threadIdx.x & (kWarp - 1)) == 0) part[threadIdx.x / kWarp] = cnt;
	__syncthreads();
	if (threadIdx.x == 0) {
		int sum = 0;
		for (int w = 0; w < kScanThreads / kWarp; ++w) sum += part[w];
		T.liveTiles[tile] = sum;
	}
}

namespace {
__device__ __forceinline__ int block_exscan(int v, int *warpSums, int *total);
}

__global__ void __launch_bounds__(kScanThreads) k_live_tiles(SimTables T, int ntiles) {
	__shared__ int warpSums[kScanThreads / kWarp];
	__shared__ int total;
	int carry = 0;
	for (int base = 0; base < ntiles; base += kScanThreads) {
		const int i = base + threadIdx.x;
		const int x = i < ntiles ? T.liveTiles[i] : 0;
		const int ex = block_exscan(x, warpSums, &total);
		if (i < ntiles) T.liveTiles[i] = carry + ex;
		carry += total;
		__syncthreads();
	}
	if (threadIdx.x == 0) *T.nLive = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_live_apply(Totals tt, SimTables T) {
	__shared__ int warpSums[kScanThreads / kWarp];
	__shared__ int total;
	const int tile = blockIdx.x;
	int carry = T.liveTiles[tile];
	for (int k = 0; k < kScanTile / kScanThreads; ++k) {
		const int t = tile * kScanTile + k * kScanThreads + threadIdx.x;
		const bool live = t < tt.ncell && T.cellCount[T.taskCell[t]] > 0;
		const int ex = block_exscan(live ? 1 : 0, warpSums, &total);
		if (live) T.liveTask[carry + ex] = t;
		carry += total;
	}
}

// ---------------------------------------------------------------------------
// Exclusive scans over cells, in three passes over tiles of kScanTile
// positions: per-tile sums, a scan of the tile sums, per-tile scans.  Three
// scans run together: the appendix counts and the entering counts in cell
// order, and the new cell counts (cellCount + appCount - leaveCount +
// enterCount) in numbering order (scenes in order, cells in colour rank).

namespace {

__device__ __forceinline__ int new_count(const SimTables &T, int c) {
	return T.cellCount[c] + T.appCount[c] - T.leaveCount[c] + T.enterCount[c];
}

// Block-wide exclusive scan of one value per thread (kScanThreads threads);
// returns the exclusive prefix and writes the block total to *total.
__device__ __forceinline__ int block_exscan(int v, int *warpSums, int *total) {
	const int lane = threadIdx.x & (kWarp - 1), warp = threadIdx.x / kWarp;
	int incl = v;
#pragma unroll
	for (int o = 1; o < kWarp; o <<= 1) {
		const int t = __shfl_up_sync(kFull, incl, o);
		if (lane >= o) incl += t;
	}
	if (lane == kWarp - 1) warpSums[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		int w = lane < kScanThreads / kWarp ? warpSums[lane] : 0;
		int wi = w;
#pragma unroll
		for (int o = 1; o < kWarp; o <<= 1) {
			const int t = __shfl_up_sync(kFull, wi, o);
			if (lane >= o) wi += t;
		}
		if (lane < kScanThreads / kWarp) warpSums[lane] = wi - w;
		if (lane == kWarp - 1) *total = wi;
	}
	__syncthreads();
	const int r = warpSums[warp] + incl - v;
	__syncthreads();
	return r;
}

}  // namespace

// Pass 1: the three sums of every tile.
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(Totals tt, SimTables T) {
	__shared__ int part[3][kScanThreads / kWarp];
	const int t = blockIdx.x;
	int a = 0, e = 0, nw = 0;
	for (int k = 0; k < kScanTile / kScanThreads; ++k) {
		const int r = t * kScanTile + k * kScanThreads + threadIdx.x;
		if (r < tt.ncell) {
			a += T.appCount[r];
			e += T.enterCount[r];
			nw += new_count(T, T.numberOrder[r]);
		}
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		a += __shfl_xor_sync(kFull, a, o);
		e += __shfl_xor_sync(kFull, e, o);
		nw += __shfl_xor_sync(kFull, nw, o);
	}
	const int lane = threadIdx.x & (kWarp - 1), warp = threadIdx.x / kWarp;
	if (lane == 0) {
		part[0][warp] = a;
		part[1][warp] = e;
		part[2][warp] = nw;
	}
	__syncthreads();
	if (threadIdx.x < 3) {
		int sum = 0;
		for (int w = 0; w < kScanThreads / kWarp; ++w) sum += part[threadIdx.x][w];
		T.scanTiles[threadIdx.x * gridDim.x + t] = sum;
	}
}

// Pass 2 (one block): exclusive scans of the tile sums; also restarts the
// per-scene neighbour-count statistics (demo4.cpp:369-370).
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(Totals tt, SimTables T, int ntiles) {
	__shared__ int warpSums[kScanThreads / kWarp];
	__shared__ int total;
	for (int s3 = 0; s3 < 3; ++s3) {
		int *v = T.scanTiles + s3 * ntiles;
		int carry = 0;
		for (int base = 0; base < ntiles; base += kScanThreads) {
			const int i = base + threadIdx.x;
			const int x = i < ntiles ? v[i] : 0;
			const int ex = block_exscan(x, warpSums, &total);
			if (i < ntiles) v[i] = carry + ex;
			carry += total;
			__syncthreads();
		}
	}
	for (int sc = threadIdx.x; sc < tt.nscenes; sc += blockDim.x) {
		T.stats[4 * sc + 0] = T.scenes[sc].nbSeed;
		T.stats[4 * sc + 1] = 0;
		if (T.springTotal) T.springTotal[sc] = 0;
	}
}

// Pass 3: per-tile scans plus the tile offsets; writes appStart, enterOffset,
// newCount and newStart.
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(Totals tt, SimTables T) {
	__shared__ int warpSums[kScanThreads / kWarp];
	__shared__ int total;
	const int t = blockIdx.x, nt = gridDim.x;
	int ca = T.scanTiles[t], ce = T.scanTiles[nt + t], cn = T.scanTiles[2 * nt + t];
	for (int k = 0; k < kScanTile / kScanThreads; ++k) {
		const int r = t * kScanTile + k * kScanThreads + threadIdx.x;
		const bool in = r < tt.ncell;
		const int a = in ? T.appCount[r] : 0;
		const int e = in ? T.enterCount[r] : 0;
		const int c = in ? T.numberOrder[r] : 0;
		const int nw = in ? new_count(T, c) : 0;
		int ex = block_exscan(a, warpSums, &total);
		if (in) T.appStart[r] = ca + ex;
		ca += total;
		ex = block_exscan(e, warpSums, &total);
		if (in) T.enterOffset[r] = ce + ex;
		ce += total;
		ex = block_exscan(nw, warpSums, &total);
		if (in) {
			T.newCount[c] = nw;
			T.newStart[c] = cn + ex;
		}
		cn += total;
	}
}

// Appendix members and movers into per-cell lists (order fixed later).
__global__ void k_scatter(Totals tt, Particles P, SimTables T) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= tt.n) return;
	const SceneDev &sc = T.scenes[T.sceneOf[i]];
	const int oc = P.cellOf[i];
	if (i - sc.pBase >= sc.n0) {
		const int slot = T.appStart[oc] + atomicAdd(&T.appCursor[oc], 1);
		T.appIdx[slot] = i;
	}
	const int nc = T.newCell[i];
	if (nc != oc) {
		const int slot = T.enterOffset[nc] + atomicAdd(&T.enterCursor[nc], 1);
		T.enterList[slot] = i;
	}
}

// ---------------------------------------------------------------------------
// Grid update, exactly as the reference's serial loop (demo4.cpp:344-352):
// particles in number order that changed cell are removed from the old cell
// by swap-with-last (demo4.cpp:56-76) and appended to the new one
// (demo4.cpp:37-54).  A cell's final array depends only on the order of its
// own events, so each warp replays one cell's events in number order.

struct GridWarp {
	int arr[kCellCap];
	int leave[kCellCap];
	int enter[kCellCap];
};

// Numbers sorted by their particles' AddParticle index (reference order).
__device__ void insertion_sort_by_id(int *a, int n, const int *id) {
	for (int i = 1; i < n; ++i) {
		const int v = a[i];
		const int key = id[v];
		int j = i - 1;
		while (j >= 0 && id[a[j]] > key) {
			a[j + 1] = a[j];
			--j;
		}
		a[j + 1] = v;
	}
}

__device__ void insertion_sort(int *a, int n) {
	for (int i = 1; i < n; ++i) {
		const int v = a[i];
		int j = i - 1;
		while (j >= 0 && a[j] > v) {
			a[j + 1] = a[j];
			--j;
		}
		a[j + 1] = v;
	}
}

__global__ void __launch_bounds__(kGridWarps * kWarp) k_grid_update(Totals tt, Particles P, Particles Q, SimTables T) {
	__shared__ GridWarp W[kGridWarps];
	GridWarp &S = W[threadIdx.x / kWarp];
	const int lane = threadIdx.x & (kWarp - 1);
	const int n = tt.n;
	const int warpsTotal = gridDim.x * kGridWarps;
	for (int c = blockIdx.x * kGridWarps + threadIdx.x / kWarp; c < tt.ncell; c += warpsTotal) {
		const int cs = T.cellStart[c], cc = T.cellCount[c];
		const int as = T.appStart[c], ac = T.appCount[c];
		const int eo = T.enterOffset[c], ec = T.enterCount[c];
		const int init = cc + ac;
		const int outStart = T.newStart[c], outCount = T.newCount[c];
		if (init == 0 && ec == 0) continue;
		uint32_t *stats = T.stats + 4 * T.sceneOfCell[c];
		if (init + ec > kCellCap || outCount > kCellCap) {
			// Over capacity: keep memory consistent (members in some order)
			// and report; the result of this update is not meaningful.
			if (lane == 0) {
				atomicOr(T.error, kErrCellOverflow);
				int w = 0;
				for (int j = 0; j < cc && w < outCount; ++j)
					if (T.newCell[cs + j] == c) T.newIdx[outStart + w++] = cs + j;
				for (int j = 0; j < ac && w < outCount; ++j)
					if (T.newCell[T.appIdx[as + j]] == c) T.newIdx[outStart + w++] = T.appIdx[as + j];
				for (int j = 0; j < ec && w < outCount; ++j) T.newIdx[outStart + w++] = T.enterList[eo + j];
				for (; w < outCount; ++w) T.newIdx[outStart + w] = 0;
				for (int j = 0; j < outCount; ++j) {
					const int p = T.newIdx[outStart + j];
					T.newLabel[p] = outStart + j;
					Q.pos[outStart + j] = P.pos[p];
				}
			}
			__syncwarp();
			continue;
		}
		for (int j = lane; j < cc; j += kWarp) S.arr[j] = cs + j;
		for (int j = lane; j < ac; j += kWarp) S.arr[cc + j] = T.appIdx[as + j];
		for (int j = lane; j < ec; j += kWarp) S.enter[j] = T.enterList[eo + j];
		__syncwarp();
		if (lane == 0) {
			// Appendix members joined in number order (their AddParticle
			// order); entering particles are applied in number order, or in
			// AddParticle order in reference order.
			insertion_sort(S.arr + cc, ac);
			if (tt.refOrder) insertion_sort_by_id(S.enter, ec, P.id); else insertion_sort(S.enter, ec);
		}
		__syncwarp();
		// Leaving particles, in number order (the array is sorted here); in
		// reference order they are sorted by AddParticle index below.
		int nl = 0;
		for (int base = 0; base < init; base += kWarp) {
			const int j = base + lane;
			bool lv = false;
			int p = 0;
			if (j < init) {
				p = S.arr[j];
				lv = T.newCell[p] != c;
			}
			const unsigned mask = __ballot_sync(kFull, lv);
			if (lv) S.leave[nl + __popc(mask & lanemask_lt())] = p;
			nl += __popc(mask);
		}
		__syncwarp();
		if (lane == 0) {
			if (tt.refOrder) insertion_sort_by_id(S.leave, nl, P.id);
			int cnt = init;
			int lo = 0x7fffffff, hi = 0;
			int a = 0, b = 0;
			while (a < nl || b < ec) {
				bool leaveFirst = b >= ec;
				if (a < nl && b < ec)
					leaveFirst = tt.refOrder ? P.id[S.leave[a]] < P.id[S.enter[b]] : S.leave[a] < S.enter[b];
				if (leaveFirst) {
					const int p = S.leave[a++];
					int at = 0;
					while (at < cnt && S.arr[at] != p) ++at;
					const int last = cnt - 1;
					if (at < cnt && at != last) {
						S.arr[at] = S.arr[last];
						S.arr[last] = p;
					}
					--cnt;
				} else {
					S.arr[cnt++] = S.enter[b++];
				}
				lo = min(lo, cnt);
				hi = max(hi, cnt);
			}
			if (nl + ec > 0) {
				atomicMin(&stats[2], (uint32_t)lo);
				atomicMax(&stats[3], (uint32_t)hi);
			}
			if (cnt != outCount) atomicOr(T.error, kErrIndex);
		}
		__syncwarp();
		// The new cell arrays are the next canonical numbering: the particle
		// at position j of cell c becomes number newStart[c] + j.  Positions
		// are gathered into that order for the density and delta passes.
		for (int j = lane; j < outCount; j += kWarp) {
			int p = S.arr[j];
			if (p < 0 || p >= n) {
				atomicOr(T.error, kErrIndex);
				p = 0;
			}
			T.newIdx[outStart + j] = p;
			T.newLabel[p] = outStart + j;
			Q.pos[outStart + j] = P.pos[p];
		}
		__syncwarp();
	}
}

// Bounding box (scene-local cell coordinates) of the new cells of each
// appendix run (in reference order: of each run of the whole scene in
// AddParticle order); one warp per run.
__global__ void k_app_boxes(Totals tt, SimTables T) {
	const int a = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
	const int lane = threadIdx.x & (kWarp - 1);
	if (a >= tt.nApp) return;
	const SceneDev &sc = T.scenes[T.appScene[a]];
	const int gx = sc.p.gx;
	const int p0 = sc.pBase + (tt.refOrder ? 0 : sc.n0) + T.appRun[a] * kAppendixRun;
	const int p1 = min(sc.pBase + sc.n, p0 + kAppendixRun);
	int bx0 = sc.p.gx, by0 = sc.p.gy, bx1 = -1, by1 = -1;
	for (int k = p0 + lane; k < p1; k += kWarp) {
		const int lc = T.newCell[tt.refOrder ? T.refOrd[k] : k] - sc.cellBase;
		bx0 = min(bx0, lc % gx);
		bx1 = max(bx1, lc % gx);
		by0 = min(by0, lc / gx);
		by1 = max(by1, lc / gx);
	}
	for (int o = 16; o > 0; o >>= 1) {
		bx0 = min(bx0, __shfl_xor_sync(kFull, bx0, o));
		by0 = min(by0, __shfl_xor_sync(kFull, by0, o));
		bx1 = max(bx1, __shfl_xor_sync(kFull, bx1, o));
		by1 = max(by1, __shfl_xor_sync(kFull, by1, o));
	}
	if (lane == 0) *reinterpret_cast<int4 *>(&T.appBox[4 * a]) = make_int4(bx0, by0, bx1, by1);
}

// ---------------------------------------------------------------------------
// Density and pressure (demo4.cpp:208-221): a pure gather.  One warp per new
// cell; each lane sums the lists of two of the cell's particles (the 3x3
// block of the new cell arrays, demo4.cpp:183-206) in list order.  The block
// is staged in chunks of kDensChunk entries, so a warp needs little shared
// memory and many warps fit on an SM.

constexpr int kDensChunk = 256;
struct DensWarp {
	float2 pos[kDensChunk];
};

namespace {

// One list entry for one particle (sph.h:465-476): sums in list order.
__device__ __forceinline__ void dens_entry(float2 xj, float2 xi, float h2, float invH, float &d0, float &d1) {
	const float rx = xj.x - xi.x, ry = xj.y - xi.y;
	const float r2 = rx * rx + ry * ry;
	if (r2 < h2) {
		const float r = sqrtf(r2);
		const float term = 1.0f - r * invH;
		d0 = d0 + term * term;
		d1 = d1 + term * term * term;
	}
}

}  // namespace

__global__ void __launch_bounds__(kDensWarps * kWarp, 4) k_density(Totals tt, Particles Q, SimTables T) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	DensWarp &S = reinterpret_cast<DensWarp *>(smem_raw)[threadIdx.x / kWarp];
	const int lane = threadIdx.x & (kWarp - 1);
	const int warpsTotal = gridDim.x * kDensWarps;
	for (int c = blockIdx.x * kDensWarps + threadIdx.x / kWarp; c < tt.ncell; c += warpsTotal) {
		const int cnt = T.newCount[c];
		if (cnt == 0) continue;
		const int sid = T.sceneOfCell[c];
		const SceneDev &sc = T.scenes[sid];
		const StepParams &s = sc.p;
		const int base = sc.cellBase;
		const int cx = (c - base) % s.gx, cy = (c - base) / s.gx;
		int segStart[9], segOff[9];
		int L = 0;
#pragma unroll
		for (int q = 0; q < 9; ++q) {
			const int x = cx + q % 3 - 1, y = cy + q / 3 - 1;
			int st = 0, nn = 0;
			if (x >= 0 && x < s.gx && y >= 0 && y < s.gy) {
				const int c2 = base + y * s.gx + x;
				st = T.newStart[c2];
				nn = T.newCount[c2];
			}
			segStart[q] = st;
			segOff[q] = L;
			L += nn;
		}
		if (lane == 0) {
			atomicMin(&T.stats[4 * sid + 0], (uint32_t)L);
			atomicMax(&T.stats[4 * sid + 1], (uint32_t)L);
		}
		if (L > kStageCap) {
			if (lane == 0) atomicOr(T.error, kErrStageOverflow);
			continue;
		}
		const float h2 = s.h2, invH = s.invH;
		const int st = T.newStart[c];
		for (int g = 0; g < cnt; g += 2 * kWarp) {
			const int j0 = g + lane, j1 = g + kWarp + lane;
			// Lanes without a particle use a position no entry is in range of.
			const float2 far = make_float2(3.0e38f, 3.0e38f);
			const float2 xi0 = j0 < cnt ? Q.pos[st + j0] : far;
			const float2 xi1 = j1 < cnt ? Q.pos[st + j1] : far;
			float d00 = 0.0f, d01 = 0.0f, d10 = 0.0f, d11 = 0.0f;
			for (int c0 = 0; c0 < L; c0 += kDensChunk) {
				const int n = min(kDensChunk, L - c0);
				__syncwarp();
				for (int e = lane; e < n; e += kWarp) S.pos[e] = Q.pos[seg_src<9>(c0 + e, segOff, segStart)];
				__syncwarp();
				int e = 0;
				for (; e + 4 <= n; e += 4) {
					float2 xj[4];
#pragma unroll
					for (int u = 0; u < 4; ++u) xj[u] = S.pos[e + u];
#pragma unroll
					for (int u = 0; u < 4; ++u) {
						dens_entry(xj[u], xi0, h2, invH, d00, d01);
						dens_entry(xj[u], xi1, h2, invH, d10, d11);
					}
				}
				for (; e < n; ++e) {
					const float2 xj = S.pos[e];
					dens_entry(xj, xi0, h2, invH, d00, d01);
					dens_entry(xj, xi1, h2, invH, d10, d11);
				}
			}
			if (j0 < cnt) {
				Q.dens[st + j0] = make_float2(d00, d01);
				Q.press[st + j0] = make_float2(s.k * (d00 - s.rho0), s.kNear * d01);
			}
			if (j1 < cnt) {
				Q.dens[st + j1] = make_float2(d10, d11);
				Q.press[st + j1] = make_float2(s.k * (d10 - s.rho0), s.kNear * d11);
			}
		}
		__syncwarp();
	}
}

// ---------------------------------------------------------------------------
// Delta sweep (double-density relaxation, demo4.cpp:239-255).  Tasks in
// number order per scene: canonical cells in rank order, then the scene's
// appendix in runs of kAppendixRun consecutive numbers.  A particle's list is
// the 3x3 block of NEW cells around its new cell.  A task stages the new
// cells of its bounding box grown by one, processes its particles in order,
// and writes back only cells inside its particles' 3x3 blocks.  Earlier tasks
// of the scene whose bounding boxes come within two cells are waited for.
// One task per block.  The block stages the task's region once.  A
// particle's list slots (three row ranges of the staged region and its own
// slot) are worked out for a chunk of particles at once, off the serial path.
//
// Particles are relaxed in a two-stage pipeline.  In phase k the producer
// warps (all but the last) scan particle k's list, compact the in-range pairs
// in list order and evaluate them (x_j += D/2), while the summer warp (the
// last) finishes particle k-1: its ordered sum dx -= D/2 and x_{k-1} += dx.
// The only pair of particle k that needs x_{k-1} after that sum is
// (k, k-1): the producers reserve its place in list order, and the summer,
// which knows from k's list ranges whether k-1 is in the list, evaluates it
// right after the sum (x_{k-1} += D/2) and keeps D/2 until the next phase,
// when it fills the reserved place before summing k.  The two roles share no
// data within a phase, so they meet only at the phase's end.  k's own (self)
// pair is kept aside (ownAfter) so that no warp sees k's position change
// before reading it.
// Particles whose lists exceed one pass, and regions staged particle by
// particle, drain the pipeline and run on the whole block in turn.
// Three shapes (sph_kernels.cuh): wide is pipelined with eleven producer
// warps, one block per SM (short per-particle latency, one scene); mid is
// pipelined with seven, two blocks per SM; lean is two warps without the
// pipeline and with smaller staging (more tasks per SM, many scenes).
template <class C>
struct DeltaSmemT {
	static constexpr int kProd = C::kWarps - 1;         // producer warps
	static constexpr int kPass = kProd * C::kChainW;    // list entries per pipelined particle
	static constexpr int kSeqPass = C::kWarps * C::kChainW;  // list entries per pass, whole block
	static constexpr int kHalf = (kSeqPass > kPass ? kSeqPass : kPass) + 16;
	static constexpr int kPhases = C::kPipelined ? 2 : 1;  // half buffers
	float2 pos[C::kStage];
	float4 cand[C::kWarps][C::kChainW];  // per warp: in-range candidates: slot, x_j.x, x_j.y, r2
	float2 half[kPhases][kHalf];  // per phase: delta * 0.5 of the in-range pairs, list order, +0 padded
	int4 meta[2];             // per phase: pairs, reserved index of (k, k-1) or -1, own slot
	float2 ownAfter[2];       // per phase: the particle's position after its self pair
	int4 pslot[C::kPrefetch];  // prefetched per particle: row ranges' first slots, own slot (or -1)
	int4 plen[C::kPrefetch];   // row ranges' lengths
	int pnc[C::kPrefetch];     // new cell and new number (per-particle staging only)
	int pjk[C::kPrefetch];
	float2 ppk[C::kPrefetch];  // pressure and near pressure
	int segOff[C::kRegion + 1];
	int segStart[C::kRegion];
	int owned[C::kRegion];
	int wcnt[C::kWarps];
	int4 oneSlot, oneLen;  // slots of a particle staged on its own
	int task;
	int pend[kPendCap];  // dependencies still pending (wait_canonical)
	int npend;
};

namespace {

struct Region {
	int x0, y0, x1, y1, w, ncells, L;
};

// Stage the new cells of [x0,x1]x[y0,y1] (row-major) from the positions in
// new-number order, where each cell is a contiguous range.  Collective over
// the block; returns false (uniformly) if the region does not fit.
template <class C>
__device__ __forceinline__ bool stage_region(DeltaSmemT<C> &S, Region &R, const Particles &Q, const SimTables &T,
                                             const StepParams &s, int cellBase, int tid) {
	constexpr int kDT = C::kWarps * kWarp;
	R.w = R.x1 - R.x0 + 1;
	R.ncells = R.w * (R.y1 - R.y0 + 1);
	if (R.ncells > C::kRegion) return false;
	if (tid < kWarp) {
		const int lane = tid;
		int carry = 0;
		for (int b0 = 0; b0 < R.ncells; b0 += kWarp) {
			const int q = b0 + lane;
			int nn = 0, st = 0;
			if (q < R.ncells) {
				const int c2 = cellBase + (R.y0 + q / R.w) * s.gx + (R.x0 + q % R.w);
				nn = T.newCount[c2];
				st = T.newStart[c2];
			}
			int incl = nn;
#pragma unroll
			for (int o = 1; o < kWarp; o <<= 1) {
				const int v = __shfl_up_sync(kFull, incl, o);
				if (lane >= o) incl += v;
			}
			if (q < R.ncells) {
				S.segOff[q] = carry + incl - nn;
				S.segStart[q] = st;
				S.owned[q] = 0;
			}
			carry += __shfl_sync(kFull, incl, kWarp - 1);
		}
		if (lane == 0) S.segOff[R.ncells] = carry;
	}
	__syncthreads();
	R.L = S.segOff[R.ncells];
	if (R.L > C::kStage) return false;
	for (int b0 = 0; b0 < R.L; b0 += 4 * kDT) {
		float2 xp[4];
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const int e = b0 + u * kDT + tid;
			if (e < R.L) {
				int lo = 0, hi = R.ncells;
				while (hi - lo > 1) {
					const int mid = (lo + hi) >> 1;
					if (S.segOff[mid] <= e) lo = mid; else hi = mid;
				}
				xp[u] = __ldcg(&Q.pos[S.segStart[lo] + (e - S.segOff[lo])]);
			}
		}
#pragma unroll
		for (int u = 0; u < 4; ++u) {
			const int e = b0 + u * kDT + tid;
			if (e < R.L) S.pos[e] = xp[u];
		}
	}
	__syncthreads();
	return true;
}

// Write the staged positions of the owned cells back.  Flat: one element
// per thread, its cell found by binary search over the region's offsets as
// in staging, so no thread walks the cells one after another.  Otherwise
// cell by cell, with fewer instructions per element.
template <class C>
__device__ __forceinline__ void write_back_owned(DeltaSmemT<C> &S, const Region &R, const Particles &Q, int tid) {
	constexpr int kDT = C::kWarps * kWarp;
	if constexpr (!C::kShortEntry) {
		for (int q = 0; q < R.ncells; ++q) {
			if (!S.owned[q]) continue;
			const int off = S.segOff[q], nn = S.segOff[q + 1] - off, st = S.segStart[q];
			for (int j = tid; j < nn; j += kDT) __stcg(&Q.pos[st + j], S.pos[off + j]);
		}
	} else {
		for (int b0 = 0; b0 < R.L; b0 += 4 * kDT) {
#pragma unroll
			for (int u = 0; u < 4; ++u) {
				const int e = b0 + u * kDT + tid;
				if (e < R.L) {
					int lo = 0, hi = R.ncells;
					while (hi - lo > 1) {
						const int mid = (lo + hi) >> 1;
						if (S.segOff[mid] <= e) lo = mid; else hi = mid;
					}
					if (S.owned[lo]) __stcg(&Q.pos[S.segStart[lo] + (e - S.segOff[lo])], S.pos[e]);
				}
			}
		}
	}
}

// List slots of the particle with new cell nc and new number jk, whose 3x3
// block lies inside the staged region: in the row-major region the three
// cells of one block row are consecutive, so the list (y-major, then x, then
// cell order, demo4.cpp:188-201) is three contiguous ranges of slots.  Marks
// the block's cells as written back.  One thread per particle.
template <class C>
__device__ __forceinline__ void particle_slots(DeltaSmemT<C> &S, const Region &R, int nc, int jk, const StepParams &s,
                                               int cellBase, uint32_t *err, int4 &slot, int4 &len) {
	const int x = (nc - cellBase) % s.gx, y = (nc - cellBase) / s.gx;
	const int xa = max(x - 1, 0), xb = min(x + 1, s.gx - 1);
	int o[3], n[3];
#pragma unroll
	for (int r = 0; r < 3; ++r) {
		const int yy = y + r - 1;
		o[r] = 0;
		n[r] = 0;
		if (yy >= 0 && yy < s.gy) {
			const int rq0 = (yy - R.y0) * R.w + (xa - R.x0);
			const int rq1 = rq0 + (xb - xa);
			o[r] = S.segOff[rq0];
			n[r] = S.segOff[rq1 + 1] - o[r];
			for (int q = rq0; q <= rq1; ++q) S.owned[q] = 1;
		}
	}
	const int ownSeg = (y - R.y0) * R.w + (x - R.x0);
	const int inCell = jk - S.segStart[ownSeg];
	int own = S.segOff[ownSeg] + inCell;
	if (inCell < 0 || inCell >= S.segOff[ownSeg + 1] - S.segOff[ownSeg]) {
		atomicOr(err, kErrIndex);
		own = -1;
	}
	slot = make_int4(o[0], o[1], o[2], own);
	len = make_int4(n[0], n[1], n[2], 0);
}

// delta * 0.5 of one in-range pair (sph.h:483-495 with demo4.cpp:250-251):
// particle at xk with pressures pk, neighbour at xj, r2 = |xj - xk|^2.
__device__ __forceinline__ float2 delta_half(float2 xj, float2 xk, float r2, float2 pk, const StepParams &s) {
	const float rx = xj.x - xk.x, ry = xj.y - xk.y;
	const float rij = sqrtf(r2);
	float len = rij;
	if (len == 0.0f) len = 1.0f;
	const float inv = 1.0f / len;
	const float nx = rx * inv, ny = ry * inv;
	const float term = 1.0f - rij * s.invH;
	const float d = s.dt2 * (pk.x * term + pk.y * (term * term));
	return make_float2(d * nx * 0.5f, d * ny * 0.5f);
}

// dx -= delta * 0.5 over the n buffered halves, in list order
// (demo4.cpp:251), in batches of eight loaded one batch ahead.  The buffer
// is padded with +0 for sixteen entries past n, and dx - (+0) == dx exactly.
__device__ __forceinline__ void sum_halves(const float2 *H, int n, float2 &dx) {
	float2 h[8];
#pragma unroll
	for (int u = 0; u < 8; ++u) h[u] = H[u];
	for (int b = 8; b < n + 8; b += 8) {
		float2 hn[8];
#pragma unroll
		for (int u = 0; u < 8; ++u) hn[u] = H[b + u];
#pragma unroll
		for (int u = 0; u < 8; ++u) {
			dx.x = dx.x - h[u].x;
			dx.y = dx.y - h[u].y;
		}
#pragma unroll
		for (int u = 0; u < 8; ++u) h[u] = hn[u];
	}
}

// Scan and compaction of one particle's list entries [p0, p0 + pl) over
// `nw` warps (this thread is warp `w` of them): each warp takes a contiguous
// range and compacts its in-range entries, in list order, into cand[w].
// Slot `skip` (or -1) is reserved whatever its distance (marked r2 = -1);
// slot `own` records the particle's unmoved position in *ownAfter.
__device__ __forceinline__ int scan_range(float4 *cand, int nw, int w, int lane, int p0, int pl, int4 sl, int len0,
                                          int l01, float2 xk, int own, int skip, const float2 *pos, float h2,
                                          float2 *ownAfter) {
	const int per = (pl + nw - 1) / nw;
	const int e0 = p0 + w * per, e1 = min(p0 + pl, e0 + per);
	int cnt = 0;
	for (int eb = e0; eb < e1; eb += kWarp) {
		const int e = eb + lane;
		bool in = false;
		int slot = 0;
		float2 xj = make_float2(0.f, 0.f);
		float r2 = 0.f;
		if (e < e1) {
			slot = e < len0 ? sl.x + e : (e < l01 ? sl.y + (e - len0) : sl.z + (e - l01));
			if (slot == skip) {
				in = true;
				r2 = -1.0f;
			} else {
				xj = pos[slot];
				const float rx = xj.x - xk.x, ry = xj.y - xk.y;
				r2 = rx * rx + ry * ry;
				in = r2 < h2;
				if (slot == own) *ownAfter = xj;  // out of range: no displacement
			}
		}
		const unsigned mk = __ballot_sync(kFull, in);
		if (in) cand[cnt + __popc(mk & lanemask_lt())] = make_float4(__int_as_float(slot), xj.x, xj.y, r2);
		cnt += __popc(mk);
	}
	return cnt;
}

// Relax one particle on the whole block, not pipelined (demo4.cpp:240-254):
// lists of any length, in passes of kSeqPass entries.  Thread 0 sums.
template <class C>
__device__ __forceinline__ void relax_particle(DeltaSmemT<C> &S, int4 sl, int4 ln, float2 pk, const StepParams &s,
                                               int tid) {
	constexpr int kW = C::kWarps, kPass = DeltaSmemT<C>::kSeqPass;
	const int lane = tid & (kWarp - 1), warp = tid / kWarp;
	const int own = sl.w;
	if (own < 0) return;  // index check failed (uniform)
	const int len0 = ln.x, l01 = ln.x + ln.y, L = l01 + ln.z;
	const float2 xk = S.pos[own];
	float2 *H = S.half[0];
	float2 dx = make_float2(0.0f, 0.0f);  // thread 0
	for (int p0 = 0; p0 < L; p0 += kPass) {
		const int pl = min(L - p0, kPass);
		const int cnt = scan_range(S.cand[warp], kW, warp, lane, p0, pl, sl, len0, l01, xk, own, -1, S.pos, s.h2,
		                           &S.ownAfter[0]);
		if (lane == 0) S.wcnt[warp] = cnt;
		__syncthreads();
		int before = 0, total = 0;
#pragma unroll
		for (int w = 0; w < kW; ++w) {
			const int c = S.wcnt[w];
			before += (w < warp) ? c : 0;
			total += c;
		}
		if (tid < 16) H[total + tid] = make_float2(0.0f, 0.0f);
		for (int q = lane; q < cnt; q += kWarp) {
			const float4 cd = S.cand[warp][q];
			const float2 xj = make_float2(cd.y, cd.z);
			const float2 h = delta_half(xj, xk, cd.w, pk, s);
			const int slot = __float_as_int(cd.x);
			const float2 moved = make_float2(h.x + xj.x, h.y + xj.y);
			if (slot == own) S.ownAfter[0] = moved; else S.pos[slot] = moved;
			H[before + q] = h;
		}
		__syncthreads();
		if (tid == 0) {
			sum_halves(H, total, dx);
			if (p0 + kPass >= L) {
				const float2 xo = S.ownAfter[0];
				S.pos[own] = make_float2(dx.x + xo.x, dx.y + xo.y);
			}
		}
		__syncthreads();
	}
}

// Summer warp, lane 0: finish the particle of phase buffer b (fill its
// reserved pair with hres, its ordered dx sum, its final position).
// Returns the final position.
template <class C>
__device__ __forceinline__ float2 finish_particle(DeltaSmemT<C> &S, int b, float2 hres) {
	const int4 m = S.meta[b];
	float2 *H = S.half[b];
	if (m.y >= 0) H[m.y] = hres;
	float2 dx = make_float2(0.0f, 0.0f);
	sum_halves(H, m.x, dx);
	const float2 xo = S.ownAfter[b];
	const float2 xp = make_float2(dx.x + xo.x, dx.y + xo.y);
	S.pos[m.z] = xp;
	return xp;
}

template <class C>
__device__ __forceinline__ void producers_bar() {
	__syncwarp();
	asm volatile("bar.sync 1, %0;" ::"r"(DeltaSmemT<C>::kProd * kWarp) : "memory");
}

// Producers' part of phase b for particle (sl, ln, pk): everything but the
// pair with slot `prev` (the particle still being finished, or -1).
template <class C>
__device__ __forceinline__ void produce(DeltaSmemT<C> &S, int b, int4 sl, int4 ln, float2 pk, int prev,
                                        const StepParams &s, int tid) {
	constexpr int kP = DeltaSmemT<C>::kProd;
	const int lane = tid & (kWarp - 1), warp = tid / kWarp;
	const int own = sl.w;
	const int len0 = ln.x, l01 = ln.x + ln.y, L = l01 + ln.z;
	const float2 xk = S.pos[own];
	float2 *H = S.half[b];
	if (tid == 0) S.meta[b].y = -1;
	const int cnt = scan_range(S.cand[warp], kP, warp, lane, 0, L, sl, len0, l01, xk, own, prev, S.pos, s.h2,
	                           &S.ownAfter[b]);
	int before = 0, total = cnt;
	if (kP > 1) {
		if (lane == 0) S.wcnt[warp] = cnt;
		producers_bar<C>();
		total = 0;
#pragma unroll
		for (int w = 0; w < kP; ++w) {
			const int c = S.wcnt[w];
			before += (w < warp) ? c : 0;
			total += c;
		}
	} else {
		__syncwarp();
	}
	if (tid < 16) H[total + tid] = make_float2(0.0f, 0.0f);
	for (int q = lane; q < cnt; q += kWarp) {
		const float4 cd = S.cand[warp][q];
		if (cd.w < 0.0f) {
			S.meta[b].y = before + q;  // (k, k-1): the summer evaluates it
			continue;
		}
		const float2 xj = make_float2(cd.y, cd.z);
		const float2 h = delta_half(xj, xk, cd.w, pk, s);
		const int slot = __float_as_int(cd.x);
		const float2 moved = make_float2(h.x + xj.x, h.y + xj.y);
		if (slot == own) S.ownAfter[b] = moved; else S.pos[slot] = moved;
		H[before + q] = h;
	}
	if (tid == 0) {
		S.meta[b].x = total;
		S.meta[b].z = own;
	}
}

// Summer's part of phase b (lane 0): finish the previous particle (buffer
// b ^ 1), then evaluate the pair (k, k-1) of particle k (list slots sl, ln,
// pressures pk) if k-1 is in k's list; its D/2 goes to hres.
template <class C>
__device__ __forceinline__ void summer(DeltaSmemT<C> &S, int b, int4 sl, int4 ln, float2 pk, const StepParams &s,
                                       float2 &hres) {
	const int prev = S.meta[b ^ 1].z;
	const float2 xp = finish_particle<C>(S, b ^ 1, hres);
	hres = make_float2(0.0f, 0.0f);
	const bool inList = (prev >= sl.x && prev < sl.x + ln.x) || (prev >= sl.y && prev < sl.y + ln.y) ||
	                    (prev >= sl.z && prev < sl.z + ln.z);
	if (!inList) return;
	const float2 xk = S.pos[sl.w];
	const float rx = xp.x - xk.x, ry = xp.y - xk.y;
	const float r2 = rx * rx + ry * ry;
	if (r2 < s.h2) {
		const float2 h = delta_half(xp, xk, r2, pk, s);
		S.pos[prev] = make_float2(h.x + xp.x, h.y + xp.y);
		hres = h;
	}
}

// Process particles [p0, p1) (old numbers, or positions in AddParticle order
// mapped to old numbers by `ord`) in order: one staged region if it fits
// (pipelined), otherwise one 3x3 region per particle.  Per-particle
// inputs (new cell, new number, pressure, list slots) are prefetched in
// chunks, off the serial path.
template <class C>
__device__ __forceinline__ unsigned long long relax_group(DeltaSmemT<C> &S, int p0, int p1, const int *ord, int bx0,
                                                          int by0, int bx1, int by1, const Particles &Q,
                                                          const SimTables &T, const StepParams &s, int cellBase,
                                                          int tid) {
	// Returns when the region was staged (global ns), for the task
	// timestamps (sph_profile_tasks).
	constexpr int kDT = C::kWarps * kWarp;
	constexpr int kP = DeltaSmemT<C>::kProd;
	const int warp = tid / kWarp, lane = tid & (kWarp - 1);
	Region R;
	R.x0 = max(bx0 - 1, 0);
	R.y0 = max(by0 - 1, 0);
	R.x1 = min(bx1 + 1, s.gx - 1);
	R.y1 = min(by1 + 1, s.gy - 1);
	// Per-particle inputs of the first chunk (one particle per thread) do not
	// depend on the staged positions: their loads can overlap the staging.
	static_assert(kDT >= C::kPrefetch, "a chunk holds at most one particle per thread");
	int jk0 = 0, nc0 = 0;
	float2 pk0 = make_float2(0.0f, 0.0f);
	if (C::kShortEntry && p0 + tid < min(p1, p0 + C::kPrefetch)) {
		const int q = ord ? ord[p0 + tid] : p0 + tid;
		jk0 = T.newLabel[q];
		nc0 = T.newCell[q];
		pk0 = Q.press[jk0];
	}
	const bool staged = stage_region<C>(S, R, Q, T, s, cellBase, tid);
	const unsigned long long tStaged = global_ns();
	bool pending = false;  // the previous particle still needs its sum (buffer ph ^ 1)
	int ph = 0;
	float2 hres = make_float2(0.0f, 0.0f);  // summer: D/2 of the pending particle's reserved pair
	for (int c0 = p0; c0 < p1; c0 += C::kPrefetch) {
		const int c1 = min(p1, c0 + C::kPrefetch);
		for (int k = c0 + tid; k < c1; k += kDT) {
			const bool first = C::kShortEntry && c0 == p0;
			const int q = ord ? ord[k] : k;
			const int jk = first ? jk0 : T.newLabel[q];
			const int nc = first ? nc0 : T.newCell[q];
			S.ppk[k - c0] = first ? pk0 : Q.press[jk];
			if (staged) {
				particle_slots<C>(S, R, nc, jk, s, cellBase, T.error, S.pslot[k - c0], S.plen[k - c0]);
			} else {
				S.pnc[k - c0] = nc;
				S.pjk[k - c0] = jk;
			}
		}
		__syncthreads();
		for (int k = c0; k < c1; ++k) {
			const float2 pk = S.ppk[k - c0];
			if (staged) {
				const int4 sl = S.pslot[k - c0], ln = S.plen[k - c0];
				if (C::kPipelined && sl.w >= 0 && ln.x + ln.y + ln.z <= DeltaSmemT<C>::kPass) {
					const int b = (ph & 1) % DeltaSmemT<C>::kPhases;
					if (warp < kP) {
						produce<C>(S, b, sl, ln, pk, pending ? S.meta[b ^ 1].z : -1, s, tid);
					} else if (pending && lane == 0) {
						summer<C>(S, b, sl, ln, pk, s, hres);
					}
					__syncthreads();
					pending = true;
					++ph;
					continue;
				}
				// Drain the pipeline, then relax this particle on the whole block.
				if (C::kPipelined && pending && warp == kP && lane == 0) finish_particle<C>(S, (ph & 1) ^ 1, hres);
				__syncthreads();
				pending = false;
				relax_particle<C>(S, sl, ln, pk, s, tid);
				continue;
			}
			const int nc = S.pnc[k - c0], jk = S.pjk[k - c0];
			Region R1;
			const int x = (nc - cellBase) % s.gx, y = (nc - cellBase) / s.gx;
			R1.x0 = max(x - 1, 0);
			R1.y0 = max(y - 1, 0);
			R1.x1 = min(x + 1, s.gx - 1);
			R1.y1 = min(y + 1, s.gy - 1);
			if (!stage_region<C>(S, R1, Q, T, s, cellBase, tid)) {
				if (tid == 0) atomicOr(T.error, kErrStageOverflow);
				__syncthreads();
				continue;
			}
			if (tid == 0) particle_slots<C>(S, R1, nc, jk, s, cellBase, T.error, S.oneSlot, S.oneLen);
			__syncthreads();
			relax_particle<C>(S, S.oneSlot, S.oneLen, pk, s, tid);
			write_back_owned<C>(S, R1, Q, tid);
			__syncthreads();
		}
		__syncthreads();
	}
	if (C::kPipelined && pending && warp == kP && lane == 0) finish_particle<C>(S, (ph & 1) ^ 1, hres);
	__syncthreads();
	if (staged) write_back_owned<C>(S, R, Q, tid);
	return tStaged;
}

// Wait for canonical tasks of the scene (old cells) near [bx0,bx1]x[by0,by1]
// whose new-cell bounding boxes come within two cells of it and whose task
// index is below `limit`.  Collective over the block.  The block first
// collects the dependencies not yet done (one acquire load each) into
// `pend`; then warp 0 alone polls them while the other warps wait at the
// barrier, so a waiting block adds one warp's polling to the memory system
// rather than every warp's (in crowded states many blocks wait at once, and
// their polling starved the running tasks' loads).  If more than kPendCap
// are pending, every warp polls its share of the window as well.
template <int kDT>
__device__ __forceinline__ void wait_canonical(int bx0, int by0, int bx1, int by1, int moveMax, int limit,
                                               int selfCell, const SimTables &T, const StepParams &s,
                                               int cellBase, int *pend, int *npend, int tid) {
	const int rad = 2 + moveMax;
	const int x0 = max(bx0 - rad, 0), x1 = min(bx1 + rad, s.gx - 1);
	const int y0 = max(by0 - rad, 0), y1 = min(by1 + rad, s.gy - 1);
	const int w = x1 - x0 + 1;
	const int total = w * (y1 - y0 + 1);
	const int lane = tid & (kWarp - 1);
	if (tid == 0) *npend = 0;
	__syncthreads();
	for (int q0 = 0; q0 < total; q0 += kDT) {
		const int q = q0 + tid;
		int r = -1;
		if (q < total) {
			const int c2 = cellBase + (y0 + q / w) * s.gx + (x0 + q % w);
			const int r2 = T.taskOfCell[c2];
			if (c2 != selfCell && r2 < limit && T.cellCount[c2] > 0) {
				const int4 b = *reinterpret_cast<const int4 *>(&T.bbox[4 * c2]);
				if (rect_dist(b.x, b.y, b.z, b.w, bx0, by0, bx1, by1) <= 2 && ld_acquire(&T.done[r2]) == 0u) r = r2;
			}
		}
		const unsigned m = __ballot_sync(kFull, r >= 0);
		int base = 0;
		if (lane == 0 && m != 0u) base = atomicAdd(npend, __popc(m));
		base = __shfl_sync(kFull, base, 0);
		if (r >= 0) {
			const int k = base + __popc(m & lanemask_lt());
			if (k < kPendCap) pend[k] = r;
		}
	}
	__syncthreads();
	const int np = *npend;
	if (np > kPendCap) {
		// Too many to list: every warp polls its share of the window.
		for (int q0 = 0; q0 < total; q0 += kDT) {
			const int q = q0 + tid;
			const uint32_t *flag = nullptr;
			if (q < total) {
				const int c2 = cellBase + (y0 + q / w) * s.gx + (x0 + q % w);
				const int r2 = T.taskOfCell[c2];
				if (c2 != selfCell && r2 < limit && T.cellCount[c2] > 0) {
					const int4 b = *reinterpret_cast<const int4 *>(&T.bbox[4 * c2]);
					if (rect_dist(b.x, b.y, b.z, b.w, bx0, by0, bx1, by1) <= 2) flag = &T.done[r2];
				}
			}
			warp_wait(flag, T.abort, T.error, T.waitLimitNs);
		}
	} else if (tid < kWarp) {
		for (int k0 = 0; k0 < np; k0 += kWarp)
			warp_wait(k0 + lane < np ? &T.done[pend[k0 + lane]] : nullptr, T.abort, T.error, T.waitLimitNs);
	}
	__syncthreads();
}

}  // namespace

template <class C>
__global__ void __launch_bounds__(C::kWarps * kWarp, C::kMinBlocks) k_delta(Totals tt, Particles Q, SimTables T) {
	constexpr int kDT = C::kWarps * kWarp;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	DeltaSmemT<C> &S = *reinterpret_cast<DeltaSmemT<C> *>(smem_raw);
	const int tid = threadIdx.x;
	const int nLive = tt.refOrder ? 0 : *T.nLive;
	const int ntask = nLive + tt.nApp;
	const int moveMax = T.moverCount[1];
	const int *ord = tt.refOrder ? T.refOrd : nullptr;
	for (;;) {
		if (tid == 0) S.task = atomicAdd(&T.taskCounter[1], 1);
		__syncthreads();
		const int i = S.task;
		__syncthreads();
		if (i >= ntask) break;
		// Task index (done flag): canonical cell task, or ncell + appendix run.
		const int t = i < nLive ? T.liveTask[i] : tt.ncell + (i - nLive);
		stamp(T, 1, t, 0, tid);
		if (i < nLive) {
			const int c = T.taskCell[t];
			const int p0 = T.cellStart[c], cnt = T.cellCount[c];
			if (cnt > 0) {
				const SceneDev &sc = T.scenes[T.sceneOfCell[c]];
				const StepParams s = sc.p;
				const int4 b = *reinterpret_cast<const int4 *>(&T.bbox[4 * c]);
				wait_canonical<kDT>(b.x, b.y, b.z, b.w, moveMax, t, c, T, s, sc.cellBase, S.pend, &S.npend, tid);
				stamp(T, 1, t, 1, tid);
				const unsigned long long staged =
				    relax_group<C>(S, p0, p0 + cnt, nullptr, b.x, b.y, b.z, b.w, Q, T, s, sc.cellBase, tid);
				if (T.prof != nullptr && tid == 0 && t < T.profStride)
					T.prof[((size_t)1 * T.profStride + t) * 4 + 2] = staged;
				__syncthreads();
				__threadfence();
			}
		} else {
			// Appendix run: particles added since the last update, after all
			// canonical tasks; it waits for the earlier runs of its scene
			// whose new cells come within two cells of its own.  In reference
			// order every task is such a run, over the whole scene in
			// AddParticle order.
			const int a = t - tt.ncell;
			const int scene = T.appScene[a];
			const SceneDev &sc = T.scenes[scene];
			const StepParams s = sc.p;
			const int base = sc.cellBase;
			const int p0 = sc.pBase + (tt.refOrder ? 0 : sc.n0) + T.appRun[a] * kAppendixRun;
			const int p1 = min(sc.pBase + sc.n, p0 + kAppendixRun);
			const int4 box = *reinterpret_cast<const int4 *>(&T.appBox[4 * a]);
			const int bx0 = box.x, by0 = box.y, bx1 = box.z, by1 = box.w;
			if (!tt.refOrder)
				wait_canonical<kDT>(bx0, by0, bx1, by1, moveMax, tt.ncell, -1, T, s, base, S.pend, &S.npend, tid);
			for (int q0 = 0; q0 < a; q0 += kDT) {
				const int q = q0 + tid;
				const uint32_t *flag = nullptr;
				if (q < a && T.appScene[q] == scene) {
					const int4 o = *reinterpret_cast<const int4 *>(&T.appBox[4 * q]);
					if (rect_dist(o.x, o.y, o.z, o.w, bx0, by0, bx1, by1) <= 2) flag = &T.done[tt.ncell + q];
				}
				warp_wait(flag, T.abort, T.error, T.waitLimitNs);
			}
			__syncthreads();
			relax_group<C>(S, p0, p1, ord, bx0, by0, bx1, by1, Q, T, s, base, tid);
			__syncthreads();
			__threadfence();
		}
		__syncthreads();
		stamp(T, 1, t, 3, tid);
		if (tid == 0 && i != T.hold[1]) st_release(&T.done[t], 1u);
	}
}

// Collisions (demo4.cpp:411-444, sph.h:514-681), velocity (demo4.cpp:446-450)
// and the renumbering into canonical order: the particle at position j of
// new cell c gets number newStart[c] + j.

namespace {

__device__ __forceinline__ float2 v2(float x, float y) { return make_float2(x, y); }

__device__ __forceinline__ float2 normalize2(float2 v) {
	float len = sqrtf(v.x * v.x + v.y * v.y);
	if (len == 0.0f) len = 1.0f;
	const float inv = 1.0f / len;
	return v2(v.x * inv, v.y * inv);
}

__device__ void solve_plane(float2 &p, const Body &b, const StepParams &s) {
	const float2 pp = v2(b.ax * b.r, b.ay * b.r);
	const float2 d = v2(p.x - pp.x, p.y - pp.y);
	const float proj = d.x * b.ax + d.y * b.ay;
	if (proj <= s.radius) {
		const float pen = s.radius - proj;
		p = v2(b.ax * pen + p.x, b.ay * pen + p.y);
	}
}

__device__ void solve_circle(float2 &p, const Body &b, const StepParams &s) {
	const float both = b.r + s.radius;
	const float2 d = v2(p.x - b.ax, p.y - b.ay);
	const float d2 = d.x * d.x + d.y * d.y;
	if (d2 <= both * both) {
		if (fabsf(d2) > 0.0f) {
			const float dist = sqrtf(d2);
			const float inv = 1.0f / dist;
			const float2 nrm = v2(d.x * inv, d.y * inv);
			const float pen = both - dist;
			p = v2(nrm.x * pen + p.x, nrm.y * pen + p.y);
		}
	}
}

__device__ void solve_segment(float2 &p, const Body &b, const StepParams &s) {
	const float both = s.margin + s.radius;
	const float2 a = v2(b.ax, b.ay), bb = v2(b.bx, b.by);
	const float2 e = v2(bb.x - a.x, bb.y - a.y);
	const float u = e.x * (bb.x - p.x) + e.y * (bb.y - p.y);
	const float v = e.x * (p.x - a.x) + e.y * (p.y - a.y);
	float2 closest, nrm;
	if (v <= 0.0f) {
		closest = a;
		const float2 d = v2(p.x - closest.x, p.y - closest.y);
		if (d.x * d.x + d.y * d.y > both * both) return;
		nrm = normalize2(v2(p.x - closest.x, p.y - closest.y));
	} else if (u <= 0.0f) {
		closest = bb;
		const float2 d = v2(p.x - closest.x, p.y - closest.y);
		if (d.x * d.x + d.y * d.y > both * both) return;
		nrm = normalize2(v2(p.x - closest.x, p.y - closest.y));
	} else {
		const float den = e.x * e.x + e.y * e.y;
		const float inv = 1.0f / den;
		closest = v2((a.x * u + bb.x * v) * inv, (a.y * u + bb.y * v) * inv);
		const float2 d = v2(p.x - closest.x, p.y - closest.y);
		if (d.x * d.x + d.y * d.y > both * both) return;
		nrm = v2(-e.y, e.x);
		if (nrm.x * (p.x - a.x) + nrm.y * (p.y - a.y) < 0.0f) nrm = v2(-nrm.x, -nrm.y);
		nrm = normalize2(nrm);
	}
	const float2 dp = v2(p.x - closest.x, p.y - closest.y);
	const float dist = nrm.x * dp.x + nrm.y * dp.y;
	const float pen = both - dist;
	p = v2(nrm.x * pen + p.x, nrm.y * pen + p.y);
}

// FindMTVCirclePolygon + SPHSolvePolygonCollision (sph.h:600-681), keeping
// the reference's Vec2DistanceSquared, which squares the product of the
// coordinate differences (vecmath.h:292-296).
__device__ void solve_polygon(float2 &p, const Body &b, const StepParams &s) {
	const float radius = s.margin + s.radius;
	const int n = b.vertexCount;
	if (n <= 0 || n > kMaxPoly) return;
	int edge = 0;
	float2 normal = v2(0.f, 0.f);
	float separation = -3.40282347e+38f;
	for (int k = 0; k < n; ++k) {
		const int k2 = (k + 1) % n;
		const float2 a = v2(b.verts[2 * k], b.verts[2 * k + 1]);
		const float2 c = v2(b.verts[2 * k2], b.verts[2 * k2 + 1]);
		const float2 ab = v2(c.x - a.x, c.y - a.y);
		const float2 nn = normalize2(v2(1.0f * ab.y, -1.0f * ab.x));
		const float sep = nn.x * (p.x - a.x) + nn.y * (p.y - a.y);
		if (sep > radius) return;
		if (sep > separation) {
			normal = nn;
			separation = sep;
			edge = k;
		}
	}
	const int e2 = (edge + 1) % n;
	const float2 v1 = v2(b.verts[2 * edge], b.verts[2 * edge + 1]);
	const float2 v2p = v2(b.verts[2 * e2], b.verts[2 * e2 + 1]);
	float2 mtv;
	if (separation < 1.1920929e-07f) {
		const float pen = radius - separation;
		mtv = v2(normal.x * pen, normal.y * pen);
	} else {
		const float u1 = (p.x - v1.x) * (v2p.x - v1.x) + (p.y - v1.y) * (v2p.y - v1.y);
		const float u2 = (p.x - v2p.x) * (v1.x - v2p.x) + (p.y - v2p.y) * (v1.y - v2p.y);
		if (u1 <= 0.0f) {
			const float f = (v1.x - p.x) * (v1.y - p.y);
			if (f * f > radius * radius) return;
			const float2 d = v2(p.x - v1.x, p.y - v1.y);
			const float2 nn = normalize2(d);
			const float pen = radius - (nn.x * d.x + nn.y * d.y);
			mtv = v2(nn.x * pen, nn.y * pen);
		} else if (u2 <= 0.0f) {
			const float f = (v2p.x - p.x) * (v2p.y - p.y);
			if (f * f > radius * radius) return;
			const float2 d = v2(p.x - v2p.x, p.y - v2p.y);
			const float2 nn = normalize2(d);
			const float pen = radius - (nn.x * d.x + nn.y * d.y);
			mtv = v2(nn.x * pen, nn.y * pen);
		} else {
			const float2 mid = v2((1.0f - 0.5f) * v1.x + 0.5f * v2p.x, (1.0f - 0.5f) * v1.y + 0.5f * v2p.y);
			const float sd = (p.x - mid.x) * normal.x + (p.y - mid.y) * normal.y;
			if (sd > radius) return;
			const float pen = radius - sd;
			mtv = v2(normal.x * pen, normal.y * pen);
		}
	}
	p = v2(mtv.x + p.x, mtv.y + p.y);
}

}  // namespace

__global__ void __launch_bounds__(kCollideThreads) k_collide(Totals tt, Particles P, Particles Q, SimTables T) {
	// j: new number.  Positions, densities and pressures are already in new
	// order; the rest is gathered from the old number.
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j < tt.ncell) T.appCount[j] = 0;
	if (j >= tt.n) return;
	const SceneDev &sc = T.scenes[T.sceneOf[j]];
	const StepParams &s = sc.p;
	float2 x = Q.pos[j];
	for (int b = 0; b < s.nbodies; ++b) {
		const Body &bd = T.bodies[sc.bodyBase + b];
		switch (bd.type) {
			case kBodyPlane: solve_plane(x, bd, s); break;
			case kBodyCircle: solve_circle(x, bd, s); break;
			case kBodySegment: solve_segment(x, bd, s); break;
			case kBodyPolygon: solve_polygon(x, bd, s); break;
			default: break;
		}
	}
	int o = T.newIdx[j];
	if (o < 0 || o >= tt.n) {
		atomicOr(T.error, kErrIndex);
		o = 0;
	}
	const float2 pv = P.prev[o];
	Q.pos[j] = x;
	Q.prev[j] = pv;
	Q.vel[j] = make_float2((x.x - pv.x) * s.invDt, (x.y - pv.y) * s.invDt);
	Q.acc[j] = make_float2(0.0f, 0.0f);
	Q.id[j] = P.id[o];
	Q.cellOf[j] = T.newCell[o];
}

// ---------------------------------------------------------------------------
// Learned correction of a finished update: x += h u, bodies as in the
// collision stage, velocity from the previous position (canonical numbering).
__global__ void __launch_bounds__(kCollideThreads) k_learned_finish(Totals tt, Particles P, const float2 *u,
                                                                   SimTables T) {
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= tt.n) return;
	const SceneDev &sc = T.scenes[T.sceneOf[j]];
	const StepParams &s = sc.p;
	const float2 d = u[j];
	float2 x = P.pos[j];
	x = make_float2(x.x + s.h * d.x, x.y + s.h * d.y);
	for (int b = 0; b < s.nbodies; ++b) {
		const Body &bd = T.bodies[sc.bodyBase + b];
		switch (bd.type) {
			case kBodyPlane: solve_plane(x, bd, s); break;
			case kBodyCircle: solve_circle(x, bd, s); break;
			case kBodySegment: solve_segment(x, bd, s); break;
			case kBodyPolygon: solve_polygon(x, bd, s); break;
			default: break;
		}
	}
	const float2 pv = P.prev[j];
	P.pos[j] = x;
	P.vel[j] = make_float2((x.x - pv.x) * s.invDt, (x.y - pv.y) * s.invDt);
}

// ---------------------------------------------------------------------------
// AddParticle (demo4.cpp:142-153) for a batch of numbers [first, first+count)
// of scene `scene`: the new particles join the appendix of their cell.
__global__ void k_add(int first, int count, int scene, int firstId, const float2 *pos, const float2 *force,
                      Particles P, SimTables T) {
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= count) return;
	const SceneDev &sc = T.scenes[scene];
	const int i = first + j;
	const float2 x = pos[j];
	P.pos[i] = x;
	P.prev[i] = x;
	P.vel[i] = make_float2(0.f, 0.f);
	P.acc[i] = force[j];
	P.dens[i] = make_float2(0.f, 0.f);
	P.press[i] = make_float2(0.f, 0.f);
	P.id[i] = firstId + j;
	if (P.springN) P.springN[i] = 0;
	T.sceneOf[i] = scene;
	const int c = sc.cellBase + cell_of(x, sc.p);
	P.cellOf[i] = c;
	const int before = atomicAdd(&T.appCount[c], 1);
	const uint32_t now = (uint32_t)(T.cellCount[c] + before + 1);
	atomicMin(&T.stats[4 * scene + 2], now);
	atomicMax(&T.stats[4 * scene + 3], now);
}

// Checks of a state given to sph_load_state, on the device (one thread per
// particle and per cell): every cell range lies within the canonical
// particles, every particle's cell and AddParticle index are in range, and
// every canonical particle lies in its cell's range, and no two particles
// share an AddParticle index (seen[] starts at zero).  Particles added since
// the last update (numbers >= n0) are counted per cell into appOut.
// verdict[0] collects failures, verdict[1] the sum of the cell counts.
__global__ void k_check_state(int n, int n0, int ncell, const int *cell, const int *start, const int *count,
                              const int *id, int *appOut, int *seen, int *verdict) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	int bad = 0;
	if (i < ncell) {
		const int st = start[i], cn = count[i];
		bad |= st < 0 || cn < 0 || (long long)st + cn > n0;
		if (!bad && cn) atomicAdd(&verdict[1], cn);
	}
	if (i < n) {
		const int c = cell[i];
		const int k = id[i];
		bad |= c < 0 || c >= ncell || k < 0 || k >= n;
		if (!bad) bad |= atomicAdd(&seen[k], 1) != 0;  // AddParticle indices are distinct
		if (!bad) {
			if (i >= n0) {
				atomicAdd(&appOut[c], 1);
			} else {
				const int st = start[c], cn = count[c];
				bad |= i < st || i >= st + cn;
			}
		}
	}
	if (bad) atomicOr(&verdict[0], 1);
}

// Scatter numbers [first, first+count) into AddParticle order for host reads.
__global__ void k_gather_by_id(int first, int count, const int *id, const float2 *src, float2 *dst) {
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= count) return;
	const int k = id[first + j];
	if (k >= 0 && k < count) dst[k] = src[first + j];
}

template <class C>
size_t visc_smem_bytes() {
	return sizeof(ViscSmemT<C>);
}
template <class C>
size_t delta_smem_bytes() {
	return sizeof(DeltaSmemT<C>);
}
cudaError_t sweep_attributes() {
	cudaError_t e = cudaFuncSetAttribute(k_viscosity<ViscWide>, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                     (int)visc_smem_bytes<ViscWide>());
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(k_viscosity_multi<ViscLean>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)sizeof(ViscMultiSmemT<ViscLean>));
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(k_delta<DeltaWide>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)delta_smem_bytes<DeltaWide>());
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(k_delta<DeltaLean>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)delta_smem_bytes<DeltaLean>());
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(k_delta<DeltaMid>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)delta_smem_bytes<DeltaMid>());
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(k_delta<DeltaTri>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)delta_smem_bytes<DeltaTri>());
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(k_delta<DeltaQuad>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)delta_smem_bytes<DeltaQuad>());
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(k_delta<DeltaDense>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)delta_smem_bytes<DeltaDense>());
	return e;
}

cudaError_t sweep_occupancy(bool viscLean, int deltaShape, int *occV, int *occD) {
	cudaError_t e = viscLean ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(occV, k_viscosity_multi<ViscLean>,
	                                                                         ViscLean::kWarps * kWarp,
	                                                                         sizeof(ViscMultiSmemT<ViscLean>))
	                         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(occV, k_viscosity<ViscWide>,
	                                                                         ViscWide::kWarps * kWarp,
	                                                                         visc_smem_bytes<ViscWide>());
	if (e != cudaSuccess) return e;
	if (deltaShape == kDeltaLean)
		return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occD, k_delta<DeltaLean>, DeltaLean::kWarps * kWarp,
		                                                     delta_smem_bytes<DeltaLean>());
	if (deltaShape == kDeltaMid)
		return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occD, k_delta<DeltaMid>, DeltaMid::kWarps * kWarp,
		                                                     delta_smem_bytes<DeltaMid>());
	if (deltaShape == kDeltaTri)
		return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occD, k_delta<DeltaTri>, DeltaTri::kWarps * kWarp,
		                                                     delta_smem_bytes<DeltaTri>());
	if (deltaShape == kDeltaQuad)
		return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occD, k_delta<DeltaQuad>, DeltaQuad::kWarps * kWarp,
		                                                     delta_smem_bytes<DeltaQuad>());
	if (deltaShape == kDeltaDense)
		return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occD, k_delta<DeltaDense>, DeltaDense::kWarps * kWarp,
		                                                     delta_smem_bytes<DeltaDense>());
	return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occD, k_delta<DeltaWide>, DeltaWide::kWarps * kWarp,
	                                                     delta_smem_bytes<DeltaWide>());
}

void launch_viscosity(bool lean, int blocks, cudaStream_t st, Totals tt, Particles P, SimTables T) {
	if (lean)
		k_viscosity_multi<ViscLean>
		    <<<blocks, ViscLean::kWarps * kWarp, sizeof(ViscMultiSmemT<ViscLean>), st>>>(tt, P, T);
	else
		k_viscosity<ViscWide><<<blocks, ViscWide::kWarps * kWarp, visc_smem_bytes<ViscWide>(), st>>>(tt, P, T);
}

void launch_delta(int shape, int blocks, cudaStream_t st, Totals tt, Particles Q, SimTables T) {
	if (shape == kDeltaLean)
		k_delta<DeltaLean><<<blocks, DeltaLean::kWarps * kWarp, delta_smem_bytes<DeltaLean>(), st>>>(tt, Q, T);
	else if (shape == kDeltaMid)
		k_delta<DeltaMid><<<blocks, DeltaMid::kWarps * kWarp, delta_smem_bytes<DeltaMid>(), st>>>(tt, Q, T);
	else if (shape == kDeltaTri)
		k_delta<DeltaTri><<<blocks, DeltaTri::kWarps * kWarp, delta_smem_bytes<DeltaTri>(), st>>>(tt, Q, T);
	else if (shape == kDeltaQuad)
		k_delta<DeltaQuad><<<blocks, DeltaQuad::kWarps * kWarp, delta_smem_bytes<DeltaQuad>(), st>>>(tt, Q, T);
	else if (shape == kDeltaDense)
		k_delta<DeltaDense><<<blocks, DeltaDense::kWarps * kWarp, delta_smem_bytes<DeltaDense>(), st>>>(tt, Q, T);
	else
		k_delta<DeltaWide><<<blocks, DeltaWide::kWarps * kWarp, delta_smem_bytes<DeltaWide>(), st>>>(tt, Q, T);
}
size_t dens_smem_bytes() { return sizeof(DensWarp) * kDensWarps; }

}  // namespace sphgb
