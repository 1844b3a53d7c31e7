// Viscoelastic springs with plasticity (Clavet et al. 2005, "Particle-based
// viscoelastic fluid simulation", Algorithms 3 and 4).  The reference's
// Demo4 step has no springs; this is the deterministic parallel form of the
// paper's two loops, run after the grid update (new numbering, predicted
// positions) and before density:
//
//  k_springs_select  per particle: adjust existing springs within h, drop
//                    those whose rest length exceeds h, and choose the nearest
//                    in-range candidates without a spring for the free slots,
//                    ordered by (r^2, AddParticle index);
//  k_springs_commit  add a spring where both ends chose each other (rest
//                    length h, adjusted like the others);
//  k_springs_apply   move every particle by -D/2 of each of its springs,
//                    D = dt^2 k (1 - L/h) (L - r) r_hat, from the positions
//                    before the phase (Jacobi), summed in slot order.
//
// Every spring is stored at both ends.  Both ends compute the same length r
// (the two difference vectors are exact negations), so they keep equal rest
// lengths and drop the spring together.  Spring partners are particle
// numbers, remapped to the new numbering here.
#include <cuda_runtime.h>

#include "sph_internal.cuh"
#include "sph_kernels.cuh"

namespace sphgb {

namespace {

constexpr unsigned kFullMask = 0xffffffffu;

// Rest length of a spring of length r < h after plasticity (Algorithm 4).
__device__ __forceinline__ float plastic(float L, float r, const StepParams &s) {
	const float d = s.springYield * L;
	if (r > L + d) return L + s.springDtAlpha * ((r - L) - d);
	if (r < L - d) return L - s.springDtAlpha * ((L - d) - r);
	return L;
}

// Candidate order: nearer first, then the smaller AddParticle index.
__device__ __forceinline__ bool before(float r2a, int ta, float r2b, int tb) {
	return r2a < r2b || (r2a == r2b && ta < tb);
}

template <int NSEG>
__device__ __forceinline__ int seg_number(int e, const int (&off)[NSEG], const int (&start)[NSEG]) {
	int src = start[0] + e;
#pragma unroll
	for (int q = 1; q < NSEG; ++q) src = (e >= off[q]) ? start[q] + (e - off[q]) : src;
	return src;
}

// Staged index of number `num` in the 3x3 block (segments of consecutive
// numbers), or -1 if it lies outside the block.
__device__ __forceinline__ int staged_index(int num, const int (&off)[9], const int (&start)[9], int L) {
	int e = -1;
#pragma unroll
	for (int q = 0; q < 9; ++q) {
		const int len = (q < 8 ? off[q + 1] : L) - off[q];
		if (num >= start[q] && num < start[q] + len) e = off[q] + (num - start[q]);
	}
	return e;
}

}  // namespace

// One warp per new cell: the 3x3 block of new cells (positions, numbers'
// AddParticle indices) is staged once; each lane handles one particle of the
// cell's existing springs.  Candidates are then chosen either by the whole
// warp for one particle at a time (when at most kSpringWarpChoice of the 32
// particles have free slots) or by every lane for its own particle with a
// converged scan over the block.
constexpr int kSpringWarpChoice = 16;
struct SpringWarp {
	float2 pos[kStageCap];
	int tag[kStageCap];
	// Per-lane lists, slot-major ([slot][lane]) so that the lanes' accesses
	// fall on distinct banks.
	int ex[kSprings][kWarp];     // existing partners (new numbers)
	uint32_t exbits[kStageCap / 32][kWarp];  // per lane: staged entries that are existing partners
	union {
		struct {
			float kr2[kSprings][kWarp];  // chosen candidates, sorted (per-lane scan)
			int ktag[kSprings][kWarp];
			int kj[kSprings][kWarp];
		};
		unsigned long long key[kStageCap];  // one particle's candidate keys (warp-wide choice)
	};
};

size_t springs_smem_bytes() { return sizeof(SpringWarp) * kSpringWarps; }

__global__ void __launch_bounds__(kSpringWarps * kWarp) k_springs_select(Totals tt, Particles P, Particles Q,
                                                                        SimTables T) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	SpringWarp &S = reinterpret_cast<SpringWarp *>(smem_raw)[threadIdx.x / kWarp];
	const int lane = threadIdx.x & (kWarp - 1);
	for (int w = 0; w < kStageCap / 32; ++w) S.exbits[w][lane] = 0u;
	const int warpsTotal = gridDim.x * kSpringWarps;
	for (int c = blockIdx.x * kSpringWarps + threadIdx.x / kWarp; c < tt.ncell; c += warpsTotal) {
		const int cnt = T.newCount[c];
		if (cnt == 0) continue;
		const SceneDev &sc = T.scenes[T.sceneOfCell[c]];
		const StepParams &s = sc.p;
		if (!s.springs) continue;
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
		if (L > kStageCap) {
			if (lane == 0) atomicOr(T.error, kErrStageOverflow);
			continue;
		}
		for (int e = lane; e < L; e += kWarp) {
			const int num = seg_number<9>(e, segOff, segStart);
			S.pos[e] = Q.pos[num];
			S.tag[e] = P.id[T.newIdx[num]];
		}
		__syncwarp();
		const int st = T.newStart[c];
		for (int g = 0; g < cnt; g += kWarp) {
			const int jj = g + lane;
			const bool active = jj < cnt;
			const int j = st + jj;
			float2 xi = make_float2(0.f, 0.f);
			int ne = 0, m = 0, kc = 0, freeSlots = 0;
			if (active) {
				xi = Q.pos[j];
				const int o = T.newIdx[j];
				ne = P.springN[o];
				if (ne > kSprings || ne < 0) {
					atomicOr(T.error, kErrIndex);
					ne = ne < 0 ? 0 : kSprings;
				}
				// The particle's spring rows, four slots per load, then the
				// partners' new numbers, all issued before any is used.
				int pn[kSprings];
				float rl[kSprings];
				const int4 *rowP = reinterpret_cast<const int4 *>(P.springP + (size_t)o * kSprings);
				const float4 *rowL = reinterpret_cast<const float4 *>(P.springL + (size_t)o * kSprings);
#pragma unroll
				for (int v = 0; v < kSprings / 4; ++v) {
					int4 a = make_int4(0, 0, 0, 0);
					float4 b = make_float4(0.f, 0.f, 0.f, 0.f);
					if (4 * v < ne) {
						a = rowP[v];
						b = rowL[v];
					}
					pn[4 * v] = a.x;
					pn[4 * v + 1] = a.y;
					pn[4 * v + 2] = a.z;
					pn[4 * v + 3] = a.w;
					rl[4 * v] = b.x;
					rl[4 * v + 1] = b.y;
					rl[4 * v + 2] = b.z;
					rl[4 * v + 3] = b.w;
				}
#pragma unroll
				for (int q = 0; q < kSprings; ++q) pn[q] = q < ne ? T.newLabel[pn[q]] : 0;
#pragma unroll
				for (int q = 0; q < kSprings; ++q) {
					if (q >= ne) break;
					float rest = rl[q];
					const int e = staged_index(pn[q], segOff, segStart, L);
					S.ex[q][lane] = e;
					if (e >= 0) S.exbits[e >> 5][lane] |= 1u << (e & 31);
					const float2 xp = e >= 0 ? S.pos[e] : Q.pos[pn[q]];
					const float rx = xp.x - xi.x, ry = xp.y - xi.y;
					const float r2 = rx * rx + ry * ry;
					if (r2 < s.h2) rest = plastic(rest, sqrtf(r2), s);
					if (rest <= s.h) {
						Q.springP[j * kSprings + m] = pn[q];
						Q.springL[j * kSprings + m] = rest;
						++m;
					}
				}
				freeSlots = s.springMax - m;
			}
			// Candidates: every list member in range without a spring,
			// nearest first, then the smaller AddParticle index.  Few
			// particles with free slots (the steady state: most hold all
			// their springs): each chooses with the whole warp, by rounds of
			// a warp-wide minimum over 64-bit keys (r^2 bits, index) -- keys
			// of distinct entries differ, and a non-negative float's bits
			// order like its value.  Many (the first updates): every lane
			// scans the list for its own particle with an ordered insertion.
			// Both give the same choices in the same order.
			const unsigned needy = __ballot_sync(kFullMask, active && freeSlots > 0);
			const bool perLane = __popc(needy) > kSpringWarpChoice;
			__syncwarp();  // every lane's existing-partner bits are in place
			for (unsigned todo = perLane ? 0u : needy; todo != 0u; todo &= todo - 1u) {
				const int lp = __ffs(todo) - 1;
				const int fs = __shfl_sync(kFullMask, freeSlots, lp);
				const float px = __shfl_sync(kFullMask, xi.x, lp), py = __shfl_sync(kFullMask, xi.y, lp);
				const int selfE = segOff[4] + g + lp;  // the particle's own entry (own cell = segment 4)
				for (int e = lane; e < L; e += kWarp) {
					const float2 xj = S.pos[e];
					const float rx = xj.x - px, ry = xj.y - py;
					const float r2 = rx * rx + ry * ry;
					const bool ok = r2 < s.h2 && e != selfE && !((S.exbits[e >> 5][lp] >> (e & 31)) & 1u);
					S.key[e] = ok ? ((unsigned long long)__float_as_uint(r2) << 32) | (unsigned)S.tag[e] : ~0ull;
				}
				__syncwarp();
				unsigned long long last = 0ull;
				int chosen = 0;
				for (; chosen < fs; ++chosen) {
					unsigned long long best = ~0ull;
					int bestE = -1;
					for (int e = lane; e < L; e += kWarp) {
						const unsigned long long k = S.key[e];
						if (k < best && (chosen == 0 || k > last)) {
							best = k;
							bestE = e;
						}
					}
					const unsigned hi = __reduce_min_sync(kFullMask, (unsigned)(best >> 32));
					const unsigned lo = __reduce_min_sync(kFullMask, (unsigned)(best >> 32) == hi ? (unsigned)best : ~0u);
					const unsigned long long mk = ((unsigned long long)hi << 32) | lo;
					if (mk == ~0ull) break;
					const int wl = __ffs(__ballot_sync(kFullMask, best == mk)) - 1;
					const int we = __shfl_sync(kFullMask, bestE, wl);
					last = mk;
					if (lane == 0) T.accP[(st + g + lp) * kSprings + chosen] = seg_number<9>(we, segOff, segStart);
				}
				if (lane == lp) kc = chosen;
				__syncwarp();
			}
			const bool scan = perLane && active && freeSlots > 0;
			const int scanLen = __any_sync(kFullMask, scan) ? L : 0;
			for (int e = 0; e < scanLen; ++e) {
				const int num = seg_number<9>(e, segOff, segStart);
				const float2 xj = S.pos[e];
				if (!scan || num == j) continue;
				const float rx = xj.x - xi.x, ry = xj.y - xi.y;
				const float r2 = rx * rx + ry * ry;
				if (!(r2 < s.h2)) continue;
				if ((S.exbits[e >> 5][lane] >> (e & 31)) & 1u) continue;
				const int tj = S.tag[e];
				if (kc == freeSlots && !before(r2, tj, S.kr2[kc - 1][lane], S.ktag[kc - 1][lane])) continue;
				int at = kc < freeSlots ? kc++ : kc - 1;
				while (at > 0 && before(r2, tj, S.kr2[at - 1][lane], S.ktag[at - 1][lane])) {
					S.kr2[at][lane] = S.kr2[at - 1][lane];
					S.ktag[at][lane] = S.ktag[at - 1][lane];
					S.kj[at][lane] = S.kj[at - 1][lane];
					--at;
				}
				S.kr2[at][lane] = r2;
				S.ktag[at][lane] = tj;
				S.kj[at][lane] = num;
			}
			if (active) {
				T.accN[j] = kc;
				if (perLane)
					for (int q = 0; q < kc; ++q) T.accP[j * kSprings + q] = S.kj[q][lane];
				Q.springN[j] = m;
				for (int q = 0; q < ne; ++q) {
					const int e = S.ex[q][lane];
					if (e >= 0) S.exbits[e >> 5][lane] = 0u;  // words touched by this particle
				}
			}
			__syncwarp();
		}
		__syncwarp();
	}
}

// A spring joins both ends where each chose the other.
__global__ void k_springs_commit(Totals tt, Particles Q, SimTables T) {
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	int m = 0, sid = -1;
	if (j < tt.n) {
		sid = T.sceneOf[j];
		const StepParams &s = T.scenes[sid].p;
		if (s.springs) {
			m = Q.springN[j];
			const float2 xi = Q.pos[j];
			const int na = T.accN[j];
			for (int q = 0; q < na; ++q) {
				const int p = T.accP[j * kSprings + q];
				const int np = T.accN[p];
				bool mutual = false;
				for (int q2 = 0; q2 < np; ++q2) mutual = mutual || T.accP[p * kSprings + q2] == j;
				if (!mutual) continue;
				const float2 xp = Q.pos[p];
				const float rx = xp.x - xi.x, ry = xp.y - xi.y;
				const float rest = plastic(s.h, sqrtf(rx * rx + ry * ry), s);
				if (rest <= s.h) {
					Q.springP[j * kSprings + m] = p;
					Q.springL[j * kSprings + m] = rest;
					++m;
				}
			}
			Q.springN[j] = m;
		}
	}
	// Springs per scene (each counted at both ends): one atomic per group of
	// lanes of one scene.
	const unsigned same = __match_any_sync(kFullMask, sid);
	const unsigned total = __reduce_add_sync(same, (unsigned)m);
	if (sid >= 0 && total && (threadIdx.x & (kWarp - 1)) == __ffs(same) - 1)
		atomicAdd(&T.springTotal[sid], (unsigned long long)total);
}

// Spring displacements from the positions before the phase.
__global__ void k_springs_apply(Totals tt, Particles Q, SimTables T) {
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= tt.n) return;
	const StepParams &s = T.scenes[T.sceneOf[j]].p;
	const float2 xi = Q.pos[j];
	if (!s.springs) {
		T.springPos[j] = xi;
		return;
	}
	float dx = 0.0f, dy = 0.0f;
	const int m = Q.springN[j];
	const float kdt2 = s.dt2 * s.springK;
	for (int q = 0; q < m; ++q) {
		const int p = Q.springP[j * kSprings + q];
		const float rest = Q.springL[j * kSprings + q];
		const float2 xp = Q.pos[p];
		const float rx = xp.x - xi.x, ry = xp.y - xi.y;
		const float r = sqrtf(rx * rx + ry * ry);
		const float len = r == 0.0f ? 1.0f : r;
		const float inv = 1.0f / len;
		const float nx = rx * inv, ny = ry * inv;
		const float f = (kdt2 * (1.0f - rest * s.invH)) * (rest - r);
		dx = dx - (f * nx) * 0.5f;
		dy = dy - (f * ny) * 0.5f;
	}
	T.springPos[j] = make_float2(dx + xi.x, dy + xi.y);
}

// Checks of spring tables given to sph_load_springs (one thread per
// particle): counts within [0, kSprings], partners within [0, n) and not the
// particle itself.  verdict[0] collects failures.
__global__ void k_check_springs(int n, const int *cnt, const int *partner, int *verdict) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const int c = cnt[i];
	int bad = c < 0 || c > kSprings;
	for (int q = 0; q < kSprings && !bad; ++q) {
		const int p = partner[i * kSprings + q];
		if (q < c) bad |= p < 0 || p >= n || p == i;
	}
	if (bad) atomicOr(&verdict[0], 1);
}

// Spring tables as sph_dump_springs reports them: slots past a particle's
// count hold partner -1 and rest length 0.
__global__ void k_clean_springs(int n, const int *cnt, const int *partner, const float *rest, int *cntOut,
                                int *partnerOut, float *restOut) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n * kSprings) return;
	const int j = i / kSprings, q = i - j * kSprings;
	const int c = min(max(cnt[j], 0), kSprings);
	if (q == 0) cntOut[j] = c;
	partnerOut[i] = q < c ? partner[i] : -1;
	restOut[i] = q < c ? rest[i] : 0.0f;
}

}  // namespace sphgb
