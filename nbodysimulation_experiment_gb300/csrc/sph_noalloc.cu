// Density and pressure for caller-provided positions, without allocating.
//
// Who needs it: callers that cannot call cudaMalloc -- code that runs
// inside someone else's memory budget or allocator (an engine that owns all
// device memory, a plugin host that forbids the runtime's allocator), a
// real-time loop that must not hit allocation latency or fragmentation.
// They hand in device pointers for the inputs and outputs; the working
// memory (cell keys, sort buffers, per-cell counts and offsets, a status
// word) lives in one fixed device array of this file, which every GPU that
// loads the library holds until the process exits.
//
// What it computes: SPHComputeDensity / SPHComputePressure
// (NBodySimulation/sph.h:465-481) for every particle over the reference's
// unfiltered 3x3-cell neighbour list (demo4.cpp:183-206), with each cell's
// array in particle order -- what one Update computes for particles that
// have just been added with zero velocity and no gravity.  Same FP32
// operation order as the update; sums run in list order.
//
// How: every particle gets its cell key (sph.h:450-463, clamped into the
// grid); a stable least-significant-digit radix sort of the particle indices
// by cell key (two passes of 9 bits: keys are below 2^18) puts each cell's
// members in particle order, which is the order AddParticle appends them
// (demo4.cpp:37-54); per-cell counts and offsets come from a count pass and
// a scan.  The domain's capacities are enforced: a cell holding more than
// max_cell_particles, or a 3x3 block listing more than max_neighbors
// particles, sets a status word and is skipped, and the call then returns
// SPH_ERR_CAPACITY -- where the reference would assert (demo4.cpp:45, 199).
// All work is O(particles x max_neighbors).
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sph_gb300.h"

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaWarps = 4;
constexpr int kNaMaxDevices = 64;
// Radix sort: digits of 9 bits, tiles of kTile particles (8 per thread).
constexpr int kRadixBits = 9;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kItems = 8;
constexpr int kTile = kNaThreads * kItems;
constexpr int kMaxTiles = (SPH_NOALLOC_MAX_PARTICLES + kTile - 1) / kTile;
static_assert(SPH_NOALLOC_MAX_CELLS <= (1 << (2 * kRadixBits)), "cell keys must fit two radix digits");

// Scratch layout (int32): per cell count and start; per particle the cell
// key, and the index and key arrays of the two sort passes; per digit and
// tile the histogram / offset table; the status word.
constexpr size_t kCountOff = 0;
constexpr size_t kStartOff = kCountOff + SPH_NOALLOC_MAX_CELLS;
constexpr size_t kKeyOff = kStartOff + SPH_NOALLOC_MAX_CELLS;
constexpr size_t kIdxAOff = kKeyOff + SPH_NOALLOC_MAX_PARTICLES;
constexpr size_t kKeyBOff = kIdxAOff + SPH_NOALLOC_MAX_PARTICLES;
constexpr size_t kIdxBOff = kKeyBOff + SPH_NOALLOC_MAX_PARTICLES;
constexpr size_t kHistOff = kIdxBOff + SPH_NOALLOC_MAX_PARTICLES;
constexpr size_t kStatusOff = kHistOff + (size_t)kRadix * kMaxTiles;
constexpr size_t kScratchInts = kStatusOff + 64;

static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

enum : int { kStatusCapacity = 1 };

struct NaParams {
	float halfW, halfH, cellSize;
	int gx, gy, ncell;
	float h2, invH, rho0, k, kNear;
	int maxCell, maxNeighbors;
	int n, tiles;
};

__device__ __forceinline__ int na_cell(float2 p, const NaParams &s) {
	int x = (int)((p.x + s.halfW) / s.cellSize);
	int y = (int)((p.y + s.halfH) / s.cellSize);
	x = min(max(x, 0), s.gx - 1);
	y = min(max(y, 0), s.gy - 1);
	return y * s.gx + x;
}

// Cell key and per-cell count of every particle.
__global__ void k_na_keys(const float2 *pos, int *scratch, NaParams s) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= s.n) return;
	const int c = na_cell(pos[i], s);
	scratch[kKeyOff + i] = c;
	atomicAdd(&scratch[kCountOff + c], 1);
}

// Per-cell exclusive scan (one block, contiguous runs per thread), and the
// cell-capacity check.
__global__ void k_na_scan(int *scratch, NaParams s) {
	__shared__ int sums[kNaThreads];
	const int tid = threadIdx.x;
	const int per = (s.ncell + kNaThreads - 1) / kNaThreads;
	const int b = tid * per, e = min(s.ncell, b + per);
	int acc = 0, over = 0;
	for (int c = b; c < e; ++c) {
		const int v = scratch[kCountOff + c];
		acc += v;
		over |= v > s.maxCell;
	}
	if (over) atomicOr(&scratch[kStatusOff], kStatusCapacity);
	sums[tid] = acc;
	__syncthreads();
	for (int off = 1; off < kNaThreads; off <<= 1) {
		const int v = tid >= off ? sums[tid - off] : 0;
		__syncthreads();
		sums[tid] += v;
		__syncthreads();
	}
	int run = tid > 0 ? sums[tid - 1] : 0;
	for (int c = b; c < e; ++c) {
		scratch[kStartOff + c] = run;
		run += scratch[kCountOff + c];
	}
}

// Radix pass, step 1: digit histogram of each tile, stored digit-major
// (hist[digit * tiles + tile]) so that one exclusive scan gives every
// (digit, tile) its output offset.  The first pass reads the keys in
// particle order (the index is the particle itself).
__global__ void k_na_hist(const int *keys, int *scratch, NaParams s, int shift) {
	__shared__ int h[kRadix];
	for (int d = threadIdx.x; d < kRadix; d += kNaThreads) h[d] = 0;
	__syncthreads();
	const int t = blockIdx.x;
	for (int k = 0; k < kItems; ++k) {
		const int i = t * kTile + k * kNaThreads + threadIdx.x;
		if (i < s.n) atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1);
	}
	__syncthreads();
	for (int d = threadIdx.x; d < kRadix; d += kNaThreads) scratch[kHistOff + (size_t)d * s.tiles + t] = h[d];
}

// Radix pass, step 2: exclusive scan of the digit-major histogram (one block).
__global__ void k_na_hist_scan(int *scratch, NaParams s) {
	__shared__ int sums[kNaThreads];
	const int tid = threadIdx.x;
	const int total = kRadix * s.tiles;
	const int per = (total + kNaThreads - 1) / kNaThreads;
	const int b = tid * per, e = min(total, b + per);
	int *h = scratch + kHistOff;
	int acc = 0;
	for (int q = b; q < e; ++q) acc += h[q];
	sums[tid] = acc;
	__syncthreads();
	for (int off = 1; off < kNaThreads; off <<= 1) {
		const int v = tid >= off ? sums[tid - off] : 0;
		__syncthreads();
		sums[tid] += v;
		__syncthreads();
	}
	int run = tid > 0 ? sums[tid - 1] : 0;
	for (int q = b; q < e; ++q) {
		const int v = h[q];
		h[q] = run;
		run += v;
	}
}

// Radix pass, step 3: stable scatter.  Warp w of a tile owns the tile's
// items [w * 8 * 32, (w + 1) * 8 * 32) in order; per-warp digit counts
// (then their exclusive scan across the warps) give each warp its first
// position per digit, and within a warp the items are placed round by round
// in lane order, equal digits ranked by __match_any_sync.  Input position q
// holds (inIdx[q], keys[q]); inIdx == nullptr means the identity (the first
// pass, over particle order).
__global__ void k_na_scatter(const int *keys, const int *inIdx, int *outKeys, int *outIdx, int *scratch, NaParams s,
                             int shift) {
	constexpr int kW = kNaThreads / 32;
	constexpr int kPerWarp = kTile / kW;  // 256 items per warp
	__shared__ int cnt[kW][kRadix];
	const int lane = threadIdx.x & 31, w = threadIdx.x / 32;
	const int t = blockIdx.x;
	for (int d = lane; d < kRadix; d += 32) cnt[w][d] = 0;
	__syncwarp();
	const int base = t * kTile + w * kPerWarp;
	// Per-warp digit counts.
	for (int r = 0; r < kPerWarp / 32; ++r) {
		const int q = base + r * 32 + lane;
		const bool in = q < s.n;
		const int d = in ? (keys[q] >> shift) & (kRadix - 1) : -1;
		const unsigned peers = __match_any_sync(0xffffffffu, d);
		if (in && lane == __ffs(peers) - 1) cnt[w][d] += __popc(peers);
	}
	__syncthreads();
	// Exclusive scan over the warps per digit, plus the tile's global offset.
	for (int d = threadIdx.x; d < kRadix; d += kNaThreads) {
		int run = scratch[kHistOff + (size_t)d * s.tiles + t];
		for (int q = 0; q < kW; ++q) {
			const int v = cnt[q][d];
			cnt[q][d] = run;
			run += v;
		}
	}
	__syncthreads();
	for (int r = 0; r < kPerWarp / 32; ++r) {
		const int q = base + r * 32 + lane;
		const bool in = q < s.n;
		const int key = in ? keys[q] : 0;
		const int d = in ? (key >> shift) & (kRadix - 1) : -1;
		const unsigned peers = __match_any_sync(0xffffffffu, d);
		const unsigned lt = peers & ((1u << lane) - 1u);
		const int leader = __ffs(peers) - 1;
		int at = 0;
		if (in) at = cnt[w][d] + __popc(lt);
		__syncwarp();
		if (in && lane == leader) cnt[w][d] += __popc(peers);
		__syncwarp();
		if (in) {
			outKeys[at] = key;
			outIdx[at] = inIdx ? inIdx[q] : q;
		}
	}
}

// One warp per cell; each lane sums one particle's list in order.  Blocks
// whose list exceeds the domain's neighbour capacity, and cells beyond its
// cell capacity, are flagged and skipped.
__global__ void k_na_density(const float2 *pos, float2 *dens, float2 *press, int *scratch, NaParams s) {
	const int lane = threadIdx.x & 31;
	const int warps = gridDim.x * (blockDim.x / 32);
	const int *sorted = scratch + kIdxAOff;
	for (int c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; c < s.ncell; c += warps) {
		const int cnt = scratch[kCountOff + c];
		if (cnt == 0) continue;
		const int cx = c % s.gx, cy = c / s.gx;
		int L = 0;
		for (int q = 0; q < 9; ++q) {
			const int x = cx + q % 3 - 1, y = cy + q / 3 - 1;
			if (x >= 0 && x < s.gx && y >= 0 && y < s.gy) L += scratch[kCountOff + y * s.gx + x];
		}
		if (cnt > s.maxCell || L > s.maxNeighbors) {
			if (lane == 0) atomicOr(&scratch[kStatusOff], kStatusCapacity);
			continue;
		}
		const int st = scratch[kStartOff + c];
		for (int g = 0; g < cnt; g += 32) {
			const bool active = g + lane < cnt;
			const int i = active ? sorted[st + g + lane] : 0;
			const float2 xi = pos[i];
			float d0 = 0.0f, d1 = 0.0f;
			for (int q = 0; q < 9; ++q) {
				const int x = cx + q % 3 - 1, y = cy + q / 3 - 1;
				if (x < 0 || x >= s.gx || y < 0 || y >= s.gy) continue;
				const int c2 = y * s.gx + x;
				const int st2 = scratch[kStartOff + c2], cnt2 = scratch[kCountOff + c2];
				for (int j = 0; j < cnt2; ++j) {
					const float2 xj = pos[sorted[st2 + j]];
					const float rx = xj.x - xi.x, ry = xj.y - xi.y;
					const float r2 = rx * rx + ry * ry;
					if (r2 < s.h2) {
						const float r = sqrtf(r2);
						const float term = 1.0f - r * s.invH;
						d0 = d0 + term * term;
						d1 = d1 + term * term * term;
					}
				}
			}
			if (active) {
				dens[i] = make_float2(d0, d1);
				press[i] = make_float2(s.k * (d0 - s.rho0), s.kNear * d1);
			}
		}
	}
}

// Device address of the scratch array, looked up once per device on the
// first call made with that device current, and kept for the life of the
// process.
std::mutex g_mutex;
int *g_ptr[kNaMaxDevices] = {};

int scratch_for_current_device(int **out) {
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return SPH_ERR_NO_DEVICE;
	if (dev < 0 || dev >= kNaMaxDevices) return SPH_ERR_NOT_SUPPORTED;
	std::lock_guard<std::mutex> lock(g_mutex);
	if (!g_ptr[dev]) {
		void *p = nullptr;
		if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SPH_ERR_CUDA;
		g_ptr[dev] = static_cast<int *>(p);
	}
	*out = g_ptr[dev];
	return SPH_OK;
}

}  // namespace

extern "C" int sph_density_pressure_noalloc(const sph_domain *domain, const sph_params *params, const sph_vec2 *pos,
                                            size_t count, sph_vec2 *dens, sph_vec2 *press, void *stream) {
	if (!domain || !params || (count > 0 && (!pos || !dens || !press))) return SPH_ERR_INVALID_ARGUMENT;
	if (!(domain->cell_size > 0.0f) || !(domain->width > 0.0f) || !(domain->height > 0.0f))
		return SPH_ERR_INVALID_ARGUMENT;
	NaParams s;
	s.gx = (int)(domain->width / domain->cell_size);
	s.gy = (int)(domain->height / domain->cell_size);
	if (s.gx <= 0 || s.gy <= 0) return SPH_ERR_INVALID_ARGUMENT;
	if (count > (size_t)SPH_NOALLOC_MAX_PARTICLES) return SPH_ERR_CAPACITY;
	if ((int64_t)s.gx * s.gy > (int64_t)SPH_NOALLOC_MAX_CELLS) return SPH_ERR_CAPACITY;
	if (domain->max_neighbors > (uint32_t)SPH_NOALLOC_MAX_NEIGHBORS) return SPH_ERR_CAPACITY;
	if (count > (size_t)domain->max_particles) return SPH_ERR_CAPACITY;
	if (count == 0) return SPH_OK;
	s.ncell = s.gx * s.gy;
	s.halfW = domain->width * 0.5f;
	s.halfH = domain->height * 0.5f;
	s.cellSize = domain->cell_size;
	s.h2 = params->kernel_height * params->kernel_height;
	s.invH = params->inv_kernel_height;
	s.rho0 = params->rest_density;
	s.k = params->stiffness;
	s.kNear = params->near_stiffness;
	s.maxCell = (int)domain->max_cell_particles;
	s.maxNeighbors = (int)domain->max_neighbors;
	s.n = (int)count;
	s.tiles = (s.n + kTile - 1) / kTile;
	int *scratch = nullptr;
	int rc = scratch_for_current_device(&scratch);
	if (rc != SPH_OK) return rc;
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	const float2 *p = reinterpret_cast<const float2 *>(pos);
	// The array keeps the previous call's contents: the counts and the status
	// word start at zero; everything else is fully rewritten before it is read.
	if (cudaMemsetAsync(scratch + kCountOff, 0, sizeof(int) * s.ncell, st) != cudaSuccess ||
	    cudaMemsetAsync(scratch + kStatusOff, 0, sizeof(int), st) != cudaSuccess)
		return SPH_ERR_CUDA;
	const int blocks = (s.n + kNaThreads - 1) / kNaThreads;
	const int cellBlocks = (s.ncell + kNaWarps - 1) / kNaWarps;
	k_na_keys<<<blocks, kNaThreads, 0, st>>>(p, scratch, s);
	k_na_scan<<<1, kNaThreads, 0, st>>>(scratch, s);
	// Pass 1 (low digit) from particle order into B; pass 2 (high digit) from
	// B into A: A then lists each cell's members in particle order.
	k_na_hist<<<s.tiles, kNaThreads, 0, st>>>(scratch + kKeyOff, scratch, s, 0);
	k_na_hist_scan<<<1, kNaThreads, 0, st>>>(scratch, s);
	k_na_scatter<<<s.tiles, kNaThreads, 0, st>>>(scratch + kKeyOff, nullptr, scratch + kKeyBOff, scratch + kIdxBOff,
	                                             scratch, s, 0);
	k_na_hist<<<s.tiles, kNaThreads, 0, st>>>(scratch + kKeyBOff, scratch, s, kRadixBits);
	k_na_hist_scan<<<1, kNaThreads, 0, st>>>(scratch, s);
	k_na_scatter<<<s.tiles, kNaThreads, 0, st>>>(scratch + kKeyBOff, scratch + kIdxBOff, scratch + kKeyOff,
	                                             scratch + kIdxAOff, scratch, s, kRadixBits);
	k_na_density<<<cellBlocks, kNaWarps * 32, 0, st>>>(p, reinterpret_cast<float2 *>(dens),
	                                                    reinterpret_cast<float2 *>(press), scratch, s);
	if (cudaGetLastError() != cudaSuccess) return SPH_ERR_CUDA;
	// The capacity verdict needs the device's status word: wait for this
	// call's work (a copy into a host variable; nothing is allocated).
	int status = 0;
	if (cudaMemcpyAsync(&status, scratch + kStatusOff, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
	    cudaStreamSynchronize(st) != cudaSuccess)
		return SPH_ERR_CUDA;
	return (status & kStatusCapacity) ? SPH_ERR_CAPACITY : SPH_OK;
}
