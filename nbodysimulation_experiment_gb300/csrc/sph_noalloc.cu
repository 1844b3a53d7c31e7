// Density and pressure for caller-provided positions, without allocating.
//
// Who needs it: callers that cannot call cudaMalloc -- code that runs
// inside someone else's memory budget or allocator (an engine that owns all
// device memory, a plugin host that forbids the runtime's allocator), a
// real-time loop that must not hit allocation latency or fragmentation.
// They hand in device pointers for the inputs and outputs; the working
// memory (cell counts, offsets, per-particle lists) lives in one fixed
// device array of this file, which every GPU that loads the library holds
// until the process exits.
//
// What it computes: SPHComputeDensity / SPHComputePressure
// (NBodySimulation/sph.h:465-481) for every particle over the reference's
// unfiltered 3x3-cell neighbour list (demo4.cpp:183-206), with each cell's
// array in particle order -- what one Update computes for particles that
// have just been added with zero velocity.  Same FP32 operation order as the
// update; sums run in list order.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sph_gb300.h"

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaWarps = 4;
constexpr int kNaMaxDevices = 64;

// Scratch layout (int32): count, start, cursor per cell; unsorted and sorted
// particle lists.
constexpr size_t kCountOff = 0;
constexpr size_t kStartOff = kCountOff + SPH_NOALLOC_MAX_CELLS;
constexpr size_t kCursorOff = kStartOff + SPH_NOALLOC_MAX_CELLS;
constexpr size_t kUnsortedOff = kCursorOff + SPH_NOALLOC_MAX_CELLS;
constexpr size_t kSortedOff = kUnsortedOff + SPH_NOALLOC_MAX_PARTICLES;
constexpr size_t kScratchInts = kSortedOff + SPH_NOALLOC_MAX_PARTICLES;

static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

struct NaParams {
	float halfW, halfH, cellSize;
	int gx, gy, ncell;
	float h2, invH, rho0, k, kNear;
};

__device__ __forceinline__ int na_cell(float2 p, const NaParams &s) {
	int x = (int)((p.x + s.halfW) / s.cellSize);
	int y = (int)((p.y + s.halfH) / s.cellSize);
	x = min(max(x, 0), s.gx - 1);
	y = min(max(y, 0), s.gy - 1);
	return y * s.gx + x;
}

__global__ void k_na_count(int n, const float2 *pos, int *scratch, NaParams s) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) atomicAdd(&scratch[kCountOff + na_cell(pos[i], s)], 1);
}

// Exclusive scan of the cell counts (one block, contiguous runs per thread).
__global__ void k_na_scan(int *scratch, NaParams s) {
	__shared__ int sums[kNaThreads];
	const int tid = threadIdx.x;
	const int per = (s.ncell + kNaThreads - 1) / kNaThreads;
	const int b = tid * per, e = min(s.ncell, b + per);
	int acc = 0;
	for (int c = b; c < e; ++c) acc += scratch[kCountOff + c];
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

__global__ void k_na_scatter(int n, const float2 *pos, int *scratch, NaParams s) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const int c = na_cell(pos[i], s);
	const int slot = scratch[kStartOff + c] + atomicAdd(&scratch[kCursorOff + c], 1);
	scratch[kUnsortedOff + slot] = i;
}

// Each cell's array in particle order (AddParticle appends in that order,
// demo4.cpp:37-54): rank of every member among the cell's members.
__global__ void k_na_order(int *scratch, NaParams s) {
	const int lane = threadIdx.x & 31;
	const int warps = gridDim.x * (blockDim.x / 32);
	for (int c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; c < s.ncell; c += warps) {
		const int st = scratch[kStartOff + c], cnt = scratch[kCountOff + c];
		for (int a = lane; a < cnt; a += 32) {
			const int v = scratch[kUnsortedOff + st + a];
			int rank = 0;
			for (int b = 0; b < cnt; ++b) rank += scratch[kUnsortedOff + st + b] < v ? 1 : 0;
			scratch[kSortedOff + st + rank] = v;
		}
	}
}

// One warp per cell; each lane sums one particle's list in order.
__global__ void k_na_density(const float2 *pos, float2 *dens, float2 *press, const int *scratch, NaParams s) {
	const int lane = threadIdx.x & 31;
	const int warps = gridDim.x * (blockDim.x / 32);
	for (int c = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; c < s.ncell; c += warps) {
		const int cnt = scratch[kCountOff + c];
		if (cnt == 0) continue;
		const int cx = c % s.gx, cy = c / s.gx;
		const int st = scratch[kStartOff + c];
		for (int g = 0; g < cnt; g += 32) {
			const bool active = g + lane < cnt;
			const int i = active ? scratch[kSortedOff + st + g + lane] : 0;
			const float2 xi = pos[i];
			float d0 = 0.0f, d1 = 0.0f;
			for (int q = 0; q < 9; ++q) {
				const int x = cx + q % 3 - 1, y = cy + q / 3 - 1;
				if (x < 0 || x >= s.gx || y < 0 || y >= s.gy) continue;
				const int c2 = y * s.gx + x;
				const int st2 = scratch[kStartOff + c2], cnt2 = scratch[kCountOff + c2];
				for (int j = 0; j < cnt2; ++j) {
					const float2 xj = pos[scratch[kSortedOff + st2 + j]];
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

// Device address of the scratch array, looked up once per device.
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
	int *scratch = nullptr;
	int rc = scratch_for_current_device(&scratch);
	if (rc != SPH_OK) return rc;
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	const int n = (int)count;
	const float2 *p = reinterpret_cast<const float2 *>(pos);
	// Counts and cursors must start at zero; the rest is fully rewritten.
	if (cudaMemsetAsync(scratch + kCountOff, 0, sizeof(int) * s.ncell, st) != cudaSuccess ||
	    cudaMemsetAsync(scratch + kCursorOff, 0, sizeof(int) * s.ncell, st) != cudaSuccess)
		return SPH_ERR_CUDA;
	const int blocks = (n + kNaThreads - 1) / kNaThreads;
	const int cellBlocks = (s.ncell + kNaWarps - 1) / kNaWarps;
	k_na_count<<<blocks, kNaThreads, 0, st>>>(n, p, scratch, s);
	k_na_scan<<<1, kNaThreads, 0, st>>>(scratch, s);
	k_na_scatter<<<blocks, kNaThreads, 0, st>>>(n, p, scratch, s);
	k_na_order<<<cellBlocks, kNaWarps * 32, 0, st>>>(scratch, s);
	k_na_density<<<cellBlocks, kNaWarps * 32, 0, st>>>(p, reinterpret_cast<float2 *>(dens),
	                                                    reinterpret_cast<float2 *>(press), scratch, s);
	return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
