// Kernel declarations and launch shapes of the GB300 Demo4 SPH step.
#pragma once

#include "sph_internal.cuh"

namespace sphgb {

// Shapes of the two ordered sweeps (one task per block).  Wide: more warps
// per task and buffers for the largest lists the reference accepts (short
// critical path for one scene).  Lean: fewer warps and smaller buffers (more
// tasks per SM for many scenes).  Results do not depend on the shape.
struct ViscWide {
	static constexpr int kWarps = 4, kProducers = 3 * kWarp, kGeom = 512, kMinBlocks = 4;
	static constexpr bool kBranchy = false;
};
// Lean viscosity: kSlots tasks per block; warp 0's lanes run their chains,
// kProd producer warps serve them (k_viscosity_multi).
struct ViscLean {
	static constexpr int kSlots = 5, kProd = 4, kWarps = 1 + kProd, kGeom = 192, kMinBlocks = 3;
};
// Delta sweep.  Pipelined shapes run kWarps - 1 producer warps and one
// summer warp per task; the others relax one particle at a time on the
// whole block.  kChainW in-range pairs are buffered per warp; a particle's
// list is relaxed in the pipeline when it has at most (kWarps - 1) * kChainW
// entries.  Wide: pipelined, twelve warps, one block per SM (short
// per-particle latency for one scene).  Lean: two warps, not pipelined,
// smaller staging (more tasks per SM for many scenes).  kShortEntry: a
// task's entry and exit take the fewest cycles (first chunk's inputs loaded
// during the staging, region written back one element per thread) rather
// than the fewest instructions.
struct DeltaWide {
	static constexpr int kWarps = 12, kStage = kDeltaStageCap, kChainW = 96, kPrefetch = 128, kMinBlocks = 1;
	static constexpr int kRegion = kRegionCells;
	static constexpr bool kPipelined = true, kShortEntry = true;
};
struct DeltaLean {
	static constexpr int kWarps = 2, kStage = 1536, kChainW = 192, kPrefetch = 64, kMinBlocks = 8;
	static constexpr int kRegion = kRegionCells;
	static constexpr bool kPipelined = false, kShortEntry = false;
};
// Mid: pipelined, eight warps, two blocks per SM (mid-size scenes, where
// more tasks run at once than one block per SM holds).
struct DeltaMid {
	static constexpr int kWarps = 8, kStage = kDeltaStageCap, kChainW = 128, kPrefetch = 128, kMinBlocks = 2;
	static constexpr int kRegion = 256;
	static constexpr bool kPipelined = true, kShortEntry = true;
};
// Small pipelined shapes for large scenes, where the sweep is bound by how
// many tasks run at once rather than by one task's latency: two (tri) or
// three (quad) producer warps and the summer warp, several blocks per SM.
struct DeltaTri {
	static constexpr int kWarps = 3, kStage = 1536, kChainW = 256, kPrefetch = 64, kMinBlocks = 5;
	static constexpr int kRegion = kRegionCells;
	static constexpr bool kPipelined = true, kShortEntry = true;
};
struct DeltaQuad {
	static constexpr int kWarps = 4, kStage = 1536, kChainW = 192, kPrefetch = 128, kMinBlocks = 4;
	static constexpr int kRegion = kRegionCells;
	static constexpr bool kPipelined = true, kShortEntry = true;
};
// Dense: pipelined, sixteen warps, one block per SM, a 12,288-entry stage,
// for crowded states where a task's region (the bounding box of its
// particles' new cells, grown by one) outgrows the other shapes' stages and
// their tasks would read unstaged from global memory.
struct DeltaDense {
	static constexpr int kWarps = 16, kStage = kDeltaDenseStageCap, kChainW = 96, kPrefetch = 128, kMinBlocks = 1;
	static constexpr int kRegion = 400;
	static constexpr bool kPipelined = true, kShortEntry = true;
};
// Delta shapes by index (sph_set_sweep_shape names them by warp count).
constexpr int kDeltaShapes = 6;
constexpr int kDeltaWide = 0, kDeltaLean = 1, kDeltaMid = 2, kDeltaTri = 3, kDeltaQuad = 4, kDeltaDense = 5;
constexpr int delta_shape_warps(int shape) {
	return shape == kDeltaLean    ? DeltaLean::kWarps
	       : shape == kDeltaMid   ? DeltaMid::kWarps
	       : shape == kDeltaTri   ? DeltaTri::kWarps
	       : shape == kDeltaQuad  ? DeltaQuad::kWarps
	       : shape == kDeltaDense ? DeltaDense::kWarps
	                              : DeltaWide::kWarps;
}
constexpr int kDensWarps = 8;
constexpr int kViscRefWarps = 4;  // reference-order viscosity sweep: one task per warp
constexpr int kGridWarps = 4;
constexpr int kScanThreads = 1024;
constexpr int kScanTile = 4 * kScanThreads;  // scan positions per block
constexpr int kElemThreads = 256;  // elementwise kernels
constexpr int kCollideThreads = 256;
constexpr int kSpringWarps = 4;

struct DensWarp;

// The two ordered sweeps in a chosen shape (lean or wide), and their set-up.
cudaError_t sweep_attributes();
cudaError_t sweep_occupancy(bool viscLean, int deltaShape, int *occV, int *occD);
// Staged entries of a delta-sweep task region in the given shape; larger
// regions are swept unstaged (from global memory).
inline int delta_stage_capacity(int shape) {
	return shape == kDeltaLean    ? DeltaLean::kStage
	       : shape == kDeltaMid   ? DeltaMid::kStage
	       : shape == kDeltaTri   ? DeltaTri::kStage
	       : shape == kDeltaQuad  ? DeltaQuad::kStage
	       : shape == kDeltaDense ? DeltaDense::kStage
	                              : DeltaWide::kStage;
}
void launch_viscosity(bool lean, int blocks, cudaStream_t st, Totals tt, Particles P, SimTables T);
void launch_delta(int shape, int blocks, cudaStream_t st, Totals tt, Particles Q, SimTables T);
size_t dens_smem_bytes();
size_t springs_smem_bytes();

__global__ void k_integrate(Totals tt, Particles P, SimTables T);
__global__ void k_ref_order(Totals tt, Particles P, SimTables T);
__global__ void k_visc_boxes(Totals tt, Particles P, SimTables T);
__global__ void k_viscosity_ref(Totals tt, Particles P, SimTables T);
__global__ void k_predict(Totals tt, Particles P, SimTables T);
__global__ void k_live_reduce(Totals tt, SimTables T);
__global__ void k_live_tiles(SimTables T, int ntiles);
__global__ void k_live_apply(Totals tt, SimTables T);
__global__ void k_scan_reduce(Totals tt, SimTables T);
__global__ void k_scan_tiles(Totals tt, SimTables T, int ntiles);
__global__ void k_scan_apply(Totals tt, SimTables T);
__global__ void k_scatter(Totals tt, Particles P, SimTables T);
__global__ void k_grid_update(Totals tt, Particles P, Particles Q, SimTables T);
__global__ void k_app_boxes(Totals tt, SimTables T);
__global__ void k_density(Totals tt, Particles Q, SimTables T);
__global__ void k_collide(Totals tt, Particles P, Particles Q, SimTables T);
__global__ void k_add(int first, int count, int scene, int firstId, const float2 *pos, const float2 *force,
                      Particles P, SimTables T);
__global__ void k_gather_by_id(int first, int count, const int *id, const float2 *src, float2 *dst);
__global__ void k_check_state(int n, int n0, int ncell, const int *cell, const int *start, const int *count,
                              const int *id, int *appOut, int *seen, int *verdict);
__global__ void k_check_springs(int n, const int *cnt, const int *partner, int *verdict);
__global__ void k_clean_springs(int n, const int *cnt, const int *partner, const float *rest, int *cntOut,
                                int *partnerOut, float *restOut);
__global__ void k_particle_colors(int first, int count, const int *id, const float2 *dens, const float2 *press,
                                  const float2 *vel, float rho0, float4 *out);
__global__ void k_splat_points(int first, int count, const int *id, const float2 *pos, const float2 *dens,
                               const float2 *press, const float2 *vel, float rho0, float halfW, float halfH,
                               float sx, float sy, int width, int height, unsigned long long *keys);
__global__ void k_keys_to_rgba8(int pixels, const unsigned long long *keys, uint32_t *rgba);
__global__ void k_springs_select(Totals tt, Particles P, Particles Q, SimTables T);
__global__ void k_springs_commit(Totals tt, Particles Q, SimTables T);
__global__ void k_springs_apply(Totals tt, Particles Q, SimTables T);
__global__ void k_learned_z0(int n, int np, const float2 *pos, const float2 *prev, float invH, float2 *z0);
__global__ void k_learned_finish(Totals tt, Particles P, const float2 *u, SimTables T);
constexpr int kErrThreads = 256;  // judge's reduction: threads per block
constexpr int kErrBlocks = 512;   // and at most this many blocks
__global__ void k_density_error(int n, const float2 *dens, float rho0, double *partial);
__global__ void k_density_error_total(int blocks, const double *partial, double *out);
__global__ void k_scatter_by_id(int n, const float2 *pos, const int *id, float2 *byId);
__global__ void k_learned_target(int n, const float2 *byId, const int *ids, const float2 *xstar, float invH,
                                 float2 *target);

}  // namespace sphgb
