// Kernel declarations and launch shapes of the GB300 Demo4 SPH step.
#pragma once

#include "sph_internal.cuh"

namespace sphgb {

constexpr int kViscTaskWarps = 4;   // warps cooperating on one viscosity task (one task per block)
constexpr int kDeltaTaskWarps = 4;  // warps cooperating on one delta task (one task per block)
constexpr int kDensWarps = 8;
constexpr int kGridWarps = 4;
constexpr int kScanThreads = 1024;
constexpr int kElemThreads = 256;  // elementwise kernels
constexpr int kCollideThreads = 256;

struct ViscSmem;
struct DeltaSmem;
struct DensWarp;

size_t visc_smem_bytes();
size_t delta_smem_bytes();
size_t dens_smem_bytes();

__global__ void k_integrate(int n, Particles P, SimTables T, StepParams s);
__global__ void k_viscosity(Particles P, SimTables T, StepParams s);
__global__ void k_predict(int n, Particles P, SimTables T, StepParams s);
__global__ void k_scan(SimTables T, StepParams s, uint32_t nbSeed);
__global__ void k_scatter(int n, int n0, Particles P, SimTables T);
__global__ void k_grid_update(int n, Particles P, Particles Q, SimTables T, StepParams s);
__global__ void k_density(int n, Particles Q, SimTables T, StepParams s);
__global__ void k_delta(int n, int n0, Particles Q, SimTables T, StepParams s);
__global__ void k_collide(int n, Particles P, Particles Q, SimTables T, StepParams s);
__global__ void k_add(int first, int count, const float2 *pos, const float2 *force, Particles P, SimTables T,
                      StepParams s);
__global__ void k_gather_by_id(int n, const int *id, const float2 *src, float2 *dst);

}  // namespace sphgb
