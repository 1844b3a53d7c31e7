// Internal device-side declarations shared by the kernels and the host code
// of the GB300 Demo4 SPH step.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sphgb {

constexpr int kWarp = 32;
// Particles staged in shared memory per sweep task: the 3x3 cell block a
// neighbour list covers.  At least kSPHMaxParticleNeighborCount (1000,
// sph.h:69), so every scene the reference accepts fits.
constexpr int kStageCap = 1024;
// Particles staged per delta-sweep task: the new cells of the task's bounding
// box grown by one (5x5 cells when particles left the cell in every
// direction).
constexpr int kDeltaStageCap = 4096;
// The dense delta shape's stage: a 5x5 region of cells of ~490 particles.
constexpr int kDeltaDenseStageCap = 12288;
// In-range pairs buffered between the parallel geometry phase and the serial
// chain of one particle; longer lists are drained in several rounds.
constexpr int kChainCap = 256;
// Per-particle inputs of the delta sweep prefetched per chunk of a task.
constexpr int kPrefetch = 128;
// Working array of one cell during the grid update (kSPHMaxCellParticleCount
// is 500, sph.h:68).
constexpr int kCellCap = 512;
// Cells of a delta-sweep staging region (bounding box of a task's new cells,
// grown by one) in the smaller shapes (the 8- and 16-warp shapes take 256
// and 400).  Larger regions fall back to per-particle staging.
constexpr int kRegionCells = 100;
constexpr int kMaxBodies = 100;  // kSPHMaxBodyCount, sph.h:71
constexpr int kMaxPoly = 8;      // kMaxScenarioPolygonCount, sph.h:161
// Appendix particles (added since the last update) are swept serially in runs
// of this many consecutive numbers.
constexpr int kAppendixRun = 32;
// Pending dependencies a delta-sweep task lists before one warp polls them.
constexpr int kPendCap = 128;
// Spring slots per particle (viscoelastic springs, not in the reference).
constexpr int kSprings = 16;

// Error bits raised by kernels into SimTables::error.
enum : uint32_t {
	kErrStageOverflow = 1u,    // a 3x3 block exceeds the staging capacity
	kErrCellOverflow = 2u,     // a cell exceeds kCellCap during the grid update
	kErrTimeout = 4u,          // a bounded wait on another task ran out
	kErrIndex = 8u,            // an index failed a bounds check (skipped)
};

enum BodyType : int { kBodyPlane = 1, kBodyCircle = 2, kBodySegment = 3, kBodyPolygon = 4 };

// One collision body (demo4.h:59-120), flattened.
struct Body {
	int type;
	int vertexCount;
	float ax, ay;  // plane normal | circle centre | segment a
	float bx, by;  // segment b
	float r;       // plane distance | circle radius
	float pad;
	float verts[2 * kMaxPoly];
};

// Scalars of one step, prepared on the host in FP32 exactly as the
// reference computes them.
struct StepParams {
	float h2;       // kernelHeight * kernelHeight   (sph.h:470)
	float invH;     // params.invKernelHeight
	float rho0, k, kNear, sigma, beta;
	float dt, invDt, dt2;  // dt, 1/dt (demo4.cpp:287), dt*dt (sph.h:492)
	float extX, extY;      // gravity + externalForce (demo4.cpp:306)
	float halfW, halfH, cellSize;  // grid mapping (sph.h:450-463)
	int gx, gy, ncell;
	float radius;   // kSPHParticleCollisionRadius
	float margin;   // kSPHCollisionMargin
	int nbodies;
	// Viscoelastic springs (Clavet et al. 2005; not in the reference).
	int springs;          // 0 = off
	int springMax;        // slots a particle may fill (<= kSprings)
	float h;              // kernel height: initial and maximum rest length
	float springYield;    // gamma: tolerable deformation = gamma * L
	float springDtAlpha;  // dt * plasticity alpha
	float springK;        // spring stiffness
};

// One scene of a simulation.  A simulation holds one or more independent
// scenes in one arena: scene s owns particle numbers pBase .. pBase+n-1
// (canonical ones first, then the appendix) and global cells
// cellBase .. cellBase+p.ncell-1 (its own grid, numbered y*gx+x).
struct SceneDev {
	StepParams p;
	int cellBase;
	int pBase;
	int n, n0;
	int bodyBase;
	uint32_t nbSeed;  // neighbour-count statistics seed (kSPHMaxParticleNeighborCount)
	int pad[2];
};

// Totals of one update over all scenes.
struct Totals {
	int n;          // particles
	int ncell;      // cells (= canonical sweep tasks)
	int nApp;       // appendix runs (delta-sweep tasks after the canonical ones)
	int nscenes;
	// Reference order (single scene): both sweeps and the grid update run in
	// AddParticle order, as the reference's Update does on its own numbering;
	// the delta sweep's tasks are then nApp runs over all particles, and the
	// viscosity sweep's nViscRuns runs over the canonical ones.
	int refOrder;
	int nViscRuns;
};

// Particle arrays of one buffer set, in the internal numbering.
struct Particles {
	float2 *pos, *prev, *vel, *acc, *dens, *press;
	int *id;      // AddParticle index
	int *cellOf;  // linear cell of the last grid insertion
	// Springs (null when off): per particle a count and kSprings slots of
	// partner number and rest length, [particle][slot]; every spring is
	// stored at both ends with the same rest length.
	int *springN, *springP;
	float *springL;
};

// Grid and scheduling tables.  Canonical numbering: the particles of cell c
// (after the last update) are numbers cellStart[c] .. +cellCount[c]-1, cells
// in colour-major rank order; numbers >= n0 are the appendix.
struct SimTables {
	int *cellStart, *cellCount;        // canonical ranges, by global cell
	int *taskOfCell, *taskCell;        // global cell <-> sweep task (scenes interleaved)
	int *numberOrder;                  // global cells in numbering order (scene-major, colour rank)
	int *sceneOfCell, *sceneOf;        // scene of a global cell / of a particle number
	SceneDev *scenes;
	int *appScene, *appRun;            // appendix run tasks: scene, run within the scene
	int *appBox;                       // per appendix run: x0, y0, x1, y1 of its particles' new cells
	// Reference order: refOrd[pBase + id] = number of the particle with
	// AddParticle index id; viscBox per viscosity run: x0, y0, x1, y1 of its
	// particles' old cells.
	int *refOrd;
	int *viscBox;
	int *appCount, *appStart, *appIdx, *appCursor;  // appendix members per cell
	int *newCell;                      // cell after predict, per particle
	int *enterCount, *leaveCount, *enterOffset, *enterCursor, *enterList;
	int *moverList, *moverCount;       // moverCount[0]: movers; [1]: max cell move
	int *bbox;                         // per cell: x0, y0, x1, y1 of new cells
	int *newCount, *newStart;
	int *scanTiles;                    // 3 x tiles: per-tile sums, then tile offsets
	int *liveTask, *liveTiles, *nLive;  // occupied canonical cells' tasks in order, per-tile offsets, count
	int *newIdx;    // new number -> old number (the new cell arrays, concatenated)
	int *newLabel;  // old number -> new number
	uint32_t *done;                    // per sweep task
	int *taskCounter;                  // [0] viscosity, [1] delta
	uint32_t *stats;                   // per scene: minNb, maxNb, minCell, maxCell
	uint32_t *error;
	uint32_t *abort;
	// Bounded waits of the ordered sweeps give up after this many
	// nanoseconds (sph_set_wait_limit; 2 s by default).
	unsigned long long waitLimitNs;
	// Tests of the timeout path only (sph_test_hold_task): the sweep task
	// claimed at position hold[sweep] (0 = viscosity, 1 = delta) does its
	// work but never publishes its done flag; -1 = off.
	int hold[2];
	Body *bodies;
	// Spring phase scratch (null when off): chosen candidates per particle
	// (count, kSprings new numbers), positions after the phase, springs per scene.
	int *accN, *accP;
	float2 *springPos;
	unsigned long long *springTotal;
	// Diagnostics: when non-null, sweep tasks record %globaltimer stamps
	// (claimed, dependencies met, staged, done) at prof[(sweep * profStride + task) * 4].
	unsigned long long *prof;
	int profStride;
};

}  // namespace sphgb
