/*
 * sph_gb300.h -- C ABI of the GB300-native Demo4 SPH step.
 *
 * One `sph_sim` is one simulation, living on one CUDA device and one CUDA
 * stream.  The entry points mirror the reference's simulation interface
 * `BaseSimulation` (NBodySimulation/base.h:8-38) as implemented by
 * `Demo4::ParticleSimulation` (NBodySimulation/demo4.h:178-267,
 * demo4.cpp:13-451); each declaration names the reference member it replaces.
 * Differences a caller must know:
 *
 *  - Every function returns an `int` status (SPH_OK or an SPH_ERR_* code);
 *    the reference returns nothing and asserts or overruns on overflow.
 *  - Vectors are passed by value as `sph_vec2` instead of `const Vec2f &`.
 *  - `Render` (base.h:25) has no counterpart: particle data is read with
 *    `sph_read_particles` (host copy) or `sph_device_arrays` (device
 *    pointers) instead of handing the AoS array to OpenGL.
 *  - What the reference fixes at compile time (sph.h:15-72: box size, grid
 *    cell size, capacities) is the `sph_domain` given to `sph_create`.
 *  - Multithreading switches are accepted for interface compatibility; the
 *    step always runs on the GPU.
 *
 * Results: one `sph_update` from a given labelled state equals the
 * reference's single-worker `Update` on the same state (same particle
 * numbering, same cell arrays, same neighbour lists) to within FP32 rounding
 * of the summation order; the neighbour structure and cell assignment are
 * bit-identical.  Between updates the library renumbers particles
 * (cell-major); `sph_read_particles` returns data in AddParticle order,
 * `sph_dump_state` in the internal numbering.
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define SPH_OK 0
#define SPH_ERR_INVALID_ARGUMENT 1
#define SPH_ERR_CAPACITY 2       /* a domain capacity would be exceeded */
#define SPH_ERR_CUDA 3           /* a CUDA runtime call failed */
#define SPH_ERR_DEVICE_OVERFLOW 4 /* a kernel flagged a capacity overflow */
#define SPH_ERR_TIMEOUT 5        /* a bounded device-side wait ran out */
#define SPH_ERR_NOT_SUPPORTED 6
#define SPH_ERR_NO_DEVICE 7

typedef struct sph_sim sph_sim;

typedef struct sph_vec2 {
	float x, y;
} sph_vec2;

/* The compile-time constants of sph.h:15-72, as runtime values. */
typedef struct sph_domain {
	float width;              /* kSPHBoundaryWidth; box centred on the origin */
	float height;             /* kSPHBoundaryHeight */
	float cell_size;          /* kSPHGridCellSize; grid = (int)(width/cell) x (int)(height/cell) */
	uint32_t max_particles;   /* kSPHMaxParticleCount */
	uint32_t max_cell_particles; /* kSPHMaxCellParticleCount (also the stats seed) */
	uint32_t max_neighbors;   /* kSPHMaxParticleNeighborCount */
	float particle_radius;    /* kSPHParticleCollisionRadius */
	float collision_margin;   /* kSPHCollisionMargin */
	float jitter_kernel_height; /* kSPHKernelHeight, as the volume/emitter jitter uses it */
	float jitter_scale;       /* kSPHVolumeParticleDistributionScale */
} sph_domain;

/* SPHParameters (sph.h:77-86), same member order. */
typedef struct sph_params {
	float kernel_height;
	float cell_size;
	float particle_spacing;
	float inv_kernel_height;
	float rest_density;
	float stiffness;
	float near_stiffness;
	float linear_viscosity;
	float quadratic_viscosity;
} sph_params;

/* SPHStatistics (sph.h:125-141); times in milliseconds (device time). */
typedef struct sph_stats {
	uint64_t min_particle_neighbor_count;
	uint64_t max_particle_neighbor_count;
	uint64_t min_cell_particle_count;
	uint64_t max_cell_particle_count;
	float time_emitters;
	float time_integration;
	float time_viscosity_forces;
	float time_predict;
	float time_update_grid;
	float time_neighbor_search;
	float time_density_and_pressure;
	float time_delta_positions;
	float time_collisions;
} sph_stats;

/* The reference's constants (sph.h:18-72) and SPHParameters() (sph.h:88-98). */
int sph_reference_domain(sph_domain *out);
int sph_default_params(sph_params *out);
const char *sph_status_string(int status);
/* No counterpart in the reference: the CUDA error name, failing call and
 * message behind the last SPH_ERR_CUDA returned on this thread ("" if none). */
const char *sph_last_error(void);

/* Demo4::ParticleSimulation() / ~ParticleSimulation() (demo4.cpp:14-35).
 * `device` selects the CUDA device; all device memory for `domain` is
 * allocated here. */
int sph_create(const sph_domain *domain, int device, sph_sim **out);
int sph_destroy(sph_sim *sim);

/* BaseSimulation::ResetStats / ClearBodies / ClearParticles / ClearEmitters
 * (base.h:10-13; demo4.cpp:78-140). */
int sph_reset_stats(sph_sim *sim);
int sph_clear_bodies(sph_sim *sim);
int sph_clear_particles(sph_sim *sim);
int sph_clear_emitters(sph_sim *sim);

/* BaseSimulation::AddPlane / AddCircle / AddLineSegment / AddPolygon
 * (base.h:15-18; demo4.cpp:82-123).  At most 100 bodies (kSPHMaxBodyCount),
 * polygons of at most 8 vertices (kMaxScenarioPolygonCount). */
int sph_add_plane(sph_sim *sim, sph_vec2 normal, float distance);
int sph_add_circle(sph_sim *sim, sph_vec2 pos, float radius);
int sph_add_line_segment(sph_sim *sim, sph_vec2 a, sph_vec2 b);
int sph_add_polygon(sph_sim *sim, size_t vertex_count, const sph_vec2 *verts);

/* BaseSimulation::AddParticle (base.h:20; demo4.cpp:142-153).  The returned
 * index is stable for the particle's lifetime (until ClearParticles). */
int sph_add_particle(sph_sim *sim, sph_vec2 position, sph_vec2 force, size_t *out_index);
/* `count` AddParticle calls in one transfer; indices first_index.. follow. */
int sph_add_particles(sph_sim *sim, size_t count, const sph_vec2 *positions, const sph_vec2 *forces,
                      size_t *first_index);
/* BaseSimulation::AddVolume (base.h:21; demo4.cpp:169-181).  Jitter draws on
 * the C library's rand(), as the reference does. */
int sph_add_volume(sph_sim *sim, sph_vec2 center, sph_vec2 force, int count_x, int count_y, float spacing);
/* BaseSimulation::AddEmitter (base.h:22; demo4.cpp:155-167). */
int sph_add_emitter(sph_sim *sim, sph_vec2 position, sph_vec2 direction, float radius, float speed, float rate,
                    float duration);

/* BaseSimulation::Update (base.h:24; demo4.cpp:286-451).  Asynchronous on
 * the simulation's stream except where emitters fire; errors flagged by
 * kernels are reported by the next call that synchronises (sph_get_stats,
 * sph_read_particles, sph_dump_state, sph_synchronize). */
int sph_update(sph_sim *sim, float delta_time);

/* BaseSimulation::AddExternalForces / ClearExternalForce (base.h:27-28). */
int sph_add_external_forces(sph_sim *sim, sph_vec2 force);
int sph_clear_external_force(sph_sim *sim);

/* BaseSimulation::GetParticleCount / SetGravity / GetParams / GetStats /
 * SetParams (base.h:30-34). */
int sph_get_particle_count(sph_sim *sim, size_t *out);
int sph_set_gravity(sph_sim *sim, sph_vec2 gravity);
int sph_get_params(sph_sim *sim, sph_params *out);
int sph_get_stats(sph_sim *sim, sph_stats *out);
int sph_set_params(sph_sim *sim, const sph_params *params);

/* BaseSimulation::SetMultiThreading / IsMultiThreadingSupported /
 * IsMultiThreading / GetWorkerThreadCount (base.h:35-38).  Kept for
 * interface compatibility: the value is stored and reported back. */
int sph_set_multithreading(sph_sim *sim, int value);
int sph_is_multithreading_supported(sph_sim *sim, int *out);
int sph_is_multithreading(sph_sim *sim, int *out);
int sph_get_worker_thread_count(sph_sim *sim, size_t *out);

/* Replaces the raw AoS pointer Render hands to OpenGL (demo4.cpp:520-531):
 * copies `count` particles (AddParticle order) to host arrays; any pointer
 * may be NULL.  dens = (density, nearDensity), press = (pressure,
 * nearPressure), as in ParticleData (demo4.h:81-109). */
int sph_read_particles(sph_sim *sim, size_t count, sph_vec2 *pos, sph_vec2 *prev, sph_vec2 *vel, sph_vec2 *acc,
                       sph_vec2 *dens, sph_vec2 *press);

/* Full state in the internal numbering, for snapshots and teacher forcing.
 * Particle arrays hold `count` entries each (any pointer may be NULL).
 * `cell` is the linear cell index y*gx+x of each particle's last grid
 * insertion (ParticleIndex::cellIndex); `id` its AddParticle index.
 * Cells: `cell_start`/`cell_count` (gx*gy entries) give each cell's array as
 * a range of internal numbers for the first `canonical_count` particles;
 * particles numbered >= canonical_count were added since the last update,
 * sit at the end of their cell's array in numbering order and have no
 * neighbour list.  Every particle below canonical_count has the neighbour
 * list the reference's NeighborSearch (demo4.cpp:183-206) builds from these
 * cell arrays. */
typedef struct sph_state_view {
	size_t count;
	size_t canonical_count;
	int grid_x, grid_y;
	sph_vec2 *pos, *prev, *vel, *acc, *dens, *press;
	int32_t *id;
	int32_t *cell;
	int32_t *cell_start, *cell_count;
} sph_state_view;
int sph_state_info(sph_sim *sim, size_t *count, size_t *canonical_count, int *grid_x, int *grid_y);
int sph_dump_state(sph_sim *sim, const sph_state_view *out);
/* Inverse of sph_dump_state (all particle pointers and the cell tables are
 * required).  The cell tables must describe a consistent canonical state. */
int sph_load_state(sph_sim *sim, const sph_state_view *in);

/* The simulation's CUDA stream (cudaStream_t) and device arrays, for callers
 * that time on the stream or consume results on the device.  Device arrays
 * are float2 in the internal numbering and are valid until the next call
 * that changes the simulation. */
int sph_get_stream(sph_sim *sim, void **stream);
int sph_device_arrays(sph_sim *sim, const void **pos, const void **vel, const void **dens, const void **press);

/* Replaces the colouring and point drawing of Render (base.h:25,
 * demo4.cpp:453-532) without a graphics API.  sph_particle_colors: RGBA
 * (4 floats per particle) of the first `count` particles in AddParticle
 * order, SPHGetParticleColor (sph.h:683-695) of the rest density, density,
 * pressure and velocity.  sph_render_points: a width x height RGBA8 image of
 * the box (row 0 at the top, pixel (x, y) spans world x in
 * [-W/2 + x W/width, ...)); each particle colours the pixel under it with
 * its colour rounded to 8 bits, later particles (AddParticle order) over
 * earlier ones; empty pixels are 0.  Both act on the first scene. */
int sph_particle_colors(sph_sim *sim, size_t count, float *rgba);
int sph_render_points(sph_sim *sim, int width, int height, unsigned char *rgba);

/* ---- Built-in scenarios (SPHScenarios[], sph.h:315-437) --------------------
 * The reference application loads a scenario with DemoApplication::
 * LoadScenario (app.cpp:477-534): reset stats, clear bodies, particles and
 * emitters, set gravity and parameters, add the bodies (planes at distance
 * dot(normal, position); segment and polygon vertices rotated by the body's
 * orientation and moved to its position), the volumes and the emitters.
 * sph_scenario_describe reports exactly the calls it makes, in order; its
 * volume loop walks the first body_count entries of the scenario's
 * zero-filled volume table (a reference quirk, app.cpp:522), so volumes past
 * the scenario's own are empty.  Scenario parameters come from the
 * 8-argument SPHParameters constructor, which keeps kSPHKernelHeight and
 * kSPHRestDensity whatever is passed (sph.h:112-122).  sph_load_scenario
 * makes those calls on `sim` (which should have the reference domain,
 * sph_reference_domain); volume and emitter jitter use the C library's
 * rand(), as the reference does. */
#define SPH_SCENARIO_MAX_BODIES 32
#define SPH_SCENARIO_MAX_VOLUMES 32
#define SPH_SCENARIO_MAX_EMITTERS 8
enum { SPH_BODY_PLANE = 1, SPH_BODY_CIRCLE = 2, SPH_BODY_LINE_SEGMENT = 3, SPH_BODY_POLYGON = 4 };
typedef struct sph_scenario_body {
	int type;           /* SPH_BODY_* */
	int vertex_count;   /* segment: 2; polygon: 3..8 */
	sph_vec2 normal;    /* plane: sph_add_plane(normal, distance) */
	float distance;
	sph_vec2 center;    /* circle: sph_add_circle(center, radius) */
	float radius;
	sph_vec2 verts[8];  /* segment a, b; polygon vertices (world coordinates) */
} sph_scenario_body;
typedef struct sph_scenario_volume {
	sph_vec2 center;
	sph_vec2 force;
	int count_x, count_y;  /* (int)floor(size / particle_spacing) */
	float spacing;
} sph_scenario_volume;
typedef struct sph_scenario_emitter {
	sph_vec2 position, direction;
	float radius, speed, rate, duration;
} sph_scenario_emitter;
typedef struct sph_scenario_desc {
	char name[100];
	sph_vec2 gravity;
	sph_params params;
	uint32_t body_count;
	sph_scenario_body bodies[SPH_SCENARIO_MAX_BODIES];
	uint32_t volume_count;
	sph_scenario_volume volumes[SPH_SCENARIO_MAX_VOLUMES];
	uint32_t emitter_count;
	sph_scenario_emitter emitters[SPH_SCENARIO_MAX_EMITTERS];
} sph_scenario_desc;
/* Number of built-in scenarios (8). */
int sph_scenario_count(int *count);
/* The calls LoadScenario makes for scenario `index`; `out` is zeroed first. */
int sph_scenario_describe(int index, sph_scenario_desc *out);
/* DemoApplication::LoadScenario (app.cpp:477-534) on this simulation. */
int sph_load_scenario(sph_sim *sim, int index);
int sph_synchronize(sph_sim *sim);
/* Number of kernels this library launched for `sim` since creation. */
int sph_kernel_launches(sph_sim *sim, uint64_t *out);
/* No counterpart in the reference.  Updates that repeat the previous one's
 * shape (same scenes, bodies, parameters and dt; no particles added since)
 * are replayed from a CUDA graph captured per step; enable = 0 launches every
 * kernel one by one instead.  Results are identical either way.  Default 1. */
int sph_use_graphs(sph_sim *sim, int enable);
/* No counterpart in the reference.  Launch shapes of the two ordered sweeps
 * (viscosity, delta): shape[4] = {viscosity warps per block (4 = wide,
 * 5 = lean), viscosity blocks, delta warps per block (12 = wide, 8 = mid,
 * 4 = quad, 3 = tri, 2 = lean, 16 = dense), delta blocks}.  The wide shapes
 * shorten one scene's critical path: one task per block; the wide viscosity
 * sweep runs each particle's head beside the previous particle's tail on two
 * lanes; the wide, mid, quad, tri and dense delta sweeps overlap each
 * particle's ordered sum with the next particle's pairs (11, 7, 3, 2 and 15
 * producer warps beside one summer warp; mid, quad and tri run several
 * blocks per SM; dense stages 12,288 entries per task, for crowded
 * states).  The lean ones
 * fit more tasks on an SM (the lean viscosity sweep runs five tasks per
 * block) for large scenes and many scenes.  Results do not depend on the
 * shape.  sph_autotune times the
 * next update (step dt) from the current state for every shape and resident
 * block count per SM, keeps the fastest for each sweep, restores the state
 * and reports the choice; it needs a state after an update. */
int sph_autotune(sph_sim *sim, float dt, int *shape);
/* Particle order of the update (single-scene simulations).  By default the
 * library renumbers particles cell by cell after every update (colour-major
 * cells, each cell's array in the reference's order) and runs the two
 * ordered passes (viscosity, delta) and the grid update in that numbering:
 * one update from a given state equals the reference's Update on the same
 * numbered state, but a run of many updates visits particles in a different
 * order from the reference's own run (demo4.cpp:223-255, 344-352 loop over
 * the reference's index order, which is AddParticle order), so its
 * trajectory drifts from the reference's by rounding from the second update
 * on.  enable = 1 selects reference order: both passes and the grid update
 * visit particles in AddParticle order, so every update equals the
 * reference's single-worker Update on the reference's own numbering, and a
 * free run reproduces the reference's trajectory bit for bit.  The storage
 * numbering (sph_dump_state) is unchanged; reference order costs speed (its
 * tasks follow AddParticle order, not the cell colouring) and is meant for
 * validation and reproduction.  Default 0. */
int sph_set_reference_order(sph_sim *sim, int enable);
int sph_get_reference_order(sph_sim *sim, int *out);
/* No counterpart in the reference (which waits on its worker threads without
 * a limit, threading.h:101-109).  Every device-side wait of the ordered
 * sweeps (a task waiting for an earlier task whose neighbourhood overlaps
 * its own) gives up after `seconds` (default 2): the sweep then stops
 * waiting, the update's results are not meaningful, and the next call that
 * synchronises returns SPH_ERR_TIMEOUT.  The simulation stays usable; load a
 * state (sph_load_state) to continue from known data. */
int sph_set_wait_limit(sph_sim *sim, double seconds);
/* No counterpart in the reference; for tests of the timeout path only.  In
 * the next updates the task claimed at position `claim` of sweep `sweep`
 * (0 = viscosity, 1 = delta) does its work but never publishes that it is
 * done, so the tasks that depend on it wait until the wait limit.  -1 turns
 * it off (the default). */
int sph_test_hold_task(sph_sim *sim, int sweep, int claim);
int sph_get_sweep_shape(sph_sim *sim, int *shape);
int sph_set_sweep_shape(sph_sim *sim, const int *shape);

/* Dense states.  With adaptive shapes on (the default), an update whose
 * previous updates saw neighbour lists longer than 440 runs the wide
 * viscosity shape, and one where a 3x3 block of the fullest cell's count
 * passes 0.65 of the tuned delta shape's stage runs the 8-warp delta shape
 * (4,096 staged entries), or the 16-warp shape (12,288) once a 5x5 region
 * of it nears 4,096, instead of the tuned shapes (results are identical in
 * every shape; only the launch differs).  Single-scene simulations only: a
 * batch keeps its tuned shapes.  The statistics come from the
 * end of earlier updates, read without waiting.  sph_last_sweep_shape
 * returns the shapes the last update ran with, in sph_get_sweep_shape's
 * form.  sph_autotune times the shapes with adaptivity off. */
int sph_set_adaptive_shapes(sph_sim *sim, int enable);
int sph_last_sweep_shape(sph_sim *sim, int shape[4]);

/* ---- Viscoelastic springs (no reference counterpart) ----------------------
 * Springs with plasticity after Clavet et al. 2005 ("Particle-based
 * viscoelastic fluid simulation", Algorithms 3 and 4), in a deterministic
 * parallel form run between the neighbour search and density: existing
 * springs within h are adjusted (tolerable deformation yield_ratio * L,
 * rate plasticity), springs whose rest length exceeds h are removed, free
 * slots go to the nearest in-range neighbours without a spring (ordered by
 * distance, then AddParticle index) and a spring is added where both ends
 * chose each other (rest length h, adjusted at once); then every particle
 * moves by -D/2 of each of its springs, D = dt^2 stiffness (1 - L/h) (L - r)
 * r_hat, from the positions before the phase.  At most max_per_particle
 * (<= 16) springs per particle.  Off by default; single-scene simulations
 * only.  Enabling allocates the spring arrays (128 B per particle per buffer
 * set). */
typedef struct sph_spring_params {
	int enabled;
	float yield_ratio;     /* gamma */
	float plasticity;      /* alpha */
	float stiffness;       /* k_spring */
	int max_per_particle;  /* <= 16 */
} sph_spring_params;
int sph_set_springs(sph_sim *sim, const sph_spring_params *params);
/* Springs after the last update (each counted once). */
int sph_get_spring_count(sph_sim *sim, uint64_t *out);
/* Spring tables in the internal numbering of sph_dump_state: per particle a
 * count and 16 slots of partner number (-1 past the count) and rest length.
 * `count` must equal the particle count.  sph_load_state clears the springs;
 * sph_load_springs (after it) sets them. */
int sph_dump_springs(sph_sim *sim, size_t count, int32_t *spring_count, int32_t *partner, float *rest);
int sph_load_springs(sph_sim *sim, size_t count, const int32_t *spring_count, const int32_t *partner,
                     const float *rest);

/* ---- Batched scenes (no single reference counterpart) ---------------------
 * Many independent Demo4 scenes advanced together: one sph_update(sim, dt)
 * advances every scene by dt with one launch per stage over all of them.
 * Each scene's update equals what a single-scene simulation holding the same
 * state computes (ParticleSimulation::Update, demo4.cpp:286-427), bit for
 * bit; scenes never interact.  A batch is fixed at creation: its scenes,
 * bodies and particles (the scene descriptions below, in the reference's
 * AddParticle/AddPlane/AddCircle/AddLineSegment/AddPolygon terms) are given
 * to sph_batch_create, and the single-scene mutators (Add*, Clear*,
 * SetGravity, SetParams, external forces, sph_load_state) return
 * SPH_ERR_NOT_SUPPORTED on a batch. */
#define SPH_BODY_PLANE 1   /* a = normal, value = distance (demo4.cpp:121-125) */
#define SPH_BODY_CIRCLE 2  /* a = centre, value = radius (demo4.cpp:127-131) */
#define SPH_BODY_SEGMENT 3 /* a, b = end points (demo4.cpp:133-137) */
#define SPH_BODY_POLYGON 4 /* verts[0..vertex_count) (demo4.cpp:139-140) */
typedef struct sph_body_desc {
	int type;
	size_t vertex_count;
	sph_vec2 a, b;
	float value;
	sph_vec2 verts[8];
} sph_body_desc;
typedef struct sph_scene_desc {
	sph_domain domain;          /* max_particles is ignored: the capacity is particle_count */
	sph_params params;
	sph_vec2 gravity;
	size_t particle_count;
	const sph_vec2 *positions;  /* AddParticle order */
	const sph_vec2 *forces;     /* NULL = zero */
	size_t body_count;
	const sph_body_desc *bodies;
} sph_scene_desc;
int sph_batch_create(const sph_scene_desc *scenes, size_t scene_count, int device, sph_sim **out);
int sph_batch_scene_count(sph_sim *sim, size_t *out);
/* Per-scene reads; `scene` indexes the creation order.  Arrays are in the
 * scene's AddParticle order; any output pointer may be NULL. */
int sph_batch_read_particles(sph_sim *sim, size_t scene, size_t count, sph_vec2 *pos, sph_vec2 *vel, sph_vec2 *dens,
                             sph_vec2 *press);
int sph_batch_get_stats(sph_sim *sim, size_t scene, sph_stats *out);
int sph_batch_state_info(sph_sim *sim, size_t scene, size_t *count, size_t *canonical_count, int *grid_x,
                         int *grid_y);
int sph_batch_dump_state(sph_sim *sim, size_t scene, const sph_state_view *out);

/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (code running inside another component's memory budget or allocator, or a
 * real-time loop that must not allocate): density and pressure
 * (SPHComputeDensity/SPHComputePressure semantics, what one update computes
 * for freshly added, motionless particles without gravity) of `count`
 * particles whose positions are on the current device at `pos`, written to
 * `dens` (density, near density) and `press` (pressure, near pressure).  The
 * work runs on `stream` (a cudaStream_t; NULL = legacy default stream) and
 * the call returns once it is done.  It allocates nothing: its working
 * memory is one fixed device array inside the library, sized for at most
 * SPH_NOALLOC_MAX_PARTICLES particles and SPH_NOALLOC_MAX_CELLS grid cells
 * (about 6.3 MiB, held by every GPU that loads the library until the process
 * exits); larger inputs, and domains allowing more than
 * SPH_NOALLOC_MAX_NEIGHBORS neighbours, return SPH_ERR_CAPACITY before any
 * work.  The domain's capacities hold as in the update: a cell with more
 * than max_cell_particles particles, or a 3x3 block listing more than
 * max_neighbors, is skipped and the call returns SPH_ERR_CAPACITY (the
 * reference asserts there).  The first call on a device looks up that
 * array's device address and keeps it for the life of the process; make it
 * before any stream capture, and do not call this entry point on a device
 * after cudaDeviceReset.  All calls share the array: calls whose work
 * overlaps on the GPU (other streams, other threads) race and must be
 * serialised by the caller. */
#define SPH_NOALLOC_MAX_PARTICLES 262144
#define SPH_NOALLOC_MAX_CELLS 262144
#define SPH_NOALLOC_MAX_NEIGHBORS 4096
int sph_density_pressure_noalloc(const sph_domain *domain, const sph_params *params, const sph_vec2 *pos,
                                 size_t count, sph_vec2 *dens, sph_vec2 *press, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GB300_H */
