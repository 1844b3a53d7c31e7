// Test infrastructure (oracle): headless C harness around the reference's own
// Demo4 solver.  Only tests, __graft_entry__.smoke() and bench.py's CPU
// baseline may load the library this file builds; the product never does.
//
// oracle/Makefile compiles this file together with the reference's
// NBodySimulation/demo4.cpp (+ demo4.h, sph.h, threading.h, base.h, utils.h
// and the vendored final_platform_layer.h) straight from the reference tree.
// Two headers are pre-empted by shims in oracle/shim: vecmath.h (MSVC-only
// anonymous unions; restated with the same arithmetic) and render.h (OpenGL
// command buffer; no-ops).  Everything on the step path -- Update(), the
// neighbour grid, the SPH kernels and collisions of sph.h, the ThreadPool --
// is the reference's code, unmodified.
//
// The C functions below map 1:1 onto BaseSimulation (base.h:8-38) plus
// state get/set for teacher forcing: the reference keeps all of its state in
// public members of Demo4::ParticleSimulation (demo4.h:178-199).
#include "vecmath_sub.h"
#include "render_stub.h"

#include <string>
#include <string.h>
#include <float.h>

#define FPL_IMPLEMENTATION
#define FPL_NO_AUDIO
#define FPL_NO_VIDEO
#define FPL_NO_WINDOW
#define FPL_NO_INPUT
#include <final_platform_layer.h>

// sph.h:75 asserts on non-constexpr float globals, which GCC refuses in a
// static_assert; the check (particle radius > collision margin) holds for the
// constants anyway.
#undef fplStaticAssert
#define fplStaticAssert(e)
#define strcpy_s(dst, n, src) strncpy(dst, src, n)

#include "demo4.cpp"

#include <stdint.h>
#include <math.h>

#include "sph_gb300.h"  // sph_scenario_desc, filled below from the reference's table

using Demo4::ParticleSimulation;

static bool g_platform_ready = false;

static ParticleSimulation *S(void *p) { return static_cast<ParticleSimulation *>(p); }

extern "C" {

void *sphref_create(void) {
	if (!g_platform_ready) {
		g_platform_ready = fplPlatformInit(fplInitFlags_None, nullptr);
	}
	ParticleSimulation *sim = new ParticleSimulation();
	// The constructor leaves cell counts uninitialised (demo4.cpp:19); the
	// application always clears before loading a scene (app.cpp:481).
	sim->ClearParticles();
	sim->ClearBodies();
	sim->ClearEmitters();
	sim->ResetStats();
	return sim;
}

void sphref_destroy(void *p) { delete S(p); }

void sphref_limits(int *gridX, int *gridY, float *cellSize, float *halfW, float *halfH,
                   uint64_t *maxParticles, uint64_t *maxCell, uint64_t *maxNeighbors) {
	*gridX = kSPHGridCountX;
	*gridY = kSPHGridCountY;
	*cellSize = kSPHGridCellSize;
	*halfW = kSPHBoundaryHalfWidth;
	*halfH = kSPHBoundaryHalfHeight;
	*maxParticles = kSPHMaxParticleCount;
	*maxCell = kSPHMaxCellParticleCount;
	*maxNeighbors = kSPHMaxParticleNeighborCount;
}

void sphref_reset_stats(void *p) { S(p)->ResetStats(); }
void sphref_clear_bodies(void *p) { S(p)->ClearBodies(); }
void sphref_clear_particles(void *p) { S(p)->ClearParticles(); }
void sphref_clear_emitters(void *p) { S(p)->ClearEmitters(); }
void sphref_set_gravity(void *p, float x, float y) { S(p)->SetGravity(Vec2f(x, y)); }
void sphref_add_external_force(void *p, float x, float y) { S(p)->AddExternalForces(Vec2f(x, y)); }
void sphref_clear_external_force(void *p) { S(p)->ClearExternalForce(); }
void sphref_set_multithreading(void *p, int on) { S(p)->SetMultiThreading(on != 0); }
uint64_t sphref_worker_count(void *p) { return S(p)->GetWorkerThreadCount(); }
uint64_t sphref_particle_count(void *p) { return S(p)->GetParticleCount(); }

// params: kernelHeight, cellSize, particleSpacing, invKernelHeight,
// restDensity, stiffness, nearStiffness, linearViscosity, quadraticViscosity
// (sph.h:77-86 member order).  Set through SetParams (member-wise copy).
void sphref_set_params(void *p, const float *v) {
	SPHParameters params;
	params.kernelHeight = v[0];
	params.cellSize = v[1];
	params.particleSpacing = v[2];
	params.invKernelHeight = v[3];
	params.restDensity = v[4];
	params.stiffness = v[5];
	params.nearStiffness = v[6];
	params.linearViscosity = v[7];
	params.quadraticViscosity = v[8];
	S(p)->SetParams(params);
}

void sphref_get_params(void *p, float *v) {
	const SPHParameters &params = S(p)->GetParams();
	v[0] = params.kernelHeight;
	v[1] = params.cellSize;
	v[2] = params.particleSpacing;
	v[3] = params.invKernelHeight;
	v[4] = params.restDensity;
	v[5] = params.stiffness;
	v[6] = params.nearStiffness;
	v[7] = params.linearViscosity;
	v[8] = params.quadraticViscosity;
}

// The 8-argument SPHParameters constructor exactly as the scenario table uses
// it (sph.h:112-122), so tests can pin what it really stores.
void sphref_params_from_ctor8(const float *a, float *out) {
	SPHParameters params(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7]);
	out[0] = params.kernelHeight;
	out[1] = params.cellSize;
	out[2] = params.particleSpacing;
	out[3] = params.invKernelHeight;
	out[4] = params.restDensity;
	out[5] = params.stiffness;
	out[6] = params.nearStiffness;
	out[7] = params.linearViscosity;
	out[8] = params.quadraticViscosity;
}

void sphref_add_plane(void *p, float nx, float ny, float d) { S(p)->AddPlane(Vec2f(nx, ny), d); }
void sphref_add_circle(void *p, float x, float y, float r) { S(p)->AddCircle(Vec2f(x, y), r); }
void sphref_add_segment(void *p, float ax, float ay, float bx, float by) {
	S(p)->AddLineSegment(Vec2f(ax, ay), Vec2f(bx, by));
}
void sphref_add_polygon(void *p, uint64_t n, const float *xy) {
	Vec2f verts[kMaxScenarioPolygonCount];
	for (uint64_t k = 0; k < n && k < kMaxScenarioPolygonCount; ++k) verts[k] = Vec2f(xy[2 * k], xy[2 * k + 1]);
	S(p)->AddPolygon(n, verts);
}
uint64_t sphref_add_particle(void *p, float x, float y, float fx, float fy) {
	return S(p)->AddParticle(Vec2f(x, y), Vec2f(fx, fy));
}
void sphref_add_volume(void *p, float cx, float cy, float fx, float fy, int nx, int ny, float spacing) {
	S(p)->AddVolume(Vec2f(cx, cy), Vec2f(fx, fy), nx, ny, spacing);
}
void sphref_add_emitter(void *p, float px, float py, float dx, float dy, float radius, float speed,
                        float rate, float duration) {
	S(p)->AddEmitter(Vec2f(px, py), Vec2f(dx, dy), radius, speed, rate, duration);
}

void sphref_update(void *p, float dt) { S(p)->Update(dt); }
void sphref_srand(unsigned seed) { srand(seed); }

// Particle state, AoS -> six float2 arrays (any may be null).
void sphref_get_particles(void *p, float *pos, float *prev, float *acc, float *vel, float *dens, float *press) {
	ParticleSimulation *s = S(p);
	for (size_t i = 0; i < s->particleCount; ++i) {
		const Demo4::ParticleData &d = s->particleDatas[i];
		if (pos) { pos[2 * i] = d.curPosition.x; pos[2 * i + 1] = d.curPosition.y; }
		if (prev) { prev[2 * i] = d.prevPosition.x; prev[2 * i + 1] = d.prevPosition.y; }
		if (acc) { acc[2 * i] = d.acceleration.x; acc[2 * i + 1] = d.acceleration.y; }
		if (vel) { vel[2 * i] = d.velocity.x; vel[2 * i + 1] = d.velocity.y; }
		if (dens) { dens[2 * i] = d.density; dens[2 * i + 1] = d.nearDensity; }
		if (press) { press[2 * i] = d.pressure; press[2 * i + 1] = d.nearPressure; }
	}
}

// Per-particle grid bookkeeping: cell (x, y), index in cell, list length.
void sphref_get_index(void *p, int *cellXY, uint64_t *indexInCell, uint64_t *neighborCount) {
	ParticleSimulation *s = S(p);
	for (size_t i = 0; i < s->particleCount; ++i) {
		const Demo4::ParticleIndex &q = s->particleIndexes[i];
		if (cellXY) { cellXY[2 * i] = q.cellIndex.x; cellXY[2 * i + 1] = q.cellIndex.y; }
		if (indexInCell) indexInCell[i] = q.indexInCell;
		if (neighborCount) neighborCount[i] = q.neighborCount;
	}
}

// Neighbour list of one particle, in list order.
void sphref_get_neighbors(void *p, uint64_t i, uint64_t *out) {
	const Demo4::ParticleIndex &q = S(p)->particleIndexes[i];
	for (size_t k = 0; k < q.neighborCount; ++k) out[k] = q.neighbors[k];
}

// Cell contents in array order; cells are numbered y * gridX + x.
uint64_t sphref_get_cell(void *p, int cell, uint64_t *indices) {
	const Demo4::Cell &c = S(p)->cells[cell];
	if (indices) {
		for (size_t k = 0; k < c.count; ++k) indices[k] = c.indices[k];
	}
	return c.count;
}

// Teacher forcing: overwrite the complete solver state.  Neighbour lists are
// given flattened in particle order (lengths in neighborCount); cells are
// given flattened in cell order (lengths in cellCount).  Returns 0, or -1 if
// a capacity of the reference would be exceeded.
int sphref_set_state(void *p, uint64_t n, const float *pos, const float *prev, const float *acc,
                     const float *vel, const float *dens, const float *press, const int *cellXY,
                     const uint64_t *indexInCell, const uint64_t *neighborCount, const uint64_t *neighbors,
                     const uint64_t *cellCount, const uint64_t *cellIndices) {
	ParticleSimulation *s = S(p);
	if (n > kSPHMaxParticleCount) return -1;
	for (int c = 0; c < kSPHGridTotalCount; ++c) {
		if (cellCount[c] > kSPHMaxCellParticleCount) return -1;
	}
	for (uint64_t i = 0; i < n; ++i) {
		if (neighborCount[i] > kSPHMaxParticleNeighborCount) return -1;
	}
	s->particleCount = n;
	const uint64_t *nb = neighbors;
	for (uint64_t i = 0; i < n; ++i) {
		Demo4::ParticleData &d = s->particleDatas[i];
		d.curPosition = Vec2f(pos[2 * i], pos[2 * i + 1]);
		d.prevPosition = Vec2f(prev[2 * i], prev[2 * i + 1]);
		d.acceleration = Vec2f(acc[2 * i], acc[2 * i + 1]);
		d.velocity = Vec2f(vel[2 * i], vel[2 * i + 1]);
		d.density = dens[2 * i];
		d.nearDensity = dens[2 * i + 1];
		d.pressure = press[2 * i];
		d.nearPressure = press[2 * i + 1];
		Demo4::ParticleIndex &q = s->particleIndexes[i];
		q.cellIndex = Vec2i(cellXY[2 * i], cellXY[2 * i + 1]);
		q.indexInCell = indexInCell[i];
		q.neighborCount = neighborCount[i];
		for (uint64_t k = 0; k < neighborCount[i]; ++k) q.neighbors[k] = *nb++;
	}
	const uint64_t *ci = cellIndices;
	for (int c = 0; c < kSPHGridTotalCount; ++c) {
		Demo4::Cell &cell = s->cells[c];
		cell.count = cellCount[c];
		for (uint64_t k = 0; k < cellCount[c]; ++k) cell.indices[k] = *ci++;
	}
	return 0;
}

// counts: minNeighbors, maxNeighbors, minCell, maxCell; times: the nine
// stage timers of SPHStatistics (sph.h:131-141), in milliseconds.
void sphref_get_stats(void *p, uint64_t *counts, float *times) {
	const SPHStatistics &st = S(p)->GetStats();
	counts[0] = st.minParticleNeighborCount;
	counts[1] = st.maxParticleNeighborCount;
	counts[2] = st.minCellParticleCount;
	counts[3] = st.maxCellParticleCount;
	times[0] = st.time.emitters;
	times[1] = st.time.integration;
	times[2] = st.time.viscosityForces;
	times[3] = st.time.predict;
	times[4] = st.time.updateGrid;
	times[5] = st.time.neighborSearch;
	times[6] = st.time.densityAndPressure;
	times[7] = st.time.deltaPositions;
	times[8] = st.time.collisions;
}

// The calls DemoApplication::LoadScenario (app.cpp:477-534) makes for
// SPHScenarios[index] (sph.h:315-437), written into the C ABI's description
// struct: bodies as placed by the loader, then the volume loop -- which walks
// bodyCount entries of the scenario's volume table -- then the emitters.
int sphref_scenario_count(void) { return (int)(sizeof(SPHScenarios) / sizeof(SPHScenarios[0])); }

int sphref_scenario_describe(int index, sph_scenario_desc *out) {
	if (index < 0 || index >= sphref_scenario_count()) return -1;
	const SPHScenario &sc = SPHScenarios[index];
	memset(out, 0, sizeof(*out));
	strncpy(out->name, sc.name, sizeof(out->name) - 1);
	out->gravity = sph_vec2{sc.gravity.x, sc.gravity.y};
	const SPHParameters &p = sc.parameters;
	out->params = sph_params{p.kernelHeight,  p.cellSize,      p.particleSpacing,  p.invKernelHeight,   p.restDensity,
	                         p.stiffness,     p.nearStiffness, p.linearViscosity,  p.quadraticViscosity};
	out->body_count = (uint32_t)sc.bodyCount;
	for (size_t b = 0; b < sc.bodyCount; ++b) {
		const SPHScenarioBody &body = sc.bodies[b];
		sph_scenario_body &o = out->bodies[b];
		switch (body.type) {
			case SPHScenarioBodyType_Plane:
				o.type = SPH_BODY_PLANE;
				o.normal = sph_vec2{body.orientation.col1.x, body.orientation.col1.y};
				o.distance = Vec2Dot(body.orientation.col1, body.position);
				break;
			case SPHScenarioBodyType_Circle:
				o.type = SPH_BODY_CIRCLE;
				o.center = sph_vec2{body.position.x, body.position.y};
				o.radius = body.radius;
				break;
			case SPHScenarioBodyType_LineSegment:
			case SPHScenarioBodyType_Polygon: {
				o.type = body.type == SPHScenarioBodyType_Polygon ? SPH_BODY_POLYGON : SPH_BODY_LINE_SEGMENT;
				o.vertex_count = (int)body.vertexCount;
				for (size_t k = 0; k < body.vertexCount; ++k) {
					const Vec2f v = Vec2MultMat2(body.orientation, body.localVerts[k]) + body.position;
					o.verts[k] = sph_vec2{v.x, v.y};
				}
			} break;
			default:
				break;
		}
	}
	const float spacing = sc.parameters.particleSpacing;
	out->volume_count = (uint32_t)sc.bodyCount;
	for (size_t v = 0; v < sc.bodyCount; ++v) {
		const SPHScenarioVolume &vol = sc.volumes[v];
		sph_scenario_volume &o = out->volumes[v];
		o.center = sph_vec2{vol.position.x, vol.position.y};
		o.force = sph_vec2{vol.force.x, vol.force.y};
		o.count_x = (int)floor(vol.size.x / spacing);
		o.count_y = (int)floor(vol.size.y / spacing);
		o.spacing = spacing;
	}
	out->emitter_count = (uint32_t)sc.emitterCount;
	for (size_t e = 0; e < sc.emitterCount; ++e) {
		const SPHScenarioEmitter &em = sc.emitters[e];
		out->emitters[e] = sph_scenario_emitter{{em.position.x, em.position.y}, {em.direction.x, em.direction.y},
		                                        em.radius, em.speed, em.rate, em.duration};
	}
	return 0;
}

}  // extern "C"
