// Host side of the GB300 Demo4 SPH step: the simulation object behind the C
// ABI of include/sph_gb300.h, mirroring Demo4::ParticleSimulation
// (NBodySimulation/demo4.h:178-267).  A simulation holds one scene
// (sph_create: the reference's interface) or many independent scenes
// (sph_batch_create) in one arena; all device memory is allocated at
// creation, and an update is one launch per stage over every scene.
//
// Host arithmetic that feeds the step (volume and emitter particle
// placement, step scalars) follows the reference's FP32 operation order; the
// library is built with -ffp-contract=off so the host compiler fuses nothing.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <utility>
#include <vector>

#include "../../include/sph_gb300.h"
#include "../../include/sph_mpnn.h"
#include "mpnn_internal.cuh"
#include "sph_internal.cuh"
#include "sph_kernels.cuh"

using namespace sphgb;

namespace {

struct Emitter {
	sph_vec2 position, direction;
	float radius, speed, rate, duration, elapsed, totalElapsed;
	int active;
};

struct BufferSet {
	float2 *pos = nullptr, *prev = nullptr, *vel = nullptr, *acc = nullptr, *dens = nullptr, *press = nullptr;
	int *id = nullptr, *cellOf = nullptr;
	int *springN = nullptr, *springP = nullptr;  // allocated when springs are first enabled
	float *springL = nullptr;
	Particles view() const {
		Particles p;
		p.pos = pos;
		p.prev = prev;
		p.vel = vel;
		p.acc = acc;
		p.dens = dens;
		p.press = press;
		p.id = id;
		p.cellOf = cellOf;
		p.springN = springN;
		p.springP = springP;
		p.springL = springL;
		return p;
	}
};

enum Stage {
	kEvBegin,
	kEvIntegrate,
	kEvVisc,
	kEvPredict,
	kEvGrid,
	kEvSprings,
	kEvDensity,
	kEvDelta,
	kEvCollide,
	kEvCount
};

// One scene: the state Demo4::ParticleSimulation keeps on the host.
struct Scene {
	sph_domain dom{};
	int gx = 0, gy = 0, ncell = 0;
	sph_params params{};
	sph_vec2 gravity{0.0f, 0.0f};
	sph_vec2 external{0.0f, 0.0f};
	std::vector<Body> bodies;
	std::vector<Emitter> emitters;
	size_t n = 0;     // particles (device-resident + pending)
	size_t n0 = 0;    // canonical particles (numbered by the last update)
	size_t nDev = 0;  // particles already on the device
	size_t cap = 0;   // particle capacity
	int cellBase = 0, pBase = 0, bodyBase = 0;  // offsets into the shared arrays
	sph_spring_params springs{};
	std::vector<float2> pendPos, pendForce;
};

}  // namespace

struct sph_sim {
	int device = 0;
	cudaStream_t stream = nullptr;
	int numSMs = 0;
	int viscBlocks = 0, deltaBlocks = 0, densBlocks = 0, gridBlocks = 0;
	int viscLean = 0;   // viscosity shape: 0 = wide, 1 = lean (sph_kernels.cuh)
	bool refOrder = false;  // sweeps and grid events in AddParticle order (sph_set_reference_order)
	int viscRefBlocks = 0;
	int deltaShape = 0;  // delta shape: kDeltaWide, kDeltaLean or kDeltaMid
	// Dense states (sph_set_adaptive_shapes): the shapes above are the tuned
	// ones; an update whose previous updates saw long neighbour lists or
	// crowded cells runs the sweep shapes that stay staged there instead.
	// The statistics arrive in pinned host memory at the end of every update
	// and are read without waiting, so the choice may lag by an update.
	bool adaptive = true;
	bool denseVisc = false, denseDelta = false, crowdedDelta = false;
	int denseViscBlocks = 0, denseDeltaBlocks = 0, crowdedDeltaBlocks = 0;
	int runViscLean = -1, runViscBlocks = 0, runDeltaShape = -1, runDeltaBlocks = 0;  // of the last update
	uint32_t *hostStats = nullptr;  // pinned: 4 per scene, as T.stats
	cudaEvent_t statsEv[2] = {nullptr, nullptr};  // after the copy, per update parity
	bool batch = false;
	int multithreading = 0;

	std::vector<Scene> scenes;
	int ncellTotal = 0;
	size_t capTotal = 0;
	size_t bodyCap = 0;
	int springBlocks = 0;
	bool sceneTableDirty = true;
	bool bodiesDirty = true;
	float tableDt = 0.0f;

	BufferSet buf[2];
	int cur = 0;
	int *cellStartA = nullptr, *cellCountA = nullptr, *cellStartB = nullptr, *cellCountB = nullptr;
	SimTables T{};
	uint32_t *doneV = nullptr, *doneD = nullptr;
	size_t doneDCap = 0;
	int nApp = 0;
	float2 *stagePos = nullptr, *stageForce = nullptr;  // device staging for adds
	float2 *hostPos = nullptr, *hostForce = nullptr;    // pinned staging
	size_t stageCap = 0;

	// Per-step CUDA graphs, one per buffer parity (the step ping-pongs its
	// particle and cell arrays), replayed while nothing but time advances.
	cudaGraphExec_t graphs[2] = {nullptr, nullptr};
	uint64_t graphKernels[2] = {0, 0};
	int steadySteps = 0;  // updates since the scene table last changed
	bool useGraphs = true;

	// Learned frames: a snapshot of the canonical state (for the fallback and
	// for sample capture), the network's input/output and judge scratch.
	BufferSet snap;
	int *snapCellStart = nullptr, *snapCellCount = nullptr;
	float2 *lz0 = nullptr, *lu = nullptr, *lbyId = nullptr, *ldens = nullptr;
	double *lerr = nullptr;  // judge's reduction: kErrBlocks partial sums, then the total
	uint32_t *lstats = nullptr;

	// Headless render output (allocated on first use).
	float4 *colorBuf = nullptr;
	size_t colorCap = 0;
	unsigned long long *imgKeys = nullptr;
	uint32_t *imgRgba = nullptr;
	size_t imgCap = 0;

	cudaEvent_t ev[kEvCount] = {};
	bool timed = false;
	float emitterMs = 0.0f;
	uint64_t launches = 0;
	unsigned long long *prof = nullptr;
	int *check = nullptr;  // verdicts of device-side input checks

	size_t totalParticles() const {
		size_t t = 0;
		for (const Scene &sc : scenes) t += sc.n;
		return t;
	}
};

namespace {

constexpr unsigned long long kDefaultWaitLimitNs = 2000000000ull;  // 2 s per bounded wait
// The learned frame's judge rejects a corrected frame whose longest
// neighbour list exceeds this fraction of the neighbour capacity.
constexpr double kLearnedCrowding = 0.7;

// Text of the last failing CUDA call on this thread (sph_last_error).
thread_local char g_last_error[256] = "";

int cuda_failed(cudaError_t e, const char *what, int line) {
	snprintf(g_last_error, sizeof(g_last_error), "%s (%s) at sph_api.cu:%d: %s", cudaGetErrorName(e), what, line,
	         cudaGetErrorString(e));
	return SPH_ERR_CUDA;
}

int cuda_status(cudaError_t e) { return e == cudaSuccess ? SPH_OK : cuda_failed(e, "CUDA call", 0); }

#define SPH_CUDA(call)                                                     \
	do {                                                                   \
		cudaError_t e_ = (call);                                           \
		if (e_ != cudaSuccess) return cuda_failed(e_, #call, __LINE__);    \
	} while (0)

#define SPH_LAUNCHED(s)                                                     \
	do {                                                                    \
		(s)->launches++;                                                    \
		cudaError_t e_ = cudaGetLastError();                                \
		if (e_ != cudaSuccess) return cuda_failed(e_, "launch", __LINE__);  \
	} while (0)

template <typename T>
int dalloc(T **p, size_t count) {
	if (count == 0) count = 1;
	cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T));
	if (e != cudaSuccess) return SPH_ERR_CUDA;
	e = cudaMemset(*p, 0, count * sizeof(T));
	return cuda_status(e);
}

int blocks_for(size_t items, int threads) { return (int)std::max<size_t>(1, (items + threads - 1) / threads); }

// Step scalars of a scene, in FP32 exactly as the reference computes them.
StepParams step_params(const Scene &sc, float dt) {
	StepParams p{};
	p.h2 = sc.params.kernel_height * sc.params.kernel_height;
	p.invH = sc.params.inv_kernel_height;
	p.rho0 = sc.params.rest_density;
	p.k = sc.params.stiffness;
	p.kNear = sc.params.near_stiffness;
	p.sigma = sc.params.linear_viscosity;
	p.beta = sc.params.quadratic_viscosity;
	p.dt = dt;
	p.invDt = 1.0f / dt;
	p.dt2 = dt * dt;
	p.extX = sc.gravity.x + sc.external.x;
	p.extY = sc.gravity.y + sc.external.y;
	p.halfW = sc.dom.width * 0.5f;
	p.halfH = sc.dom.height * 0.5f;
	p.cellSize = sc.dom.cell_size;
	p.gx = sc.gx;
	p.gy = sc.gy;
	p.ncell = sc.ncell;
	p.radius = sc.dom.particle_radius;
	p.margin = sc.dom.collision_margin;
	p.nbodies = (int)sc.bodies.size();
	p.springs = sc.springs.enabled ? 1 : 0;
	p.springMax = sc.springs.max_per_particle;
	p.h = sc.params.kernel_height;
	p.springYield = sc.springs.yield_ratio;
	p.springDtAlpha = dt * sc.springs.plasticity;
	p.springK = sc.springs.stiffness;
	return p;
}

SimTables tables(sph_sim *s) {
	SimTables t = s->T;
	t.cellStart = s->cellStartA;
	t.cellCount = s->cellCountA;
	t.newStart = s->cellStartB;
	t.newCount = s->cellCountB;
	t.prof = s->prof;
	t.profStride = s->prof ? (int)s->doneDCap : 0;
	return t;
}

Totals totals(const sph_sim *s) {
	Totals tt;
	tt.n = (int)s->totalParticles();
	tt.ncell = s->ncellTotal;
	tt.nApp = s->nApp;
	tt.nscenes = (int)s->scenes.size();
	tt.refOrder = s->refOrder ? 1 : 0;
	tt.nViscRuns = s->refOrder ? (int)((s->scenes[0].n0 + kAppendixRun - 1) / kAppendixRun) : 0;
	return tt;
}

void drop_graphs(sph_sim *s) {
	for (int k = 0; k < 2; ++k) {
		if (s->graphs[k]) cudaGraphExecDestroy(s->graphs[k]);
		s->graphs[k] = nullptr;
		s->graphKernels[k] = 0;
	}
	s->steadySteps = 0;
}

// Body tables of all scenes to the device (scene after scene) when they changed.
int upload_bodies(sph_sim *s) {
	if (!s->bodiesDirty) return SPH_OK;
	std::vector<Body> all;
	for (Scene &sc : s->scenes) {
		sc.bodyBase = (int)all.size();
		all.insert(all.end(), sc.bodies.begin(), sc.bodies.end());
	}
	if (all.size() > s->bodyCap) return SPH_ERR_CAPACITY;
	// A pageable source: the call returns once the bytes are staged.
	if (!all.empty())
		SPH_CUDA(cudaMemcpyAsync(s->T.bodies, all.data(), all.size() * sizeof(Body), cudaMemcpyHostToDevice,
		                         s->stream));
	s->bodiesDirty = false;
	s->sceneTableDirty = true;
	return SPH_OK;
}

// Scene table (step scalars, offsets, counts) to the device when it changed.
int upload_scenes(sph_sim *s, float dt) {
	int rc = upload_bodies(s);
	if (rc) return rc;
	if (!s->sceneTableDirty && dt == s->tableDt) return SPH_OK;
	std::vector<SceneDev> host(s->scenes.size());
	for (size_t k = 0; k < s->scenes.size(); ++k) {
		const Scene &sc = s->scenes[k];
		SceneDev &d = host[k];
		std::memset(&d, 0, sizeof(d));
		d.p = step_params(sc, dt);
		d.cellBase = sc.cellBase;
		d.pBase = sc.pBase;
		d.n = (int)sc.nDev;
		d.n0 = (int)sc.n0;
		d.bodyBase = sc.bodyBase;
		d.nbSeed = sc.dom.max_neighbors;
	}
	SPH_CUDA(cudaMemcpyAsync(s->T.scenes, host.data(), host.size() * sizeof(SceneDev), cudaMemcpyHostToDevice,
	                         s->stream));
	drop_graphs(s);
	s->sceneTableDirty = false;
	s->tableDt = dt;
	return SPH_OK;
}

int ensure_stage(sph_sim *s, size_t count) {
	if (count <= s->stageCap) return SPH_OK;
	size_t cap = std::max<size_t>(count, 4096);
	if (s->stagePos) cudaFree(s->stagePos);
	if (s->stageForce) cudaFree(s->stageForce);
	if (s->hostPos) cudaFreeHost(s->hostPos);
	if (s->hostForce) cudaFreeHost(s->hostForce);
	s->stagePos = s->stageForce = s->hostPos = s->hostForce = nullptr;
	s->stageCap = 0;
	SPH_CUDA(cudaMalloc(&s->stagePos, cap * sizeof(float2)));
	SPH_CUDA(cudaMalloc(&s->stageForce, cap * sizeof(float2)));
	SPH_CUDA(cudaMallocHost(&s->hostPos, cap * sizeof(float2)));
	SPH_CUDA(cudaMallocHost(&s->hostForce, cap * sizeof(float2)));
	s->stageCap = cap;
	return SPH_OK;
}

// Pending AddParticle calls reach the device in order, before anything that
// reads or changes device state.
int flush_adds(sph_sim *s) {
	for (size_t k = 0; k < s->scenes.size(); ++k) {
		Scene &sc = s->scenes[k];
		const size_t count = sc.pendPos.size();
		if (count == 0) continue;
		int rc = ensure_stage(s, count);
		if (rc != SPH_OK) return rc;
		// The cell of an added particle needs the scene's grid, not dt.
		rc = upload_scenes(s, s->tableDt > 0.0f ? s->tableDt : 1.0f);
		if (rc != SPH_OK) return rc;
		SPH_CUDA(cudaStreamSynchronize(s->stream));  // host staging is reused
		std::memcpy(s->hostPos, sc.pendPos.data(), count * sizeof(float2));
		std::memcpy(s->hostForce, sc.pendForce.data(), count * sizeof(float2));
		SPH_CUDA(cudaMemcpyAsync(s->stagePos, s->hostPos, count * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
		SPH_CUDA(
		    cudaMemcpyAsync(s->stageForce, s->hostForce, count * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
		k_add<<<blocks_for(count, kElemThreads), kElemThreads, 0, s->stream>>>(
		    sc.pBase + (int)sc.nDev, (int)count, (int)k, (int)sc.nDev, s->stagePos, s->stageForce,
		    s->buf[s->cur].view(), tables(s));
		SPH_LAUNCHED(s);
		sc.nDev += count;
		sc.pendPos.clear();
		sc.pendForce.clear();
		s->sceneTableDirty = true;
	}
	return SPH_OK;
}

int push_particle(Scene &sc, float2 p, float2 f, size_t *index) {
	if (sc.n >= sc.cap) return SPH_ERR_CAPACITY;
	sc.pendPos.push_back(p);
	sc.pendForce.push_back(f);
	if (index) *index = sc.n;
	sc.n++;
	return SPH_OK;
}

// Vec2RandomDirection (vecmath.h:317-322): the reference's jitter source.
float2 random_direction() {
	float d = rand() / (float)RAND_MAX;
	float angle = d * ((float)M_PI * 2.0f);
	return make_float2(cosf(angle), sinf(angle));
}

float2 jitter(const Scene &sc) {
	float2 r = random_direction();
	r = make_float2(r.x * sc.dom.jitter_kernel_height, r.y * sc.dom.jitter_kernel_height);
	return make_float2(r.x * sc.dom.jitter_scale, r.y * sc.dom.jitter_scale);
}

// UpdateEmitter (demo4.cpp:257-284).
int update_emitter(Scene &sc, Emitter &e, float dt) {
	const float spacing = sc.params.particle_spacing;
	const float invDt = 1.0f / dt;
	if (!e.active) return SPH_OK;
	const float rate = 1.0f / e.rate;
	e.elapsed = dt + e.elapsed;
	e.totalElapsed = dt + e.totalElapsed;
	if (e.elapsed >= rate) {
		e.elapsed = 0;
		float2 accel = make_float2(e.direction.x * e.speed, e.direction.y * e.speed);
		accel = make_float2(accel.x * invDt, accel.y * invDt);
		const float2 dir = make_float2(-1.0f * e.direction.y, 1.0f * e.direction.x);  // Vec2Cross(1, d)
		const int count = (int)std::floor(e.radius / spacing);
		float2 offset = make_float2(dir.x * (float)count, dir.y * (float)count);
		offset = make_float2(offset.x * spacing, offset.y * spacing);
		offset = make_float2(offset.x * 0.5f, offset.y * 0.5f);
		for (int k = 0; k < count; ++k) {
			float2 p = make_float2(dir.x * (float)k, dir.y * (float)k);
			p = make_float2(p.x * spacing, p.y * spacing);
			float2 h = make_float2(dir.x * spacing, dir.y * spacing);
			h = make_float2(h.x * 0.5f, h.y * 0.5f);
			p = make_float2(h.x + p.x, h.y + p.y);
			const float2 base = make_float2(e.position.x - offset.x, e.position.y - offset.y);
			p = make_float2(base.x + p.x, base.y + p.y);
			const float2 j = jitter(sc);
			p = make_float2(j.x + p.x, j.y + p.y);
			int rc = push_particle(sc, p, accel, nullptr);
			if (rc != SPH_OK) return rc;
		}
	}
	if (e.totalElapsed >= e.duration) e.active = 0;
	return SPH_OK;
}

int check_device_errors(sph_sim *s) {
	uint32_t err = 0;
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	SPH_CUDA(cudaMemcpy(&err, s->T.error, sizeof(err), cudaMemcpyDeviceToHost));
	if (err) {
		uint32_t zero = 0;
		SPH_CUDA(cudaMemcpy(s->T.error, &zero, sizeof(zero), cudaMemcpyHostToDevice));
		SPH_CUDA(cudaMemcpy(s->T.abort, &zero, sizeof(zero), cudaMemcpyHostToDevice));
		if (err & kErrTimeout) return SPH_ERR_TIMEOUT;
		return SPH_ERR_DEVICE_OVERFLOW;
	}
	return SPH_OK;
}

// Appendix runs (particles added since the last update, kAppendixRun at a
// time) of every scene as delta-sweep tasks after the canonical ones,
// interleaved across scenes; in reference order, runs of the whole scene in
// AddParticle order are the only delta-sweep tasks.  A run waits for the earlier runs of its scene
// whose particles' new cells come within two cells of its own, so a scene's
// appendix is relaxed as in AddParticle order.
int upload_appendix_tasks(sph_sim *s) {
	const size_t S = s->scenes.size();
	std::vector<int> runs(S);
	int maxRuns = 0;
	for (size_t k = 0; k < S; ++k) {
		const Scene &sc = s->scenes[k];
		// In reference order the delta sweep runs over the whole scene.
		const size_t first = s->refOrder ? 0 : sc.n0;
		runs[k] = (int)((sc.nDev - first + kAppendixRun - 1) / kAppendixRun);
		maxRuns = std::max(maxRuns, runs[k]);
	}
	s->nApp = 0;
	if (maxRuns == 0) return SPH_OK;
	std::vector<int> scene, run;
	for (int r = 0; r < maxRuns; ++r) {
		for (size_t k = 0; k < S; ++k) {
			if (r >= runs[k]) continue;
			scene.push_back((int)k);
			run.push_back(r);
		}
	}
	if ((size_t)s->ncellTotal + scene.size() > s->doneDCap) return SPH_ERR_CAPACITY;
	s->nApp = (int)scene.size();
	const size_t bytes = scene.size() * sizeof(int);
	SPH_CUDA(cudaMemcpyAsync(s->T.appScene, scene.data(), bytes, cudaMemcpyHostToDevice, s->stream));
	SPH_CUDA(cudaMemcpyAsync(s->T.appRun, run.data(), bytes, cudaMemcpyHostToDevice, s->stream));
	return SPH_OK;
}

// Every launch, memset and stage event of one update, on the simulation's
// stream (also what a per-step graph captures).
int enqueue_step(sph_sim *s, bool capturing) {
	const Totals tt = totals(s);
	cudaStream_t st = s->stream;
	BufferSet &A = s->buf[s->cur];
	BufferSet &B = s->buf[1 - s->cur];
	SimTables T = tables(s);
	const int cellOrN = std::max(tt.n, tt.ncell);
	bool anyCanonical = false;
	for (const Scene &sc : s->scenes) anyCanonical = anyCanonical || sc.n0 > 0;
	// Under capture, stage events become event-record nodes of the graph.
	auto mark = [&](int k) {
		return capturing ? cudaEventRecordWithFlags(s->ev[k], st, cudaEventRecordExternal)
		                 : cudaEventRecord(s->ev[k], st);
	};

	SPH_CUDA(mark(kEvBegin));
	k_integrate<<<blocks_for(cellOrN, kElemThreads), kElemThreads, 0, st>>>(tt, A.view(), T);
	SPH_LAUNCHED(s);
	{
		// The sweeps' task list: occupied canonical cells in task order.
		const int ntiles = (tt.ncell + kScanTile - 1) / kScanTile;
		k_live_reduce<<<ntiles, kScanThreads, 0, st>>>(tt, T);
		SPH_LAUNCHED(s);
		k_live_tiles<<<1, kScanThreads, 0, st>>>(T, ntiles);
		SPH_LAUNCHED(s);
		k_live_apply<<<ntiles, kScanThreads, 0, st>>>(tt, T);
		SPH_LAUNCHED(s);
	}
	SPH_CUDA(mark(kEvIntegrate));

	if (tt.refOrder) {
		k_ref_order<<<blocks_for(tt.n, kElemThreads), kElemThreads, 0, st>>>(tt, A.view(), T);
		SPH_LAUNCHED(s);
	}
	if (anyCanonical && tt.refOrder) {
		SPH_CUDA(cudaMemsetAsync(s->doneV, 0, sizeof(uint32_t) * std::max(tt.nViscRuns, 1), st));
		SPH_CUDA(cudaMemsetAsync(T.taskCounter, 0, sizeof(int), st));
		SimTables v = T;
		v.done = s->doneV;
		k_visc_boxes<<<blocks_for((size_t)tt.nViscRuns * kWarp, kElemThreads), kElemThreads, 0, st>>>(tt, A.view(),
		                                                                                          v);
		SPH_LAUNCHED(s);
		k_viscosity_ref<<<s->viscRefBlocks, kViscRefWarps * kWarp, 0, st>>>(tt, A.view(), v);
		SPH_LAUNCHED(s);
	} else if (anyCanonical) {
		SPH_CUDA(cudaMemsetAsync(s->doneV, 0, sizeof(uint32_t) * s->ncellTotal, st));
		SPH_CUDA(cudaMemsetAsync(T.taskCounter, 0, sizeof(int), st));
		SimTables v = T;
		v.done = s->doneV;
		launch_viscosity(s->runViscLean != 0, s->runViscBlocks, st, tt, A.view(), v);
		SPH_LAUNCHED(s);
	}
	SPH_CUDA(mark(kEvVisc));

	k_predict<<<blocks_for(tt.n, kElemThreads), kElemThreads, 0, st>>>(tt, A.view(), T);
	SPH_LAUNCHED(s);
	SPH_CUDA(mark(kEvPredict));

	{
		const int ntiles = (tt.ncell + kScanTile - 1) / kScanTile;
		k_scan_reduce<<<ntiles, kScanThreads, 0, st>>>(tt, T);
		SPH_LAUNCHED(s);
		k_scan_tiles<<<1, kScanThreads, 0, st>>>(tt, T, ntiles);
		SPH_LAUNCHED(s);
		k_scan_apply<<<ntiles, kScanThreads, 0, st>>>(tt, T);
		SPH_LAUNCHED(s);
	}
	k_scatter<<<blocks_for(tt.n, kElemThreads), kElemThreads, 0, st>>>(tt, A.view(), T);
	SPH_LAUNCHED(s);
	k_grid_update<<<s->gridBlocks, kGridWarps * kWarp, 0, st>>>(tt, A.view(), B.view(), T);
	SPH_LAUNCHED(s);
	SPH_CUDA(mark(kEvGrid));

	bool anySprings = false;
	for (const Scene &sc : s->scenes) anySprings = anySprings || sc.springs.enabled;
	if (anySprings) {
		k_springs_select<<<s->springBlocks, kSpringWarps * kWarp, springs_smem_bytes(), st>>>(tt, A.view(),
		                                                                                      B.view(), T);
		SPH_LAUNCHED(s);
		k_springs_commit<<<blocks_for(tt.n, kElemThreads), kElemThreads, 0, st>>>(tt, B.view(), T);
		SPH_LAUNCHED(s);
		k_springs_apply<<<blocks_for(tt.n, kElemThreads), kElemThreads, 0, st>>>(tt, B.view(), T);
		SPH_LAUNCHED(s);
		SPH_CUDA(cudaMemcpyAsync(B.pos, T.springPos, sizeof(float2) * tt.n, cudaMemcpyDeviceToDevice, st));
	}
	SPH_CUDA(mark(kEvSprings));

	k_density<<<s->densBlocks, kDensWarps * kWarp, dens_smem_bytes(), st>>>(tt, B.view(), T);
	SPH_LAUNCHED(s);
	SPH_CUDA(mark(kEvDensity));

	if (tt.nApp > 0) {
		k_app_boxes<<<blocks_for((size_t)tt.nApp * kWarp, kElemThreads), kElemThreads, 0, st>>>(tt, T);
		SPH_LAUNCHED(s);
	}
	SPH_CUDA(cudaMemsetAsync(s->doneD, 0, sizeof(uint32_t) * (s->ncellTotal + s->nApp), st));
	SPH_CUDA(cudaMemsetAsync(T.taskCounter + 1, 0, sizeof(int), st));
	{
		SimTables d = T;
		d.done = s->doneD;
		launch_delta(s->runDeltaShape, s->runDeltaBlocks, st, tt, B.view(), d);
		SPH_LAUNCHED(s);
	}
	SPH_CUDA(mark(kEvDelta));

	k_collide<<<blocks_for(cellOrN, kCollideThreads), kCollideThreads, 0, st>>>(tt, A.view(), B.view(), T);
	SPH_LAUNCHED(s);
	SPH_CUDA(mark(kEvCollide));
	// This update's neighbourhood statistics, for the next updates' choice
	// of sweep shapes (read on the host without waiting).
	SPH_CUDA(cudaMemcpyAsync(s->hostStats, T.stats, sizeof(uint32_t) * 4 * s->scenes.size(), cudaMemcpyDeviceToHost, st));
	return SPH_OK;
}

// Viscosity pair lists longer than this send the lean viscosity shape's
// chains through several rounds; the wide shape stays staged.
constexpr uint32_t kDenseNeighbors = 440;

// The sweep shapes of the next update: the tuned ones, or in dense states
// (see sph_sim::adaptive) the wide viscosity shape and a delta shape whose
// stage holds the task regions: the 8-warp shape (4,096 entries) once a 3x3
// block of the fullest cell passes 0.65 of the tuned shape's stage, the
// 16-warp shape (12,288 entries) once a 5x5 region of it nears 4,096.  The statistics are those of the update
// before last at the latest: the host waits for its copy, so it never runs
// more than two updates ahead.  Changing shapes drops the update graphs.
void choose_shapes(sph_sim *s) {
	int vl = s->viscLean, vb = s->viscBlocks, ds = s->deltaShape, db = s->deltaBlocks;
	// A batch of many scenes keeps its tuned shapes: its sweeps are bound by
	// how many tasks run at once, not by one crowded scene's tasks.
	const bool adapt = s->adaptive && !s->batch && s->hostStats;
	if (adapt && s->statsEv[s->cur]) cudaEventSynchronize(s->statsEv[s->cur]);
	if (adapt) {
		uint32_t maxNb = 0, maxCell = 0;
		const volatile uint32_t *h = s->hostStats;
		for (size_t k = 0; k < s->scenes.size(); ++k) {
			const uint32_t nb = h[4 * k + 1], cell = h[4 * k + 3];
			maxNb = std::max(maxNb, nb);
			maxCell = std::max(maxCell, cell);
		}
		// Hysteresis: back to the tuned shape only well below the threshold.
		s->denseVisc = s->denseVisc ? maxNb * 5 > kDenseNeighbors * 4 : maxNb > kDenseNeighbors;
		const uint32_t cap = (uint32_t)delta_stage_capacity(ds);
		const uint32_t block = 9 * maxCell;   // a 3x3 block at the fullest cell's count
		const uint32_t spread = 25 * maxCell;  // a 5x5 region: a cell's particles spread over 3x3 new cells
		// Thresholds from measured crossovers on the collapsing 1M column:
		// the 8-warp shape wins from ~110 particles in the fullest cell (a
		// 3x3 block at 0.65 of the 1,536-entry stage), the 16-warp one from
		// ~160 (a 5x5 region near 4,096).
		s->denseDelta = s->denseDelta ? block * 2 > cap : block * 20 > cap * 13;
		s->crowdedDelta =
		    s->crowdedDelta ? spread * 5 > (uint32_t)kDeltaStageCap * 4 : spread * 20 > (uint32_t)kDeltaStageCap * 19;
		if (vl && s->denseVisc) {
			vl = 0;
			vb = s->denseViscBlocks;
		}
		if (cap < (uint32_t)kDeltaDenseStageCap && s->crowdedDelta) {
			ds = kDeltaDense;
			db = s->crowdedDeltaBlocks;
		} else if (cap < (uint32_t)kDeltaStageCap && s->denseDelta) {
			ds = kDeltaMid;
			db = s->denseDeltaBlocks;
		}
	}
	if (vl != s->runViscLean || vb != s->runViscBlocks || ds != s->runDeltaShape || db != s->runDeltaBlocks) {
		drop_graphs(s);
		s->runViscLean = vl;
		s->runViscBlocks = vb;
		s->runDeltaShape = ds;
		s->runDeltaBlocks = db;
	}
}

// Capture one update into an executable graph (nothing runs).
int capture_step(sph_sim *s, cudaGraphExec_t *out, uint64_t *kernels) {
	SPH_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
	const uint64_t before = s->launches;
	const int rc = enqueue_step(s, true);
	cudaGraph_t g = nullptr;
	const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
	*kernels = s->launches - before;
	s->launches = before;
	if (rc != SPH_OK || e != cudaSuccess) {
		if (g) cudaGraphDestroy(g);
		cudaGetLastError();
		return rc != SPH_OK ? rc : SPH_ERR_CUDA;
	}
	const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
	cudaGraphDestroy(g);
	return cuda_status(ei);
}

int run_step(sph_sim *s, float dt) {
	int rc = upload_scenes(s, dt);
	if (rc) return rc;
	rc = upload_appendix_tasks(s);
	if (rc) return rc;
	choose_shapes(s);
	// A graph is captured once the same update has run eagerly (scene table,
	// bodies and dt unchanged, no appendix), then replayed.
	const bool replay = s->useGraphs && s->nApp == 0 && s->steadySteps >= 1;
	if (replay) {
		cudaGraphExec_t &g = s->graphs[s->cur];
		if (!g) {
			rc = capture_step(s, &g, &s->graphKernels[s->cur]);
			if (rc) return rc;
		}
		SPH_CUDA(cudaGraphLaunch(g, s->stream));
		s->launches += s->graphKernels[s->cur];
	} else {
		rc = enqueue_step(s, false);
		if (rc) return rc;
	}
	SPH_CUDA(cudaEventRecord(s->statsEv[s->cur], s->stream));
	if (s->nApp == 0) s->steadySteps++;

	// The new cell arrays are the canonical ranges of the next step.
	s->cur = 1 - s->cur;
	std::swap(s->cellStartA, s->cellStartB);
	std::swap(s->cellCountA, s->cellCountB);
	for (Scene &sc : s->scenes) {
		if (sc.n0 != sc.nDev) s->sceneTableDirty = true;
		sc.n0 = sc.nDev;
	}
	s->nApp = 0;
	s->timed = true;
	return SPH_OK;
}

bool valid_geometry(const sph_domain &d) {
	if (!(d.cell_size > 0.0f) || !(d.width > 0.0f) || !(d.height > 0.0f)) return false;
	const int gx = (int)(d.width / d.cell_size), gy = (int)(d.height / d.cell_size);
	return gx > 0 && gy > 0 && (int64_t)gx * gy <= (1 << 26);
}

void init_scene(Scene &sc, const sph_domain &d, size_t cap) {
	sc.dom = d;
	sc.gx = (int)(d.width / d.cell_size);
	sc.gy = (int)(d.height / d.cell_size);
	sc.ncell = sc.gx * sc.gy;
	sc.cap = cap;
	sph_default_params(&sc.params);
}

std::vector<uint32_t> stats_seed(const sph_sim *s) {
	// SPHStatistics() (sph.h:143-149): both minimums start at the cell capacity.
	std::vector<uint32_t> seed(4 * s->scenes.size());
	for (size_t k = 0; k < s->scenes.size(); ++k) {
		seed[4 * k + 0] = s->scenes[k].dom.max_cell_particles;
		seed[4 * k + 1] = 0;
		seed[4 * k + 2] = s->scenes[k].dom.max_cell_particles;
		seed[4 * k + 3] = 0;
	}
	return seed;
}

// Device memory and tables for the scenes described in s->scenes.
int allocate(sph_sim *s) {
	int64_t ncell = 0, pBase = 0;
	for (Scene &sc : s->scenes) {
		sc.cellBase = (int)ncell;
		sc.pBase = (int)pBase;
		ncell += sc.ncell;
		pBase += (int64_t)sc.cap;
		if (ncell > (1 << 28) || pBase > (1 << 30)) return SPH_ERR_CAPACITY;
	}
	s->ncellTotal = (int)ncell;
	s->capTotal = (size_t)pBase;
	const size_t N = (size_t)pBase, C = (size_t)ncell, S = s->scenes.size();
	int rc = SPH_OK;
	if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return SPH_ERR_CUDA;
	for (int k = 0; k < kEvCount; ++k)
		if (cudaEventCreate(&s->ev[k]) != cudaSuccess) return SPH_ERR_CUDA;
	for (int k = 0; k < 2; ++k)
		if (cudaEventCreateWithFlags(&s->statsEv[k], cudaEventDisableTiming) != cudaSuccess) return SPH_ERR_CUDA;
	for (int b = 0; b < 2; ++b) {
		BufferSet &B = s->buf[b];
		if ((rc = dalloc(&B.pos, N)) || (rc = dalloc(&B.prev, N)) || (rc = dalloc(&B.vel, N)) ||
		    (rc = dalloc(&B.acc, N)) || (rc = dalloc(&B.dens, N)) || (rc = dalloc(&B.press, N)) ||
		    (rc = dalloc(&B.id, N)) || (rc = dalloc(&B.cellOf, N)))
			return rc;
	}
	size_t bodies = 0;
	for (const Scene &sc : s->scenes) bodies += sc.bodies.size();
	s->bodyCap = s->batch ? std::max<size_t>(bodies, 1) : (size_t)kMaxBodies;
	SimTables &T = s->T;
	if ((rc = dalloc(&s->cellStartA, C)) || (rc = dalloc(&s->cellCountA, C)) || (rc = dalloc(&s->cellStartB, C)) ||
	    (rc = dalloc(&s->cellCountB, C)) || (rc = dalloc(&T.taskOfCell, C)) || (rc = dalloc(&T.taskCell, C)) ||
	    (rc = dalloc(&T.numberOrder, C)) || (rc = dalloc(&T.sceneOfCell, C)) || (rc = dalloc(&T.sceneOf, N)) ||
	    (rc = dalloc(&T.scenes, S)) || (rc = dalloc(&T.appCount, C)) || (rc = dalloc(&T.appStart, C)) ||
	    (rc = dalloc(&T.appIdx, N)) || (rc = dalloc(&T.appCursor, C)) || (rc = dalloc(&T.newCell, N)) ||
	    (rc = dalloc(&T.enterCount, C)) || (rc = dalloc(&T.leaveCount, C)) || (rc = dalloc(&T.enterOffset, C)) ||
	    (rc = dalloc(&T.enterCursor, C)) || (rc = dalloc(&T.enterList, N)) || (rc = dalloc(&T.moverCount, 2)) ||
	    (rc = dalloc(&T.bbox, 4 * C)) || (rc = dalloc(&T.newIdx, N)) || (rc = dalloc(&T.newLabel, N)) ||
	    (rc = dalloc(&T.taskCounter, 2)) || (rc = dalloc(&T.stats, 4 * S)) || (rc = dalloc(&T.error, 1)) ||
	    (rc = dalloc(&T.scanTiles, 3 * ((C + kScanTile - 1) / kScanTile))) ||
	    (rc = dalloc(&T.liveTask, C)) || (rc = dalloc(&T.liveTiles, (C + kScanTile - 1) / kScanTile)) ||
	    (rc = dalloc(&T.nLive, 1)) ||
	    (rc = dalloc(&T.abort, 1)) || (rc = dalloc(&T.bodies, s->bodyCap)))
		return rc;
	// Appendix runs: at most one partial run per scene beyond N / kAppendixRun.
	const size_t appCap = (N + kAppendixRun - 1) / kAppendixRun + S + 1;
	s->doneDCap = C + appCap;
	// Viscosity done flags: one per cell, or per run in reference order.
	if ((rc = dalloc(&s->doneD, s->doneDCap)) || (rc = dalloc(&T.appScene, appCap)) ||
	    (rc = dalloc(&T.appRun, appCap)) || (rc = dalloc(&T.appBox, 4 * appCap)) ||
	    (rc = dalloc(&s->doneV, std::max(C, appCap))) || (rc = dalloc(&T.refOrd, N)) ||
	    (rc = dalloc(&T.viscBox, 4 * appCap)) || (rc = dalloc(&s->check, 4)))
		return rc;
	T.moverList = nullptr;
	T.waitLimitNs = kDefaultWaitLimitNs;
	T.hold[0] = T.hold[1] = -1;

	// Per scene: colour-major cell rank -- colour (y%3, x%3), then sub-colour
	// ((y/3)%2, (x/3)%2), then row-major.  Cells of one colour are >= 3
	// apart; within a colour, the sub-colour order keeps conflicts between
	// cells that particles move across short.  Particles are numbered scene
	// after scene in that order.  The sweep tasks interleave the scenes by
	// relative rank, so that every scene's ordered sweep advances at once.
	std::vector<int> numberOrder, sceneOfCell(C), taskCell(C), taskOfCell(C);
	std::vector<std::pair<double, int>> interleave;
	numberOrder.reserve(C);
	interleave.reserve(C);
	for (size_t k = 0; k < S; ++k) {
		const Scene &sc = s->scenes[k];
		std::vector<int> order(sc.ncell);
		for (int c = 0; c < sc.ncell; ++c) order[c] = c;
		const int gx = sc.gx;
		auto key = [gx](int c) {
			const int x = c % gx, y = c / gx;
			return (int64_t)(((y % 3) * 3 + (x % 3)) * 4 + ((y / 3) % 2) * 2 + ((x / 3) % 2)) * (int64_t)(1 << 26) + c;
		};
		std::sort(order.begin(), order.end(), [&](int a, int b) { return key(a) < key(b); });
		for (int r = 0; r < sc.ncell; ++r) {
			const int g = sc.cellBase + order[r];
			numberOrder.push_back(g);
			sceneOfCell[g] = (int)k;
			interleave.push_back({(double)r / (double)sc.ncell, g});
		}
	}
	// Stable: equal fractions keep scene order; within a scene the rank
	// order is kept because the fraction grows with the rank.
	std::stable_sort(interleave.begin(), interleave.end(),
	                 [](const std::pair<double, int> &a, const std::pair<double, int> &b) { return a.first < b.first; });
	for (size_t t = 0; t < C; ++t) {
		taskCell[t] = interleave[t].second;
		taskOfCell[interleave[t].second] = (int)t;
	}
	std::vector<int> sceneOf(std::max<size_t>(N, 1), 0);
	for (size_t k = 0; k < S; ++k)
		for (size_t j = 0; j < s->scenes[k].cap; ++j) sceneOf[s->scenes[k].pBase + j] = (int)k;
	const std::vector<uint32_t> seed = stats_seed(s);
	if (cudaMemcpy(T.numberOrder, numberOrder.data(), C * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(T.sceneOfCell, sceneOfCell.data(), C * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(T.taskCell, taskCell.data(), C * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(T.taskOfCell, taskOfCell.data(), C * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(T.sceneOf, sceneOf.data(), sceneOf.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(T.stats, seed.data(), seed.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
		return SPH_ERR_CUDA;
	if (s->hostStats) cudaFreeHost(s->hostStats);
	s->hostStats = nullptr;
	if (cudaMallocHost(&s->hostStats, sizeof(uint32_t) * 4 * S) != cudaSuccess) return SPH_ERR_CAPACITY;
	std::memcpy(s->hostStats, seed.data(), seed.size() * 4);

	cudaDeviceProp prop;
	if (cudaGetDeviceProperties(&prop, s->device) != cudaSuccess) return SPH_ERR_CUDA;
	s->numSMs = prop.multiProcessorCount;
	if (sweep_attributes() != cudaSuccess ||
	    cudaFuncSetAttribute(k_density, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dens_smem_bytes()) !=
	        cudaSuccess ||
	    cudaFuncSetAttribute(k_springs_select, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                         (int)springs_smem_bytes()) != cudaSuccess)
		return SPH_ERR_CUDA;
	int occV = 0, occD = 0;
	if (sweep_occupancy(false, kDeltaWide, &occV, &occD) != cudaSuccess || occV < 1 || occD < 1) return SPH_ERR_CUDA;
	s->viscBlocks = occV * s->numSMs;
	s->deltaBlocks = occD * s->numSMs;
	s->denseViscBlocks = s->viscBlocks;  // the wide viscosity shape
	{
		int v2 = 0, d2 = 0;
		if (sweep_occupancy(false, kDeltaMid, &v2, &d2) != cudaSuccess || d2 < 1) return SPH_ERR_CUDA;
		s->denseDeltaBlocks = d2 * s->numSMs;
		if (sweep_occupancy(false, kDeltaDense, &v2, &d2) != cudaSuccess || d2 < 1) return SPH_ERR_CUDA;
		s->crowdedDeltaBlocks = d2 * s->numSMs;
	}
	s->densBlocks = std::max(1, std::min(blocks_for(C, kDensWarps), 64 * s->numSMs));
	s->springBlocks = std::max(1, std::min(blocks_for(C, kSpringWarps), 64 * s->numSMs));
	s->gridBlocks = std::max(1, std::min(blocks_for(C, kGridWarps), 64 * s->numSMs));
	s->viscRefBlocks = 8 * s->numSMs;
	return SPH_OK;
}

int create_common(sph_sim *s, int device) {
	int devices = 0;
	if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) return SPH_ERR_NO_DEVICE;
	if (device < 0 || device >= devices) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(device));
	s->device = device;
	return allocate(s);
}

// Scene 0 of a single-scene simulation: what the reference interface mutates.
Scene *single(sph_sim *s) { return (s && !s->batch) ? &s->scenes[0] : nullptr; }
int not_single(sph_sim *s) { return s ? SPH_ERR_NOT_SUPPORTED : SPH_ERR_INVALID_ARGUMENT; }

int push_body(sph_sim *s, const Body &b) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	if (sc->bodies.size() >= (size_t)kMaxBodies) return SPH_ERR_CAPACITY;
	sc->bodies.push_back(b);
	s->bodiesDirty = true;
	return SPH_OK;
}

Body plane_body(sph_vec2 normal, float distance) {
	Body b{};
	b.type = kBodyPlane;
	b.ax = normal.x;
	b.ay = normal.y;
	b.r = distance;
	return b;
}

Body circle_body(sph_vec2 pos, float radius) {
	Body b{};
	b.type = kBodyCircle;
	b.ax = pos.x;
	b.ay = pos.y;
	b.r = radius;
	return b;
}

Body segment_body(sph_vec2 a, sph_vec2 bb) {
	Body b{};
	b.type = kBodySegment;
	b.ax = a.x;
	b.ay = a.y;
	b.bx = bb.x;
	b.by = bb.y;
	return b;
}

Body polygon_body(size_t count, const sph_vec2 *verts) {
	Body b{};
	b.type = kBodyPolygon;
	b.vertexCount = (int)count;
	for (size_t k = 0; k < count; ++k) {
		b.verts[2 * k] = verts[k].x;
		b.verts[2 * k + 1] = verts[k].y;
	}
	return b;
}

int body_from_desc(const sph_body_desc &d, Body *out) {
	switch (d.type) {
		case SPH_BODY_PLANE: *out = plane_body(d.a, d.value); return SPH_OK;
		case SPH_BODY_CIRCLE: *out = circle_body(d.a, d.value); return SPH_OK;
		case SPH_BODY_SEGMENT: *out = segment_body(d.a, d.b); return SPH_OK;
		case SPH_BODY_POLYGON:
			if (d.vertex_count > (size_t)kMaxPoly) return SPH_ERR_CAPACITY;
			*out = polygon_body(d.vertex_count, d.verts);
			return SPH_OK;
		default: return SPH_ERR_INVALID_ARGUMENT;
	}
}

int read_scene(sph_sim *s, size_t scene, size_t count, sph_vec2 *pos, sph_vec2 *prev, sph_vec2 *vel, sph_vec2 *acc,
               sph_vec2 *dens, sph_vec2 *press) {
	if (!s || scene >= s->scenes.size()) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	const Scene &sc = s->scenes[scene];
	if (count > sc.n) return SPH_ERR_INVALID_ARGUMENT;
	const int n = (int)sc.n;
	BufferSet &A = s->buf[s->cur];
	BufferSet &Z = s->buf[1 - s->cur];  // free between updates: scratch
	struct Item {
		float2 *src, *scratch;
		sph_vec2 *dst;
	} items[] = {{A.pos, Z.pos, pos}, {A.prev, Z.prev, prev}, {A.vel, Z.vel, vel},
	             {A.acc, Z.acc, acc}, {A.dens, Z.dens, dens}, {A.press, Z.press, press}};
	for (const Item &it : items) {
		if (!it.dst || count == 0) continue;
		float2 *dst = it.scratch + sc.pBase;
		k_gather_by_id<<<blocks_for(n, kElemThreads), kElemThreads, 0, s->stream>>>(sc.pBase, n, A.id, it.src, dst);
		SPH_LAUNCHED(s);
		SPH_CUDA(cudaMemcpyAsync(it.dst, dst, count * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
	}
	return check_device_errors(s);
}

int scene_info(sph_sim *s, size_t scene, size_t *count, size_t *canonical, int *gx, int *gy) {
	if (!s || scene >= s->scenes.size()) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	const Scene &sc = s->scenes[scene];
	if (count) *count = sc.n;
	if (canonical) *canonical = sc.n0;
	if (gx) *gx = sc.gx;
	if (gy) *gy = sc.gy;
	return SPH_OK;
}

// The state of one scene in scene-local numbers and cells.
int dump_scene(sph_sim *s, size_t scene, const sph_state_view *v) {
	if (!s || !v || scene >= s->scenes.size()) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	const Scene &sc = s->scenes[scene];
	if (v->count != sc.n) return SPH_ERR_INVALID_ARGUMENT;
	const size_t n = sc.n, p0 = (size_t)sc.pBase, c0 = (size_t)sc.cellBase;
	BufferSet &A = s->buf[s->cur];
	cudaStream_t st = s->stream;
	auto d2h = [&](void *dst, const void *src, size_t bytes) -> int {
		if (!dst || bytes == 0) return SPH_OK;
		return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
	};
	if ((rc = d2h(v->pos, A.pos + p0, n * 8)) || (rc = d2h(v->prev, A.prev + p0, n * 8)) ||
	    (rc = d2h(v->vel, A.vel + p0, n * 8)) || (rc = d2h(v->acc, A.acc + p0, n * 8)) ||
	    (rc = d2h(v->dens, A.dens + p0, n * 8)) || (rc = d2h(v->press, A.press + p0, n * 8)) ||
	    (rc = d2h(v->id, A.id + p0, n * 4)) || (rc = d2h(v->cell, A.cellOf + p0, n * 4)) ||
	    (rc = d2h(v->cell_start, s->cellStartA + c0, sc.ncell * 4)) ||
	    (rc = d2h(v->cell_count, s->cellCountA + c0, sc.ncell * 4)))
		return rc;
	rc = check_device_errors(s);
	if (rc) return rc;
	if (v->cell && c0 != 0)
		for (size_t k = 0; k < n; ++k) v->cell[k] -= (int32_t)c0;
	if (v->cell_start && p0 != 0)
		for (int c = 0; c < sc.ncell; ++c) v->cell_start[c] -= (int32_t)p0;
	return SPH_OK;
}

// ---- Learned frames -------------------------------------------------------

int ensure_learned(sph_sim *s) {
	if (s->lz0) return SPH_OK;
	const size_t N = (size_t)round_up128((int)s->capTotal), C = (size_t)s->ncellTotal;
	int rc;
	BufferSet &B = s->snap;
	if ((rc = dalloc(&B.pos, N)) || (rc = dalloc(&B.prev, N)) || (rc = dalloc(&B.vel, N)) ||
	    (rc = dalloc(&B.acc, N)) || (rc = dalloc(&B.dens, N)) || (rc = dalloc(&B.press, N)) ||
	    (rc = dalloc(&B.id, N)) || (rc = dalloc(&B.cellOf, N)) || (rc = dalloc(&s->snapCellStart, C)) ||
	    (rc = dalloc(&s->snapCellCount, C)) || (rc = dalloc(&s->lz0, N)) || (rc = dalloc(&s->lu, N)) ||
	    (rc = dalloc(&s->lbyId, N)) || (rc = dalloc(&s->ldens, N)) || (rc = dalloc(&s->lerr, kErrBlocks + 1)) ||
	    (rc = dalloc(&s->lstats, 4)))
		return rc;
	return SPH_OK;
}

// Copy the canonical state (particle arrays and cell ranges) to or from the
// snapshot.
int copy_state(sph_sim *s, bool save) {
	BufferSet &A = s->buf[s->cur];
	BufferSet &Z = s->snap;
	const size_t n = s->totalParticles(), C = (size_t)s->ncellTotal;
	cudaStream_t st = s->stream;
	auto cp = [&](void *live, void *snap, size_t bytes) {
		return cudaMemcpyAsync(save ? snap : live, save ? live : snap, bytes, cudaMemcpyDeviceToDevice, st);
	};
	const size_t f2 = n * sizeof(float2), i4 = n * sizeof(int);
	if (n) {
		SPH_CUDA(cp(A.pos, Z.pos, f2));
		SPH_CUDA(cp(A.prev, Z.prev, f2));
		SPH_CUDA(cp(A.vel, Z.vel, f2));
		SPH_CUDA(cp(A.acc, Z.acc, f2));
		SPH_CUDA(cp(A.dens, Z.dens, f2));
		SPH_CUDA(cp(A.press, Z.press, f2));
		SPH_CUDA(cp(A.id, Z.id, i4));
		SPH_CUDA(cp(A.cellOf, Z.cellOf, i4));
	}
	SPH_CUDA(cp(s->cellStartA, s->snapCellStart, C * sizeof(int)));
	SPH_CUDA(cp(s->cellCountA, s->snapCellCount, C * sizeof(int)));
	return SPH_OK;
}

// Mean |rho - rho0| / rho0 of the canonical state's final positions (density
// from the cell ranges, as the step computes it), on scratch arrays.
// Mean |rho - rho0| / rho0 of the current positions (over the current cell
// arrays) and, in *maxNb, the longest neighbour list.
int density_error(sph_sim *s, float *out, uint32_t *maxNb = nullptr) {
	const Scene &sc = s->scenes[0];
	int rc = upload_scenes(s, s->tableDt > 0.0f ? s->tableDt : 1.0f);
	if (rc) return rc;
	const uint32_t seed[4] = {0xffffffffu, 0u, 0xffffffffu, 0u};
	SPH_CUDA(cudaMemcpyAsync(s->lstats, seed, sizeof(seed), cudaMemcpyHostToDevice, s->stream));
	const Totals tt = totals(s);
	SimTables T = tables(s);
	T.newStart = s->cellStartA;
	T.newCount = s->cellCountA;
	T.stats = s->lstats;
	Particles Q = s->buf[s->cur].view();
	Q.dens = s->ldens;
	Q.press = s->lbyId;
	k_density<<<s->densBlocks, kDensWarps * kWarp, dens_smem_bytes(), s->stream>>>(tt, Q, T);
	SPH_LAUNCHED(s);
	const int blocks = std::min(blocks_for(tt.n, kErrThreads), kErrBlocks);
	k_density_error<<<blocks, kErrThreads, 0, s->stream>>>(tt.n, s->ldens, sc.params.rest_density, s->lerr);
	SPH_LAUNCHED(s);
	k_density_error_total<<<1, kErrBlocks, 0, s->stream>>>(blocks, s->lerr, s->lerr + kErrBlocks);
	SPH_LAUNCHED(s);
	double sum = 0.0;
	uint32_t st[4] = {0u, 0u, 0u, 0u};
	SPH_CUDA(cudaMemcpyAsync(&sum, s->lerr + kErrBlocks, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
	SPH_CUDA(cudaMemcpyAsync(st, s->lstats, sizeof(st), cudaMemcpyDeviceToHost, s->stream));
	rc = check_device_errors(s);
	if (rc) return rc;
	*out = tt.n > 0 ? (float)(sum / ((double)tt.n * (double)sc.params.rest_density)) : 0.0f;
	if (maxNb) *maxNb = st[1];
	return SPH_OK;
}

int learned_checks(sph_sim *s, sph_mpnn *m, float dt, int substeps) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	if (!m || !(dt > 0.0f) || substeps < 1) return SPH_ERR_INVALID_ARGUMENT;
	if (sc->springs.enabled) return SPH_ERR_NOT_SUPPORTED;
	if (mpnn_device(m) != s->device) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(s->device));
	int rc = flush_adds(s);
	if (rc) return rc;
	if ((size_t)round_up128((int)sc->n) > mpnn_capacity(m)) return SPH_ERR_CAPACITY;
	return ensure_learned(s);
}

int plain_frame(sph_sim *s, float dt, int substeps) {
	for (int k = 0; k < substeps; ++k) {
		int rc = run_step(s, dt / (float)substeps);
		if (rc) return rc;
	}
	return SPH_OK;
}

// The network's graph on the canonical state after an update: positions,
// z0 = v dt / h (written to s->lz0 by the caller) and the cell ranges.
MpnnGraph learned_graph(sph_sim *s, const Scene &sc) {
	MpnnGraph g;
	g.pos = s->buf[s->cur].pos;
	g.z0 = s->lz0;
	g.cellStart = s->cellStartA;
	g.cellCount = s->cellCountA;
	g.n = (int)sc.n;
	g.gx = sc.gx;
	g.gy = sc.gy;
	g.h = sc.params.kernel_height;
	g.invH = sc.params.inv_kernel_height;
	return g;
}

int learned_z0(sph_sim *s, const Scene &sc) {
	const int n = (int)sc.n, np = round_up128(n);
	const BufferSet &A = s->buf[s->cur];
	k_learned_z0<<<blocks_for(np, kElemThreads), kElemThreads, 0, s->stream>>>(n, np, A.pos, A.prev,
	                                                                            sc.params.inv_kernel_height, s->lz0);
	SPH_LAUNCHED(s);
	return SPH_OK;
}

}  // namespace

extern "C" {

int sph_learned_frame(sph_sim *s, sph_mpnn *m, float dt, int substeps, float bound, int *used_learned,
                      float *density_err) {
	int rc = learned_checks(s, m, dt, substeps);
	if (rc) return rc;
	Scene &sc = s->scenes[0];
	int used = 0;
	float err = 0.0f;
	if (sc.n == 0) {
		rc = SPH_OK;
	} else if (sc.n0 != sc.nDev) {
		// Particles added since the last update: the frame runs plainly.
		rc = plain_frame(s, dt, substeps);
		if (!rc) rc = density_error(s, &err);
	} else {
		// One plain update over the whole frame, corrected by the network
		// towards the `substeps` updates it stands in for.  A capacity
		// overflow anywhere on this path (the long plain update, or the
		// corrected positions) rejects the learned frame: the plain frame
		// takes over from the snapshot taken before it.
		rc = copy_state(s, true);
		if (!rc) rc = run_step(s, dt);
		float err1 = 0.0f;
		if (!rc) rc = density_error(s, &err1);
		bool reject = false;
		if (rc == SPH_ERR_DEVICE_OVERFLOW) {
			reject = true;
			rc = SPH_OK;
		}
		if (rc) return rc;
		if (!reject) {
			rc = learned_z0(s, sc);
			if (!rc) rc = mpnn_forward_dev(m, learned_graph(s, sc), s->lu, s->stream);
			if (rc) return rc;
			const Totals tt = totals(s);
			k_learned_finish<<<blocks_for(tt.n, kCollideThreads), kCollideThreads, 0, s->stream>>>(
			    tt, s->buf[s->cur].view(), s->lu, tables(s));
			SPH_LAUNCHED(s);
			uint32_t maxNb = 0;
			rc = density_error(s, &err, &maxNb);
			if (rc == SPH_ERR_DEVICE_OVERFLOW) {
				reject = true;
				rc = SPH_OK;
			}
			if (rc) return rc;
			// Local crowding does not show in the mean deviation: a frame
			// whose densest neighbourhood lists more than kLearnedCrowding of
			// the neighbour capacity is rejected too, so the plain method
			// relaxes crowding before it nears the capacity.
			const uint32_t cap = std::min<uint32_t>(sc.dom.max_neighbors, (uint32_t)kStageCap);
			if ((double)maxNb > kLearnedCrowding * (double)cap) reject = true;
		}
		// The judge: the correction stands if it leaves the mean density
		// deviation of the plain update it corrects at most `bound` (a
		// fraction of the rest density) higher.
		if (!reject && std::isfinite(err) && err <= err1 + bound) {
			used = 1;
		} else {
			rc = copy_state(s, false);
			if (!rc) rc = plain_frame(s, dt, substeps);
			if (!rc) rc = density_error(s, &err);
			if (rc) return rc;
		}
	}
	if (used_learned) *used_learned = used;
	if (density_err) *density_err = err;
	return rc ? rc : check_device_errors(s);
}

int sph_mpnn_capture(sph_sim *s, sph_mpnn *m, float dt, int substeps) {
	int rc = learned_checks(s, m, dt, substeps);
	if (rc) return rc;
	Scene &sc = s->scenes[0];
	if (sc.n == 0 || sc.n0 != sc.nDev) return SPH_ERR_NOT_SUPPORTED;  // needs a canonical state: update first
	const int n = (int)sc.n;
	// Inputs: the state after one plain update over the whole frame.
	rc = copy_state(s, true);
	if (!rc) rc = run_step(s, dt);
	if (!rc) rc = learned_z0(s, sc);
	if (rc) return rc;
	float2 *x1 = nullptr, *target = nullptr;
	int *ids = nullptr;
	rc = mpnn_add_sample(m, learned_graph(s, sc), s->stream, &x1, &target, &ids);
	if (rc) return rc;
	SPH_CUDA(cudaMemcpyAsync(ids, s->buf[s->cur].id, sizeof(int) * n, cudaMemcpyDeviceToDevice, s->stream));
	// Target: where `substeps` plain updates of dt / substeps take each
	// particle, relative to x1, in units of h.
	rc = copy_state(s, false);
	if (!rc) rc = plain_frame(s, dt, substeps);
	if (rc) return rc;
	const BufferSet &F = s->buf[s->cur];
	k_scatter_by_id<<<blocks_for(n, kElemThreads), kElemThreads, 0, s->stream>>>(n, F.pos, F.id, s->lbyId);
	SPH_LAUNCHED(s);
	k_learned_target<<<blocks_for(n, kElemThreads), kElemThreads, 0, s->stream>>>(
	    n, s->lbyId, ids, x1, sc.params.inv_kernel_height, target);
	SPH_LAUNCHED(s);
	return check_device_errors(s);
}

}  // extern "C"

extern "C" {

const char *sph_last_error(void) { return g_last_error; }

const char *sph_status_string(int status) {
	switch (status) {
		case SPH_OK: return "ok";
		case SPH_ERR_INVALID_ARGUMENT: return "invalid argument";
		case SPH_ERR_CAPACITY: return "capacity exceeded";
		case SPH_ERR_CUDA: return "CUDA runtime error";
		case SPH_ERR_DEVICE_OVERFLOW: return "device-side capacity overflow";
		case SPH_ERR_TIMEOUT: return "device-side wait timed out";
		case SPH_ERR_NOT_SUPPORTED: return "not supported";
		case SPH_ERR_NO_DEVICE: return "no CUDA device";
		default: return "unknown status";
	}
}

int sph_reference_domain(sph_domain *d) {
	if (!d) return SPH_ERR_INVALID_ARGUMENT;
	// sph.h:18-72 (kSPHBoundaryHeight = width / (16/9); cell = 6 * 0.05).
	d->width = 10.0f;
	d->height = 10.0f / (16.0f / 9.0f);
	d->cell_size = 6.0f * 0.05f;
	d->max_particles = 10000;
	d->max_cell_particles = 500;
	d->max_neighbors = 1000;
	d->particle_radius = 0.05f;
	d->collision_margin = 0.005f * 2.0f;
	d->jitter_kernel_height = 6.0f * 0.05f;
	d->jitter_scale = 0.01f;
	return SPH_OK;
}

int sph_default_params(sph_params *p) {
	if (!p) return SPH_ERR_INVALID_ARGUMENT;
	// SPHParameters() (sph.h:88-98).
	const float h = 6.0f * 0.05f;
	p->kernel_height = h;
	p->cell_size = h;
	p->particle_spacing = h * 0.5f;
	p->inv_kernel_height = 1.0f / h;
	p->rest_density = 20.0f;
	p->stiffness = 0.6f;
	p->near_stiffness = 0.6f * 10.0f;
	p->linear_viscosity = 0.5f;
	p->quadratic_viscosity = 0.3f;
	return SPH_OK;
}

int sph_create(const sph_domain *domain, int device, sph_sim **out) {
	if (!domain || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	if (!valid_geometry(*domain) || domain->max_particles == 0 || domain->max_particles > (1u << 30))
		return SPH_ERR_INVALID_ARGUMENT;
	sph_sim *s = new (std::nothrow) sph_sim();
	if (!s) return SPH_ERR_CAPACITY;
	s->scenes.resize(1);
	init_scene(s->scenes[0], *domain, domain->max_particles);
	int rc = create_common(s, device);
	if (rc == SPH_OK) rc = cuda_status(cudaStreamSynchronize(s->stream));
	if (rc != SPH_OK) {
		sph_destroy(s);
		return rc;
	}
	*out = s;
	return SPH_OK;
}

int sph_batch_create(const sph_scene_desc *descs, size_t scene_count, int device, sph_sim **out) {
	if (!descs || !out || scene_count == 0) return SPH_ERR_INVALID_ARGUMENT;
	*out = nullptr;
	for (size_t k = 0; k < scene_count; ++k) {
		const sph_scene_desc &d = descs[k];
		if (!valid_geometry(d.domain) || (d.particle_count > 0 && !d.positions) || (d.body_count > 0 && !d.bodies) ||
		    d.particle_count > (size_t)(1u << 30))
			return SPH_ERR_INVALID_ARGUMENT;
	}
	sph_sim *s = new (std::nothrow) sph_sim();
	if (!s) return SPH_ERR_CAPACITY;
	s->batch = true;
	s->scenes.resize(scene_count);
	int rc = SPH_OK;
	for (size_t k = 0; rc == SPH_OK && k < scene_count; ++k) {
		const sph_scene_desc &d = descs[k];
		Scene &sc = s->scenes[k];
		init_scene(sc, d.domain, d.particle_count);
		sc.params = d.params;
		sc.gravity = d.gravity;
		for (size_t b = 0; rc == SPH_OK && b < d.body_count; ++b) {
			Body body;
			rc = body_from_desc(d.bodies[b], &body);
			if (rc == SPH_OK && sc.bodies.size() >= (size_t)kMaxBodies) rc = SPH_ERR_CAPACITY;
			if (rc == SPH_OK) sc.bodies.push_back(body);
		}
		for (size_t j = 0; rc == SPH_OK && j < d.particle_count; ++j) {
			const float2 f = d.forces ? make_float2(d.forces[j].x, d.forces[j].y) : make_float2(0.0f, 0.0f);
			push_particle(sc, make_float2(d.positions[j].x, d.positions[j].y), f, nullptr);
		}
	}
	if (rc == SPH_OK) rc = create_common(s, device);
	if (rc == SPH_OK) rc = flush_adds(s);
	if (rc == SPH_OK) rc = check_device_errors(s);
	if (rc != SPH_OK) {
		sph_destroy(s);
		return rc;
	}
	*out = s;
	return SPH_OK;
}

int sph_batch_scene_count(sph_sim *s, size_t *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->scenes.size();
	return SPH_OK;
}

int sph_destroy(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	cudaSetDevice(s->device);
	if (s->stream) cudaStreamSynchronize(s->stream);
	drop_graphs(s);
	for (int b = 0; b < 2; ++b) {
		BufferSet &B = s->buf[b];
		void *ptrs[] = {B.pos, B.prev, B.vel, B.acc, B.dens, B.press, B.id, B.cellOf, B.springN, B.springP, B.springL};
		for (void *p : ptrs)
			if (p) cudaFree(p);
	}
	SimTables &T = s->T;
	void *ptrs[] = {s->cellStartA, s->cellCountA, s->cellStartB, s->cellCountB, T.taskOfCell,  T.taskCell,
	                T.numberOrder, T.sceneOfCell, T.sceneOf,     T.scenes,      T.appScene,    T.appRun,
	                T.appBox,      T.appCount,    T.appStart,    T.appIdx,      T.appCursor,   T.newCell,
	                T.enterCount,  T.leaveCount,  T.enterOffset, T.enterCursor, T.enterList,   T.moverCount,
	                T.bbox,        T.newIdx,      T.newLabel,    T.taskCounter, T.stats,       T.error,
	                T.scanTiles,   T.liveTask,    T.liveTiles,   T.nLive,
	                T.abort,       T.bodies,      s->doneV,      s->doneD,      s->stagePos,   s->stageForce,
	                s->prof,       T.accN,        T.accP,        T.springPos,   T.springTotal,
	                s->snap.pos,   s->snap.prev,  s->snap.vel,   s->snap.acc,   s->snap.dens,  s->snap.press,
	                s->snap.id,    s->snap.cellOf, s->snapCellStart, s->snapCellCount, s->lz0, s->lu,
	                s->lbyId,      s->ldens,      s->lerr,       s->lstats,     s->colorBuf,   s->imgKeys,
	                s->imgRgba,    T.refOrd,      T.viscBox,     s->check};
	for (void *p : ptrs)
		if (p) cudaFree(p);
	if (s->hostStats) cudaFreeHost(s->hostStats);
	if (s->hostPos) cudaFreeHost(s->hostPos);
	if (s->hostForce) cudaFreeHost(s->hostForce);
	for (int k = 0; k < kEvCount; ++k)
		if (s->ev[k]) cudaEventDestroy(s->ev[k]);
	for (int k = 0; k < 2; ++k)
		if (s->statsEv[k]) cudaEventDestroy(s->statsEv[k]);
	if (s->stream) cudaStreamDestroy(s->stream);
	delete s;
	return SPH_OK;
}

int sph_reset_stats(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	const std::vector<uint32_t> seed = stats_seed(s);
	SPH_CUDA(cudaMemcpyAsync(s->T.stats, seed.data(), seed.size() * 4, cudaMemcpyHostToDevice, s->stream));
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	s->timed = false;
	s->emitterMs = 0.0f;
	return SPH_OK;
}

int sph_clear_bodies(sph_sim *s) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	sc->bodies.clear();
	s->bodiesDirty = true;
	return SPH_OK;
}

int sph_clear_particles(sph_sim *s) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	sc->pendPos.clear();
	sc->pendForce.clear();
	SPH_CUDA(cudaMemsetAsync(s->cellCountA, 0, sizeof(int) * s->ncellTotal, s->stream));
	SPH_CUDA(cudaMemsetAsync(s->cellStartA, 0, sizeof(int) * s->ncellTotal, s->stream));
	SPH_CUDA(cudaMemsetAsync(s->T.appCount, 0, sizeof(int) * s->ncellTotal, s->stream));
	sc->n = sc->n0 = sc->nDev = 0;
	s->sceneTableDirty = true;
	return SPH_OK;
}

int sph_clear_emitters(sph_sim *s) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	sc->emitters.clear();
	return SPH_OK;
}

int sph_add_plane(sph_sim *s, sph_vec2 normal, float distance) { return push_body(s, plane_body(normal, distance)); }

int sph_add_circle(sph_sim *s, sph_vec2 pos, float radius) { return push_body(s, circle_body(pos, radius)); }

int sph_add_line_segment(sph_sim *s, sph_vec2 a, sph_vec2 b) { return push_body(s, segment_body(a, b)); }

int sph_add_polygon(sph_sim *s, size_t count, const sph_vec2 *verts) {
	if (!s || (count > 0 && !verts)) return SPH_ERR_INVALID_ARGUMENT;
	if (count > (size_t)kMaxPoly) return SPH_ERR_CAPACITY;
	return push_body(s, polygon_body(count, verts));
}

int sph_add_particle(sph_sim *s, sph_vec2 position, sph_vec2 force, size_t *out_index) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	return push_particle(*sc, make_float2(position.x, position.y), make_float2(force.x, force.y), out_index);
}

int sph_add_particles(sph_sim *s, size_t count, const sph_vec2 *positions, const sph_vec2 *forces,
                      size_t *first_index) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	if (count > 0 && !positions) return SPH_ERR_INVALID_ARGUMENT;
	if (sc->n + count > sc->cap) return SPH_ERR_CAPACITY;
	if (first_index) *first_index = sc->n;
	for (size_t k = 0; k < count; ++k) {
		const float2 f = forces ? make_float2(forces[k].x, forces[k].y) : make_float2(0.0f, 0.0f);
		push_particle(*sc, make_float2(positions[k].x, positions[k].y), f, nullptr);
	}
	return SPH_OK;
}

int sph_add_volume(sph_sim *s, sph_vec2 center, sph_vec2 force, int count_x, int count_y, float spacing) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	if (count_x < 0 || count_y < 0) return SPH_ERR_INVALID_ARGUMENT;
	if (sc->n + (size_t)count_x * (size_t)count_y > sc->cap) return SPH_ERR_CAPACITY;
	// AddVolume (demo4.cpp:169-181), same operation order.
	float2 offset = make_float2((float)count_x * spacing, (float)count_y * spacing);
	offset = make_float2(offset.x * 0.5f, offset.y * 0.5f);
	const float2 f = make_float2(force.x, force.y);
	for (int yi = 0; yi < count_y; ++yi) {
		for (int xi = 0; xi < count_x; ++xi) {
			float2 p = make_float2((float)xi * spacing, (float)yi * spacing);
			const float hs = spacing * 0.5f;
			p = make_float2(hs + p.x, hs + p.y);
			const float2 base = make_float2(center.x - offset.x, center.y - offset.y);
			p = make_float2(base.x + p.x, base.y + p.y);
			const float2 j = jitter(*sc);
			p = make_float2(j.x + p.x, j.y + p.y);
			push_particle(*sc, p, f, nullptr);
		}
	}
	return SPH_OK;
}

int sph_add_emitter(sph_sim *s, sph_vec2 position, sph_vec2 direction, float radius, float speed, float rate,
                    float duration) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	if (sc->emitters.size() >= 8) return SPH_ERR_CAPACITY;  // kSPHMaxEmitterCount
	Emitter e{};
	e.position = position;
	e.direction = direction;
	e.radius = radius;
	e.speed = speed;
	e.rate = rate;
	e.duration = duration;
	e.elapsed = 0;
	e.totalElapsed = 0;
	e.active = 1;
	sc->emitters.push_back(e);
	return SPH_OK;
}

int sph_update(sph_sim *s, float dt) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	if (!(dt > 0.0f)) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(s->device));
	int rc = flush_adds(s);
	if (rc) return rc;
	const auto t0 = std::chrono::high_resolution_clock::now();
	for (Scene &sc : s->scenes) {
		for (Emitter &e : sc.emitters) {
			rc = update_emitter(sc, e, dt);
			if (rc) return rc;
		}
	}
	rc = flush_adds(s);
	if (rc) return rc;
	s->emitterMs = (float)std::chrono::duration_cast<std::chrono::nanoseconds>(
	                   std::chrono::high_resolution_clock::now() - t0)
	                   .count() *
	               (1.0f / 1000000);
	if (s->totalParticles() == 0) {
		// NeighborSearch restarts the neighbour statistics even with no particles.
		for (size_t k = 0; k < s->scenes.size(); ++k) {
			const uint32_t seed[2] = {s->scenes[k].dom.max_neighbors, 0u};
			SPH_CUDA(cudaMemcpyAsync(s->T.stats + 4 * k, seed, sizeof(seed), cudaMemcpyHostToDevice, s->stream));
		}
		SPH_CUDA(cudaStreamSynchronize(s->stream));
		s->timed = false;
		return SPH_OK;
	}
	return run_step(s, dt);
}

int sph_add_external_forces(sph_sim *s, sph_vec2 f) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	sc->external = sph_vec2{f.x + sc->external.x, f.y + sc->external.y};
	s->sceneTableDirty = true;
	return SPH_OK;
}

int sph_clear_external_force(sph_sim *s) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	sc->external = sph_vec2{0.0f, 0.0f};
	s->sceneTableDirty = true;
	return SPH_OK;
}

int sph_get_particle_count(sph_sim *s, size_t *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->totalParticles();
	return SPH_OK;
}

int sph_set_gravity(sph_sim *s, sph_vec2 g) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	sc->gravity = g;
	s->sceneTableDirty = true;
	return SPH_OK;
}

int sph_get_params(sph_sim *s, sph_params *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->scenes[0].params;
	return SPH_OK;
}

int sph_set_params(sph_sim *s, const sph_params *p) {
	if (!p) return SPH_ERR_INVALID_ARGUMENT;
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	sc->params = *p;
	s->sceneTableDirty = true;
	return SPH_OK;
}

int sph_batch_get_stats(sph_sim *s, size_t scene, sph_stats *out) {
	if (!s || !out || scene >= s->scenes.size()) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	rc = check_device_errors(s);
	uint32_t st[4];
	SPH_CUDA(cudaMemcpy(st, s->T.stats + 4 * scene, sizeof(st), cudaMemcpyDeviceToHost));
	out->min_particle_neighbor_count = st[0];
	out->max_particle_neighbor_count = st[1];
	out->min_cell_particle_count = st[2];
	out->max_cell_particle_count = st[3];
	out->time_emitters = s->emitterMs;
	// Stage times cover the whole update (every scene of a batch).
	float t[kEvCount] = {};
	if (s->timed) {
		for (int k = 1; k < kEvCount; ++k) {
			if (cudaEventElapsedTime(&t[k], s->ev[k - 1], s->ev[k]) != cudaSuccess) t[k] = 0.0f;
		}
	}
	out->time_integration = t[kEvIntegrate];
	out->time_viscosity_forces = t[kEvVisc];
	out->time_predict = t[kEvPredict];
	out->time_update_grid = t[kEvGrid];
	// The grid update builds the neighbour structure; this slot holds the
	// spring phase, which runs on the fresh lists (0 when springs are off).
	out->time_neighbor_search = t[kEvSprings];
	out->time_density_and_pressure = t[kEvDensity];
	out->time_delta_positions = t[kEvDelta];
	out->time_collisions = t[kEvCollide];
	return rc;
}

int sph_get_stats(sph_sim *s, sph_stats *out) { return sph_batch_get_stats(s, 0, out); }

int sph_set_multithreading(sph_sim *s, int value) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	s->multithreading = value ? 1 : 0;
	return SPH_OK;
}

int sph_is_multithreading_supported(sph_sim *s, int *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = 1;
	return SPH_OK;
}

int sph_is_multithreading(sph_sim *s, int *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->multithreading;
	return SPH_OK;
}

int sph_get_worker_thread_count(sph_sim *s, size_t *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = (size_t)s->numSMs;
	return SPH_OK;
}

int sph_read_particles(sph_sim *s, size_t count, sph_vec2 *pos, sph_vec2 *prev, sph_vec2 *vel, sph_vec2 *acc,
                       sph_vec2 *dens, sph_vec2 *press) {
	return read_scene(s, 0, count, pos, prev, vel, acc, dens, press);
}

int sph_batch_read_particles(sph_sim *s, size_t scene, size_t count, sph_vec2 *pos, sph_vec2 *vel, sph_vec2 *dens,
                             sph_vec2 *press) {
	return read_scene(s, scene, count, pos, nullptr, vel, nullptr, dens, press);
}

// Demo4::Render (demo4.cpp:520-531) colours every particle with
// SPHGetParticleColor (sph.h:683-695) from its density, pressure and
// velocity; here the colours are computed on the device and copied out in
// AddParticle order.
int sph_particle_colors(sph_sim *s, size_t count, float *rgba) {
	if (!s || (count && !rgba)) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(s->device));
	int rc = flush_adds(s);
	if (rc) return rc;
	const Scene &sc = s->scenes[0];
	if (count > sc.n) return SPH_ERR_INVALID_ARGUMENT;
	if (count == 0) return SPH_OK;
	if (s->colorCap < sc.n) {
		SPH_CUDA(cudaStreamSynchronize(s->stream));
		if (s->colorBuf) cudaFree(s->colorBuf);
		s->colorBuf = nullptr;
		s->colorCap = 0;
		if ((rc = dalloc(&s->colorBuf, sc.n))) return rc;
		s->colorCap = sc.n;
	}
	const BufferSet &A = s->buf[s->cur];
	const int n = (int)sc.n;
	k_particle_colors<<<blocks_for(n, kElemThreads), kElemThreads, 0, s->stream>>>(
	    sc.pBase, n, A.id, A.dens, A.press, A.vel, sc.params.rest_density, s->colorBuf);
	SPH_LAUNCHED(s);
	SPH_CUDA(cudaMemcpyAsync(rgba, s->colorBuf, count * sizeof(float4), cudaMemcpyDeviceToHost, s->stream));
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	return check_device_errors(s);
}

// A point image of the scene instead of Render's OpenGL points: width x
// height RGBA8 pixels spanning the box (row 0 at the top); each particle
// colours the pixel under it, later particles (AddParticle order) over
// earlier ones; empty pixels are 0.
int sph_render_points(sph_sim *s, int width, int height, unsigned char *rgba) {
	if (!s || !rgba || width <= 0 || height <= 0 || (int64_t)width * height > (1 << 26))
		return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(s->device));
	int rc = flush_adds(s);
	if (rc) return rc;
	const Scene &sc = s->scenes[0];
	const size_t pixels = (size_t)width * height;
	if (s->imgCap < pixels) {
		SPH_CUDA(cudaStreamSynchronize(s->stream));
		if (s->imgKeys) cudaFree(s->imgKeys);
		if (s->imgRgba) cudaFree(s->imgRgba);
		s->imgKeys = nullptr;
		s->imgRgba = nullptr;
		s->imgCap = 0;
		if ((rc = dalloc(&s->imgKeys, pixels)) || (rc = dalloc(&s->imgRgba, pixels))) return rc;
		s->imgCap = pixels;
	}
	SPH_CUDA(cudaMemsetAsync(s->imgKeys, 0, pixels * sizeof(unsigned long long), s->stream));
	const BufferSet &A = s->buf[s->cur];
	const int n = (int)sc.n;
	const float halfW = sc.dom.width * 0.5f, halfH = sc.dom.height * 0.5f;
	const float sx = (float)width / sc.dom.width, sy = (float)height / sc.dom.height;
	if (n > 0) {
		k_splat_points<<<blocks_for(n, kElemThreads), kElemThreads, 0, s->stream>>>(
		    sc.pBase, n, A.id, A.pos, A.dens, A.press, A.vel, sc.params.rest_density, halfW, halfH, sx, sy, width,
		    height, s->imgKeys);
		SPH_LAUNCHED(s);
	}
	k_keys_to_rgba8<<<blocks_for(pixels, kElemThreads), kElemThreads, 0, s->stream>>>((int)pixels, s->imgKeys,
	                                                                                    s->imgRgba);
	SPH_LAUNCHED(s);
	SPH_CUDA(cudaMemcpyAsync(rgba, s->imgRgba, pixels * 4, cudaMemcpyDeviceToHost, s->stream));
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	return check_device_errors(s);
}

int sph_state_info(sph_sim *s, size_t *count, size_t *canonical, int *gx, int *gy) {
	return scene_info(s, 0, count, canonical, gx, gy);
}

int sph_batch_state_info(sph_sim *s, size_t scene, size_t *count, size_t *canonical, int *gx, int *gy) {
	return scene_info(s, scene, count, canonical, gx, gy);
}

int sph_dump_state(sph_sim *s, const sph_state_view *v) { return dump_scene(s, 0, v); }

int sph_batch_dump_state(sph_sim *s, size_t scene, const sph_state_view *v) { return dump_scene(s, scene, v); }

int sph_load_state(sph_sim *s, const sph_state_view *v) {
	if (!v) return SPH_ERR_INVALID_ARGUMENT;
	Scene *scp = single(s);
	if (!scp) return not_single(s);
	Scene &sc = *scp;
	if (!v->pos || !v->prev || !v->vel || !v->acc || !v->dens || !v->press || !v->id || !v->cell ||
	    !v->cell_start || !v->cell_count)
		return SPH_ERR_INVALID_ARGUMENT;
	if (v->count > sc.cap || v->canonical_count > v->count) return SPH_ERR_INVALID_ARGUMENT;
	if (v->grid_x != sc.gx || v->grid_y != sc.gy) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(s->device));
	const size_t n = v->count;
	// The state goes into the back buffer set and the back cell tables (free
	// between updates) and is checked there on the device; only a valid
	// state becomes current, so an invalid one leaves the simulation as it
	// was.  With pinned host arrays the copies run at full link speed and
	// the host does no per-particle work.
	BufferSet &B = s->buf[1 - s->cur];
	cudaStream_t st = s->stream;
	auto h2d = [&](void *dst, const void *src, size_t bytes) -> int {
		if (bytes == 0) return SPH_OK;
		return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
	};
	int rc;
	if ((rc = h2d(B.pos, v->pos, n * 8)) || (rc = h2d(B.prev, v->prev, n * 8)) || (rc = h2d(B.vel, v->vel, n * 8)) ||
	    (rc = h2d(B.acc, v->acc, n * 8)) || (rc = h2d(B.dens, v->dens, n * 8)) ||
	    (rc = h2d(B.press, v->press, n * 8)) || (rc = h2d(B.id, v->id, n * 4)) ||
	    (rc = h2d(B.cellOf, v->cell, n * 4)) || (rc = h2d(s->cellStartB, v->cell_start, sc.ncell * 4)) ||
	    (rc = h2d(s->cellCountB, v->cell_count, sc.ncell * 4)))
		return rc;
	// Per-step scratch, free between updates: enterCount counts the added
	// particles per cell, newLabel marks the AddParticle indices seen.
	SPH_CUDA(cudaMemsetAsync(s->T.enterCount, 0, sc.ncell * sizeof(int), st));
	SPH_CUDA(cudaMemsetAsync(s->T.newLabel, 0, std::max<size_t>(n, 1) * sizeof(int), st));
	SPH_CUDA(cudaMemsetAsync(s->check, 0, 2 * sizeof(int), st));
	const size_t items = std::max(n, (size_t)sc.ncell);
	k_check_state<<<blocks_for(items, kElemThreads), kElemThreads, 0, st>>>(
	    (int)n, (int)v->canonical_count, sc.ncell, B.cellOf, s->cellStartB, s->cellCountB, B.id, s->T.enterCount,
	    s->T.newLabel, s->check);
	SPH_LAUNCHED(s);
	int verdict[2] = {0, 0};
	SPH_CUDA(cudaMemcpyAsync(verdict, s->check, sizeof(verdict), cudaMemcpyDeviceToHost, st));
	SPH_CUDA(cudaStreamSynchronize(st));
	if (verdict[0] != 0 || (size_t)verdict[1] != v->canonical_count) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaMemcpyAsync(s->T.appCount, s->T.enterCount, sc.ncell * 4, cudaMemcpyDeviceToDevice, st));
	if (B.springN && n) SPH_CUDA(cudaMemsetAsync(B.springN, 0, n * sizeof(int), st));  // sph_load_springs sets them
	s->cur = 1 - s->cur;
	std::swap(s->cellStartA, s->cellStartB);
	std::swap(s->cellCountA, s->cellCountB);
	sc.pendPos.clear();
	sc.pendForce.clear();
	sc.n = sc.nDev = n;
	sc.n0 = v->canonical_count;
	s->sceneTableDirty = true;
	drop_graphs(s);
	return SPH_OK;
}

int sph_get_stream(sph_sim *s, void **stream) {
	if (!s || !stream) return SPH_ERR_INVALID_ARGUMENT;
	*stream = (void *)s->stream;
	return SPH_OK;
}

int sph_device_arrays(sph_sim *s, const void **pos, const void **vel, const void **dens, const void **press) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	BufferSet &A = s->buf[s->cur];
	if (pos) *pos = A.pos;
	if (vel) *vel = A.vel;
	if (dens) *dens = A.dens;
	if (press) *press = A.press;
	return SPH_OK;
}

int sph_synchronize(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	return check_device_errors(s);
}

// Diagnostics (not part of the reference interface): per-task timestamps of
// the two ordered sweeps of the next updates.
int sph_profile_tasks(sph_sim *s, int enable) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	drop_graphs(s);  // graphs hold the timestamp buffer's address
	if (enable && !s->prof) {
		SPH_CUDA(cudaMalloc(&s->prof, sizeof(unsigned long long) * 8 * s->doneDCap));
		SPH_CUDA(cudaMemset(s->prof, 0, sizeof(unsigned long long) * 8 * s->doneDCap));
	} else if (!enable && s->prof) {
		cudaFree(s->prof);
		s->prof = nullptr;
	}
	return SPH_OK;
}

int sph_profile_read(sph_sim *s, unsigned long long *out, size_t capacity, size_t *stride) {
	if (!s || !stride) return SPH_ERR_INVALID_ARGUMENT;
	*stride = s->doneDCap;
	if (!s->prof || !out) return SPH_OK;
	const size_t total = std::min(capacity, (size_t)8 * s->doneDCap);
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	SPH_CUDA(cudaMemcpy(out, s->prof, total * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
	return SPH_OK;
}

int sph_set_springs(sph_sim *s, const sph_spring_params *p) {
	if (!p) return SPH_ERR_INVALID_ARGUMENT;
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	if (p->enabled && (p->max_per_particle < 0 || p->max_per_particle > kSprings || !(p->yield_ratio >= 0.0f) ||
	                   !(p->plasticity >= 0.0f)))
		return SPH_ERR_INVALID_ARGUMENT;
	if (p->enabled && !s->buf[0].springN) {
		const size_t N = s->capTotal, S = s->scenes.size();
		SPH_CUDA(cudaStreamSynchronize(s->stream));
		int rc;
		for (int b = 0; b < 2; ++b) {
			BufferSet &B = s->buf[b];
			if ((rc = dalloc(&B.springN, N)) || (rc = dalloc(&B.springP, N * kSprings)) ||
			    (rc = dalloc(&B.springL, N * kSprings)))
				return rc;
		}
		if ((rc = dalloc(&s->T.accN, N)) || (rc = dalloc(&s->T.accP, N * kSprings)) ||
		    (rc = dalloc(&s->T.springPos, N)) || (rc = dalloc(&s->T.springTotal, S)))
			return rc;
	}
	if (p->enabled && !sc->springs.enabled) {
		// Springs start empty whenever they are switched on.
		for (int b = 0; b < 2; ++b)
			SPH_CUDA(cudaMemsetAsync(s->buf[b].springN, 0, s->capTotal * sizeof(int), s->stream));
	}
	sc->springs = *p;
	s->sceneTableDirty = true;
	return SPH_OK;
}

int sph_get_spring_count(sph_sim *s, uint64_t *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = 0;
	if (!s->T.springTotal) return SPH_OK;
	int rc = check_device_errors(s);
	if (rc) return rc;
	std::vector<unsigned long long> t(s->scenes.size());
	SPH_CUDA(cudaMemcpy(t.data(), s->T.springTotal, t.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
	unsigned long long total = 0;
	for (unsigned long long v : t) total += v;
	*out = total / 2;  // each spring is stored at both ends
	return SPH_OK;
}

int sph_dump_springs(sph_sim *s, size_t count, int32_t *spring_count, int32_t *partner, float *rest) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	int rc = flush_adds(s);
	if (rc) return rc;
	if (count != sc->n) return SPH_ERR_INVALID_ARGUMENT;
	const BufferSet &A = s->buf[s->cur];
	const BufferSet &B = s->buf[1 - s->cur];  // free between updates: the cleaned copy
	cudaStream_t st = s->stream;
	if (!A.springN) {
		// Springs were never enabled: no particle has one.
		for (size_t i = 0; i < count; ++i) {
			if (spring_count) spring_count[i] = 0;
			for (int q = 0; q < kSprings; ++q) {
				if (partner) partner[i * kSprings + q] = -1;
				if (rest) rest[i * kSprings + q] = 0.0f;
			}
		}
		return check_device_errors(s);
	}
	if (count) {
		k_clean_springs<<<blocks_for(count * kSprings, kElemThreads), kElemThreads, 0, st>>>(
		    (int)count, A.springN, A.springP, A.springL, B.springN, B.springP, B.springL);
		SPH_LAUNCHED(s);
		if (spring_count)
			SPH_CUDA(cudaMemcpyAsync(spring_count, B.springN, count * 4, cudaMemcpyDeviceToHost, st));
		if (partner)
			SPH_CUDA(cudaMemcpyAsync(partner, B.springP, count * kSprings * 4, cudaMemcpyDeviceToHost, st));
		if (rest) SPH_CUDA(cudaMemcpyAsync(rest, B.springL, count * kSprings * 4, cudaMemcpyDeviceToHost, st));
	}
	return check_device_errors(s);
}

int sph_load_springs(sph_sim *s, size_t count, const int32_t *spring_count, const int32_t *partner,
                     const float *rest) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	if (!spring_count || !partner || !rest) return SPH_ERR_INVALID_ARGUMENT;
	if (!s->buf[0].springN) return SPH_ERR_NOT_SUPPORTED;  // springs were never enabled
	int rc = flush_adds(s);
	if (rc) return rc;
	if (count != sc->n) return SPH_ERR_INVALID_ARGUMENT;
	// Into the back buffer set's spring tables, checked on the device, then
	// swapped in: invalid tables leave the current springs as they were.
	BufferSet &A = s->buf[s->cur];
	BufferSet &B = s->buf[1 - s->cur];
	cudaStream_t st = s->stream;
	if (count) {
		SPH_CUDA(cudaMemcpyAsync(B.springN, spring_count, count * 4, cudaMemcpyHostToDevice, st));
		SPH_CUDA(cudaMemcpyAsync(B.springP, partner, count * kSprings * 4, cudaMemcpyHostToDevice, st));
		SPH_CUDA(cudaMemcpyAsync(B.springL, rest, count * kSprings * 4, cudaMemcpyHostToDevice, st));
		SPH_CUDA(cudaMemsetAsync(s->check, 0, sizeof(int), st));
		k_check_springs<<<blocks_for(count, kElemThreads), kElemThreads, 0, st>>>((int)count, B.springN, B.springP,
		                                                                          s->check);
		SPH_LAUNCHED(s);
	}
	int bad = 0;
	if (count) SPH_CUDA(cudaMemcpyAsync(&bad, s->check, sizeof(int), cudaMemcpyDeviceToHost, st));
	SPH_CUDA(cudaStreamSynchronize(st));
	if (bad) return SPH_ERR_INVALID_ARGUMENT;
	std::swap(A.springN, B.springN);
	std::swap(A.springP, B.springP);
	std::swap(A.springL, B.springL);
	drop_graphs(s);  // graphs hold the spring tables' addresses
	return SPH_OK;
}

// Launch-shape autotuner: the ordered sweeps are persistent kernels; each
// has shapes (wide: short per-particle latency for one scene; the delta
// sweep's mid: the same pipeline with two blocks per SM; lean: more tasks per
// SM for many scenes) and a resident block count that trades parallel tasks
// against polling traffic.  Every shape gives the same results
// (the task order fixes them), so each candidate is timed on the same update
// from a snapshot and the fastest kept for each sweep.
int sph_autotune(sph_sim *s, float dt, int *shape) {
	if (!s || !(dt > 0.0f)) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(s->device));
	int rc = flush_adds(s);
	if (rc) return rc;
	for (const Scene &sc : s->scenes)
		if (sc.n0 != sc.nDev) return SPH_ERR_NOT_SUPPORTED;  // needs a canonical state: update first
	if (s->totalParticles() == 0) return SPH_ERR_NOT_SUPPORTED;
	rc = ensure_learned(s);
	if (rc) return rc;
	const bool graphs = s->useGraphs, adaptive = s->adaptive;
	s->useGraphs = false;
	s->adaptive = false;  // time the shapes as given
	rc = copy_state(s, true);
	if (rc) return rc;
	// Median of three timed updates per shape (after one warm-up update); the
	// current shape is kept unless another is faster by more than 2%.
	auto measure = [&](int vLean, int vBlocks, int dShape, int dBlocks, float *tv, float *td) -> int {
		s->viscLean = vLean;
		s->viscBlocks = vBlocks;
		s->deltaShape = dShape;
		s->deltaBlocks = dBlocks;
		float v[3], d[3];
		for (int rep = 0; rep < 4; ++rep) {
			int r = copy_state(s, false);
			if (!r) r = run_step(s, dt);
			if (!r) r = check_device_errors(s);
			if (r) return r;
			if (rep == 0) continue;
			SPH_CUDA(cudaEventElapsedTime(&v[rep - 1], s->ev[kEvIntegrate], s->ev[kEvVisc]));
			SPH_CUDA(cudaEventElapsedTime(&d[rep - 1], s->ev[kEvDensity], s->ev[kEvDelta]));
		}
		std::sort(v, v + 3);
		std::sort(d, d + 3);
		*tv = v[1];
		*td = d[1];
		return SPH_OK;
	};
	int pick[4] = {s->viscLean, s->viscBlocks, s->deltaShape, s->deltaBlocks};
	float bestV = 0.f, bestD = 0.f;
	rc = measure(pick[0], pick[1], pick[2], pick[3], &bestV, &bestD);
	// Candidates: every delta shape, each timed with the viscosity shape of
	// the same kind (lean with lean, wide with both pipelined delta shapes),
	// at every resident block count per SM.
	for (int dShape = 0; dShape < kDeltaShapes && !rc; ++dShape) {
		const int lean = dShape == kDeltaLean ? 1 : 0;
		int occV = 0, occD = 0;
		rc = cuda_status(sweep_occupancy(lean != 0, dShape, &occV, &occD));
		const int maxPer = std::max(occV, occD);
		for (int per = 1; per <= maxPer && !rc; ++per) {
			const int vb = std::min(per, occV) * s->numSMs, db = std::min(per, occD) * s->numSMs;
			float tv = 0.f, td = 0.f;
			rc = measure(lean, vb, dShape, db, &tv, &td);
			if (rc) break;
			if (tv < 0.98f * bestV) {
				bestV = tv;
				pick[0] = lean;
				pick[1] = vb;
			}
			if (td < 0.98f * bestD) {
				bestD = td;
				pick[2] = dShape;
				pick[3] = db;
			}
		}
	}
	if (!rc) rc = copy_state(s, false);
	s->viscLean = pick[0];
	s->viscBlocks = pick[1];
	s->deltaShape = pick[2];
	s->deltaBlocks = pick[3];
	s->useGraphs = graphs;
	s->adaptive = adaptive;
	drop_graphs(s);
	s->timed = false;
	if (rc) return rc;
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	if (shape) {
		shape[0] = s->viscLean ? ViscLean::kWarps : ViscWide::kWarps;
		shape[1] = s->viscBlocks;
		shape[2] = delta_shape_warps(s->deltaShape);
		shape[3] = s->deltaBlocks;
	}
	return SPH_OK;
}

int sph_get_sweep_shape(sph_sim *s, int *shape) {
	if (!s || !shape) return SPH_ERR_INVALID_ARGUMENT;
	shape[0] = s->viscLean ? ViscLean::kWarps : ViscWide::kWarps;
	shape[1] = s->viscBlocks;
	shape[2] = delta_shape_warps(s->deltaShape);
	shape[3] = s->deltaBlocks;
	return SPH_OK;
}

int sph_set_sweep_shape(sph_sim *s, const int *shape) {
	if (!s || !shape) return SPH_ERR_INVALID_ARGUMENT;
	const bool vOk = shape[0] == ViscLean::kWarps || shape[0] == ViscWide::kWarps;
	int dShape = -1;
	for (int k = 0; k < kDeltaShapes; ++k)
		if (shape[2] == delta_shape_warps(k)) dShape = k;
	const bool dOk = dShape >= 0;
	if (!vOk || !dOk || shape[1] < 1 || shape[3] < 1 || shape[1] > (1 << 20) || shape[3] > (1 << 20))
		return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	s->viscLean = shape[0] == ViscLean::kWarps;
	s->viscBlocks = shape[1];
	s->deltaShape = dShape;
	s->deltaBlocks = shape[3];
	drop_graphs(s);
	return SPH_OK;
}

int sph_set_adaptive_shapes(sph_sim *s, int enable) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	s->adaptive = enable != 0;
	return SPH_OK;
}

int sph_last_sweep_shape(sph_sim *s, int *shape) {
	if (!s || !shape) return SPH_ERR_INVALID_ARGUMENT;
	if (s->runViscLean < 0) return sph_get_sweep_shape(s, shape);
	shape[0] = s->runViscLean ? ViscLean::kWarps : ViscWide::kWarps;
	shape[1] = s->runViscBlocks;
	shape[2] = delta_shape_warps(s->runDeltaShape);
	shape[3] = s->runDeltaBlocks;
	return SPH_OK;
}

int sph_set_reference_order(sph_sim *s, int enable) {
	Scene *sc = single(s);
	if (!sc) return not_single(s);
	if (s->refOrder != (enable != 0)) drop_graphs(s);
	s->refOrder = enable != 0;
	s->sceneTableDirty = true;
	return SPH_OK;
}

int sph_get_reference_order(sph_sim *s, int *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->refOrder ? 1 : 0;
	return SPH_OK;
}

int sph_set_wait_limit(sph_sim *s, double seconds) {
	if (!s || !(seconds > 0.0) || !(seconds <= 3600.0)) return SPH_ERR_INVALID_ARGUMENT;
	const double ns = seconds * 1e9;
	s->T.waitLimitNs = ns < 1.0 ? 1ull : (unsigned long long)ns;
	drop_graphs(s);  // graphs hold the tables by value
	return SPH_OK;
}

int sph_test_hold_task(sph_sim *s, int sweep, int claim) {
	if (!s || sweep < 0 || sweep > 1 || claim < -1) return SPH_ERR_INVALID_ARGUMENT;
	s->T.hold[sweep] = claim;
	drop_graphs(s);
	return SPH_OK;
}

int sph_use_graphs(sph_sim *s, int enable) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	drop_graphs(s);
	s->useGraphs = enable != 0;
	return SPH_OK;
}

int sph_kernel_launches(sph_sim *s, uint64_t *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->launches;
	return SPH_OK;
}

}  // extern "C"
