// Host side of the GB300 Demo4 SPH step: the simulation object behind the C
// ABI of include/sph_gb300.h, mirroring Demo4::ParticleSimulation
// (NBodySimulation/demo4.h:178-267).  All device memory is allocated once in
// sph_create for the domain's capacities; an update is a fixed sequence of
// kernel launches on the simulation's stream.
//
// Host arithmetic that feeds the step (volume and emitter particle
// placement, step scalars) follows the reference's FP32 operation order; the
// library is built with -ffp-contract=off so the host compiler fuses nothing.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/sph_gb300.h"
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
		return p;
	}
};

enum Stage { kEvBegin, kEvIntegrate, kEvVisc, kEvPredict, kEvGrid, kEvDensity, kEvDelta, kEvCollide, kEvCount };

}  // namespace

struct sph_sim {
	int device = 0;
	cudaStream_t stream = nullptr;
	sph_domain dom{};
	int gx = 0, gy = 0, ncell = 0;
	int numSMs = 0;
	int viscBlocks = 0, deltaBlocks = 0, densBlocks = 0, gridBlocks = 0;

	sph_params params{};
	sph_vec2 gravity{0.0f, 0.0f};
	sph_vec2 external{0.0f, 0.0f};
	int multithreading = 0;

	std::vector<Body> bodies;
	bool bodiesDirty = true;
	std::vector<Emitter> emitters;

	size_t n = 0;   // particles (device-resident + pending)
	size_t n0 = 0;  // canonical count
	size_t nDev = 0;  // particles already on the device
	std::vector<float2> pendPos, pendForce;

	BufferSet buf[2];
	int cur = 0;
	int *cellStartA = nullptr, *cellCountA = nullptr, *cellStartB = nullptr, *cellCountB = nullptr;
	SimTables T{};
	uint32_t *doneV = nullptr, *doneD = nullptr;
	size_t doneDCap = 0;
	float2 *stagePos = nullptr, *stageForce = nullptr;  // device staging for adds
	float2 *hostPos = nullptr, *hostForce = nullptr;    // pinned staging
	size_t stageCap = 0;

	cudaEvent_t ev[kEvCount] = {};
	bool timed = false;
	float emitterMs = 0.0f;
	uint64_t launches = 0;
	int stickyError = SPH_OK;
	unsigned long long *prof = nullptr;

	uint32_t maxNbSeed() const { return dom.max_neighbors; }
};

namespace {

int cuda_status(cudaError_t e) { return e == cudaSuccess ? SPH_OK : SPH_ERR_CUDA; }

#define SPH_CUDA(call)                                 \
	do {                                               \
		cudaError_t e_ = (call);                       \
		if (e_ != cudaSuccess) return SPH_ERR_CUDA;    \
	} while (0)

template <typename T>
int dalloc(T **p, size_t count) {
	if (count == 0) count = 1;
	cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T));
	if (e != cudaSuccess) return SPH_ERR_CUDA;
	e = cudaMemset(*p, 0, count * sizeof(T));
	return cuda_status(e);
}

StepParams step_params(const sph_sim *s, float dt) {
	StepParams p{};
	p.h2 = s->params.kernel_height * s->params.kernel_height;
	p.invH = s->params.inv_kernel_height;
	p.rho0 = s->params.rest_density;
	p.k = s->params.stiffness;
	p.kNear = s->params.near_stiffness;
	p.sigma = s->params.linear_viscosity;
	p.beta = s->params.quadratic_viscosity;
	p.dt = dt;
	p.invDt = 1.0f / dt;
	p.dt2 = dt * dt;
	p.extX = s->gravity.x + s->external.x;
	p.extY = s->gravity.y + s->external.y;
	p.halfW = s->dom.width * 0.5f;
	p.halfH = s->dom.height * 0.5f;
	p.cellSize = s->dom.cell_size;
	p.gx = s->gx;
	p.gy = s->gy;
	p.ncell = s->ncell;
	p.radius = s->dom.particle_radius;
	p.margin = s->dom.collision_margin;
	p.nbodies = (int)s->bodies.size();
	return p;
}

SimTables tables(sph_sim *s) {
	SimTables t = s->T;
	t.prof = s->prof;
	t.profStride = s->prof ? (int)s->doneDCap : 0;
	t.cellStart = s->cellStartA;
	t.cellCount = s->cellCountA;
	t.newStart = s->cellStartB;
	t.newCount = s->cellCountB;
	return t;
}

int blocks_for(size_t items, int threads) { return (int)std::max<size_t>(1, (items + threads - 1) / threads); }

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
	const size_t count = s->pendPos.size();
	if (count == 0) return SPH_OK;
	int rc = ensure_stage(s, count);
	if (rc != SPH_OK) return rc;
	SPH_CUDA(cudaStreamSynchronize(s->stream));  // host staging is reused
	std::memcpy(s->hostPos, s->pendPos.data(), count * sizeof(float2));
	std::memcpy(s->hostForce, s->pendForce.data(), count * sizeof(float2));
	SPH_CUDA(cudaMemcpyAsync(s->stagePos, s->hostPos, count * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
	SPH_CUDA(cudaMemcpyAsync(s->stageForce, s->hostForce, count * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
	StepParams sp = step_params(s, 1.0f);
	k_add<<<blocks_for(count, kElemThreads), kElemThreads, 0, s->stream>>>(
	    (int)s->nDev, (int)count, s->stagePos, s->stageForce, s->buf[s->cur].view(), tables(s), sp);
	s->launches++;
	SPH_CUDA(cudaGetLastError());
	s->nDev += count;
	s->pendPos.clear();
	s->pendForce.clear();
	return SPH_OK;
}

int push_particle(sph_sim *s, float2 p, float2 f, size_t *index) {
	if (s->n >= s->dom.max_particles) return SPH_ERR_CAPACITY;
	s->pendPos.push_back(p);
	s->pendForce.push_back(f);
	if (index) *index = s->n;
	s->n++;
	return SPH_OK;
}

// Vec2RandomDirection (vecmath.h:317-322): the reference's jitter source.
float2 random_direction() {
	float d = rand() / (float)RAND_MAX;
	float angle = d * ((float)M_PI * 2.0f);
	return make_float2(cosf(angle), sinf(angle));
}

float2 jitter(const sph_sim *s) {
	float2 r = random_direction();
	r = make_float2(r.x * s->dom.jitter_kernel_height, r.y * s->dom.jitter_kernel_height);
	return make_float2(r.x * s->dom.jitter_scale, r.y * s->dom.jitter_scale);
}

// UpdateEmitter (demo4.cpp:257-284).
int update_emitter(sph_sim *s, Emitter &e, float dt) {
	const float spacing = s->params.particle_spacing;
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
			const float2 j = jitter(s);
			p = make_float2(j.x + p.x, j.y + p.y);
			int rc = push_particle(s, p, accel, nullptr);
			if (rc != SPH_OK) return rc;
		}
	}
	if (e.totalElapsed >= e.duration) e.active = 0;
	return SPH_OK;
}

int upload_bodies(sph_sim *s) {
	if (!s->bodiesDirty) return SPH_OK;
	if (!s->bodies.empty()) {
		SPH_CUDA(cudaMemcpyAsync(s->T.bodies, s->bodies.data(), s->bodies.size() * sizeof(Body),
		                         cudaMemcpyHostToDevice, s->stream));
	}
	s->bodiesDirty = false;
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
	int sticky = s->stickyError;
	s->stickyError = SPH_OK;
	return sticky;
}

#define SPH_LAUNCHED(s)                                 \
	do {                                                \
		(s)->launches++;                                \
		cudaError_t e_ = cudaGetLastError();            \
		if (e_ != cudaSuccess) return SPH_ERR_CUDA;     \
	} while (0)

int run_step(sph_sim *s, float dt) {
	const int n = (int)s->n;
	const int n0 = (int)s->n0;
	StepParams sp = step_params(s, dt);
	cudaStream_t st = s->stream;
	BufferSet &A = s->buf[s->cur];
	BufferSet &B = s->buf[1 - s->cur];
	SimTables T = tables(s);
	const int cellOrN = std::max(n, s->ncell);

	SPH_CUDA(cudaEventRecord(s->ev[kEvBegin], st));
	k_integrate<<<blocks_for(cellOrN, kElemThreads), kElemThreads, 0, st>>>(n, A.view(), T, sp);
	SPH_LAUNCHED(s);
	SPH_CUDA(cudaEventRecord(s->ev[kEvIntegrate], st));

	if (n0 > 0) {
		SPH_CUDA(cudaMemsetAsync(s->doneV, 0, sizeof(uint32_t) * s->ncell, st));
		SPH_CUDA(cudaMemsetAsync(T.taskCounter, 0, sizeof(int), st));
		k_viscosity<<<s->viscBlocks, kViscTaskWarps * kWarp, visc_smem_bytes(), st>>>(A.view(), [&] {
			SimTables v = T;
			v.done = s->doneV;
			return v;
		}(), sp);
		SPH_LAUNCHED(s);
	}
	SPH_CUDA(cudaEventRecord(s->ev[kEvVisc], st));

	k_predict<<<blocks_for(n, kElemThreads), kElemThreads, 0, st>>>(n, A.view(), T, sp);
	SPH_LAUNCHED(s);
	SPH_CUDA(cudaEventRecord(s->ev[kEvPredict], st));

	k_scan<<<1, kScanThreads, 0, st>>>(T, sp, s->maxNbSeed());
	SPH_LAUNCHED(s);
	k_scatter<<<blocks_for(n, kElemThreads), kElemThreads, 0, st>>>(n, n0, A.view(), T);
	SPH_LAUNCHED(s);
	k_grid_update<<<s->gridBlocks, kGridWarps * kWarp, 0, st>>>(n, A.view(), B.view(), T, sp);
	SPH_LAUNCHED(s);
	SPH_CUDA(cudaEventRecord(s->ev[kEvGrid], st));

	k_density<<<s->densBlocks, kDensWarps * kWarp, dens_smem_bytes(), st>>>(n, B.view(), T, sp);
	SPH_LAUNCHED(s);
	SPH_CUDA(cudaEventRecord(s->ev[kEvDensity], st));

	const size_t runs = (size_t)(n - n0 + kAppendixRun - 1) / kAppendixRun;
	SPH_CUDA(cudaMemsetAsync(s->doneD, 0, sizeof(uint32_t) * (s->ncell + runs), st));
	SPH_CUDA(cudaMemsetAsync(T.taskCounter + 1, 0, sizeof(int), st));
	{
		SimTables d = T;
		d.done = s->doneD;
		k_delta<<<s->deltaBlocks, kDeltaTaskWarps * kWarp, delta_smem_bytes(), st>>>(n, n0, B.view(), d, sp);
		SPH_LAUNCHED(s);
	}
	SPH_CUDA(cudaEventRecord(s->ev[kEvDelta], st));

	k_collide<<<blocks_for(cellOrN, kCollideThreads), kCollideThreads, 0, st>>>(n, A.view(), B.view(), T, sp);
	SPH_LAUNCHED(s);
	SPH_CUDA(cudaEventRecord(s->ev[kEvCollide], st));

	// The new cell arrays are the canonical ranges of the next step.
	s->cur = 1 - s->cur;
	std::swap(s->cellStartA, s->cellStartB);
	std::swap(s->cellCountA, s->cellCountB);
	s->n0 = s->n;
	s->timed = true;
	return SPH_OK;
}

}  // namespace

extern "C" {

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
	if (!(domain->cell_size > 0.0f) || !(domain->width > 0.0f) || !(domain->height > 0.0f) ||
	    domain->max_particles == 0 || domain->max_particles > (1u << 30))
		return SPH_ERR_INVALID_ARGUMENT;
	int devices = 0;
	if (cudaGetDeviceCount(&devices) != cudaSuccess || devices == 0) return SPH_ERR_NO_DEVICE;
	if (device < 0 || device >= devices) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(device));
	sph_sim *s = new (std::nothrow) sph_sim();
	if (!s) return SPH_ERR_CAPACITY;
	s->device = device;
	s->dom = *domain;
	s->gx = (int)(domain->width / domain->cell_size);
	s->gy = (int)(domain->height / domain->cell_size);
	if (s->gx <= 0 || s->gy <= 0 || (int64_t)s->gx * s->gy > (1 << 26)) {
		delete s;
		return SPH_ERR_INVALID_ARGUMENT;
	}
	s->ncell = s->gx * s->gy;
	sph_default_params(&s->params);
	int rc = SPH_OK;
	auto fail = [&](int code) {
		sph_destroy(s);
		return code;
	};
	if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(SPH_ERR_CUDA);
	for (int k = 0; k < kEvCount; ++k)
		if (cudaEventCreate(&s->ev[k]) != cudaSuccess) return fail(SPH_ERR_CUDA);
	const size_t N = domain->max_particles, C = (size_t)s->ncell;
	for (int b = 0; b < 2; ++b) {
		BufferSet &B = s->buf[b];
		if ((rc = dalloc(&B.pos, N)) || (rc = dalloc(&B.prev, N)) || (rc = dalloc(&B.vel, N)) ||
		    (rc = dalloc(&B.acc, N)) || (rc = dalloc(&B.dens, N)) || (rc = dalloc(&B.press, N)) ||
		    (rc = dalloc(&B.id, N)) || (rc = dalloc(&B.cellOf, N)))
			return fail(rc);
	}
	SimTables &T = s->T;
	if ((rc = dalloc(&s->cellStartA, C)) || (rc = dalloc(&s->cellCountA, C)) || (rc = dalloc(&s->cellStartB, C)) ||
	    (rc = dalloc(&s->cellCountB, C)) || (rc = dalloc(&T.rankOfCell, C)) || (rc = dalloc(&T.cellOfRank, C)) ||
	    (rc = dalloc(&T.appCount, C)) || (rc = dalloc(&T.appStart, C)) || (rc = dalloc(&T.appIdx, N)) ||
	    (rc = dalloc(&T.appCursor, C)) || (rc = dalloc(&T.newCell, N)) || (rc = dalloc(&T.enterCount, C)) ||
	    (rc = dalloc(&T.leaveCount, C)) || (rc = dalloc(&T.enterOffset, C)) || (rc = dalloc(&T.enterCursor, C)) ||
	    (rc = dalloc(&T.enterList, N)) || (rc = dalloc(&T.moverCount, 2)) || (rc = dalloc(&T.bbox, 4 * C)) ||
	    (rc = dalloc(&T.newIdx, N)) || (rc = dalloc(&T.newLabel, N)) || (rc = dalloc(&T.taskCounter, 2)) ||
	    (rc = dalloc(&T.stats, 4)) || (rc = dalloc(&T.error, 1)) || (rc = dalloc(&T.abort, 1)) ||
	    (rc = dalloc(&T.bodies, kMaxBodies)) || (rc = dalloc(&s->doneV, C)))
		return fail(rc);
	s->doneDCap = C + (N + kAppendixRun - 1) / kAppendixRun + 1;
	if ((rc = dalloc(&s->doneD, s->doneDCap))) return fail(rc);
	T.moverList = nullptr;

	// Colour-major cell rank: colour (y%3, x%3), then sub-colour
	// ((y/3)%2, (x/3)%2), then row-major.  Cells of one colour are >= 3 apart;
	// within a colour, the sub-colour order keeps conflicts between cells that
	// particles move across short.
	std::vector<int> order(C), rank(C);
	for (size_t c = 0; c < C; ++c) order[c] = (int)c;
	const int gx = s->gx;
	auto key = [gx](int c) {
		const int x = c % gx, y = c / gx;
		return (int64_t)(((y % 3) * 3 + (x % 3)) * 4 + ((y / 3) % 2) * 2 + ((x / 3) % 2)) * (int64_t)(1 << 26) + c;
	};
	std::sort(order.begin(), order.end(), [&](int a, int b) { return key(a) < key(b); });
	for (size_t r = 0; r < C; ++r) rank[order[r]] = (int)r;
	if (cudaMemcpy(T.cellOfRank, order.data(), C * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(T.rankOfCell, rank.data(), C * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
		return fail(SPH_ERR_CUDA);

	cudaDeviceProp prop;
	if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return fail(SPH_ERR_CUDA);
	s->numSMs = prop.multiProcessorCount;
	if (cudaFuncSetAttribute(k_viscosity, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)visc_smem_bytes()) !=
	        cudaSuccess ||
	    cudaFuncSetAttribute(k_delta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)delta_smem_bytes()) !=
	        cudaSuccess ||
	    cudaFuncSetAttribute(k_density, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dens_smem_bytes()) !=
	        cudaSuccess)
		return fail(SPH_ERR_CUDA);
	int occ = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_viscosity, kViscTaskWarps * kWarp, visc_smem_bytes()) !=
	        cudaSuccess ||
	    occ < 1)
		return fail(SPH_ERR_CUDA);
	s->viscBlocks = occ * s->numSMs;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_delta, kDeltaTaskWarps * kWarp, delta_smem_bytes()) !=
	        cudaSuccess ||
	    occ < 1)
		return fail(SPH_ERR_CUDA);
	s->deltaBlocks = occ * s->numSMs;
	s->densBlocks = std::max(1, std::min(blocks_for(C, kDensWarps), 64 * s->numSMs));
	s->gridBlocks = std::max(1, std::min(blocks_for(C, kGridWarps), 64 * s->numSMs));
	sph_reset_stats(s);
	if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(SPH_ERR_CUDA);
	*out = s;
	return SPH_OK;
}

int sph_destroy(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	cudaSetDevice(s->device);
	if (s->stream) cudaStreamSynchronize(s->stream);
	for (int b = 0; b < 2; ++b) {
		BufferSet &B = s->buf[b];
		cudaFree(B.pos);
		cudaFree(B.prev);
		cudaFree(B.vel);
		cudaFree(B.acc);
		cudaFree(B.dens);
		cudaFree(B.press);
		cudaFree(B.id);
		cudaFree(B.cellOf);
	}
	SimTables &T = s->T;
	void *ptrs[] = {s->cellStartA, s->cellCountA, s->cellStartB, s->cellCountB, T.rankOfCell, T.cellOfRank,
	                T.appCount,    T.appStart,    T.appIdx,      T.appCursor,   T.newCell,     T.enterCount,
	                T.leaveCount,  T.enterOffset, T.enterCursor, T.enterList,   T.moverCount,  T.bbox,
	                T.newIdx,      T.newLabel, T.taskCounter, T.stats,      T.error,       T.abort,
	                T.bodies,      s->doneV,      s->doneD,      s->stagePos,   s->stageForce, s->prof};
	for (void *p : ptrs)
		if (p) cudaFree(p);
	if (s->hostPos) cudaFreeHost(s->hostPos);
	if (s->hostForce) cudaFreeHost(s->hostForce);
	for (int k = 0; k < kEvCount; ++k)
		if (s->ev[k]) cudaEventDestroy(s->ev[k]);
	if (s->stream) cudaStreamDestroy(s->stream);
	delete s;
	return SPH_OK;
}

int sph_reset_stats(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	// SPHStatistics() (sph.h:143-149): both minimums start at the cell capacity.
	const uint32_t seed[4] = {s->dom.max_cell_particles, 0u, s->dom.max_cell_particles, 0u};
	SPH_CUDA(cudaMemcpyAsync(s->T.stats, seed, sizeof(seed), cudaMemcpyHostToDevice, s->stream));
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	s->timed = false;
	s->emitterMs = 0.0f;
	return SPH_OK;
}

int sph_clear_bodies(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	s->bodies.clear();
	s->bodiesDirty = true;
	return SPH_OK;
}

int sph_clear_particles(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	s->pendPos.clear();
	s->pendForce.clear();
	SPH_CUDA(cudaMemsetAsync(s->cellCountA, 0, sizeof(int) * s->ncell, s->stream));
	SPH_CUDA(cudaMemsetAsync(s->cellStartA, 0, sizeof(int) * s->ncell, s->stream));
	SPH_CUDA(cudaMemsetAsync(s->T.appCount, 0, sizeof(int) * s->ncell, s->stream));
	s->n = s->n0 = s->nDev = 0;
	return SPH_OK;
}

int sph_clear_emitters(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	s->emitters.clear();
	return SPH_OK;
}

static int push_body(sph_sim *s, const Body &b) {
	if (s->bodies.size() >= (size_t)kMaxBodies) return SPH_ERR_CAPACITY;
	s->bodies.push_back(b);
	s->bodiesDirty = true;
	return SPH_OK;
}

int sph_add_plane(sph_sim *s, sph_vec2 normal, float distance) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	Body b{};
	b.type = kBodyPlane;
	b.ax = normal.x;
	b.ay = normal.y;
	b.r = distance;
	return push_body(s, b);
}

int sph_add_circle(sph_sim *s, sph_vec2 pos, float radius) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	Body b{};
	b.type = kBodyCircle;
	b.ax = pos.x;
	b.ay = pos.y;
	b.r = radius;
	return push_body(s, b);
}

int sph_add_line_segment(sph_sim *s, sph_vec2 a, sph_vec2 bb) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	Body b{};
	b.type = kBodySegment;
	b.ax = a.x;
	b.ay = a.y;
	b.bx = bb.x;
	b.by = bb.y;
	return push_body(s, b);
}

int sph_add_polygon(sph_sim *s, size_t count, const sph_vec2 *verts) {
	if (!s || (count > 0 && !verts)) return SPH_ERR_INVALID_ARGUMENT;
	if (count > (size_t)kMaxPoly) return SPH_ERR_CAPACITY;
	Body b{};
	b.type = kBodyPolygon;
	b.vertexCount = (int)count;
	for (size_t k = 0; k < count; ++k) {
		b.verts[2 * k] = verts[k].x;
		b.verts[2 * k + 1] = verts[k].y;
	}
	return push_body(s, b);
}

int sph_add_particle(sph_sim *s, sph_vec2 position, sph_vec2 force, size_t *out_index) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	return push_particle(s, make_float2(position.x, position.y), make_float2(force.x, force.y), out_index);
}

int sph_add_particles(sph_sim *s, size_t count, const sph_vec2 *positions, const sph_vec2 *forces,
                      size_t *first_index) {
	if (!s || (count > 0 && !positions)) return SPH_ERR_INVALID_ARGUMENT;
	if (s->n + count > s->dom.max_particles) return SPH_ERR_CAPACITY;
	if (first_index) *first_index = s->n;
	for (size_t k = 0; k < count; ++k) {
		const float2 f = forces ? make_float2(forces[k].x, forces[k].y) : make_float2(0.0f, 0.0f);
		push_particle(s, make_float2(positions[k].x, positions[k].y), f, nullptr);
	}
	return SPH_OK;
}

int sph_add_volume(sph_sim *s, sph_vec2 center, sph_vec2 force, int count_x, int count_y, float spacing) {
	if (!s || count_x < 0 || count_y < 0) return SPH_ERR_INVALID_ARGUMENT;
	if (s->n + (size_t)count_x * (size_t)count_y > s->dom.max_particles) return SPH_ERR_CAPACITY;
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
			const float2 j = jitter(s);
			p = make_float2(j.x + p.x, j.y + p.y);
			push_particle(s, p, f, nullptr);
		}
	}
	return SPH_OK;
}

int sph_add_emitter(sph_sim *s, sph_vec2 position, sph_vec2 direction, float radius, float speed, float rate,
                    float duration) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	if (s->emitters.size() >= 8) return SPH_ERR_CAPACITY;  // kSPHMaxEmitterCount
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
	s->emitters.push_back(e);
	return SPH_OK;
}

int sph_update(sph_sim *s, float dt) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	if (!(dt > 0.0f)) return SPH_ERR_INVALID_ARGUMENT;
	SPH_CUDA(cudaSetDevice(s->device));
	int rc = flush_adds(s);
	if (rc) return rc;
	const auto t0 = std::chrono::high_resolution_clock::now();
	for (Emitter &e : s->emitters) {
		rc = update_emitter(s, e, dt);
		if (rc) return rc;
	}
	rc = flush_adds(s);
	if (rc) return rc;
	s->emitterMs = (float)std::chrono::duration_cast<std::chrono::nanoseconds>(
	                   std::chrono::high_resolution_clock::now() - t0)
	                   .count() *
	               (1.0f / 1000000);
	rc = upload_bodies(s);
	if (rc) return rc;
	if (s->n == 0) {
		const uint32_t seed[2] = {s->dom.max_neighbors, 0u};
		SPH_CUDA(cudaMemcpyAsync(s->T.stats, seed, sizeof(seed), cudaMemcpyHostToDevice, s->stream));
		s->timed = false;
		return SPH_OK;
	}
	return run_step(s, dt);
}

int sph_add_external_forces(sph_sim *s, sph_vec2 f) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	s->external = sph_vec2{f.x + s->external.x, f.y + s->external.y};
	return SPH_OK;
}

int sph_clear_external_force(sph_sim *s) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	s->external = sph_vec2{0.0f, 0.0f};
	return SPH_OK;
}

int sph_get_particle_count(sph_sim *s, size_t *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->n;
	return SPH_OK;
}

int sph_set_gravity(sph_sim *s, sph_vec2 g) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	s->gravity = g;
	return SPH_OK;
}

int sph_get_params(sph_sim *s, sph_params *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->params;
	return SPH_OK;
}

int sph_set_params(sph_sim *s, const sph_params *p) {
	if (!s || !p) return SPH_ERR_INVALID_ARGUMENT;
	s->params = *p;
	return SPH_OK;
}

int sph_get_stats(sph_sim *s, sph_stats *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	rc = check_device_errors(s);
	uint32_t st[4];
	SPH_CUDA(cudaMemcpy(st, s->T.stats, sizeof(st), cudaMemcpyDeviceToHost));
	out->min_particle_neighbor_count = st[0];
	out->max_particle_neighbor_count = st[1];
	out->min_cell_particle_count = st[2];
	out->max_cell_particle_count = st[3];
	out->time_emitters = s->emitterMs;
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
	out->time_neighbor_search = 0.0f;  // the grid update builds the neighbour structure
	out->time_density_and_pressure = t[kEvDensity];
	out->time_delta_positions = t[kEvDelta];
	out->time_collisions = t[kEvCollide];
	return rc;
}

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
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	if (count > s->n) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	const int n = (int)s->n;
	BufferSet &A = s->buf[s->cur];
	BufferSet &Z = s->buf[1 - s->cur];  // free between updates: scratch
	struct Item {
		float2 *src, *scratch;
		sph_vec2 *dst;
	} items[] = {{A.pos, Z.pos, pos}, {A.prev, Z.prev, prev}, {A.vel, Z.vel, vel},
	             {A.acc, Z.acc, acc}, {A.dens, Z.dens, dens}, {A.press, Z.press, press}};
	for (const Item &it : items) {
		if (!it.dst || count == 0) continue;
		k_gather_by_id<<<blocks_for(n, kElemThreads), kElemThreads, 0, s->stream>>>(n, A.id, it.src, it.scratch);
		SPH_LAUNCHED(s);
		SPH_CUDA(cudaMemcpyAsync(it.dst, it.scratch, count * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
	}
	return check_device_errors(s);
}

int sph_state_info(sph_sim *s, size_t *count, size_t *canonical, int *gx, int *gy) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	if (count) *count = s->n;
	if (canonical) *canonical = s->n0;
	if (gx) *gx = s->gx;
	if (gy) *gy = s->gy;
	return SPH_OK;
}

int sph_dump_state(sph_sim *s, const sph_state_view *v) {
	if (!s || !v) return SPH_ERR_INVALID_ARGUMENT;
	int rc = flush_adds(s);
	if (rc) return rc;
	if (v->count != s->n) return SPH_ERR_INVALID_ARGUMENT;
	const size_t n = s->n;
	BufferSet &A = s->buf[s->cur];
	cudaStream_t st = s->stream;
	auto d2h = [&](void *dst, const void *src, size_t bytes) -> int {
		if (!dst || bytes == 0) return SPH_OK;
		return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
	};
	if ((rc = d2h(v->pos, A.pos, n * 8)) || (rc = d2h(v->prev, A.prev, n * 8)) || (rc = d2h(v->vel, A.vel, n * 8)) ||
	    (rc = d2h(v->acc, A.acc, n * 8)) || (rc = d2h(v->dens, A.dens, n * 8)) ||
	    (rc = d2h(v->press, A.press, n * 8)) || (rc = d2h(v->id, A.id, n * 4)) ||
	    (rc = d2h(v->cell, A.cellOf, n * 4)) || (rc = d2h(v->cell_start, s->cellStartA, s->ncell * 4)) ||
	    (rc = d2h(v->cell_count, s->cellCountA, s->ncell * 4)))
		return rc;
	return check_device_errors(s);
}

int sph_load_state(sph_sim *s, const sph_state_view *v) {
	if (!s || !v) return SPH_ERR_INVALID_ARGUMENT;
	if (!v->pos || !v->prev || !v->vel || !v->acc || !v->dens || !v->press || !v->id || !v->cell ||
	    !v->cell_start || !v->cell_count)
		return SPH_ERR_INVALID_ARGUMENT;
	if (v->count > s->dom.max_particles || v->canonical_count > v->count) return SPH_ERR_INVALID_ARGUMENT;
	if (v->grid_x != s->gx || v->grid_y != s->gy) return SPH_ERR_INVALID_ARGUMENT;
	const size_t n = v->count;
	// Validate the cell tables so that no kernel can index out of range.
	size_t total = 0;
	for (int c = 0; c < s->ncell; ++c) {
		if (v->cell_count[c] < 0 || v->cell_start[c] < 0) return SPH_ERR_INVALID_ARGUMENT;
		if ((size_t)v->cell_start[c] + (size_t)v->cell_count[c] > v->canonical_count) return SPH_ERR_INVALID_ARGUMENT;
		total += (size_t)v->cell_count[c];
	}
	if (total != v->canonical_count) return SPH_ERR_INVALID_ARGUMENT;
	std::vector<int> app(s->ncell, 0);
	for (size_t k = 0; k < n; ++k) {
		if (v->cell[k] < 0 || v->cell[k] >= s->ncell) return SPH_ERR_INVALID_ARGUMENT;
		if (k >= v->canonical_count) app[v->cell[k]]++;
	}
	for (size_t k = 0; k < v->canonical_count; ++k) {
		const int c = v->cell[k];
		if ((int)k < v->cell_start[c] || (int)k >= v->cell_start[c] + v->cell_count[c])
			return SPH_ERR_INVALID_ARGUMENT;
	}
	s->pendPos.clear();
	s->pendForce.clear();
	BufferSet &A = s->buf[s->cur];
	cudaStream_t st = s->stream;
	auto h2d = [&](void *dst, const void *src, size_t bytes) -> int {
		if (bytes == 0) return SPH_OK;
		return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
	};
	int rc;
	if ((rc = h2d(A.pos, v->pos, n * 8)) || (rc = h2d(A.prev, v->prev, n * 8)) || (rc = h2d(A.vel, v->vel, n * 8)) ||
	    (rc = h2d(A.acc, v->acc, n * 8)) || (rc = h2d(A.dens, v->dens, n * 8)) ||
	    (rc = h2d(A.press, v->press, n * 8)) || (rc = h2d(A.id, v->id, n * 4)) ||
	    (rc = h2d(A.cellOf, v->cell, n * 4)) || (rc = h2d(s->cellStartA, v->cell_start, s->ncell * 4)) ||
	    (rc = h2d(s->cellCountA, v->cell_count, s->ncell * 4)))
		return rc;
	SPH_CUDA(cudaMemcpyAsync(s->T.appCount, app.data(), s->ncell * 4, cudaMemcpyHostToDevice, st));
	SPH_CUDA(cudaStreamSynchronize(st));  // `app` is a host temporary
	s->n = s->nDev = n;
	s->n0 = v->canonical_count;
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
extern "C" int sph_profile_tasks(sph_sim *s, int enable) {
	if (!s) return SPH_ERR_INVALID_ARGUMENT;
	if (enable && !s->prof) {
		SPH_CUDA(cudaMalloc(&s->prof, sizeof(unsigned long long) * 8 * s->doneDCap));
		SPH_CUDA(cudaMemset(s->prof, 0, sizeof(unsigned long long) * 8 * s->doneDCap));
	} else if (!enable && s->prof) {
		cudaFree(s->prof);
		s->prof = nullptr;
	}
	return SPH_OK;
}

extern "C" int sph_profile_read(sph_sim *s, unsigned long long *out, size_t capacity, size_t *stride) {
	if (!s || !stride) return SPH_ERR_INVALID_ARGUMENT;
	*stride = s->doneDCap;
	if (!s->prof || !out) return SPH_OK;
	const size_t total = std::min(capacity, (size_t)8 * s->doneDCap);
	SPH_CUDA(cudaStreamSynchronize(s->stream));
	SPH_CUDA(cudaMemcpy(out, s->prof, total * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
	return SPH_OK;
}

int sph_kernel_launches(sph_sim *s, uint64_t *out) {
	if (!s || !out) return SPH_ERR_INVALID_ARGUMENT;
	*out = s->launches;
	return SPH_OK;
}

}  // extern "C"
