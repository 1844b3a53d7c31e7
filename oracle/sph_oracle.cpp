// Test infrastructure (oracle): CPU restatement of the reference's Demo4 SPH
// step.  Only tests, __graft_entry__.smoke() and bench.py's CPU baseline may
// load the library this file builds; the product never does.
//
// It restates NBodySimulation/demo4.cpp:37-451 and sph.h:439-681 stage by
// stage, in the same serial order and with the same floating-point operation
// sequence (built with -ffp-contract=off), templated on the scalar type so the
// same step also runs in FP64.  Differences from the reference are only in
// what the reference fixes at compile time: the domain (sph.h:18-23), the grid
// derived from it (sph.h:60-65) and the capacities (sph.h:68-72) are runtime
// values here, so scenes larger than the reference's 10 x 5.625 box and 10,000
// particles can be checked.  With the reference's domain and one worker the
// FP32 instantiation is bit-identical to the reference (pinned by tests
// against the reference compiled headless, oracle/ref_harness.cpp).
//
// The data layout deliberately mirrors the reference (48-byte AoS particle
// record, a fixed-capacity 64-bit neighbour array per particle, fixed-capacity
// cells), so that its multi-worker mode is a fair CPU baseline.  Multi-worker
// mode reproduces the reference's ThreadPool chunking (threading.h:111-129)
// and, like the reference, lets workers scatter into shared neighbours without
// locks; here the shared loads and stores are relaxed atomics, which keeps the
// race well-defined in C++ while generating the same plain loads and stores.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "sph_oracle.h"

namespace {

template <typename T>
struct V2 {
	T x, y;
	V2() : x(0), y(0) {}
	V2(T a, T b) : x(a), y(b) {}
};

template <typename T> inline V2<T> mul(const V2<T> &v, T s) { return V2<T>(v.x * s, v.y * s); }
template <typename T> inline V2<T> add(const V2<T> &p, const V2<T> &q) { return V2<T>(p.x + q.x, p.y + q.y); }
template <typename T> inline V2<T> sub(const V2<T> &p, const V2<T> &q) { return V2<T>(p.x - q.x, p.y - q.y); }
template <typename T> inline T dot(const V2<T> &p, const V2<T> &q) { return p.x * q.x + p.y * q.y; }
template <typename T> inline T sqrt_t(T v) { return std::sqrt(v); }
template <typename T> inline V2<T> normalize(const V2<T> &v) {
	T len = sqrt_t(v.x * v.x + v.y * v.y);
	if (len == 0) len = 1;
	T inv = T(1) / len;
	return mul(v, inv);
}

// Relaxed atomic access to a scalar that other workers may scatter into.
template <typename T> inline T ld(const T &v) { return std::atomic_ref<T>(const_cast<T &>(v)).load(std::memory_order_relaxed); }
template <typename T> inline void st(T &v, T x) { std::atomic_ref<T>(v).store(x, std::memory_order_relaxed); }

// ThreadPool equivalent: contiguous [start, end] chunks of max(1, n/threads)
// items (threading.h:111-129), executed by a fixed set of workers; the caller
// waits until all chunks are done (threading.h:101-109).
class ChunkPool {
public:
	explicit ChunkPool(size_t threads) : threads_(std::max<size_t>(1, threads)) {
		for (size_t w = 0; w < threads_; ++w) workers_.emplace_back([this] { Loop(); });
	}
	~ChunkPool() {
		{
			std::lock_guard<std::mutex> g(m_);
			stop_ = true;
		}
		cv_.notify_all();
		for (auto &t : workers_) t.join();
	}
	size_t threads() const { return threads_; }
	void Run(size_t items, const std::function<void(size_t, size_t)> &fn) {
		if (items == 0) return;
		size_t per = std::max<size_t>(1, items / threads_);
		std::vector<std::pair<size_t, size_t>> chunks;
		for (size_t s = 0; s < items; s += per) chunks.push_back({s, std::min(s + per - 1, items - 1)});
		{
			std::lock_guard<std::mutex> g(m_);
			chunks_ = std::move(chunks);
			fn_ = &fn;
			next_ = 0;
			pending_ = chunks_.size();
			++generation_;
		}
		cv_.notify_all();
		std::unique_lock<std::mutex> lk(m_);
		done_cv_.wait(lk, [this] { return pending_ == 0; });
		fn_ = nullptr;
	}

private:
	void Loop() {
		uint64_t seen = 0;
		for (;;) {
			std::unique_lock<std::mutex> lk(m_);
			cv_.wait(lk, [&] { return stop_ || (generation_ != seen && next_ < chunks_.size()); });
			if (stop_) return;
			while (next_ < chunks_.size()) {
				std::pair<size_t, size_t> c = chunks_[next_++];
				const std::function<void(size_t, size_t)> *fn = fn_;
				lk.unlock();
				(*fn)(c.first, c.second);
				lk.lock();
				if (--pending_ == 0) done_cv_.notify_all();
			}
			seen = generation_;
		}
	}
	size_t threads_;
	std::vector<std::thread> workers_;
	std::mutex m_;
	std::condition_variable cv_, done_cv_;
	std::vector<std::pair<size_t, size_t>> chunks_;
	const std::function<void(size_t, size_t)> *fn_ = nullptr;
	size_t next_ = 0, pending_ = 0;
	uint64_t generation_ = 0;
	bool stop_ = false;
};

enum BodyKind { kPlane = 1, kCircle = 2, kSegment = 3, kPolygon = 4 };

template <typename T>
struct Body {
	int kind = 0;
	V2<T> a, b;  // plane: normal, (distance in r); circle: centre; segment: a, b
	T r = 0;
	V2<T> verts[SPH_ORACLE_MAX_POLY];
	size_t vertexCount = 0;
};

template <typename T>
struct Emitter {
	V2<T> position, direction;
	T radius, speed, rate, duration, elapsed, totalElapsed;
	int active;
};

// The simulation interface every instantiation implements.
struct SimBase {
	virtual ~SimBase() {}
	virtual void ResetStats() = 0;
	virtual void ClearBodies() = 0;
	virtual void ClearParticles() = 0;
	virtual void ClearEmitters() = 0;
	virtual int AddPlane(float nx, float ny, float d) = 0;
	virtual int AddCircle(float x, float y, float r) = 0;
	virtual int AddSegment(float ax, float ay, float bx, float by) = 0;
	virtual int AddPolygon(size_t n, const float *xy) = 0;
	virtual int64_t AddParticle(float x, float y, float fx, float fy) = 0;
	virtual int AddVolume(float cx, float cy, float fx, float fy, int nx, int ny, float spacing) = 0;
	virtual int AddEmitter(float px, float py, float dx, float dy, float radius, float speed, float rate, float duration) = 0;
	virtual int Update(float dt) = 0;
	virtual void SetGravity(float x, float y) = 0;
	virtual void AddExternalForce(float x, float y) = 0;
	virtual void ClearExternalForce() = 0;
	virtual void SetParams(const float *p) = 0;
	virtual void GetParams(float *p) = 0;
	virtual size_t Count() = 0;
	virtual void SetSpringSerial(int serial) = 0;
	virtual void GetParticles(double *pos, double *prev, double *acc, double *vel, double *dens, double *press) = 0;
	virtual void GetIndex(int *cellXY, uint64_t *inCell, uint64_t *nbCount) = 0;
	virtual void GetNeighbors(size_t i, uint64_t *out) = 0;
	virtual uint64_t GetCell(int c, uint64_t *out) = 0;
	virtual int SetState(size_t n, const double *pos, const double *prev, const double *acc, const double *vel,
	                     const double *dens, const double *press, const int *cellXY, const uint64_t *inCell,
	                     const uint64_t *nbCount, const uint64_t *nb, const uint64_t *cellCount,
	                     const uint64_t *cellIdx) = 0;
	virtual void GetStats(uint64_t *counts, float *times) = 0;
	virtual size_t Workers() = 0;
	virtual void SetWorkers(size_t w) = 0;
	virtual void SetSprings(int enabled, float yield, float plasticity, float stiffness, int maxPer) = 0;
	virtual int SetSpringState(size_t n, const int32_t *count, const int32_t *partner, const float *rest,
	                           const int64_t *tag) = 0;
	virtual void GetSpringState(int32_t *count, int32_t *partner, float *rest) = 0;
	virtual uint64_t SpringTotal() = 0;
};

template <typename T>
struct Sim : SimBase {
	// Particle record laid out like demo4.h ParticleData.
	struct Particle {
		V2<T> cur, prev, acc, vel;
		T density, nearDensity, pressure, nearPressure;
	};

	sph_oracle_domain dom;
	T halfW, halfH, cellSize;
	int gx, gy;
	size_t capN, capCell, capNb;

	T h, cellSizeParam, spacing, invH, rho0, k, kNear, sigma, beta;
	V2<T> gravity, extForce;

	size_t n = 0;
	std::vector<Particle> parts;
	std::vector<int> cellX, cellY;
	std::vector<size_t> inCell, nbCount, nb;
	std::vector<size_t> cellIdx, cellCnt;

	std::vector<Body<T>> bodies;
	std::vector<Emitter<T>> emitters;

	uint64_t statMinNb, statMaxNb, statMinCell, statMaxCell;
	float times[9];
	int error = 0;

	size_t workers = 1;
	ChunkPool *pool = nullptr;

	// Viscoelastic springs (not in the reference; Clavet et al. 2005,
	// "Particle-based viscoelastic fluid simulation", Algorithms 3 and 4):
	// up to kSprings per particle, stored at both ends, partner = particle
	// index, rest length per spring; tag = AddParticle index (tie-break).
	static constexpr int kSprings = 16;
	int springsOn = 0, springMax = kSprings;
	int springSerial = 0;  // 1: displacements applied one spring at a time (Clavet 2005, Algorithm 3)
	T springYield = 0, springPlastic = 0, springK = 0;
	std::vector<int32_t> sN, sP, accN, accP;
	std::vector<T> sL;
	std::vector<int64_t> tag;
	std::vector<V2<T>> springPos;
	uint64_t springTotal = 0;

	explicit Sim(const sph_oracle_domain &d) : dom(d) {
		halfW = T(d.width * 0.5f);
		halfH = T(d.height * 0.5f);
		cellSize = T(d.cell_size);
		gx = (int)(d.width / d.cell_size);
		gy = (int)(d.height / d.cell_size);
		capN = d.max_particles;
		capCell = d.max_cell_particles;
		capNb = d.max_neighbors;
		parts.resize(capN);
		cellX.resize(capN);
		cellY.resize(capN);
		inCell.resize(capN);
		nbCount.resize(capN);
		nb.resize(capN * capNb);
		cellIdx.resize((size_t)gx * gy * capCell);
		cellCnt.assign((size_t)gx * gy, 0);
		tag.resize(capN);
		float defaults[9];
		sph_oracle_default_params(defaults);
		SetParams(defaults);
		ResetStats();
	}
	~Sim() { delete pool; }

	// sph.h:439-463
	bool InGrid(int x, int y) const { return x >= 0 && x < gx && y >= 0 && y < gy; }
	size_t CellOffset(int x, int y) const { return (size_t)y * gx + x; }
	void CellOf(const V2<T> &p, int *cx, int *cy) const {
		int x = (int)((p.x + halfW) / cellSize);
		int y = (int)((p.y + halfH) / cellSize);
		*cx = std::min(std::max(x, 0), gx - 1);
		*cy = std::min(std::max(y, 0), gy - 1);
	}

	// demo4.cpp:37-54
	void Insert(size_t i) {
		int cx, cy;
		CellOf(parts[i].cur, &cx, &cy);
		size_t c = CellOffset(cx, cy);
		if (cellCnt[c] >= capCell) { error = SPH_ORACLE_ERR_CAPACITY; return; }
		size_t slot = cellCnt[c]++;
		cellIdx[c * capCell + slot] = i;
		cellX[i] = cx;
		cellY[i] = cy;
		inCell[i] = slot;
		statMinCell = std::min<uint64_t>(cellCnt[c], statMinCell);
		statMaxCell = std::max<uint64_t>(cellCnt[c], statMaxCell);
	}

	// demo4.cpp:56-76
	void Remove(size_t i) {
		size_t c = CellOffset(cellX[i], cellY[i]);
		size_t at = inCell[i];
		size_t last = cellCnt[c] - 1;
		if (at != last) {
			cellIdx[c * capCell + at] = cellIdx[c * capCell + last];
			cellIdx[c * capCell + last] = i;
			inCell[cellIdx[c * capCell + at]] = at;
		}
		--cellCnt[c];
		statMinCell = std::min<uint64_t>(cellCnt[c], statMinCell);
		statMaxCell = std::max<uint64_t>(cellCnt[c], statMaxCell);
	}

	void ResetStats() override {
		// SPHStatistics() (sph.h:143-149): note both minimums start at the
		// cell capacity constant.
		statMinNb = dom.stats_min_init;
		statMaxNb = 0;
		statMinCell = dom.stats_min_init;
		statMaxCell = 0;
		for (float &t : times) t = 0;
	}
	void ClearBodies() override { bodies.clear(); }
	void ClearParticles() override {
		std::fill(cellCnt.begin(), cellCnt.end(), 0);
		n = 0;
	}
	void ClearEmitters() override { emitters.clear(); }

	int PushBody(const Body<T> &b) {
		if (bodies.size() >= SPH_ORACLE_MAX_BODIES) return SPH_ORACLE_ERR_CAPACITY;
		bodies.push_back(b);
		return 0;
	}
	int AddPlane(float nx, float ny, float d) override {
		Body<T> b;
		b.kind = kPlane;
		b.a = V2<T>(nx, ny);
		b.r = d;
		return PushBody(b);
	}
	int AddCircle(float x, float y, float r) override {
		Body<T> b;
		b.kind = kCircle;
		b.a = V2<T>(x, y);
		b.r = r;
		return PushBody(b);
	}
	int AddSegment(float ax, float ay, float bx, float by) override {
		Body<T> b;
		b.kind = kSegment;
		b.a = V2<T>(ax, ay);
		b.b = V2<T>(bx, by);
		return PushBody(b);
	}
	int AddPolygon(size_t count, const float *xy) override {
		if (count > SPH_ORACLE_MAX_POLY) return SPH_ORACLE_ERR_CAPACITY;
		Body<T> b;
		b.kind = kPolygon;
		for (size_t k = 0; k < count; ++k) b.verts[k] = V2<T>(xy[2 * k], xy[2 * k + 1]);
		b.vertexCount = count;
		return PushBody(b);
	}

	// demo4.cpp:142-153
	int64_t AddParticleT(const V2<T> &p, const V2<T> &force) {
		if (n >= capN) { error = SPH_ORACLE_ERR_CAPACITY; return -1; }
		size_t i = n++;
		Particle &q = parts[i];
		q.cur = q.prev = p;
		q.vel = V2<T>();
		q.acc = force;
		q.density = q.nearDensity = q.pressure = q.nearPressure = 0;
		nbCount[i] = 0;
		inCell[i] = 0;
		tag[i] = (int64_t)i;
		if (springsOn) sN[i] = 0;
		Insert(i);
		return (int64_t)i;
	}
	int64_t AddParticle(float x, float y, float fx, float fy) override {
		return AddParticleT(V2<T>(x, y), V2<T>(fx, fy));
	}

	// Vec2RandomDirection (vecmath.h:317-322), the reference's jitter source.
	static V2<T> RandomDirection() {
		float d = rand() / (float)RAND_MAX;
		float angle = d * ((float)M_PI * 2.0f);
		return V2<T>(cosf(angle), sinf(angle));
	}

	// demo4.cpp:169-181; jitter scale kSPHKernelHeight * 0.01 (sph.h:36, 51).
	int AddVolume(float cxf, float cyf, float fxf, float fyf, int nx, int ny, float spacingf) override {
		const T sp = spacingf;
		const V2<T> center(cxf, cyf), force(fxf, fyf);
		V2<T> offset = mul(V2<T>(T(nx) * sp, T(ny) * sp), T(0.5f));
		for (int yi = 0; yi < ny; ++yi) {
			for (int xi = 0; xi < nx; ++xi) {
				V2<T> p = mul(V2<T>((T)(float)xi, (T)(float)yi), sp);
				p = add(V2<T>(sp * T(0.5f), sp * T(0.5f)), p);
				p = add(sub(center, offset), p);
				V2<T> jitter = mul(mul(RandomDirection(), T(dom.jitter_kernel_height)), T(0.01f));
				p = add(jitter, p);
				if (AddParticleT(p, force) < 0) return SPH_ORACLE_ERR_CAPACITY;
			}
		}
		return 0;
	}

	int AddEmitter(float px, float py, float dx, float dy, float radius, float speed, float rate, float duration) override {
		if (emitters.size() >= SPH_ORACLE_MAX_EMITTERS) return SPH_ORACLE_ERR_CAPACITY;
		Emitter<T> e;
		e.position = V2<T>(px, py);
		e.direction = V2<T>(dx, dy);
		e.radius = radius;
		e.speed = speed;
		e.rate = rate;
		e.duration = duration;
		e.elapsed = 0;
		e.totalElapsed = 0;
		e.active = 1;
		emitters.push_back(e);
		return 0;
	}

	// demo4.cpp:257-284
	void UpdateEmitter(Emitter<T> &e, T dt) {
		const T sp = spacing;
		const T invDt = T(1) / dt;
		if (!e.active) return;
		const T rate = T(1) / e.rate;
		e.elapsed += dt;
		e.totalElapsed += dt;
		if (e.elapsed >= rate) {
			e.elapsed = 0;
			V2<T> accel = mul(mul(e.direction, e.speed), invDt);
			V2<T> dir(-T(1) * e.direction.y, T(1) * e.direction.x);  // Vec2Cross(1, d)
			int count = (int)std::floor(e.radius / sp);
			V2<T> offset = mul(mul(mul(dir, (T)(float)count), sp), T(0.5f));
			for (int k = 0; k < count; ++k) {
				V2<T> p = mul(mul(dir, (T)(float)k), sp);
				p = add(mul(mul(dir, sp), T(0.5f)), p);
				p = add(sub(e.position, offset), p);
				V2<T> jitter = mul(mul(RandomDirection(), T(dom.jitter_kernel_height)), T(0.01f));
				p = add(jitter, p);
				AddParticleT(p, accel);
			}
		}
		if (e.totalElapsed >= e.duration) e.active = 0;
	}

	// demo4.cpp:183-206: every particle of the clamped 3x3 cell block, y-major,
	// then x, then cell array order; self included, no distance filter.
	void NeighborSearch(size_t s, size_t e) {
		for (size_t a = s; a <= e; ++a) {
			size_t cnt = 0;
			for (int y = -1; y <= 1; ++y) {
				for (int x = -1; x <= 1; ++x) {
					int px = cellX[a] + x, py = cellY[a] + y;
					if (!InGrid(px, py)) continue;
					size_t c = CellOffset(px, py);
					for (size_t k = 0; k < cellCnt[c]; ++k) {
						if (cnt >= capNb) { error = SPH_ORACLE_ERR_CAPACITY; break; }
						nb[a * capNb + cnt++] = cellIdx[c * capCell + k];
					}
				}
			}
			nbCount[a] = cnt;
		}
	}

	// demo4.cpp:208-221 + sph.h:465-481
	void DensityAndPressure(size_t s, size_t e) {
		const T h2 = h * h;
		for (size_t i = s; i <= e; ++i) {
			Particle &pi = parts[i];
			T d0 = 0, d1 = 0;
			const V2<T> xi = pi.cur;
			for (size_t k = 0; k < nbCount[i]; ++k) {
				const V2<T> xj = parts[nb[i * capNb + k]].cur;
				V2<T> r = sub(xj, xi);
				T r2 = dot(r, r);
				if (r2 < h2) {
					T rij = sqrt_t(r2);
					T term = T(1) - rij * invH;
					d0 += term * term;
					d1 += term * term * term;
				}
			}
			pi.density = d0;
			pi.nearDensity = d1;
			pi.pressure = k * (d0 - rho0);
			pi.nearPressure = kNear * d1;
		}
	}

	// demo4.cpp:223-237 + sph.h:497-512.  v_i and v_j change inside the loop.
	void Viscosity(size_t s, size_t e, T dt) {
		const T h2 = h * h;
		for (size_t i = s; i <= e; ++i) {
			Particle &pi = parts[i];
			for (size_t k = 0; k < nbCount[i]; ++k) {
				Particle &pj = parts[nb[i * capNb + k]];
				V2<T> xi(ld(pi.cur.x), ld(pi.cur.y)), xj(ld(pj.cur.x), ld(pj.cur.y));
				V2<T> vi(ld(pi.vel.x), ld(pi.vel.y)), vj(ld(pj.vel.x), ld(pj.vel.y));
				V2<T> force;
				V2<T> r = sub(xj, xi);
				T r2 = dot(r, r);
				if (r2 < h2) {
					T rij = sqrt_t(r2);
					T q = rij * invH;
					V2<T> nrm = normalize(r);
					T u = dot(sub(vi, vj), nrm);
					if (u > T(0)) {
						T f = (T(1) - q) * (sigma * u + beta * (u * u));
						force = V2<T>(f * nrm.x, f * nrm.y);
					}
				}
				V2<T> imp = mul(mul(force, T(0.5f)), dt);
				st(pi.vel.x, ld(pi.vel.x) - imp.x);
				st(pi.vel.y, ld(pi.vel.y) - imp.y);
				st(pj.vel.x, imp.x + ld(pj.vel.x));
				st(pj.vel.y, imp.y + ld(pj.vel.y));
			}
		}
	}

	// demo4.cpp:239-255 + sph.h:483-495.  x_j moves inside the loop, x_i after.
	void Delta(size_t s, size_t e, T dt) {
		const T h2 = h * h;
		for (size_t i = s; i <= e; ++i) {
			Particle &pi = parts[i];
			V2<T> dx;
			for (size_t k = 0; k < nbCount[i]; ++k) {
				Particle &pj = parts[nb[i * capNb + k]];
				V2<T> xi(ld(pi.cur.x), ld(pi.cur.y)), xj(ld(pj.cur.x), ld(pj.cur.y));
				V2<T> delta;
				V2<T> r = sub(xj, xi);
				T r2 = dot(r, r);
				if (r2 < h2) {
					T rij = sqrt_t(r2);
					V2<T> nrm = normalize(r);
					T term = T(1) - rij * invH;
					T d = (dt * dt) * (pi.pressure * term + pi.nearPressure * (term * term));
					delta = V2<T>(d * nrm.x, d * nrm.y);
				}
				V2<T> half = mul(delta, T(0.5f));
				st(pj.cur.x, half.x + ld(pj.cur.x));
				st(pj.cur.y, half.y + ld(pj.cur.y));
				dx = sub(dx, half);
			}
			st(pi.cur.x, dx.x + ld(pi.cur.x));
			st(pi.cur.y, dx.y + ld(pi.cur.y));
		}
	}

	// sph.h:514-524; collision radius kSPHParticleCollisionRadius = 0.05.
	void SolvePlane(V2<T> *pos, const V2<T> &normal, T distance) const {
		const T radius = T(dom.particle_radius);
		V2<T> p = mul(normal, distance);
		V2<T> x = *pos;
		T proj = dot(sub(x, p), normal);
		if (proj <= radius) {
			T pen = radius - proj;
			*pos = add(mul(normal, pen), x);
		}
	}

	// sph.h:526-542
	void SolveCircle(V2<T> *pos, const V2<T> &c, T cr) const {
		const T both = cr + T(dom.particle_radius);
		V2<T> x = *pos;
		V2<T> d = sub(x, c);
		T d2 = dot(d, d);
		if (d2 <= both * both) {
			if (std::fabs(d2) > T(0)) {
				T dist = sqrt_t(d2);
				V2<T> nrm = mul(d, T(1) / dist);
				T pen = both - dist;
				*pos = add(mul(nrm, pen), x);
			}
		}
	}

	// sph.h:544-598; margin kSPHCollisionMargin = 0.01.
	void SolveSegment(V2<T> *pos, const V2<T> &a, const V2<T> &b) const {
		const T both = T(dom.collision_margin) + T(dom.particle_radius);
		V2<T> x = *pos;
		V2<T> e = sub(b, a);
		T u = dot(e, sub(b, x));
		T v = dot(e, sub(x, a));
		V2<T> closest, nrm;
		if (v <= T(0)) {
			closest = a;
			V2<T> d = sub(x, closest);
			if (dot(d, d) > both * both) return;
			nrm = normalize(sub(x, closest));
		} else if (u <= T(0)) {
			closest = b;
			V2<T> d = sub(x, closest);
			if (dot(d, d) > both * both) return;
			nrm = normalize(sub(x, closest));
		} else {
			T den = dot(e, e);
			closest = mul(add(mul(a, u), mul(b, v)), T(1) / den);
			V2<T> d = sub(x, closest);
			if (dot(d, d) > both * both) return;
			nrm = V2<T>(-e.y, e.x);
			if (dot(nrm, sub(x, a)) < T(0)) nrm = V2<T>(-nrm.x, -nrm.y);
			nrm = normalize(nrm);
		}
		T dist = dot(nrm, sub(x, closest));
		T pen = both - dist;
		*pos = add(mul(nrm, pen), x);
	}

	// sph.h:600-681, including the reference's Vec2DistanceSquared, which
	// squares the product of the coordinate differences (vecmath.h:292-296).
	void SolvePolygon(V2<T> *pos, size_t count, const V2<T> *verts) const {
		const T radius = T(dom.collision_margin) + T(dom.particle_radius);
		const V2<T> c = *pos;
		size_t edge = 0;
		V2<T> normal;
		T separation = -T(FLT_MAX_VALUE);
		for (size_t k = 0; k < count; ++k) {
			V2<T> a = verts[k], b = verts[(k + 1) % count];
			V2<T> ab = sub(b, a);
			V2<T> nrm = normalize(V2<T>(T(1) * ab.y, -T(1) * ab.x));  // Vec2Cross(v, 1)
			T s = dot(nrm, sub(c, a));
			if (s > radius) return;
			if (s > separation) {
				normal = nrm;
				separation = s;
				edge = k;
			}
		}
		V2<T> v1 = verts[edge], v2 = verts[(edge + 1) % count];
		V2<T> mtv;
		if (separation < T(FLT_EPSILON_VALUE)) {
			mtv = mul(normal, radius - separation);
		} else {
			T u1 = dot(sub(c, v1), sub(v2, v1));
			T u2 = dot(sub(c, v2), sub(v1, v2));
			auto distSqBug = [](const V2<T> &p, const V2<T> &q) {
				T f = (q.x - p.x) * (q.y - p.y);
				return f * f;
			};
			if (u1 <= T(0)) {
				if (distSqBug(c, v1) > radius * radius) return;
				V2<T> d = sub(c, v1);
				V2<T> nrm = normalize(d);
				mtv = mul(nrm, radius - dot(nrm, d));
			} else if (u2 <= T(0)) {
				if (distSqBug(c, v2) > radius * radius) return;
				V2<T> d = sub(c, v2);
				V2<T> nrm = normalize(d);
				mtv = mul(nrm, radius - dot(nrm, d));
			} else {
				V2<T> mid((T(1) - T(0.5f)) * v1.x + T(0.5f) * v2.x, (T(1) - T(0.5f)) * v1.y + T(0.5f) * v2.y);
				T s = dot(sub(c, mid), normal);
				if (s > radius) return;
				mtv = mul(normal, radius - s);
			}
		}
		*pos = add(mtv, c);
	}
	static constexpr double FLT_MAX_VALUE = 3.40282346638528859811704183484516925440e+38;
	static constexpr double FLT_EPSILON_VALUE = 1.1920928955078125e-07;

	void ForEachChunk(size_t items, const std::function<void(size_t, size_t)> &fn) {
		if (items == 0) return;
		if (workers <= 1 || !pool) {
			fn(0, items - 1);
		} else {
			pool->Run(items, fn);
		}
	}

	static float Ms(std::chrono::high_resolution_clock::time_point t0) {
		auto d = std::chrono::high_resolution_clock::now() - t0;
		return (float)std::chrono::duration_cast<std::chrono::nanoseconds>(d).count() * (1.0f / 1000000);
	}

	// Plasticity of one spring of rest length L at length r < h (Clavet
	// 2005, Algorithm 4): outside the tolerable deformation d = yield * L the
	// rest length moves towards r at rate alpha.
	T Plastic(T L, T r, T dtAlpha) const {
		const T d = springYield * L;
		if (r > L + d) L = L + dtAlpha * ((r - L) - d);
		else if (r < L - d) L = L - dtAlpha * ((L - d) - r);
		return L;
	}

	// Springs, after the neighbour search and before density (Clavet 2005:
	// adjust springs, then apply spring displacements).  Restated for a
	// deterministic parallel form:
	//  1. per particle: existing springs within h are adjusted, springs
	//     whose rest length exceeds h are removed; the free slots go to the
	//     nearest candidates (in-range list members without a spring),
	//     ordered by (r^2, AddParticle index);
	//  2. a spring is added where both ends chose each other; its rest
	//     length starts at h and is adjusted like the others;
	//  3. every particle moves by -D/2 of each of its springs, from the
	//     positions before this phase (Jacobi), summed in slot order, with
	//     D = dt^2 k_spring (1 - L/h) (L - r) r_hat -- or, with springSerial,
	//     the paper's serial loop over the springs with immediate updates.
	void Springs(T dt) {
		const T h2 = h * h;
		const T dtAlpha = dt * springPlastic;
		const T dt2 = dt * dt;
		const int K = kSprings;
		std::vector<int32_t> nN(n);
		std::vector<int32_t> nP(n * K);
		std::vector<T> nL(n * K);
		// Chunks are inclusive ranges [s, e], as the reference's ThreadPool's.
		ForEachChunk(n, [&](size_t s, size_t e) {
			for (size_t i = s; i <= e; ++i) {
				const V2<T> xi = parts[i].cur;
				int m = 0;
				for (int q = 0; q < sN[i]; ++q) {
					const int p = sP[i * K + q];
					T L = sL[i * K + q];
					const V2<T> rij = sub(parts[p].cur, xi);
					const T r2 = dot(rij, rij);
					if (r2 < h2) L = Plastic(L, sqrt_t(r2), dtAlpha);
					if (L <= h) {
						nP[i * K + m] = p;
						nL[i * K + m] = L;
						++m;
					}
				}
				nN[i] = m;
				const int freeSlots = springMax - m;
				T kr2[kSprings];
				int64_t ktag[kSprings];
				int kj[kSprings];
				int cnt = 0;
				for (size_t t = 0; t < nbCount[i] && freeSlots > 0; ++t) {
					const size_t j = nb[i * capNb + t];
					if (j == i) continue;
					const V2<T> rij = sub(parts[j].cur, xi);
					const T r2 = dot(rij, rij);
					if (!(r2 < h2)) continue;
					bool has = false;
					for (int q = 0; q < sN[i]; ++q) has = has || (size_t)sP[i * K + q] == j;
					if (has) continue;
					const int64_t tj = tag[j];
					if (cnt == freeSlots && !(r2 < kr2[cnt - 1] || (r2 == kr2[cnt - 1] && tj < ktag[cnt - 1])))
						continue;
					int at = cnt < freeSlots ? cnt++ : cnt - 1;
					while (at > 0 && (r2 < kr2[at - 1] || (r2 == kr2[at - 1] && tj < ktag[at - 1]))) {
						kr2[at] = kr2[at - 1];
						ktag[at] = ktag[at - 1];
						kj[at] = kj[at - 1];
						--at;
					}
					kr2[at] = r2;
					ktag[at] = tj;
					kj[at] = (int)j;
				}
				accN[i] = cnt;
				for (int q = 0; q < cnt; ++q) accP[i * K + q] = kj[q];
			}
		});
		ForEachChunk(n, [&](size_t s, size_t e) {
			for (size_t i = s; i <= e; ++i) {
				const V2<T> xi = parts[i].cur;
				int m = nN[i];
				for (int q = 0; q < accN[i]; ++q) {
					const int p = accP[i * K + q];
					bool mutual = false;
					for (int q2 = 0; q2 < accN[p]; ++q2) mutual = mutual || (size_t)accP[p * K + q2] == i;
					if (!mutual) continue;
					const V2<T> rij = sub(parts[p].cur, xi);
					const T L = Plastic(h, sqrt_t(dot(rij, rij)), dtAlpha);
					if (L <= h) {
						nP[i * K + m] = p;
						nL[i * K + m] = L;
						++m;
					}
				}
				nN[i] = m;
			}
		});
		if (springSerial) {
			// The paper's loop as published: foreach spring ij, D from the
			// current positions, x_i -= D/2 and x_j += D/2 at once.  Springs
			// in particle-number order of their lower end, then slot order.
			for (size_t i = 0; i < n; ++i) {
				for (int q = 0; q < nN[i]; ++q) {
					const size_t p = (size_t)nP[i * K + q];
					if (p <= i) continue;
					const T L = nL[i * K + q];
					const V2<T> rij = sub(parts[p].cur, parts[i].cur);
					const T r = sqrt_t(dot(rij, rij));
					const T len = r == T(0) ? T(1) : r;
					const T inv = T(1) / len;
					const T nx = rij.x * inv, ny = rij.y * inv;
					const T f = ((dt2 * springK) * (T(1) - L * invH)) * (L - r);
					const V2<T> half((f * nx) * T(0.5f), (f * ny) * T(0.5f));
					parts[i].cur = sub(parts[i].cur, half);
					parts[p].cur = add(parts[p].cur, half);
				}
			}
			for (size_t i = 0; i < n; ++i) springPos[i] = parts[i].cur;
		} else
		ForEachChunk(n, [&](size_t s, size_t e) {
			for (size_t i = s; i <= e; ++i) {
				const V2<T> xi = parts[i].cur;
				V2<T> dx;
				for (int q = 0; q < nN[i]; ++q) {
					const int p = nP[i * K + q];
					const T L = nL[i * K + q];
					const V2<T> rij = sub(parts[p].cur, xi);
					const T r = sqrt_t(dot(rij, rij));
					const T len = r == T(0) ? T(1) : r;
					const T inv = T(1) / len;
					const T nx = rij.x * inv, ny = rij.y * inv;
					const T f = ((dt2 * springK) * (T(1) - L * invH)) * (L - r);
					dx.x = dx.x - (f * nx) * T(0.5f);
					dx.y = dx.y - (f * ny) * T(0.5f);
				}
				springPos[i] = add(dx, xi);
			}
		});
		uint64_t total = 0;
		for (size_t i = 0; i < n; ++i) {
			parts[i].cur = springPos[i];
			sN[i] = nN[i];
			for (int q = 0; q < nN[i]; ++q) {
				sP[i * K + q] = nP[i * K + q];
				sL[i * K + q] = nL[i * K + q];
			}
			total += (uint64_t)nN[i];
		}
		springTotal = total;
	}

	// demo4.cpp:286-451
	int Update(float dtf) override {
		error = 0;
		const T dt = dtf;
		const T invDt = T(1) / dt;
		using clk = std::chrono::high_resolution_clock;
		auto t0 = clk::now();
		for (auto &e : emitters) UpdateEmitter(e, dt);
		times[0] = Ms(t0);

		t0 = clk::now();
		const V2<T> ext = add(gravity, extForce);
		for (size_t i = 0; i < n; ++i) {
			Particle &p = parts[i];
			p.acc = add(ext, p.acc);
			p.vel = add(mul(p.acc, dt), p.vel);
			p.acc = V2<T>();
		}
		times[1] = Ms(t0);

		t0 = clk::now();
		ForEachChunk(n, [&](size_t s, size_t e) { Viscosity(s, e, dt); });
		times[2] = Ms(t0);

		t0 = clk::now();
		for (size_t i = 0; i < n; ++i) {
			Particle &p = parts[i];
			p.prev = p.cur;
			p.cur = add(mul(p.vel, dt), p.cur);
		}
		times[3] = Ms(t0);

		t0 = clk::now();
		for (size_t i = 0; i < n; ++i) {
			int cx, cy;
			CellOf(parts[i].cur, &cx, &cy);
			if (cx != cellX[i] || cy != cellY[i]) {
				Remove(i);
				Insert(i);
			}
		}
		times[4] = Ms(t0);

		t0 = clk::now();
		ForEachChunk(n, [&](size_t s, size_t e) { NeighborSearch(s, e); });
		statMinNb = dom.max_neighbors_stat;
		statMaxNb = 0;
		for (size_t i = 0; i < n; ++i) {
			statMinNb = std::min<uint64_t>(nbCount[i], statMinNb);
			statMaxNb = std::max<uint64_t>(nbCount[i], statMaxNb);
		}
		if (springsOn) Springs(dt);
		times[5] = Ms(t0);

		t0 = clk::now();
		ForEachChunk(n, [&](size_t s, size_t e) { DensityAndPressure(s, e); });
		times[6] = Ms(t0);

		t0 = clk::now();
		ForEachChunk(n, [&](size_t s, size_t e) { Delta(s, e, dt); });
		times[7] = Ms(t0);

		t0 = clk::now();
		for (size_t i = 0; i < n; ++i) {
			V2<T> *pos = &parts[i].cur;
			for (const Body<T> &b : bodies) {
				switch (b.kind) {
					case kPlane: SolvePlane(pos, b.a, b.r); break;
					case kCircle: SolveCircle(pos, b.a, b.r); break;
					case kSegment: SolveSegment(pos, b.a, b.b); break;
					case kPolygon: SolvePolygon(pos, b.vertexCount, b.verts); break;
				}
			}
		}
		times[8] = Ms(t0);

		for (size_t i = 0; i < n; ++i) {
			Particle &p = parts[i];
			p.vel = mul(sub(p.cur, p.prev), invDt);
		}
		return error;
	}

	void SetGravity(float x, float y) override { gravity = V2<T>(x, y); }
	void AddExternalForce(float x, float y) override { extForce = add(V2<T>(x, y), extForce); }
	void ClearExternalForce() override { extForce = V2<T>(); }

	void SetParams(const float *p) override {
		h = p[0];
		cellSizeParam = p[1];
		spacing = p[2];
		invH = p[3];
		rho0 = p[4];
		k = p[5];
		kNear = p[6];
		sigma = p[7];
		beta = p[8];
	}
	void GetParams(float *p) override {
		p[0] = (float)h;
		p[1] = (float)cellSizeParam;
		p[2] = (float)spacing;
		p[3] = (float)invH;
		p[4] = (float)rho0;
		p[5] = (float)k;
		p[6] = (float)kNear;
		p[7] = (float)sigma;
		p[8] = (float)beta;
	}
	size_t Count() override { return n; }

	void GetParticles(double *pos, double *prev, double *acc, double *vel, double *dens, double *press) override {
		for (size_t i = 0; i < n; ++i) {
			const Particle &d = parts[i];
			if (pos) { pos[2 * i] = d.cur.x; pos[2 * i + 1] = d.cur.y; }
			if (prev) { prev[2 * i] = d.prev.x; prev[2 * i + 1] = d.prev.y; }
			if (acc) { acc[2 * i] = d.acc.x; acc[2 * i + 1] = d.acc.y; }
			if (vel) { vel[2 * i] = d.vel.x; vel[2 * i + 1] = d.vel.y; }
			if (dens) { dens[2 * i] = d.density; dens[2 * i + 1] = d.nearDensity; }
			if (press) { press[2 * i] = d.pressure; press[2 * i + 1] = d.nearPressure; }
		}
	}
	void GetIndex(int *cellXY, uint64_t *ic, uint64_t *cnt) override {
		for (size_t i = 0; i < n; ++i) {
			if (cellXY) { cellXY[2 * i] = cellX[i]; cellXY[2 * i + 1] = cellY[i]; }
			if (ic) ic[i] = inCell[i];
			if (cnt) cnt[i] = nbCount[i];
		}
	}
	void GetNeighbors(size_t i, uint64_t *out) override {
		for (size_t k = 0; k < nbCount[i]; ++k) out[k] = nb[i * capNb + k];
	}
	uint64_t GetCell(int c, uint64_t *out) override {
		if (out) {
			for (size_t k = 0; k < cellCnt[c]; ++k) out[k] = cellIdx[(size_t)c * capCell + k];
		}
		return cellCnt[c];
	}
	int SetState(size_t cnt, const double *pos, const double *prev, const double *acc, const double *vel,
	             const double *dens, const double *press, const int *cellXY, const uint64_t *ic,
	             const uint64_t *nbc, const uint64_t *nbl, const uint64_t *cellCount, const uint64_t *cidx) override {
		if (cnt > capN) return SPH_ORACLE_ERR_CAPACITY;
		for (size_t c = 0; c < (size_t)gx * gy; ++c)
			if (cellCount[c] > capCell) return SPH_ORACLE_ERR_CAPACITY;
		for (size_t i = 0; i < cnt; ++i)
			if (nbc[i] > capNb) return SPH_ORACLE_ERR_CAPACITY;
		n = cnt;
		const uint64_t *q = nbl;
		for (size_t i = 0; i < cnt; ++i) {
			Particle &d = parts[i];
			d.cur = V2<T>((T)pos[2 * i], (T)pos[2 * i + 1]);
			d.prev = V2<T>((T)prev[2 * i], (T)prev[2 * i + 1]);
			d.acc = V2<T>((T)acc[2 * i], (T)acc[2 * i + 1]);
			d.vel = V2<T>((T)vel[2 * i], (T)vel[2 * i + 1]);
			d.density = (T)dens[2 * i];
			d.nearDensity = (T)dens[2 * i + 1];
			d.pressure = (T)press[2 * i];
			d.nearPressure = (T)press[2 * i + 1];
			cellX[i] = cellXY[2 * i];
			cellY[i] = cellXY[2 * i + 1];
			inCell[i] = ic[i];
			nbCount[i] = nbc[i];
			for (size_t k = 0; k < nbc[i]; ++k) nb[i * capNb + k] = *q++;
		}
		const uint64_t *ci = cidx;
		for (size_t c = 0; c < (size_t)gx * gy; ++c) {
			cellCnt[c] = cellCount[c];
			for (size_t k = 0; k < cellCount[c]; ++k) cellIdx[c * capCell + k] = *ci++;
		}
		return 0;
	}
	void GetStats(uint64_t *counts, float *t) override {
		counts[0] = statMinNb;
		counts[1] = statMaxNb;
		counts[2] = statMinCell;
		counts[3] = statMaxCell;
		for (int k = 0; k < 9; ++k) t[k] = times[k];
	}
	void SetSpringSerial(int serial) override { springSerial = serial ? 1 : 0; }
	void SetSprings(int enabled, float yield, float plasticity, float stiffness, int maxPer) override {
		springYield = yield;
		springPlastic = plasticity;
		springK = stiffness;
		springMax = std::min(std::max(maxPer, 0), (int)kSprings);
		if (enabled && !springsOn) {
			sN.assign(capN, 0);
			sP.assign(capN * kSprings, 0);
			sL.assign(capN * kSprings, T(0));
			accN.assign(capN, 0);
			accP.assign(capN * kSprings, 0);
			springPos.assign(capN, V2<T>());
		}
		springsOn = enabled ? 1 : 0;
	}
	int SetSpringState(size_t cnt, const int32_t *count, const int32_t *partner, const float *rest,
	                   const int64_t *tags) override {
		if (!springsOn || cnt != n) return SPH_ORACLE_ERR_CAPACITY;
		for (size_t i = 0; i < cnt; ++i) {
			if (count[i] < 0 || count[i] > kSprings) return SPH_ORACLE_ERR_CAPACITY;
			sN[i] = count[i];
			for (int q = 0; q < count[i]; ++q) {
				const int32_t p = partner[i * kSprings + q];
				if (p < 0 || (size_t)p >= cnt) return SPH_ORACLE_ERR_CAPACITY;
				sP[i * kSprings + q] = p;
				sL[i * kSprings + q] = (T)rest[i * kSprings + q];
			}
			if (tags) tag[i] = tags[i];
		}
		return 0;
	}
	void GetSpringState(int32_t *count, int32_t *partner, float *rest) override {
		for (size_t i = 0; i < n; ++i) {
			const int c = springsOn ? sN[i] : 0;
			if (count) count[i] = c;
			for (int q = 0; q < kSprings; ++q) {
				if (partner) partner[i * kSprings + q] = q < c ? sP[i * kSprings + q] : -1;
				if (rest) rest[i * kSprings + q] = q < c ? (float)sL[i * kSprings + q] : 0.0f;
			}
		}
	}
	uint64_t SpringTotal() override { return springTotal; }
	size_t Workers() override { return workers; }
	void SetWorkers(size_t w) override {
		w = std::max<size_t>(1, w);
		if (w == workers) return;
		delete pool;
		pool = nullptr;
		workers = w;
		if (w > 1) pool = new ChunkPool(w);
	}
};

SimBase *B(void *p) { return static_cast<SimBase *>(p); }

}  // namespace

extern "C" {

void sph_oracle_reference_domain(sph_oracle_domain *d) {
	// sph.h:18-23, 35-36, 54, 60, 68-70 and the SPHStatistics initialiser.
	d->width = 10.0f;
	d->height = 10.0f / (16.0f / 9.0f);
	d->cell_size = 6.0f * 0.05f;
	d->max_particles = 10000;
	d->max_cell_particles = 500;
	d->max_neighbors = 1000;
	d->stats_min_init = 500;
	d->max_neighbors_stat = 1000;
	d->particle_radius = 0.05f;
	d->collision_margin = 0.005f * 2.0f;
	d->jitter_kernel_height = 6.0f * 0.05f;
}

void sph_oracle_default_params(float *p) {
	// SPHParameters() (sph.h:88-98).
	const float h = 6.0f * 0.05f;
	p[0] = h;
	p[1] = h;
	p[2] = h * 0.5f;
	p[3] = 1.0f / h;
	p[4] = 20.0f;
	p[5] = 0.6f;
	p[6] = 0.6f * 10.0f;
	p[7] = 0.5f;
	p[8] = 0.3f;
}

void *sph_oracle_create(const sph_oracle_domain *d, int fp64) {
	if (fp64) return static_cast<SimBase *>(new Sim<double>(*d));
	return static_cast<SimBase *>(new Sim<float>(*d));
}
void sph_oracle_destroy(void *p) { delete B(p); }
void sph_oracle_reset_stats(void *p) { B(p)->ResetStats(); }
void sph_oracle_clear_bodies(void *p) { B(p)->ClearBodies(); }
void sph_oracle_clear_particles(void *p) { B(p)->ClearParticles(); }
void sph_oracle_clear_emitters(void *p) { B(p)->ClearEmitters(); }
int sph_oracle_add_plane(void *p, float nx, float ny, float d) { return B(p)->AddPlane(nx, ny, d); }
int sph_oracle_add_circle(void *p, float x, float y, float r) { return B(p)->AddCircle(x, y, r); }
int sph_oracle_add_segment(void *p, float ax, float ay, float bx, float by) { return B(p)->AddSegment(ax, ay, bx, by); }
int sph_oracle_add_polygon(void *p, uint64_t n, const float *xy) { return B(p)->AddPolygon(n, xy); }
int64_t sph_oracle_add_particle(void *p, float x, float y, float fx, float fy) { return B(p)->AddParticle(x, y, fx, fy); }
int sph_oracle_add_volume(void *p, float cx, float cy, float fx, float fy, int nx, int ny, float spacing) {
	return B(p)->AddVolume(cx, cy, fx, fy, nx, ny, spacing);
}
int sph_oracle_add_emitter(void *p, float px, float py, float dx, float dy, float radius, float speed, float rate,
                           float duration) {
	return B(p)->AddEmitter(px, py, dx, dy, radius, speed, rate, duration);
}
int sph_oracle_update(void *p, float dt) { return B(p)->Update(dt); }
void sph_oracle_set_gravity(void *p, float x, float y) { B(p)->SetGravity(x, y); }
void sph_oracle_add_external_force(void *p, float x, float y) { B(p)->AddExternalForce(x, y); }
void sph_oracle_clear_external_force(void *p) { B(p)->ClearExternalForce(); }
void sph_oracle_set_params(void *p, const float *v) { B(p)->SetParams(v); }
void sph_oracle_get_params(void *p, float *v) { B(p)->GetParams(v); }
uint64_t sph_oracle_particle_count(void *p) { return B(p)->Count(); }
void sph_oracle_get_particles(void *p, double *pos, double *prev, double *acc, double *vel, double *dens,
                              double *press) {
	B(p)->GetParticles(pos, prev, acc, vel, dens, press);
}
void sph_oracle_get_index(void *p, int *cellXY, uint64_t *inCell, uint64_t *nbCount) {
	B(p)->GetIndex(cellXY, inCell, nbCount);
}
void sph_oracle_get_neighbors(void *p, uint64_t i, uint64_t *out) { B(p)->GetNeighbors(i, out); }
uint64_t sph_oracle_get_cell(void *p, int c, uint64_t *out) { return B(p)->GetCell(c, out); }
int sph_oracle_set_state(void *p, uint64_t n, const double *pos, const double *prev, const double *acc,
                         const double *vel, const double *dens, const double *press, const int *cellXY,
                         const uint64_t *inCell, const uint64_t *nbCount, const uint64_t *nb,
                         const uint64_t *cellCount, const uint64_t *cellIdx) {
	return B(p)->SetState(n, pos, prev, acc, vel, dens, press, cellXY, inCell, nbCount, nb, cellCount, cellIdx);
}
void sph_oracle_get_stats(void *p, uint64_t *counts, float *times) { B(p)->GetStats(counts, times); }
void sph_oracle_set_workers(void *p, uint64_t w) { B(p)->SetWorkers(w); }
uint64_t sph_oracle_workers(void *p) { return B(p)->Workers(); }
void sph_oracle_set_springs(void *p, int enabled, float yield, float plasticity, float stiffness, int max_per) {
	B(p)->SetSprings(enabled, yield, plasticity, stiffness, max_per);
}
int sph_oracle_set_spring_state(void *p, uint64_t n, const int32_t *count, const int32_t *partner, const float *rest,
                                const int64_t *tag) {
	return B(p)->SetSpringState(n, count, partner, rest, tag);
}
void sph_oracle_get_spring_state(void *p, int32_t *count, int32_t *partner, float *rest) {
	B(p)->GetSpringState(count, partner, rest);
}
uint64_t sph_oracle_spring_total(void *p) { return B(p)->SpringTotal(); }
void sph_oracle_set_spring_serial(void *p, int serial) { B(p)->SetSpringSerial(serial); }
uint64_t sph_oracle_hardware_threads(void) {
	unsigned t = std::thread::hardware_concurrency();
	return t ? t : 1;
}
void sph_oracle_srand(unsigned seed) { srand(seed); }

}  // extern "C"
