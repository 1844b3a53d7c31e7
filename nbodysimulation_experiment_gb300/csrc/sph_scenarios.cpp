// The reference application's built-in scenarios (SPHScenarios[],
// NBodySimulation/sph.h:315-437) and its loader
// (DemoApplication::LoadScenario, NBodySimulation/app.cpp:477-534), restated
// on the C ABI.  The table is data the scenes are defined by, so its values
// and the float expressions that derive them (sph.h:15-72, 300-313) are kept
// as the reference writes them; the loader makes the same calls in the same
// order, including its walk over body_count entries of the volume table.
#include <cmath>
#include <cstring>

#include "../../include/sph_gb300.h"

namespace {

// sph.h:18-46 (box, kernel and stiffness constants).
const float kWidth = 10.0f;
const float kHeight = kWidth / (16.0f / 9.0f);
const float kHalfWidth = kWidth * 0.5f;
const float kHalfHeight = kHeight * 0.5f;
const float kParticleRadius = 0.05f;
const float kKernelHeight = 6.0f * kParticleRadius;
const float kCollisionRadius = kParticleRadius;
const float kRestDensity = 20.0f;
const float kStiffness = 0.6f;
const float kNearStiffness = kStiffness * 10.0f;
const float kLinearViscosity = 0.5f;
const float kQuadraticViscosity = 0.3f;
const float kCellSize = kKernelHeight;
// sph.h:300-306: dam-break wall and volume, blob volume.
const float kWallWidth = kWidth * 0.05f;
const float kWallHeight = kHeight * 0.85f;
const float kDamWidth = kWidth * 0.25f;
const float kDamHeight = kHeight * 0.95f;
const float kBlobWidth = kWidth * 0.5f;
const float kBlobHeight = kHeight * 0.5f;
const float kDeg2Rad = (float)M_PI / 180.0f;  // vecmath.h:9

struct V2 {
	float x, y;
};

enum Kind { kPlane, kCircle, kBox };
struct BodySpec {
	Kind kind;
	V2 position;
	V2 normal;  // plane
	float radius;
	float rotation;  // box
	V2 ext;          // box half extents
};
struct VolumeSpec {
	V2 position, size, force;
};
struct EmitterSpec {
	V2 position, direction;
	float radius, speed, rate, duration;
};
struct ScenarioSpec {
	const char *name;
	V2 gravity;
	int nv;
	VolumeSpec volumes[2];
	int ne;
	EmitterSpec emitters[1];
	int nb;
	BodySpec bodies[7];
	float spacing, nearStiffness;  // the SPHParameters arguments that differ
};

BodySpec plane(V2 p, V2 n) { return BodySpec{kPlane, p, n, 0.0f, 0.0f, {0.0f, 0.0f}}; }
BodySpec circle(V2 p, float r) { return BodySpec{kCircle, p, {0.0f, 0.0f}, r, 0.0f, {0.0f, 0.0f}}; }
BodySpec box(V2 p, float rot, V2 ext) { return BodySpec{kBox, p, {0.0f, 0.0f}, 0.0f, rot, ext}; }

#define WALLS4                                                                                     \
	plane({0, -kHalfHeight}, {0, 1}), plane({0, kHalfHeight}, {0, -1}), plane({-kHalfWidth, 0}, {1, 0}), \
	    plane({kHalfWidth, 0}, {-1, 0})

const ScenarioSpec kScenarios[] = {
	{"Dambreak", {0, -10}, 1, {{{-kHalfWidth + kDamWidth * 0.5f, 0}, {kDamWidth, kDamHeight}, {0, 0}}}, 0, {}, 5,
	 {WALLS4, box({-kHalfWidth + kDamWidth + kWallWidth * 0.5f + kCollisionRadius, kHeight * 0.1f}, 0.0f,
	              {kWallWidth * 0.5f, kWallHeight * 0.5f})},
	 kKernelHeight / 6.0f, kNearStiffness},
	{"Dambreak x 2", {0, -10}, 2,
	 {{{-kHalfWidth + kDamWidth * 0.5f, 0}, {kDamWidth, kDamHeight}, {0, 0}},
	  {{kHalfWidth - kDamWidth * 0.5f, 0}, {kDamWidth, kDamHeight}, {0, 0}}},
	 0, {}, 4, {WALLS4}, kKernelHeight / 3.0f, kStiffness * 20.0f},
	{"Blob", {0, 0}, 1, {{{0, 0}, {kBlobWidth, kBlobHeight}, {0, 0}}}, 0, {}, 4, {WALLS4}, kKernelHeight / 3.0f,
	 kNearStiffness},
	{"Blob x 2", {0, 0}, 2,
	 {{{-kBlobHeight * 0.75f, 0}, {kBlobHeight * 0.75f, kBlobHeight * 0.75f}, {10, 0}},
	  {{kBlobHeight * 0.75f, 0}, {kBlobHeight * 0.75f, kBlobHeight * 0.75f}, {-10, 0}}},
	 0, {}, 4, {WALLS4}, kKernelHeight / 3.0f, kNearStiffness},
	{"Liquid", {0, -2}, 0, {}, 1, {{{-3.5f, 0.0f}, {1, 0}, kKernelHeight * 3, 2.5f, 15.0f, 30.0f}}, 4, {WALLS4},
	 kKernelHeight / 4.0f, kStiffness * 10.0f},
	{"Glass", {0, -10}, 0, {}, 1, {{{-1.5f, 2.0f}, {1, 0}, kKernelHeight * 3, 2.5f, 15.0f, 25.0f}}, 7,
	 {WALLS4, box({0.0f, -2.0f}, 0.0f, {1.0f, 0.2f}), box({-1.0f, -0.5f}, 0.0f, {0.2f, 1.5f}),
	  box({1.0f, -0.5f}, 0.0f, {0.2f, 1.5f})},
	 kKernelHeight / 4.0f, kStiffness * 6.0f},
	{"Fontain", {0, -10}, 0, {}, 1, {{{0, -kHalfHeight + 1.0f}, {0, 1}, kKernelHeight * 4, 8.0f, 15.0f, 25.0f}}, 4,
	 {WALLS4}, kKernelHeight / 4.0f, kStiffness * 2.0f},
	// "Fun" has no top wall.
	{"Fun", {0, -10}, 0, {}, 1, {{{-4, 2}, {1, 0}, kKernelHeight * 4, 3.5f, 15.0f, 20.0f}}, 7,
	 {plane({0, -kHalfHeight}, {0, 1}), plane({-kHalfWidth, 0}, {1, 0}), plane({kHalfWidth, 0}, {-1, 0}),
	  box({-1.5f, 1.0f}, kDeg2Rad * -2.5f, {3.5f, 0.1f}), box({1.5f, -0.25f}, kDeg2Rad * 2.5f, {3.5f, 0.1f}),
	  circle({-4.0f, -1.5f}, 0.5f), box({0, -kHalfHeight + 0.5f}, 0, {0.3f, 1.0f})},
	 kKernelHeight / 4.0f, kStiffness * 6.0f},
};
const int kScenarioCount = (int)(sizeof(kScenarios) / sizeof(kScenarios[0]));

// Vec2MultMat2(orientation, v) + position with orientation = Mat2FromAngle
// (vecmath.h:287-290, 358-365).
sph_vec2 place(V2 v, float rotation, V2 position) {
	const float s = sinf(rotation), c = cosf(rotation);
	const float x = c * v.x + -s * v.y;
	const float y = s * v.x + c * v.y;
	return sph_vec2{x + position.x, y + position.y};
}

}  // namespace

extern "C" {

int sph_scenario_count(int *count) {
	if (!count) return SPH_ERR_INVALID_ARGUMENT;
	*count = kScenarioCount;
	return SPH_OK;
}

int sph_scenario_describe(int index, sph_scenario_desc *out) {
	if (!out || index < 0 || index >= kScenarioCount) return SPH_ERR_INVALID_ARGUMENT;
	const ScenarioSpec &sc = kScenarios[index];
	memset(out, 0, sizeof(*out));
	strncpy(out->name, sc.name, sizeof(out->name) - 1);
	out->gravity = sph_vec2{sc.gravity.x, sc.gravity.y};
	// SPHParameters' 8-argument constructor (sph.h:112-122).
	sph_params &p = out->params;
	p.kernel_height = kKernelHeight;
	p.cell_size = kCellSize;
	p.particle_spacing = sc.spacing;
	p.inv_kernel_height = 1.0f / kKernelHeight;
	p.rest_density = kRestDensity;
	p.stiffness = kStiffness;
	p.near_stiffness = sc.nearStiffness;
	p.linear_viscosity = kLinearViscosity;
	p.quadratic_viscosity = kQuadraticViscosity;
	// Bodies (app.cpp:488-517).
	out->body_count = (uint32_t)sc.nb;
	for (int b = 0; b < sc.nb; ++b) {
		const BodySpec &bs = sc.bodies[b];
		sph_scenario_body &o = out->bodies[b];
		if (bs.kind == kPlane) {
			// Mat2FromAxis(normal).col1 == normal; distance = dot(normal, position).
			o.type = SPH_BODY_PLANE;
			o.normal = sph_vec2{bs.normal.x, bs.normal.y};
			o.distance = bs.normal.x * bs.position.x + bs.normal.y * bs.position.y;
		} else if (bs.kind == kCircle) {
			o.type = SPH_BODY_CIRCLE;
			o.center = sph_vec2{bs.position.x, bs.position.y};
			o.radius = bs.radius;
		} else {
			// SPHScenarioBody::CreateBox (sph.h:204-216).
			o.type = SPH_BODY_POLYGON;
			o.vertex_count = 4;
			const V2 local[4] = {{bs.ext.x, bs.ext.y}, {-bs.ext.x, bs.ext.y}, {-bs.ext.x, -bs.ext.y},
			                     {bs.ext.x, -bs.ext.y}};
			for (int k = 0; k < 4; ++k) o.verts[k] = place(local[k], bs.rotation, bs.position);
		}
	}
	// Volumes: the loader walks body_count entries of the volume table, whose
	// entries past the scenario's own are zero (app.cpp:521-527).
	out->volume_count = (uint32_t)sc.nb;
	for (int v = 0; v < sc.nb; ++v) {
		const VolumeSpec zero = {{0, 0}, {0, 0}, {0, 0}};
		const VolumeSpec &vs = v < sc.nv ? sc.volumes[v] : zero;
		sph_scenario_volume &o = out->volumes[v];
		o.center = sph_vec2{vs.position.x, vs.position.y};
		o.force = sph_vec2{vs.force.x, vs.force.y};
		o.count_x = (int)std::floor(vs.size.x / sc.spacing);
		o.count_y = (int)std::floor(vs.size.y / sc.spacing);
		o.spacing = sc.spacing;
	}
	out->emitter_count = (uint32_t)sc.ne;
	for (int e = 0; e < sc.ne; ++e) {
		const EmitterSpec &es = sc.emitters[e];
		out->emitters[e] = sph_scenario_emitter{{es.position.x, es.position.y}, {es.direction.x, es.direction.y},
		                                        es.radius, es.speed, es.rate, es.duration};
	}
	return SPH_OK;
}

int sph_load_scenario(sph_sim *sim, int index) {
	if (!sim) return SPH_ERR_INVALID_ARGUMENT;
	sph_scenario_desc d;
	int rc = sph_scenario_describe(index, &d);
	if (rc) return rc;
	if ((rc = sph_reset_stats(sim)) || (rc = sph_clear_bodies(sim)) || (rc = sph_clear_particles(sim)) ||
	    (rc = sph_clear_emitters(sim)) || (rc = sph_set_gravity(sim, d.gravity)) || (rc = sph_set_params(sim, &d.params)))
		return rc;
	for (uint32_t b = 0; b < d.body_count; ++b) {
		const sph_scenario_body &o = d.bodies[b];
		if (o.type == SPH_BODY_PLANE) rc = sph_add_plane(sim, o.normal, o.distance);
		else if (o.type == SPH_BODY_CIRCLE) rc = sph_add_circle(sim, o.center, o.radius);
		else if (o.type == SPH_BODY_LINE_SEGMENT) rc = sph_add_line_segment(sim, o.verts[0], o.verts[1]);
		else rc = sph_add_polygon(sim, (size_t)o.vertex_count, o.verts);
		if (rc) return rc;
	}
	for (uint32_t v = 0; v < d.volume_count; ++v) {
		const sph_scenario_volume &o = d.volumes[v];
		if ((rc = sph_add_volume(sim, o.center, o.force, o.count_x, o.count_y, o.spacing))) return rc;
	}
	for (uint32_t e = 0; e < d.emitter_count; ++e) {
		const sph_scenario_emitter &o = d.emitters[e];
		if ((rc = sph_add_emitter(sim, o.position, o.direction, o.radius, o.speed, o.rate, o.duration))) return rc;
	}
	return SPH_OK;
}

}  // extern "C"
