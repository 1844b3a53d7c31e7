// Headless replacement for Demo4's point render (NBodySimulation/demo4.cpp:
// 453-532): per-particle colours from SPHGetParticleColor (sph.h:683-695) and
// a point image of the scene.  The reference hands its AoS particle array and
// a colour array to OpenGL; here the colours go to a caller buffer and the
// points are splatted into an RGBA8 image on the device, with no graphics API.
#include "sph_internal.cuh"
#include "sph_kernels.cuh"

namespace sphgb {

namespace {

// std::max(std::min(v, 1.0f), 0.0f) with std's comparisons (a NaN stays NaN).
__device__ __forceinline__ float clamp01(float v) {
	const float lo = (1.0f < v) ? 1.0f : v;
	return (lo < 0.0f) ? 0.0f : lo;
}

// SPHGetParticleColor(restDensity, density, pressure, velocity): red from the
// pressure, green from the density ratio, blue from the speed.
__device__ __forceinline__ float4 particle_color(float rho0, float density, float pressure, float2 v) {
	const float r = pressure / (-10.0f);
	const float g = density / rho0;
	const float b = sqrtf(v.x * v.x + v.y * v.y) / 10.0f;  // Vec2Length (vecmath.h:267-270)
	return make_float4(clamp01(r), clamp01(g), clamp01(b), 1.0f);
}

__device__ __forceinline__ uint32_t rgba8(float4 c) {
	// Round to nearest of c * 255; NaN channels map to 0.
	auto q = [](float x) -> uint32_t {
		const float y = x * 255.0f + 0.5f;
		return (y >= 1.0f) ? (uint32_t)fminf(y, 255.0f) : 0u;
	};
	return q(c.x) | (q(c.y) << 8) | (q(c.z) << 16) | (q(c.w) << 24);
}

}  // namespace

// Colour of every particle of one scene, stored at its AddParticle index.
__global__ void k_particle_colors(int first, int count, const int *id, const float2 *dens, const float2 *press,
                                  const float2 *vel, float rho0, float4 *out) {
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= count) return;
	const int k = id[first + j];
	if (k < 0 || k >= count) return;
	out[k] = particle_color(rho0, dens[first + j].x, press[first + j].x, vel[first + j]);
}

// Splat each particle into the pixel under it.  Particles are drawn in
// AddParticle order (later over earlier, as the reference's point array
// draws): each pixel keeps the largest key (AddParticle index + 1) << 32 |
// colour.  The image spans the scene's box, row 0 at the top.
__global__ void k_splat_points(int first, int count, const int *id, const float2 *pos, const float2 *dens,
                               const float2 *press, const float2 *vel, float rho0, float halfW, float halfH,
                               float sx, float sy, int width, int height, unsigned long long *keys) {
	const int j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= count) return;
	const int k = id[first + j];
	if (k < 0 || k >= count) return;
	const float2 p = pos[first + j];
	const float fx = (p.x + halfW) * sx;
	const float fy = (halfH - p.y) * sy;
	if (!(fx >= 0.0f) || !(fy >= 0.0f) || !(fx < (float)width) || !(fy < (float)height)) return;
	const int px = min((int)fx, width - 1), py = min((int)fy, height - 1);
	const uint32_t c = rgba8(particle_color(rho0, dens[first + j].x, press[first + j].x, vel[first + j]));
	const unsigned long long key = ((unsigned long long)(k + 1) << 32) | c;
	atomicMax(&keys[(size_t)py * width + px], key);
}

__global__ void k_keys_to_rgba8(int pixels, const unsigned long long *keys, uint32_t *rgba) {
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t < pixels) rgba[t] = (uint32_t)(keys[t] & 0xffffffffull);
}

}  // namespace sphgb
