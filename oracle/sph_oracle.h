// Test infrastructure (oracle): C interface of the CPU restatement of the
// reference's Demo4 step (sph_oracle.cpp).  Only tests, the smoke check and
// the benchmark's CPU-baseline leg use it.
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>

#define SPH_ORACLE_ERR_CAPACITY 2
#define SPH_ORACLE_MAX_POLY 8       /* kMaxScenarioPolygonCount, sph.h:161 */
#define SPH_ORACLE_MAX_BODIES 100   /* kSPHMaxBodyCount, sph.h:71 */
#define SPH_ORACLE_MAX_EMITTERS 8   /* kSPHMaxEmitterCount, sph.h:72 */

#ifdef __cplusplus
extern "C" {
#endif

/* What the reference fixes at compile time (sph.h:15-72). */
typedef struct sph_oracle_domain {
	float width, height, cell_size;
	uint64_t max_particles, max_cell_particles, max_neighbors;
	uint64_t stats_min_init;     /* SPHStatistics() minimums (sph.h:143-147) */
	uint64_t max_neighbors_stat; /* neighbour-count minimum seed (demo4.cpp:369) */
	float particle_radius;       /* kSPHParticleCollisionRadius */
	float collision_margin;      /* kSPHCollisionMargin */
	float jitter_kernel_height;  /* kSPHKernelHeight used by the volume jitter */
} sph_oracle_domain;

void sph_oracle_reference_domain(sph_oracle_domain *d);
void sph_oracle_default_params(float *p);
void *sph_oracle_create(const sph_oracle_domain *d, int fp64);
void sph_oracle_destroy(void *p);

#ifdef __cplusplus
}
#endif

#endif
