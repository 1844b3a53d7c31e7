/*
 * sph_mpnn.h -- C ABI of the learned frame (no counterpart in the reference).
 *
 * A small message-passing network stands in for one frame of the plain
 * method (the reference's four Update(dt/4) substeps per frame,
 * kSPHSubsteps, sph.h:32-34 / app.cpp:231-233).  Its layers run on the
 * GB300's 5th-generation tensor cores (tcgen05; BF16 operands for the dense
 * layers, TF32 for the edge layer; FP32 accumulation); the plain step stays
 * its judge and fallback.
 */
#ifndef SPH_MPNN_H
#define SPH_MPNN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* C[M x N] (+)= A[M x K] * B[N x K]^T on the tensor cores: A and B bf16
 * row-major device arrays (leading dimensions lda, ldb in elements, multiples
 * of 8, 16-byte aligned), C FP32 row-major (ldc).  N a multiple of 16 up to
 * 256, K a multiple of 16, any M.  Optional bias [N] and ReLU; accumulate = 1
 * adds into C atomically (required when splits > 1 divides K over CTAs).
 * staging = 0 feeds the operands with TMA (cp.async.bulk.tensor, 128-byte
 * swizzle): with splits = 1 and B small enough to stay in shared memory
 * (N x K <= 48K elements), persistent CTAs (one per SM) loop over the row
 * tiles with B resident, A through a 4-stage ring and the accumulator
 * double-buffered in tensor memory; otherwise one CTA per row tile and K
 * split.  staging = 2 forces the one-tile-per-CTA TMA form, 1 stages with
 * plain loads.  Enqueued on `stream` (cudaStream_t) and waited for. */
int sph_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, int lda, int ldb, int ldc,
                  const float *bias, int relu, int accumulate, int splits, int staging, void *stream);

/* The network.  Two rounds of message passing over the radius-h neighbour
 * graph (the 3x3 cell block of each particle, pairs closer than h), each
 * with an edge MLP 6 -> 128 -> 128 (summed over a particle's edges) and a
 * node MLP 130 -> 128 -> 2 updating a 2-vector node state; BF16 weights for
 * the tensor-core layers, FP32 master weights and accumulation.  A learned
 * frame of length dt is one plain update over the whole frame (instead of the
 * reference's `substeps` updates of dt / substeps), corrected by the network:
 * input the positions x1 after that update and the node state
 * z0 = (x1 - x_prev) / h, output u, positions x1 + h u (then bodies and
 * velocities as in the plain step).  Trained with Adam on samples captured
 * from plain frames.  A model serves one device; its calls must not
 * overlap. */
typedef struct sph_mpnn sph_mpnn;
typedef struct sph_sim sph_sim;
int sph_mpnn_create(int device, size_t max_particles, uint64_t seed, sph_mpnn **out);
int sph_mpnn_destroy(sph_mpnn *model);
int sph_mpnn_param_count(size_t *out);
/* Flat FP32 parameters, per round: W1[128][6], b1[128], W2[128][128],
 * b2[128], W3[128][144] (columns 130.. are zero padding), b3[128],
 * W4[2][128], b4[2].  Setting them resets the optimizer state. */
int sph_mpnn_get_params(sph_mpnn *model, float *out);
int sph_mpnn_set_params(sph_mpnn *model, const float *in);

/* Where the edge MLP's first layer (6 -> 128, summed over a particle's
 * edges) runs in the forward pass: path 0 (default) on the tensor cores
 * (per tile of 128 edges one kind::tf32 MMA computes W1 e + b1 for every
 * edge into tensor memory; the ReLU and the per-particle sums are read out
 * of it with packed FP32 adds; four CTAs per SM share its tensor memory and
 * overlap one another's building, MMA and read-out phases), path 1 on the
 * CUDA cores (FP32 FMAs).  Both round the edge features, W1 and b1 to TF32, so they compute
 * the same function up to summation order. */
int sph_mpnn_set_edge_path(sph_mpnn *model, int path);
int sph_mpnn_get_edge_path(sph_mpnn *model, int *path);

/* Training samples, stored on the device.  sph_mpnn_capture takes one from
 * `sim` (a single-scene simulation in a canonical state, i.e. after an
 * update): the network's inputs after one plain update of frame_dt, and as
 * target (x - x1) / h with x the positions the plain method reaches in
 * `substeps` updates of frame_dt / substeps (the reference's kSPHSubsteps
 * loop), which `sim` then holds. */
int sph_mpnn_capture(sph_sim *sim, sph_mpnn *model, float frame_dt, int substeps);
int sph_mpnn_sample_count(sph_mpnn *model, size_t *out);
int sph_mpnn_clear_samples(sph_mpnn *model);
int sph_mpnn_sample_info(sph_mpnn *model, size_t index, size_t *count, int *grid_x, int *grid_y, float *h);
/* Host copies of a sample: x1 (count), z0 (count), target u (count), the cell
 * ranges of the particles' numbering (grid_x * grid_y each). */
int sph_mpnn_read_sample(sph_mpnn *model, size_t index, void *pos, void *z0, void *target, int32_t *cell_start,
                         int32_t *cell_count);
/* Mean squared error of u on a sample (u copied out if u_host is given). */
int sph_mpnn_eval(sph_mpnn *model, size_t index, float *loss, void *u_host);
/* Loss and gradient of every parameter (grad_host: param_count floats). */
int sph_mpnn_gradient(sph_mpnn *model, size_t index, float *loss, float *grad_host);
/* One Adam step (learning rate lr) on a sample; returns the loss before it. */
int sph_mpnn_train_step(sph_mpnn *model, size_t index, float lr, float *loss);

/* One learned frame of length frame_dt, judged by the plain method: the
 * network's correction stands if the mean |rho - rho0| / rho0 of the
 * corrected positions exceeds that of the plain update it corrects by at
 * most `bound`, its densest neighbourhood lists at most 70% of the neighbour
 * capacity, and no capacity overflowed on the way; otherwise the state is
 * restored and the frame runs as `substeps` plain updates of
 * frame_dt / substeps.  Reports which ran and the density error of the
 * result (summed in a fixed order: the verdict is reproducible).
 * Single-scene simulations without springs. */
int sph_learned_frame(sph_sim *sim, sph_mpnn *model, float frame_dt, int substeps, float bound, int *used_learned,
                      float *density_error);

#ifdef __cplusplus
}
#endif

#endif /* SPH_MPNN_H */
