/*
 * pdflow_net.h - the learned warm start of the GB300 PD-Flow solver
 * (no counterpart in the reference, which always starts from the coarsest
 * level at zero flow).
 *
 * A 4-level convolutional encoder-decoder (338 k parameters, 3x3
 * convolutions, BF16 weights and activations, FP32 accumulation on the
 * tcgen05 tensor cores) maps both frames' intensity and depth at the 60x80
 * pyramid level to that level's flow.  pdflow_solve_batch_learned starts the
 * coarse-to-fine solve at the 60x80 level from the prediction, with scaled
 * iteration counts, and falls back to the plain solve per pair when the
 * energy rule rejects the prediction (a rejected pair continues from the
 * plain 60x80 solution, so its result is the plain solve's bit for bit).  The network is trained by the same
 * library (pdflow_net_train_step) on flows the plain solver produces.
 */
#ifndef PDFLOW_NET_H
#define PDFLOW_NET_H

#include <stddef.h>

#include "pdflow.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pdflow_net pdflow_net;

/* Creates a network for batches of up to max_batch inputs with He-normal
 * weights drawn from `seed` (device buffers for training included). */
int pdflow_net_create(unsigned max_batch, unsigned long long seed, pdflow_net** out);
int pdflow_net_destroy(pdflow_net* n);
/* Device memory the network holds (weights, optimiser state, activation and
 * gradient buffers for max_batch inputs), in bytes. */
size_t pdflow_net_device_bytes(const pdflow_net* n);

/* Parameters: FP32, per convolution (in network order) the weights
 * [cout][3*3*cin] (tap-major: tap = 3*dh + dw, then input channel) followed
 * by the biases [cout]. */
size_t pdflow_net_param_count(const pdflow_net* n);
int pdflow_net_get_params(pdflow_net* n, float* params, size_t count);
int pdflow_net_set_params(pdflow_net* n, const float* params, size_t count);   /* also resets Adam */
int pdflow_net_set_stream(pdflow_net* n, void* stream);

/* Inputs (device) [n][4][4800]: intensity of frame 1 and 2 (0..255), depth of
 * frame 1 and 2 (metres, 0 = invalid), each the column-major 60x80 level
 * plane (idx = v + 60 u).  Output (device) [n][3][4800]: du, dv (pixels of the
 * 60x80 level), dw (metres).  Blocks until done. */
int pdflow_net_forward(pdflow_net* n, unsigned nb, const float* d_input, float* d_output);

/* One Adam step (lr; betas 0.9, 0.999) on the masked mean squared error
 * against labels [n][3][4800] (du, dv, 20 dw) over pixels with valid frame-1
 * depth.  *loss (may be NULL) receives the loss before the step. */
int pdflow_net_train_step(pdflow_net* n, unsigned nb, const float* d_input, const float* d_label, float lr,
                          float* loss);

/* Loss and gradients (host [param_count], the parameter layout) without an
 * update. */
int pdflow_net_gradients(pdflow_net* n, unsigned nb, const float* d_input, const float* d_label, float* grads,
                         float* loss);

/* Learned solve options / report. */
typedef struct pdflow_learned_opts {
    float iter_scale;        /* iterations per level from the seed level on: ceil(num_max_iter * iter_scale) */
    float energy_margin;     /* fall back when E(learned) > (1 + margin) * E(plain) at the seed level; < 0: never */
} pdflow_learned_opts;

typedef struct pdflow_learned_report {
    unsigned fallbacks;      /* pairs finished by the plain schedule (from the plain 60x80 solution) */
    float max_energy_ratio;  /* max over pairs of E(learned) / E(plain) at the seed level */
} pdflow_learned_report;

/* Solves pairs [0, n) of a batch handle (frames pushed for the whole batch)
 * with the learned warm start:
 *   1. the plain schedule up to the 60x80 level, and that level's energy;
 *   2. the network's prediction from the 60x80 level images seeds the 60x80
 *      level (zero duals); it and every finer level run
 *      ceil(num_max_iter * iter_scale) iterations; the 60x80 energy of this
 *      path is taken after its median;
 *   3. pairs whose learned energy exceeds (1 + energy_margin) times the plain
 *      one are solved again with the plain schedule (bit-identical to
 *      pdflow_solve_batch for those pairs).
 * Needs rows >= 120 (a level finer than 60x80) and n <= the network's batch.
 * Waits for step 2 (the energies decide step 3) and returns with step 3
 * queued on the handle's stream; *report may be NULL.  The network's stream
 * is not used: all work runs on the solver's stream. */
int pdflow_solve_batch_learned(pdflow_solver* s, unsigned n, pdflow_net* net, const pdflow_learned_opts* opts,
                               pdflow_learned_report* report);

/* The same for the listed slots of a slot-addressed handle (serving): each
 * slot's previous and newest frame form its pair. */
int pdflow_solve_slots_learned(pdflow_solver* s, unsigned n, const unsigned* slots, pdflow_net* net,
                               const pdflow_learned_opts* opts, pdflow_learned_report* report);

/* The seed-level energies of the last learned solve's first n grid entries
 * (pairs, or the listed slots in list order): plain path and learned path
 * (host arrays, either may be NULL). */
int pdflow_learned_energies(const pdflow_solver* s, unsigned n, float* plain, float* learned);

/* Training data from a batch handle (frames pushed for the whole batch):
 * the network's input for pairs [0, n) — the seed level's images, exactly
 * what pdflow_solve_batch_learned feeds it — and, after a plain solve, the
 * label: the finest-level solution averaged over s x s blocks (s = cols / 80)
 * in 60x80-level units.  Device outputs [n][4][4800] and [n][3][4800]; both
 * block until written. */
int pdflow_seed_level_inputs(pdflow_solver* s, unsigned n, float* d_out);
int pdflow_seed_level_labels(pdflow_solver* s, unsigned n, float* d_out);

/* The tcgen05 GEMM the network runs on, for tests: C[M][N] (FP32, ldc) =
 * A[M][K] * B[N][K]^T with bf16 A, B (device, K contiguous; K, lda, ldb
 * multiples of 8); k_per_split > 0 splits K (partials summed in a fixed
 * order).  Blocks until done. */
int pdflow_gemm_bf16(int M, int N, int K, const void* d_a, int lda, const void* d_b, int ldb, float* d_c, int ldc,
                     int k_per_split, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PDFLOW_NET_H */
