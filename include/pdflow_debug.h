/*
 * pdflow_debug.h - inspection entry points of the GB300 PD-Flow solver, for
 * stage-by-stage parity checks.  They have no production use and are not on
 * the solve path.
 */
#ifndef PDFLOW_DEBUG_H
#define PDFLOW_DEBUG_H

#include "pdflow.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Receives one named plane (host memory, valid during the call). */
typedef void (*pdflow_dump_fn)(void* ctx, const char* name, int level, const float* data, long n);

/* Runs pdflow_solve kernel by kernel, synchronising after every stage and
 * handing each intermediate to `fn` under the names of the reference's device
 * arrays: per level `dct dcu dcv ddt ddu ddv mu ri rj ri_2 rj_2 du_prev dv_prev
 * sigma_* tau_* init_*` after the set-up, `du_new ... pwv` after the
 * iterations, `sat_du sat_dv sat_dw` after saturateVariables and
 * `du_l dv_l dw_l` after the weighted median (the arrays the reference keeps
 * in CSF_cuda, pdflow_cudalib.h:71-122).  The final flow equals pdflow_solve's. */
int pdflow_debug_solve(pdflow_solver* s, pdflow_dump_fn fn, void* ctx);

/* Selects how pdflow_solve runs a level's iterations: 10 (default) = as 8
 * below, but each CTA walks rows of regions (24-row bands of a pair, or
 * column pieces of them; taken from a device counter as CTAs finish) left to
 * right and hands each region's last exact column's exchange values to the
 * next one, so that only a right halo is recomputed (28 of 32 columns exact
 * at 4 iterations per launch); levels with fewer bands than SMs run 8
 * instead, or 9 where all of the level's 16x16 tiles fit in one round of
 * CTAs (a single pair's 60x80 and 120x160 levels); 9 = as 8 with 16x16
 * interiors and a halo of 8 (up to 8 iterations per launch); 8 = every
 * level of a batch (more than one pair), and a single pair's levels above 300
 * pixels, as temporally blocked 24x24 tiles (halo 4, up to 4 iterations per
 * launch) walked by one persistent CTA per SM, each tile's state and
 * constants in registers (one pixel pair per thread, packed FP32x2) while
 * the next tile's region streams into shared memory by two 4D TMA tensor
 * copies; levels whose row count is even but not a multiple of 4 (30x40)
 * load each pixel pair directly instead, and 15x20 runs form 5 there;
 * 7 = the same tiles as one CTA per tile, four rows per
 * thread with the state in registers and the constants in shared memory;
 * 5 = every level of a batch, and a single pair's levels above
 * 300 pixels (all but 15x20), as temporally blocked shared-memory tiles (several
 * iterations per launch; 24x24 tiles, one pixel pair per thread in packed
 * FP32x2 arithmetic, two CTAs per SM so that one CTA's region load and store
 * overlap the other's iterations), a single pair's 15x20 level as one
 * launch; 6 = the same with 24x28 tiles (288 threads owning two
 * pairs each, two CTAs per SM); 4 = the same with 40x34 tiles (1008 threads,
 * one CTA per SM); 3 = the same with 40x40 tiles and two pairs per thread; 2 = one pixel
 * per lane; 1 = one launch per level (slab-persistent kernel; batches use two
 * kernels per iteration for the large levels); 0 = two kernels per iteration
 * (the reference's launch structure with gradient+dual and divergence+primal
 * fused).  All give the same bits. */
int pdflow_set_iteration_form(pdflow_solver* s, int form);

/* Number of kernels the last pdflow_solve / pdflow_solve_batch launched
 * (graph replays count the kernels of the captured solve). */
int pdflow_last_solve_launches(const pdflow_solver* s, unsigned* count);

/* Runs `iters` iterations of coarse-to-fine level `level` (0 = coarsest) for
 * pairs [0, n) in the launch form pdflow_solve uses, on the handle's stream,
 * after a solve has left that level's constants in place, and returns the
 * elapsed device time (CUDA events on that stream) in *ms.  The handle's state
 * is overwritten; push frames again before the next solve. */
int pdflow_time_level_iterations(pdflow_solver* s, unsigned n, unsigned level, unsigned iters, float* ms);

/* The 3x3 weighted median of filterSolution (pdflow_cudalib.cu:1040-1148) on
 * caller planes (device pointers, R*C floats, column-major).  `sel` (device,
 * 3*R*C int32, may be NULL) receives, per component, the bracketing index the
 * median picked (-1 where depth_old == 0). */
int pdflow_stage_median(unsigned R, unsigned C, const float* depth_old, const float* ddt, const float* du,
                        const float* dv, const float* dw, float* du_l, float* dv_l, float* dw_l, int32_t* sel,
                        void* stream);

/* Runs levels [first, last] of the coarse-to-fine schedule for pairs [0, n)
 * (no graph, on the handle's stream, blocking).  `d_seed` (device,
 * [n][3][N_first] floats: du, dv in level pixels, dw in metres; may be NULL)
 * replaces level `first`'s upsampled start, with zero duals; every solved
 * level runs ceil(num_max_iter * iter_scale) iterations.  With energy_level in
 * [first, last], energies[n] (host) receives that level's solution energy
 * (the functional of pdflow_energy_batch).  first = 0, last >= the finest
 * level, no seed, scale 1 is pdflow_solve_batch. */
int pdflow_solve_levels(pdflow_solver* s, unsigned n, unsigned first, unsigned last, const float* d_seed,
                        float iter_scale, int energy_level, float* energies);

/* How the paired tile kernels move a tile's region between HBM and shared
 * memory (process-wide; graphs captured afterwards use it): shape 0 = 40x40
 * tiles (iteration form 3), 1 = 40x34 tiles (form 4), 2 = 24x24 tiles
 * (form 5), 3 = 24x28 tiles (form 6); mode bit 0 = TMA bulk
 * copies for the region load, bit 1 = for the interior store, else plain
 * loads/stores; bit 2 (with bit 0) = the region load as one TMA tensor copy
 * per plane (the whole region as one box through a 3D tensor map of rows,
 * columns and arena slots) instead of one bulk copy per plane column.
 * Default: mode 5 (tensor-copy loads, plain stores) for every shape.  Levels
 * whose row count is not a multiple of 4 always use plain loads and stores.
 * All modes give the same bits. */
int pdflow_set_tile_copy_mode(int shape, int mode);

/* Process-wide L2 prefetch distance of the register-resident quad tiles
 * (iteration form 7), in CTAs: each CTA prefetches into L2 (one TMA tensor
 * prefetch per plane) the region of the CTA that many launch positions later,
 * which starts about when it finishes; 0 = no prefetch.  Same bits. */
int pdflow_set_quad_prefetch(unsigned ctas_ahead);

/* Check of the shrinkage's division (no counterpart in the reference): the
 * register tiles divide by a pixel's fixed denominator with its correctly
 * rounded reciprocal and two FMA corrections (Markstein's theorem) instead
 * of an IEEE division; this compares that quotient with the IEEE one
 * (__fdiv_rn) bit for bit on `pairs` random pairs of the range the kernels
 * use it in and returns how many differ (0 expected). */
int pdflow_check_div_rcp(unsigned long long pairs, unsigned long long seed, unsigned long long* mismatches);

/* The strip walk's work units (iteration form 10; no counterpart in the
 * reference), as the launcher computes them for `bands` 24-row bands of
 * `cols` columns on `ctas` CTAs at `iters_per_launch` iterations per launch:
 * bands [0, *whole) are whole units, then for tier i = 0, 1, 2 the next
 * tier_n[i] bands are cut into tier_p[i] column pieces each (host
 * arithmetic only, no GPU needed). */
int pdflow_strip_units(unsigned bands, unsigned cols, unsigned iters_per_launch, unsigned ctas, unsigned* whole,
                       unsigned* tier_n, unsigned* tier_p);

/* Copy bandwidth of this GPU for a working set of `bytes` per buffer (the
 * roofline denominators; no counterpart in the reference): allocates two
 * buffers of `bytes` and copies them into each other `reps` times within one
 * launch (alternating directions; 16-byte loads and stores that bypass L1,
 * 4 CTAs of 512 threads per SM, grid-stride) after a warm-up launch, timed
 * with CUDA events on `stream`; returns read + written bytes per second in
 * GB/s.  With 2 * bytes well inside L2 (e.g. 2 x 24 MiB on a 126 MB L2)
 * every copy after the first is served by L2: the L2 bandwidth ceiling; with
 * buffers far above L2 it is the HBM copy bandwidth. */
int pdflow_measure_copy_gbs(size_t bytes, unsigned reps, void* stream, float* gbs);

/* Per-level, per-phase timing of a plain solve of pairs [0, n) (tracing; no
 * counterpart in the reference, whose only timing is a host clock around the
 * whole solve): runs the solve eagerly (no graph) on the handle's stream with
 * CUDA events before each level's set-up (upsampling, gradients, warping),
 * iterations and median, and fills ms[3 * level + phase] (phase 0 = set-up,
 * 1 = iterations, 2 = median and motion field) for every level, coarsest
 * first (ms has 3 * ctf_levels entries).  The flow is the plain solve's. */
int pdflow_trace_solve(pdflow_solver* s, unsigned n, float* ms);

/* Failure detection without a fault: on the handle's stream, two CTAs where
 * one waits, through the bounded neighbour wait of the one-launch grid form
 * limited to `polls` polls (1..1e7), for a progress counter the other never
 * sets.  The wait runs out, the kernel records a timeout in the handle's
 * status word and returns; this call then reports it the way every
 * synchronising call does (PDFLOW_ERR_TIMEOUT, the status word reset) and
 * the handle stays usable.  No counterpart in the reference, which checks no
 * errors. */
int pdflow_debug_wait_timeout(pdflow_solver* s, unsigned polls);

#ifdef __cplusplus
}
#endif
#endif /* PDFLOW_DEBUG_H */
