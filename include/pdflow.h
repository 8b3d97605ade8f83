/*
 * pdflow.h - C ABI of the GB300-native PD-Flow scene-flow solver.
 *
 * The entry points replace the host interface of the reference solver:
 *   class PD_flow_opencv  (scene_flow_impair.h:53-115, scene_flow_impair.cpp:31-193)
 *   class CSF_cuda host methods and bridges (pdflow_cudalib.h:125-134, :159-174)
 * with plain pointers, sizes and integer status codes.  All image buffers use
 * the reference's layout: column-major, rows contiguous, idx = v + u*height
 * (scene_flow_impair.cpp:230-232).  Flow outputs are rows x cols, idx = v + u*rows
 * (pdflow_cudalib.cu:239-244).  Axis convention of the flow (pdflow_cudalib.cu:1157-1159):
 * dx = motion along the optical axis, dy = horizontal, dz = vertical, metres.
 *
 * Threading: a handle is not re-entrant; calls on one handle must be serialised
 * by the caller (as the reference's object).  Distinct handles are independent.
 * Every call returns PDFLOW_OK (0) or a negative pdflow_status.
 */
#ifndef PDFLOW_H
#define PDFLOW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pdflow_status {
    PDFLOW_OK = 0,
    PDFLOW_ERR_ARG = -1,          /* bad size, null pointer or unsupported configuration */
    PDFLOW_ERR_OOM = -2,          /* device arena could not be allocated / admission refused */
    PDFLOW_ERR_CUDA = -3,         /* a CUDA runtime call failed (see pdflow_last_error) */
    PDFLOW_ERR_STATE = -4,        /* call out of order (e.g. solve before two frames) */
    PDFLOW_ERR_TIMEOUT = -5,      /* a bounded device-side wait gave up */
    PDFLOW_ERR_NO_DEVICE = -6     /* no CUDA device of the supported architecture */
} pdflow_status;

/* Solver parameters.  Defaults (pdflow_default_params) are the reference's:
 * lambda_i = 0.04, lambda_d = 0.35, mu = 75 (scene_flow_impair.cpp:67-69),
 * fovh = 62.5 deg, fovv = 48.5 deg (:41-42), and the iteration schedule
 * num_max_iter[i] = 100 at the finest level, -15 per coarser level (:46-52). */
typedef struct pdflow_params {
    float lambda_i;
    float lambda_d;
    float mu;
    float fovh;                   /* radians */
    float fovv;                   /* radians (kept for interface parity; unused by the solver) */
    unsigned num_max_iter[6];     /* iterations per coarse-to-fine level, coarse -> fine */
} pdflow_params;

typedef struct pdflow_solver pdflow_solver;    /* opaque handle */

/* Fills `p` with the reference defaults for `rows` (PD_flow_opencv ctor,
 * scene_flow_impair.cpp:31-69). rows in {15,30,60,120,240,480}. */
int pdflow_default_params(unsigned rows, pdflow_params* p);

/* Creates a solver: replaces PD_flow_opencv::PD_flow_opencv + initializeCUDA
 * (scene_flow_impair.cpp:31-77, :175-193) and CSF_cuda::readParameters +
 * allocateDevMemory (pdflow_cudalib.cu:29-72, :176-193).
 * rows in {15,30,60,120,240,480} (main_scene_flow_impair.cpp:83); image
 * width x height is 640x480 or 320x240 (cam_mode 1 / 2, scene_flow_impair.cpp:182);
 * cols = rows*4/3 must not exceed width.  `params` may be NULL for defaults.
 * All device memory of the solver is allocated here, once. */
int pdflow_create(unsigned rows, unsigned width, unsigned height, const pdflow_params* params,
                  pdflow_solver** out);

/* Releases the handle: replaces PD_flow_opencv::freeGPUMemory /
 * CSF_cuda::freeDeviceMemory (scene_flow_impair.cpp:170-173, pdflow_cudalib.cu:249-288). */
int pdflow_destroy(pdflow_solver* s);

/* Pushes a new frame from the float staging buffers I, Z (host, width*height,
 * column-major; Z in metres): replaces PD_flow_opencv::createImagePyramidGPU
 * (scene_flow_impair.cpp:80-93), i.e. CSF_cuda::copyNewFrames + the Gaussian
 * pyramid (pdflow_cudalib.cu:195-222, :1172-1184).  The previous frame becomes
 * the old frame. */
int pdflow_push_frame(pdflow_solver* s, const float* I, const float* Z);

/* Same, from raw camera images as a PNG decoder returns them: row-major
 * uint8 intensity and uint16 depth (metres * 5000), decoded on the device
 * bit-exactly as the reference's host loop (scene_flow_impair.cpp:230-245,
 * depth = uint16 * (float)(1/5000)). */
int pdflow_push_frame_u16(pdflow_solver* s, const uint8_t* intensity, const uint16_t* depth);

/* Same as pdflow_push_frame_u16 with device pointers (no host copy). */
int pdflow_push_frame_u16_device(pdflow_solver* s, const uint8_t* d_intensity, const uint16_t* d_depth);

/* Same, from an RGB-D camera's raw frames as the reference's live application
 * converts them (PD_flow_mrpt::CaptureFrame, scene_flow_visualization.cpp:313-323):
 * row-major RGB888 and uint16 depth in millimetres, converted on the device
 * bit-exactly as its host loop (gray = 0.299 r + 0.587 g + 0.114 b in double,
 * each product and sum rounded once, then to float; depth = 0.001f * mm).
 * rotate180 != 0 stores camera pixel (y, x) at (height-1-y, width-1-x), as that
 * loop does.  The host variant allocates a device staging buffer on first use. */
int pdflow_push_frame_rgb8_mm(pdflow_solver* s, const uint8_t* rgb, const uint16_t* depth_mm, int rotate180);

/* Runs the coarse-to-fine solve on the last two pushed frames: replaces
 * PD_flow_opencv::solveSceneFlowGPU (scene_flow_impair.cpp:95-168).  Asynchronous
 * on the solver's stream; pdflow_read_flow or pdflow_synchronize waits. */
int pdflow_solve(pdflow_solver* s);

/* Copies the motion field (rows*cols floats each, column-major) to host
 * memory: replaces CSF_cuda::copyMotionField (pdflow_cudalib.cu:239-244) and
 * the public dxp/dyp/dzp buffers of PD_flow_opencv.  Blocks until the solve ends. */
int pdflow_read_flow(pdflow_solver* s, float* dx, float* dy, float* dz);

/* Device pointers of the solver's motion-field planes (valid until destroy). */
int pdflow_flow_device(pdflow_solver* s, const float** dx, const float** dy, const float** dz);

/* Copies the motion fields of pairs [0, n) into caller device buffers
 * [n][rows*cols] (column-major per pair) on the solver's stream and returns
 * without waiting (no counterpart in the reference): a pipeline can then copy
 * them to the host on another stream while the next batch is solved. */
int pdflow_copy_flow_device(pdflow_solver* s, unsigned n, float* d_dx, float* d_dy, float* d_dz);

/* Copies pyramid level `level` (0 = full image resolution) of the old
 * (frame = 0) or new (frame = 1) frame: intensity, depth and the
 * back-projected xx, yy, each (height>>level)*(width>>level) floats,
 * column-major.  Any pointer may be NULL.  Replaces the image part of
 * CSF_cuda::copyAllSolutions (pdflow_cudalib.cu:224-237). */
int pdflow_read_level_images(pdflow_solver* s, unsigned level, int frame, float* colour, float* depth, float* xx,
                             float* yy);

/* CSF_cuda::copyAllSolutions (pdflow_cudalib.cu:224-237): the motion field
 * and both frames' depth, intensity and back-projected xx, yy at the finest
 * solved level (rows*cols floats each, column-major; the point cloud the
 * reference's live viewer draws).  Any pointer may be NULL; blocks. */
int pdflow_read_all_solutions(pdflow_solver* s, float* dx, float* dy, float* dz, float* depth, float* depth_old,
                              float* colour, float* colour_old, float* xx, float* xx_old, float* yy, float* yy_old);

/* Waits for all work queued on the solver's stream. */
int pdflow_synchronize(pdflow_solver* s);

/* Uses `stream` (a cudaStream_t, or NULL for the solver's own stream) for all
 * later work of this handle. */
int pdflow_set_stream(pdflow_solver* s, void* stream);

/* rows, cols, ctf_levels, pyr_levels, cam_mode of a handle (out may be NULL). */
int pdflow_get_config(const pdflow_solver* s, unsigned* rows, unsigned* cols, unsigned* ctf_levels,
                      unsigned* pyr_levels, unsigned* cam_mode);

/* Selects the execution form of pdflow_solve: 0 = stream of kernels,
 * 1 = the whole solve replayed as one captured CUDA graph (default). */
int pdflow_set_graph_mode(pdflow_solver* s, int use_graph);

/* ---- Batches: many independent pairs of one configuration in one handle ----
 * The reference solves one pair per object; a batch handle holds `max_pairs`
 * solver states in one device allocation and runs the same coarse-to-fine
 * schedule for pairs [0, n) with one launch per kernel for all of them.  Each
 * pair's result equals a single-pair solve of the same frames, bit for bit.
 * Multi-pair buffers are contiguous arrays of per-pair buffers with the
 * layouts of the single-pair calls above. */

/* Creates a handle for up to max_pairs pairs (pdflow_create == max_pairs 1). */
int pdflow_create_batch(unsigned rows, unsigned width, unsigned height, const pdflow_params* params,
                        unsigned max_pairs, pdflow_solver** out);

/* Pushes one frame for each of pairs [0, n): float column-major staging
 * buffers [n][width*height] (as pdflow_push_frame). */
int pdflow_push_frames(pdflow_solver* s, unsigned n, const float* I, const float* Z);

/* Pushes raw frames [n][height][width] uint8 / uint16 (as pdflow_push_frame_u16). */
int pdflow_push_frames_u16(pdflow_solver* s, unsigned n, const uint8_t* intensity, const uint16_t* depth);

/* Pushes RGB888 [n][height][width][3] + millimetre depth [n][height][width]
 * frames (as pdflow_push_frame_rgb8_mm); host and device-pointer variants. */
int pdflow_push_frames_rgb8_mm(pdflow_solver* s, unsigned n, const uint8_t* rgb, const uint16_t* depth_mm,
                               int rotate180);
int pdflow_push_frames_rgb8_mm_device(pdflow_solver* s, unsigned n, const uint8_t* d_rgb, const uint16_t* d_depth_mm,
                                      int rotate180);

/* Same with device pointers (contiguous [n][height][width]). */
int pdflow_push_frames_u16_device(pdflow_solver* s, unsigned n, const uint8_t* d_intensity,
                                  const uint16_t* d_depth);

/* Solves pairs [0, n) (asynchronous on the handle's stream). */
int pdflow_solve_batch(pdflow_solver* s, unsigned n);

/* Copies the motion fields of pairs [0, n) to host arrays [n][rows*cols]. */
int pdflow_read_flow_batch(pdflow_solver* s, unsigned n, float* dx, float* dy, float* dz);

/* Capacity of a handle and the byte distance between consecutive pairs'
 * device buffers (pdflow_flow_device returns pair 0's planes). */
int pdflow_batch_info(const pdflow_solver* s, unsigned* max_pairs, size_t* pair_stride_bytes);

/* Device memory held by the handle, in bytes (0 for NULL). */
size_t pdflow_device_bytes(const pdflow_solver* s);

/* ---- Slot-addressed batches (serving; no counterpart in the reference) ----
 * Each of the handle's max_pairs slots is an independent camera stream: a
 * push moves the slot's newest frame (pyramid kept on the device) to the
 * previous-frame position and decodes the new one into its place, so a
 * stream's frame t is decoded once and reused as frame t-1 of the next pair.
 * slots[k] (distinct, < max_pairs) is the slot of input k; inputs are
 * [n][height][width].  Once a handle has been pushed per slot it accepts only
 * slot calls (and vice versa: PDFLOW_ERR_STATE). */
int pdflow_push_frames_slots_u16(pdflow_solver* s, unsigned n, const unsigned* slots, const uint8_t* intensity,
                                 const uint16_t* depth);
int pdflow_push_frames_slots_u16_device(pdflow_solver* s, unsigned n, const unsigned* slots,
                                        const uint8_t* d_intensity, const uint16_t* d_depth);
/* Solves the listed slots (each must hold two frames) in one batch. */
int pdflow_solve_slots(pdflow_solver* s, unsigned n, const unsigned* slots);
/* Copies the listed slots' motion fields to host arrays [n][rows*cols]. */
int pdflow_read_flow_slots(pdflow_solver* s, unsigned n, const unsigned* slots, float* dx, float* dy, float* dz);

/* ---- Mixed-resolution batches (no counterpart in the reference) ----
 * One handle holds pairs of different rows (15..480; rows 480 take 640x480
 * frames, smaller rows 320x240 frames, as the reference's cam_mode) and
 * solves them with one launch per kernel per coarse-to-fine step: all rows
 * classes share the 15x20 -> 480x640 ladder, so at every step the pairs that
 * have that level solve the same size.  Each pair's iteration schedule is the
 * reference default for its rows, and each pair's result equals a single-pair
 * solve of the same frames, bit for bit.  Iterations run in the tile form. */
int pdflow_create_mixed(unsigned max_pairs, pdflow_solver** out);
/* Pushes one frame for each of pairs [0, n): rows[k] is pair k's rows; the
 * frames of the rows-480 pairs come, in pair order, from vga_* ([m][480][640])
 * and the others' from qvga_* ([m'][240][320]).  A rows vector that differs
 * from the previous push starts new pairs. */
int pdflow_push_frames_mixed(pdflow_solver* s, unsigned n, const unsigned* rows, const uint8_t* vga_intensity,
                             const uint16_t* vga_depth, const uint8_t* qvga_intensity, const uint16_t* qvga_depth);
int pdflow_solve_mixed(pdflow_solver* s, unsigned n);
/* Copies pair k's motion field (rows_k x cols_k floats each) to host memory; blocks. */
int pdflow_read_flow_mixed(pdflow_solver* s, unsigned k, float* dx, float* dy, float* dz);

/* ---- Launch-form autotuner (no counterpart in the reference) ----
 * A level's iterations can run as two kernels per iteration (form 0), one
 * persistent launch per level (form 1: one CTA, a cluster, or, for a single
 * pair, the cooperative grid) or temporally blocked shared-memory tiles with
 * 2..4 iterations per launch (the iterations between two grid-wide
 * synchronisations), one pixel per lane (form 2) or pixel pairs in packed
 * FP32x2 arithmetic (form 3: 40x40 tiles, 576 threads; form 4: 40x34 tiles,
 * 1008 threads; form 5: 24x24 tiles, 512 threads, two CTAs per SM; form 6:
 * 24x28 tiles, 288 threads owning two pairs each, two CTAs per SM; form 7:
 * 24x24 tiles with the state in registers, 256 threads owning four rows each,
 * two CTAs per SM, levels with rows % 4 == 0; form 8: the same regions
 * walked by one persistent CTA per SM with the state and constants in
 * registers while the next region streams into shared memory by TMA (levels
 * with rows % 4 == 0; other even row counts load each pixel pair directly);
 * form 9: the same with 16x16 interiors and a halo of 8,
 * up to 8 iterations per launch, for levels whose launches are latency-bound;
 * form 10: rows of regions walked left to right, each handing the next its
 * last exact column's exchange values, so no left halo is recomputed; levels
 * with rows % 4 == 0).
 * pdflow_autotune times every eligible candidate of every
 * level for pairs [0, n) of the pushed frames (probe_iters iterations each,
 * 0 = 12; use a multiple of 12 so every candidate runs whole launches) and keeps the fastest per level; all forms give the same bits.  The
 * handle's solution state is overwritten (the pushed frames are kept).  On a
 * mixed-resolution handle (pdflow_create_mixed) it tunes per coarse-to-fine
 * step (report level i = the 15*2^i x 20*2^i step) over the pairs active at
 * that step, among the tile forms 3..8 (2, 3 or 4 iterations per launch);
 * pdflow_solve_mixed then runs each step in its chosen form. */
#define PDFLOW_TUNE_CANDIDATES 29     /* form 0, form 1, forms 2..8 x {2, 3, 4}, form 9 x {4, 6, 8}, form 10 x {2, 3, 4} */
typedef struct pdflow_tune_level {
    int form;                         /* chosen form */
    unsigned iters_per_launch;        /* chosen iterations per launch (forms 2..10) */
    float ms_per_iter[PDFLOW_TUNE_CANDIDATES];   /* per candidate; NaN if not eligible */
} pdflow_tune_level;
typedef struct pdflow_tune_report {
    unsigned levels;
    pdflow_tune_level level[8];
} pdflow_tune_report;
int pdflow_autotune(pdflow_solver* s, unsigned n, unsigned probe_iters, pdflow_tune_report* report);
/* Sets level `level`'s form by hand (-1 restores the default choice). */
int pdflow_set_level_form(pdflow_solver* s, unsigned level, int form, unsigned iters_per_launch);

/* ---- Energy of a solution (no counterpart in the reference) ----
 * The functional the iterations minimise, evaluated at the last solve's
 * finest-level solution of pairs [0, n) (blocks; host array [n]):
 *   sum over pixels of |I2(x+u) - I1(x)| + mu(x) |Z2(x+u) - Z1(x) - dw|
 *   + lambda_i (|r grad du| + |r grad dv|) + lambda_d |r grad dw|
 * with the warped data terms and the data weight mu(x) of the solver's own
 * warping at the solution's flow (pdflow_cudalib.cu:629-808) and the
 * ri/rj-weighted forward differences of its gradient (:982-1013). */
int pdflow_energy_batch(pdflow_solver* s, unsigned n, float* energies);

/* Device planes of pair 0's finest-level image-plane solution (du, dv in
 * pixels of the finest solved level, dw in metres; column-major rows*cols;
 * pair k at + k * pair_stride_bytes), valid after a solve completes. */
int pdflow_image_flow_device(pdflow_solver* s, const float** du, const float** dv, const float** dw);

/* ---- Allocation-free solve (no counterpart in the reference) ----
 * For callers that cannot allocate device memory after start-up (a real-time
 * or safety-critical camera loop with a fixed memory budget, or a plugin whose
 * host framework owns every allocation): one pair solved entirely in scratch
 * memory compiled into this library, a 12 MiB __device__ array.  A GPU holds
 * those 12 MiB from the first call on it (when the driver loads the array's
 * module; with CUDA_MODULE_LOADING=EAGER from context creation) until the
 * process exits.  It fits 320x240 frames with rows <= 120; larger
 * configurations return PDFLOW_ERR_ARG.
 * Inputs: both frames as device pointers, row-major uint8 intensity and
 * uint16 depth (metres * 5000), height x width.  Outputs: device planes of
 * rows*cols floats (column-major, as pdflow_read_flow).  Work is queued on
 * `stream` (a cudaStream_t, NULL = the legacy default stream) and the call
 * returns without waiting.  The first call on a device resolves the scratch
 * array's device address (cudaGetSymbolAddress) and sets kernel attributes:
 * make it before any stream capture.  All calls share the scratch array, which
 * keeps the last call's contents; calls that overlap on the GPU race on it and
 * must be serialised by the caller.  No cudaMalloc or cudaFree is called.
 * The kernels it runs (one-CTA launch at 15x20, scalar tiles above) contain
 * no bounded device-side wait, so no device timeout can arise; launch errors
 * are returned, and asynchronous execution errors surface at the caller's next
 * synchronisation of `stream`. */
int pdflow_solve_pair_noalloc(unsigned rows, unsigned width, unsigned height, const pdflow_params* params,
                              const uint8_t* d_intensity1, const uint16_t* d_depth1, const uint8_t* d_intensity2,
                              const uint16_t* d_depth2, float* d_dx, float* d_dy, float* d_dz, void* stream);

/* ---- Per-level record (copyAllSolutions after every level) ----
 * The reference's live application copies every solved level's motion field
 * and images to the host as the solve climbs the pyramid
 * (scene_flow_visualization.cpp:194-199, CSF_cuda::copyAllSolutions,
 * pdflow_cudalib.cu:224-237).  pdflow_keep_level_solutions(s, 1) makes every
 * later solve record, per pair and per solved level, the median-filtered
 * image-plane flow (du, dv in that level's pixels, dw in metres) and its
 * motion field (computeMotionField at that level, pdflow_cudalib.cu:1150-1167,
 * which uses the focal length of the finest solved width at every level).
 * The record (6 planes per level per pair) is allocated by the first call
 * that turns it on; 0 turns recording off.  Mixed-resolution handles refuse
 * (PDFLOW_ERR_STATE).  Levels are numbered as the schedule visits them:
 * 0 = the coarsest (15x20), ctf_levels - 1 = the finest (rows x cols); level
 * i has (rows >> (L-1-i)) x (cols >> (L-1-i)) pixels, column-major. */
int pdflow_keep_level_solutions(pdflow_solver* s, int keep);
/* copyAllSolutions at solved level `level` for pair 0: its motion field and
 * both frames' depth, intensity and back-projected xx, yy at that level's
 * pyramid image (any pointer may be NULL; blocks).  Needs the record. */
int pdflow_read_level_solutions(pdflow_solver* s, unsigned level, float* dx, float* dy, float* dz, float* depth,
                                float* depth_old, float* colour, float* colour_old, float* xx, float* xx_old,
                                float* yy, float* yy_old);
/* Pair `pair`'s record at solved level `level`: image-plane flow (du, dv, dw;
 * the reference's du_l, dv_l, dw_l after filterSolution) and motion field
 * (dx, dy, dz); any pointer may be NULL; blocks. */
int pdflow_read_level_flow(pdflow_solver* s, unsigned pair, unsigned level, float* du, float* dv, float* dw,
                           float* dx, float* dy, float* dz);

/* Human-readable text of the last error on this thread. */
const char* pdflow_last_error(void);

/* Library version string. */
const char* pdflow_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PDFLOW_H */
