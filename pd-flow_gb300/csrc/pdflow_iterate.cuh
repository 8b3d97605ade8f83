// One-launch iteration of a pyramid level (see pdflow_iterate.cu).
#pragma once
#include <cuda_runtime.h>

#include "pdflow_kernels.cuh"

namespace pdflow {

enum IterMode { kIterSingle = 0, kIterCluster = 1, kIterGrid = 2 };

// Value left in the status word when a bounded wait gives up.
constexpr unsigned kStatusTimeout = 1u;

struct IterArgs {
    LevelGeom g;
    LevelConsts L;
    float *du, *dv, *dw;          // primal increments (updated in place; saturated after the last iteration)
    float* acc[2][3];             // over-relaxed primal, double buffered: [buffer][du, dv, dw]
    float* p_[2][7];              // duals, double buffered: [buffer][pd, puu, puv, pvu, pvv, pwu, pwv]
    Params p;
    const float* depth_old;       // old frame depth at this level (saturation)
    unsigned iters;
    unsigned* flags;              // per-CTA completed-iteration counters (grid form)
    unsigned* status;             // 0, or kStatusTimeout after a bounded wait gave up
    unsigned smem_plane;          // floats per shared plane of new duals (set by launch_iterate)
    unsigned smem_state_plane;    // floats per shared state plane (set by launch_iterate)
};

struct IterPlan {
    int mode = kIterSingle;
    unsigned ctas = 1;
    unsigned smem_plane = 0;
    unsigned smem_state_plane = 0;
    size_t smem_bytes = 0;
};

// Launch shape for a level on a GPU with `num_sms` SMs.
IterPlan plan_iterate(LevelGeom g, int num_sms);
// Dynamic shared memory the iteration kernels may use (after prepare_iterate).
unsigned iterate_smem_limit();
// One-time function attributes (dynamic shared memory, cluster size).
cudaError_t prepare_iterate();
// Temporally blocked form (pdflow_tiles.cu): `kk` iterations of every tile of
// the level, state read from `src` and the tiles' interiors written to `dst`.
cudaError_t prepare_tiles();
unsigned tiles_halo();
size_t tiles_smem_bytes();
unsigned tiles_per_level(LevelGeom g);
cudaError_t launch_iterate_tiles(LevelGeom g, LevelConsts L, State src, State dst, Params p, const float* depth_old,
                                 unsigned kk, bool last, cudaStream_t st);
// The paired FP32x2 variant of the same tiling (pdflow_tiles2.cu); same bits.
// Shapes: 0 = 40x40 tiles (iteration form 3), 1 = 40x34 (form 4), 2 = 24x24
// (form 5, two CTAs per SM).  set_tile_copy_mode: bit 0 = bulk load, bit 1 = bulk store.
void set_tile_copy_mode(int shape, int mode);
cudaError_t prepare_tiles2();
cudaError_t launch_iterate_tiles2(LevelGeom g, LevelConsts L, State src, State dst, Params p, const float* depth_old,
                                  unsigned kk, bool last, cudaStream_t st, int shape = 0,
                                  unsigned* status = nullptr);
// Register-resident quad tiles (pdflow_quads.cu, iteration form 7): 32x32
// regions, one thread per 4-row quad, constants by TMA (the step products
// in L.qs, written by a kStepsQuads / kStepsAll set-up); same bits.  Needs
// rows % 4 == 0 and 16-byte aligned planes (quads_eligible).
cudaError_t prepare_quads();
// Persistent streamed tiles (pdflow_ptiles.cu, iteration forms 8-10): one
// CTA per SM (`ctas` CTAs) walks 32x32 regions of the launch with their
// state in registers while the next region streams into shared memory by
// TMA: 24x24 interiors and a halo of 4 (form 8), 16x16 interiors and a halo
// of 8 (form 9, up to 8 iterations per launch), or rows of regions walked
// left to right that carry their left neighbour's exchange values (form 10,
// 24-row interiors, 32 - kk exact columns per region); same preconditions
// (quads_eligible) and same bits.  `status` is the handle's four device
// words: [0] the status word, [2] and [3] the strip walk's unit counters
// (zero between launches; the kernel leaves them so).
enum class StreamLayout { Tiles24, Tiles16, Strips };
// Whether a level can run register-resident tile form `form` (7-10): the
// quad tiles and the strips need quads_eligible (tensor copies); the
// streamed tiles (8, 9) also run on direct loads where the rows are even.
bool stream_eligible(const LevelGeom& g, const LevelConsts& L, const State& src, const State& dst, int form);
bool stream_direct_eligible(const LevelGeom& g, const LevelConsts& L, const State& src, const State& dst);
// The strip walk's units for `strips_n` bands of C columns on `grid` CTAs at
// kk iterations per launch: bands [0, whole) whole, then for tier i = 0..2
// the next tier_n[i] bands in tier_p[i] column pieces each.
struct StripUnits {
    unsigned whole, tier_n[3], tier_p[3];
};
StripUnits strip_units(unsigned strips_n, unsigned C, unsigned kk, unsigned grid);
inline StreamLayout stream_layout(int form)
{
    return form == 9 ? StreamLayout::Tiles16 : (form == 10 ? StreamLayout::Strips : StreamLayout::Tiles24);
}
cudaError_t prepare_stream_tiles();
size_t stream_smem_bytes();
cudaError_t launch_iterate_stream(LevelGeom g, LevelConsts L, State src, State dst, Params p, const float* depth_old,
                                  unsigned kk, bool last, cudaStream_t st, unsigned* status, unsigned ctas,
                                  StreamLayout layout);
// L2 prefetch distance of the quad tiles in CTAs (0 = off).
void set_quad_prefetch(unsigned ctas_ahead);
size_t quads_smem_bytes();
bool quads_eligible(const LevelGeom& g, const LevelConsts& L, const State& src, const State& dst);
cudaError_t launch_iterate_quads(LevelGeom g, LevelConsts L, State src, State dst, Params p, const float* depth_old,
                                 unsigned kk, bool last, cudaStream_t st, unsigned* status);
// Failure-detection probe: two CTAs where one waits (the grid form's bounded
// neighbour wait, `polls` polls) for a progress counter the other never sets;
// the wait runs out and records kStatusTimeout in *status.  flags: 2 counters.
cudaError_t launch_wait_probe(unsigned* flags, unsigned* status, unsigned polls, cudaStream_t st);
// Enqueues the level's iterations (and, in the grid form, the reset of the progress counters).
cudaError_t launch_iterate(const IterPlan& pl, IterArgs a, cudaStream_t st);

}  // namespace pdflow
