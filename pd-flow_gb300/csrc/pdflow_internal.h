// Internal definition of the solver handle (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/pdflow.h"
#include "../../include/pdflow_net.h"
#include "pdflow_iterate.cuh"
#include "pdflow_kernels.cuh"

struct pdflow_solver {
    int device = 0;
    unsigned rows = 0, cols = 0, width = 0, height = 0, cam_mode = 0, ctf_levels = 0, pyr_levels = 0;
    pdflow_params prm{};
    cudaStream_t stream = nullptr;       // stream used for all work of the handle
    cudaStream_t own_stream = nullptr;
    void* arena = nullptr;               // the one device allocation of the handle
    size_t arena_bytes = 0;
    // Pyramid of the two frames [slot][level]; `new_slot` holds the newest frame.
    pdflow::PyrLevel pyr[2][8]{};
    int new_slot = 1;
    int frames = 0;                      // frames pushed (saturates at 2)
    float* stage_I = nullptr;            // device staging of a float frame
    float* stage_Z = nullptr;
    uint8_t* stage_u8 = nullptr;         // device staging of a raw frame
    uint16_t* stage_u16 = nullptr;
    uint8_t* stage_rgb = nullptr;        // device staging of RGB888 frames (allocated on first use)
    double* energy_part = nullptr;       // energy partial sums [batch][1024]
    float* sol_keep = nullptr;           // learned path: the plain 60x80 solutions [slot][10][4800] and ...
    unsigned* map2 = nullptr;            // ... a second slot map [batch] (one allocation, on first use)
    int keep_levels = 0;                 // record every solved level's solution (pdflow_keep_level_solutions)
    float* lvl_keep = nullptr;           // per slot: per level du, dv, dw, dx, dy, dz planes (on first use)
    size_t lvl_keep_stride = 0;          // floats per slot of lvl_keep
    pdflow::LevelConsts L{};
    pdflow::State S{};
    float* alt[10] = {};                 // second buffer of du_acc,dv_acc,dw_acc,pd,puu,puv,pvu,pvv,pwu,pwv
    float* alt_d[3] = {};                // second buffer of du,dv,dw (tile form)
    pdflow::LevelSol sol{};
    unsigned* flags = nullptr;           // per-CTA progress counters of the grid-form iteration
    unsigned* status = nullptr;          // device status word (0 = ok)
    int num_sms = 0;
    int iter_form = 10;                  // 10 = streamed strips (levels with a strip per SM; others 9 or 8),
                                         // 9 = deep streamed tiles,
                                         // 8 = streamed register tiles (persistent, one CTA per SM), 7 = quad
                                         // register tiles, 5 / 4 / 3 = paired tiles 24x24 (two CTAs per SM) / 40x34 / 40x40,
                                         // 2 = scalar tiles for large levels,
                                         // 1 = one launch per level, 0 = two kernels per iteration
    int level_form[8] = {-1, -1, -1, -1, -1, -1, -1, -1};   // per-level override (autotuner); -1 = iter_form's choice
    unsigned level_kk[8] = {};           // tile form: iterations per launch (0 = the halo width)
    float* dx = nullptr;
    float* dy = nullptr;
    float* dz = nullptr;
    int use_graph = 1;
    unsigned batch = 1;                  // pairs the arena holds
    size_t pair_stride = 0;              // bytes between pair k and pair k+1 buffers
    unsigned launches = 0;               // kernel launches of the last enqueued solve
    unsigned* map = nullptr;             // device [batch]: arena slots of a slot-addressed push / solve
    float* energy = nullptr;             // device [2 * batch]: energies written by a solve
    float* seed = nullptr;               // device [batch][3][seed level N]: warm-start fields
    int slot_mode = 0;                   // 1 once frames were pushed per slot (then only per slot)
    std::vector<unsigned char> slot_frames;   // frames pushed per slot (saturates at 2)
    struct GraphEntry {
        int slot;
        unsigned pairs;
        int form;
        unsigned kind;                   // which enqueue sequence (plain, slot-mapped, learned ...)
        unsigned long long key;          // identity of the object the sequence reads (the network's uid), or 0
        cudaGraphExec_t exec;
        unsigned launches;
    };
    std::vector<GraphEntry> graphs;      // captured solves, per (slot, pair count, iteration form)
    // mixed-resolution batches (pdflow_mixed.cu): VGA-sized slots holding pairs of any rows
    int mixed = 0;
    std::vector<unsigned> mixed_rows;    // rows of the pair in each slot (0: none)
    unsigned* map_table = nullptr;       // device: the slot maps of every launch of the mixed plan
    size_t map_table_cap = 0;
    std::vector<unsigned> plan_rows;     // rows vector + per-step choices the current table / graph were built for
    cudaGraphExec_t mixed_graph = nullptr;
    int mixed_graph_slot = -1;
    int mixed_form[8] = {-1, -1, -1, -1, -1, -1, -1, -1};   // per coarse-to-fine step: tile form (-1: the handle's)
    unsigned mixed_kk[8] = {};           // per step: iterations per tile launch (0: 4)
};

namespace pdflow {

// Which part of the coarse-to-fine schedule an enqueue runs, and how.
struct SolvePlan {
    unsigned first = 0;                  // first level solved
    unsigned last = ~0u;                 // last level solved (clamped to the finest)
    const float* seed = nullptr;         // device [pairs][3][N_first]: level `first` starts from it
    float iter_scale = 1.f;              // iterations of every solved level: ceil(num_max_iter * scale)
    int energy_level = -1;               // after this level's median, its energy goes to ...
    float* energy = nullptr;             // ... device [pairs]
    const unsigned* map = nullptr;       // device [pairs] arena slots (null: slots 0..pairs-1)
    bool all_steps = false;              // write the step-size planes even for levels run as tiles
    cudaEvent_t* trace = nullptr;        // eager runs only: 3 per solved level + 1, recorded before
                                         // each level's set-up, iterations and median, and at the end
};

constexpr unsigned kSeedLevel = 2;       // the 60x80 level (15x20 -> 30x40 -> 60x80)
constexpr unsigned kSeedN = 60 * 80;

void carve_solver(pdflow_solver* s, char* base, size_t* used);
int enqueue_pyramid(pdflow_solver* s, cudaStream_t st, unsigned pairs, const unsigned* map = nullptr);
int enqueue_solve(pdflow_solver* s, cudaStream_t st, unsigned pairs, const SolvePlan& plan = SolvePlan());
int enqueue_energy(pdflow_solver* s, cudaStream_t st, unsigned pairs, unsigned level, float* out,
                   const unsigned* map = nullptr);
unsigned scaled_iters(unsigned iters, float scale);
// Float offset of level `level`'s six planes in a slot of the per-level record.
size_t level_keep_offset(const pdflow_solver* s, unsigned level);
// Runs fn(s, stream, pairs, ctx) on the handle's stream, through a cached CUDA
// graph keyed by (new frame slot, pairs, iteration form, kind) in graph mode.
// Whatever fn reads from ctx is baked into the graph: equal kinds must mean
// equal ctx contents.
using EnqueueFn = int (*)(pdflow_solver* s, cudaStream_t st, unsigned pairs, const void* ctx);
int run_graphed(pdflow_solver* s, unsigned pairs, unsigned kind, EnqueueFn fn, const void* ctx,
                unsigned long long key = 0);
int set_error_code(int code, const char* what, cudaError_t e = cudaSuccess);
// The learned slot solve with every pair sent down the fallback path (the
// serving lanes' graph warm-up uses it to capture the fallback graphs).
// An NVTX range over a host-side scope (tracing: nsys / ncu --nvtx show the
// library's calls and phases; without a tool attached it costs a function call).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Device bytes of the learned path's buffers (kept 60x80 solutions + second slot map).
inline size_t learned_keep_bytes(unsigned batch)
{
    return (sizeof(float) * 10 * kSeedN + sizeof(unsigned)) * size_t(batch);
}
int learned_solve_all_fallback(pdflow_solver* s, unsigned n, const unsigned* slots, ::pdflow_net* net,
                               const ::pdflow_learned_opts* opts);
int enqueue_level_iterations(pdflow_solver* s, cudaStream_t st, unsigned pairs, unsigned level, unsigned iters);
// Autotuner of a mixed-resolution handle (pdflow_mixed.cu): per coarse-to-fine
// step, the tile form and iterations per launch over the pairs active there.
int mixed_autotune(pdflow_solver* s, unsigned n, unsigned probe_iters, pdflow_tune_report* report);

// Candidate c (0 <= c < PDFLOW_TUNE_CANDIDATES) of the launch-form autotuners:
// its iteration form and iterations per launch (0 for forms 0 and 1).
struct TuneCandidate {
    int form;
    unsigned kk;
};
TuneCandidate tune_candidate(int c);
int check_status(pdflow_solver* s);
void set_last_error(const char* text);   // the text pdflow_last_error returns on this thread
LevelGeom level_geom(const pdflow_solver* s, unsigned i, unsigned* level_image, unsigned pairs = 1);
}  // namespace pdflow
