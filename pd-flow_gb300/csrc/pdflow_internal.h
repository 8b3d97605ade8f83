// Internal definition of the solver handle (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/pdflow.h"
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
    pdflow::LevelConsts L{};
    pdflow::State S{};
    float* alt[10] = {};                 // second buffer of du_acc,dv_acc,dw_acc,pd,puu,puv,pvu,pvv,pwu,pwv
    float* alt_d[3] = {};                // second buffer of du,dv,dw (tile form)
    pdflow::LevelSol sol{};
    unsigned* flags = nullptr;           // per-CTA progress counters of the grid-form iteration
    unsigned* status = nullptr;          // device status word (0 = ok)
    int num_sms = 0;
    int iter_form = 2;                   // 2 = tiles for large levels, 1 = one launch per level, 0 = two kernels per iteration
    float* dx = nullptr;
    float* dy = nullptr;
    float* dz = nullptr;
    int use_graph = 1;
    unsigned batch = 1;                  // pairs the arena holds
    size_t pair_stride = 0;              // bytes between pair k and pair k+1 buffers
    unsigned launches = 0;               // kernel launches of the last enqueued solve
    struct GraphEntry {
        int slot;
        unsigned pairs;
        int form;
        cudaGraphExec_t exec;
        unsigned launches;
    };
    std::vector<GraphEntry> graphs;      // captured solves, per (slot, pair count, iteration form)
};

namespace pdflow {
void carve_solver(pdflow_solver* s, char* base, size_t* used);
int enqueue_pyramid(pdflow_solver* s, cudaStream_t st, unsigned pairs);
int enqueue_solve(pdflow_solver* s, cudaStream_t st, unsigned pairs);
int enqueue_level_iterations(pdflow_solver* s, cudaStream_t st, unsigned pairs, unsigned level, unsigned iters);
int check_status(pdflow_solver* s);
void set_last_error(const char* text);   // the text pdflow_last_error returns on this thread
LevelGeom level_geom(const pdflow_solver* s, unsigned i, unsigned* level_image, unsigned pairs = 1);
}  // namespace pdflow
