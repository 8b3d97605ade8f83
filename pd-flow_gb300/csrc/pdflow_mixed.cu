// Mixed-resolution batches (include/pdflow.h): pairs with rows 15..480 in one
// handle, one launch per kernel per coarse-to-fine step for all of them.
//
// Every rows class starts at a 15x20 level and doubles, so at step i every
// pair that has an i-th level solves the same 15*2^i x 20*2^i size.  Slots are
// sized for 640x480 frames; a 320x240 frame is decoded into the second
// pyramid slot (320x240, the size of a VGA pyramid's level 1), so at step i
// all pairs also read the same pyramid slot (5 - i).  What differs per pair
// is carried by its slot-map entry: the active pairs of a step, whether a tile
// launch ends the pair's level (its iteration count: 100 at its finest level,
// 15 fewer per coarser one), which state buffer its level ended in, and
// whether the step is its finest level (motion field).  The per-launch maps of
// the whole solve are built on the host once per rows vector, uploaded as one
// table, and the solve is replayed as one CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/pdflow.h"
#include "pdflow_internal.h"

using namespace pdflow;

namespace {

constexpr unsigned kSteps = 6;   // 15x20 .. 480x640

unsigned levels_of(unsigned rows)
{
    unsigned l = 0;
    for (unsigned r = rows / 15; r > 1; r >>= 1) ++l;
    return l + 1;
}

bool is_rows(unsigned r) { return r == 15 || r == 30 || r == 60 || r == 120 || r == 240 || r == 480; }

struct LaunchRec {
    int kind;            // 0 set-up (init, gradients, warp), 1 tiles, 2 median
    unsigned step, kk, off, count;
};

// The launches of a solve and their slot maps (flags in the high bits).
void build_plan(const std::vector<unsigned>& rows, std::vector<LaunchRec>& plan, std::vector<unsigned>& table)
{
    plan.clear();
    table.clear();
    const unsigned n = unsigned(rows.size());
    for (unsigned i = 0; i < kSteps; ++i) {
        std::vector<unsigned> act;
        for (unsigned k = 0; k < n; ++k)
            if (levels_of(rows[k]) > i) act.push_back(k);
        if (act.empty()) continue;
        plan.push_back({0, i, 0, unsigned(table.size()), unsigned(act.size())});
        table.insert(table.end(), act.begin(), act.end());
        std::vector<unsigned> remaining(act.size()), launches(act.size(), 0);
        for (size_t a = 0; a < act.size(); ++a) remaining[a] = 100u - 15u * (levels_of(rows[act[a]]) - 1u - i);
        for (;;) {
            unsigned kk = 4, live = 0;
            for (unsigned r : remaining)
                if (r > 0) {
                    kk = std::min(kk, r);
                    ++live;
                }
            if (!live) break;
            plan.push_back({1, i, kk, unsigned(table.size()), live});
            for (size_t a = 0; a < act.size(); ++a)
                if (remaining[a] > 0) {
                    remaining[a] -= kk;
                    ++launches[a];
                    table.push_back(act[a] | (remaining[a] == 0 ? kMapLast : 0u));
                }
        }
        plan.push_back({2, i, 0, unsigned(table.size()), unsigned(act.size())});
        for (size_t a = 0; a < act.size(); ++a)
            table.push_back(act[a] | ((launches[a] & 1u) ? kMapAlt : 0u) |
                            (levels_of(rows[act[a]]) == i + 1 ? kMapFinest : 0u));
    }
}

int enqueue_mixed(pdflow_solver* s, cudaStream_t st, const std::vector<LaunchRec>& plan, unsigned* count)
{
    Params p{s->prm.lambda_i, s->prm.lambda_d, s->prm.mu, s->prm.fovh, s->cols};
    const int fn = s->new_slot, fo = fn ^ 1;
    const State alt{s->alt_d[0], s->alt_d[1], s->alt_d[2], s->alt[0], s->alt[1], s->alt[2], s->alt[3], s->alt[4],
                    s->alt[5], s->alt[6], s->alt[7], s->alt[8], s->alt[9]};
    State cur = s->S, nxt = alt;
    for (const LaunchRec& r : plan) {
        const unsigned R = 15u << r.step, C = 20u << r.step;
        LevelGeom g{R, C, R * C};
        g.pairs = r.count;
        g.pstride = s->pair_stride;
        g.slots = s->batch;
        g.map = s->map_table + r.off;
        const unsigned li = kSteps - 1 - r.step;
        const PyrLevel o = s->pyr[fo][li], n = s->pyr[fn][li];
        cudaError_t e = cudaSuccess;
        if (r.kind == 0) {
            e = launch_level_init(g, r.step == 0, s->sol, o, n, s->L, s->S, st);
            if (e == cudaSuccess) e = launch_im_gradients(g, n, s->L, st);
            if (e == cudaSuccess) e = launch_warp_steps(g, o, n, s->L, p, st, false);   // tiles only
            *count += 3;
            cur = s->S;
            nxt = alt;
        } else if (r.kind == 1) {
            const int shape = s->iter_form >= 3 ? s->iter_form - 3 : 2;   // the paired tiles of the handle's form
            e = launch_iterate_tiles2(g, s->L, cur, nxt, p, o.dep, r.kk, false, st, shape, s->status);
            std::swap(cur, nxt);
            *count += 1;
        } else {
            e = launch_median(g, false, o, s->L, s->S, s->sol, s->dx, s->dy, s->dz, p, nullptr, st, &alt, true);
            *count += 1;
        }
        if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "mixed batch launch", e);
    }
    return PDFLOW_OK;
}

}  // namespace

extern "C" {

int pdflow_create_mixed(unsigned max_pairs, pdflow_solver** out)
{
    int rc = pdflow_create_batch(480, 640, 480, nullptr, max_pairs, out);
    if (rc) return rc;
    (*out)->mixed = 1;
    (*out)->mixed_rows.assign(max_pairs, 0);
    return PDFLOW_OK;
}

int pdflow_push_frames_mixed(pdflow_solver* s, unsigned n, const unsigned* rows, const uint8_t* vga_intensity,
                             const uint16_t* vga_depth, const uint8_t* qvga_intensity, const uint16_t* qvga_depth)
{
    if (!s || !rows) {
        set_last_error("null argument");
        return PDFLOW_ERR_ARG;
    }
    if (!s->mixed) {
        set_last_error("not a mixed-resolution handle (pdflow_create_mixed)");
        return PDFLOW_ERR_STATE;
    }
    if (n == 0 || n > s->batch) {
        set_last_error("pair count out of range");
        return PDFLOW_ERR_ARG;
    }
    std::vector<unsigned> vga, qvga;
    for (unsigned k = 0; k < n; ++k) {
        if (!is_rows(rows[k])) {
            set_last_error("rows must be one of 15,30,60,120,240,480");
            return PDFLOW_ERR_ARG;
        }
        (rows[k] == 480 ? vga : qvga).push_back(k);
    }
    if ((!vga.empty() && (!vga_intensity || !vga_depth)) || (!qvga.empty() && (!qvga_intensity || !qvga_depth))) {
        set_last_error("missing frames for the VGA or QVGA pairs");
        return PDFLOW_ERR_ARG;
    }
    bool same = s->frames > 0;
    for (unsigned k = 0; k < n && same; ++k) same = s->mixed_rows[k] == rows[k];
    if (!same) s->frames = 0;   // a new rows assignment starts new pairs
    for (unsigned k = 0; k < n; ++k) s->mixed_rows[k] = rows[k];
    for (unsigned k = n; k < s->batch; ++k) s->mixed_rows[k] = 0;
    s->new_slot ^= 1;
    const int f = s->new_slot;
    const size_t vimg = 640u * 480u, qimg = 320u * 240u;
    // VGA frames: level 0 of the slot; QVGA frames: pyramid slot 1 (320x240)
    struct Group {
        const std::vector<unsigned>* slots;
        const uint8_t* I;
        const uint16_t* Z;
        size_t img;
        unsigned W, H, level;
    } groups[2] = {{&vga, vga_intensity, vga_depth, vimg, 640, 480, 0}, {&qvga, qvga_intensity, qvga_depth, qimg, 320, 240, 1}};
    for (const Group& gr : groups) {
        const unsigned m = unsigned(gr.slots->size());
        if (!m) continue;
        cudaError_t e = cudaMemcpyAsync(s->map, gr.slots->data(), sizeof(unsigned) * m, cudaMemcpyHostToDevice,
                                        s->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(s->stage_u8, gr.I, gr.img * m, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->stage_u16, gr.Z, gr.img * 2 * m, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess)
            e = launch_decode_u16(s->stage_u8, s->stage_u16, gr.W, gr.H, s->pyr[f][gr.level], s->prm.fovh, m,
                                  s->pair_stride, s->stream, s->map);
        if (e == cudaSuccess && gr.level == 0)   // VGA pairs: their 320x240 level
            e = launch_pyr_down(s->pyr[f][0], 240, 320, s->pyr[f][1], s->prm.fovh, m, s->pair_stride, s->stream,
                                s->map);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);   // the map and staging are reused
        if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "mixed push", e);
    }
    // levels 2.. for every pair (slots 0..n-1)
    for (unsigned l = 2; l < s->pyr_levels; ++l) {
        cudaError_t e = launch_pyr_down(s->pyr[f][l - 1], 480u >> l, 640u >> l, s->pyr[f][l], s->prm.fovh, n,
                                        s->pair_stride, s->stream);
        if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "mixed pyramid", e);
    }
    if (s->frames < 2) ++s->frames;
    return PDFLOW_OK;
}

int pdflow_solve_mixed(pdflow_solver* s, unsigned n)
{
    const NvtxRange trace_range("pdflow_solve_mixed");
    if (!s) {
        set_last_error("null handle");
        return PDFLOW_ERR_ARG;
    }
    if (!s->mixed) {
        set_last_error("not a mixed-resolution handle (pdflow_create_mixed)");
        return PDFLOW_ERR_STATE;
    }
    if (n == 0 || n > s->batch || s->frames < 2) {
        set_last_error("pair count out of range or fewer than two frames pushed");
        return n == 0 || n > s->batch ? PDFLOW_ERR_ARG : PDFLOW_ERR_STATE;
    }
    std::vector<unsigned> rows(s->mixed_rows.begin(), s->mixed_rows.begin() + n);
    for (unsigned r : rows)
        if (!r) {
            set_last_error("a pair of the batch has no frames");
            return PDFLOW_ERR_STATE;
        }
    std::vector<LaunchRec> plan;
    std::vector<unsigned> table;
    build_plan(rows, plan, table);
    const bool replan = rows != s->plan_rows;
    if (replan) {
        if (table.size() > s->map_table_cap) {
            if (s->map_table) cudaFree(s->map_table);
            s->map_table = nullptr;
            cudaError_t e = cudaMalloc(&s->map_table, sizeof(unsigned) * table.size());
            if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_OOM, "map table", e);
            s->map_table_cap = table.size();
        }
        cudaError_t e = cudaMemcpyAsync(s->map_table, table.data(), sizeof(unsigned) * table.size(),
                                        cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "map table upload", e);
        if (s->mixed_graph) cudaGraphExecDestroy(s->mixed_graph);
        s->mixed_graph = nullptr;
        s->plan_rows = rows;
    }
    unsigned count = 0;
    if (!s->use_graph) {
        int rc = enqueue_mixed(s, s->stream, plan, &count);
        s->launches = count;
        return rc;
    }
    if (!s->mixed_graph || s->mixed_graph_slot != s->new_slot) {
        if (s->mixed_graph) cudaGraphExecDestroy(s->mixed_graph);
        s->mixed_graph = nullptr;
        cudaStream_t cap;
        cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "capture stream", e);
        cudaGraph_t graph = nullptr;
        e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        int rc = PDFLOW_OK;
        if (e == cudaSuccess) {
            rc = enqueue_mixed(s, cap, plan, &count);
            cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
            if (e == cudaSuccess) e = e2;
        }
        if (e == cudaSuccess && rc == PDFLOW_OK) e = cudaGraphInstantiate(&s->mixed_graph, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cap);
        if (rc) return rc;
        if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "mixed graph capture", e);
        s->mixed_graph_slot = s->new_slot;
        s->launches = count;
    }
    cudaError_t e = cudaGraphLaunch(s->mixed_graph, s->stream);
    if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "mixed graph launch", e);
    return PDFLOW_OK;
}

int pdflow_read_flow_mixed(pdflow_solver* s, unsigned k, float* dx, float* dy, float* dz)
{
    if (!s || !s->mixed || k >= s->batch || !s->mixed_rows[k]) {
        set_last_error("not a mixed handle or no pair in that slot");
        return PDFLOW_ERR_ARG;
    }
    const unsigned r = s->mixed_rows[k];
    const size_t N = size_t(r) * (r * 4 / 3), po = size_t(k) * s->pair_stride;
    float* dst[3] = {dx, dy, dz};
    const float* src[3] = {s->dx, s->dy, s->dz};
    for (int a = 0; a < 3; ++a)
        if (dst[a]) {
            cudaError_t e = cudaMemcpyAsync(dst[a], at(src[a], po), N * 4, cudaMemcpyDeviceToHost, s->stream);
            if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "D2H flow", e);
        }
    return check_status(s);
}

}  // extern "C"
