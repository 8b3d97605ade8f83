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
// the whole solve are built on the host once per rows vector (and per-step
// launch choice), uploaded as one table, and the solve is replayed as one CUDA
// graph.  Each step's iterations run in the tile form and iterations per
// launch that pdflow_autotune picked for it over the pairs active at that step
// (mixed_autotune), by default the handle's paired tiles with 4 iterations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
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

// Iterations per tile launch at step i in form `form` (the autotuned choice,
// else the halo width: 8 for the deep streamed tiles of form 9, else 4).
unsigned step_kk(const pdflow_solver* s, unsigned i, int form)
{
    const unsigned k = s->mixed_kk[i], h = form == 9 ? 8u : 4u;
    return (k >= 1 && k <= h) ? k : h;
}

// Tile form at step i: the autotuned choice, else the handle's paired form
// (forms 7 and 10 need rows % 4 == 0, forms 8 and 9 even rows; the 15x20
// level runs form 5; by default the strips, form 10, need a strip per SM and
// rows % 4 == 0, else form 8 runs, or form 9 where the 16x16 tiles fit in one
// round of CTAs).
int step_form(const pdflow_solver* s, unsigned i, const LevelGeom& g)
{
    int f = s->mixed_form[i] >= 3 ? s->mixed_form[i] : (s->iter_form >= 3 ? s->iter_form : 5);
    if (s->mixed_form[i] < 3 && f == 10 &&
        (g.pairs * ((g.R + 23u) / 24u) < unsigned(s->num_sms) || !stream_eligible(g, s->L, s->S, s->S, 10)))
        f = g.pairs * ((g.R + 15u) / 16u) * ((g.C + 15u) / 16u) <= unsigned(s->num_sms) ? 9 : 8;
    if (f >= 7 && !stream_eligible(g, s->L, s->S, s->S, f)) f = 5;
    return f;
}

LevelGeom step_geom(const pdflow_solver* s, unsigned step, unsigned pairs, const unsigned* map)
{
    const unsigned R = 15u << step, C = 20u << step;
    LevelGeom g{R, C, R * C};
    g.pairs = pairs;
    g.pstride = s->pair_stride;
    g.slots = s->batch;
    g.map = map;
    return g;
}

// kk iterations of the pairs of `g` in form `form`, state from cur to nxt.
cudaError_t launch_step_tiles(pdflow_solver* s, const LevelGeom& g, const State& cur, const State& nxt,
                              const Params& p, const PyrLevel& o, unsigned kk, cudaStream_t st, int form)
{
    if (form >= 8)
        return launch_iterate_stream(g, s->L, cur, nxt, p, o.dep, kk, false, st, s->status, s->num_sms,
                                     stream_layout(form));
    if (form == 7) return launch_iterate_quads(g, s->L, cur, nxt, p, o.dep, kk, false, st, s->status);
    return launch_iterate_tiles2(g, s->L, cur, nxt, p, o.dep, kk, false, st, form - 3, s->status);
}

// The launches of a solve and their slot maps (flags in the high bits).
void build_plan(const pdflow_solver* s, const std::vector<unsigned>& rows, std::vector<LaunchRec>& plan,
                std::vector<unsigned>& table)
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
        const unsigned step_k = step_kk(s, i, step_form(s, i, step_geom(s, i, unsigned(act.size()), nullptr)));
        for (;;) {
            unsigned kk = step_k, live = 0;
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

// Builds the plan of `rows` with the handle's per-step choices; uploads its
// map table and drops the captured graph when the rows or the choices changed.
int prepare_plan(pdflow_solver* s, const std::vector<unsigned>& rows, std::vector<LaunchRec>& plan)
{
    std::vector<unsigned> table;
    build_plan(s, rows, plan, table);
    std::vector<unsigned> sig(rows);
    for (unsigned i = 0; i < kSteps; ++i) {
        sig.push_back(s->mixed_kk[i]);
        sig.push_back(unsigned(s->mixed_form[i] + 1));
    }
    sig.push_back(unsigned(s->iter_form + 1));   // the default iterations per launch follow the form
    if (sig == s->plan_rows) return PDFLOW_OK;
    if (table.size() > s->map_table_cap) {
        if (s->map_table) cudaFree(s->map_table);
        s->map_table = nullptr;
        s->map_table_cap = 0;
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
    s->plan_rows = sig;
    return PDFLOW_OK;
}

// Launches plan[0, end) (the whole plan by default).  all_steps: the set-ups
// write every step-size plane (the autotuner then runs any form on them).
int enqueue_mixed(pdflow_solver* s, cudaStream_t st, const std::vector<LaunchRec>& plan, unsigned* count,
                  size_t end = ~size_t(0), bool all_steps = false)
{
    Params p{s->prm.lambda_i, s->prm.lambda_d, s->prm.mu, s->prm.fovh, s->cols};
    const int fn = s->new_slot, fo = fn ^ 1;
    const State alt{s->alt_d[0], s->alt_d[1], s->alt_d[2], s->alt[0], s->alt[1], s->alt[2], s->alt[3], s->alt[4],
                    s->alt[5], s->alt[6], s->alt[7], s->alt[8], s->alt[9]};
    State cur = s->S, nxt = alt;
    for (size_t q = 0; q < plan.size() && q < end; ++q) {
        const LaunchRec& r = plan[q];
        const LevelGeom g = step_geom(s, r.step, r.count, s->map_table + r.off);
        const int form = step_form(s, r.step, g);
        const unsigned li = kSteps - 1 - r.step;
        const PyrLevel o = s->pyr[fo][li], n = s->pyr[fn][li];
        cudaError_t e = cudaSuccess;
        if (r.kind == 0) {
            e = launch_level_init(g, r.step == 0, s->sol, o, n, s->L, s->S, st);
            if (e == cudaSuccess) e = launch_im_gradients(g, n, s->L, st);
            if (e == cudaSuccess)
                e = launch_warp_steps(g, o, n, s->L, p, st,
                                      all_steps ? kStepsAll : (form >= 7 ? kStepsQuads : kStepsNone));
            *count += 3;
            cur = s->S;
            nxt = alt;
        } else if (r.kind == 1) {
            e = launch_step_tiles(s, g, cur, nxt, p, o, r.kk, st, form);
            std::swap(cur, nxt);
            *count += 1;
        } else {
            e = launch_median(g, false, o, s->L, s->S, s->sol, s->dx, s->dy, s->dz, p, nullptr, st, &alt,
                              !all_steps);
            *count += 1;
        }
        if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "mixed batch launch", e);
    }
    return PDFLOW_OK;
}

}  // namespace

// Per coarse-to-fine step i: replay the plan through step i's set-up (earlier
// steps with the choices made so far), then time every tile form and
// iterations per launch on the pairs active at step i (probe_iters
// iterations, best of three runs after a warm-up) and keep the fastest.
int pdflow::mixed_autotune(pdflow_solver* s, unsigned n, unsigned probe_iters, pdflow_tune_report* report)
{
    if (n == 0 || n > s->batch) return set_error_code(PDFLOW_ERR_ARG, "pair count out of range");
    if (s->frames < 2) return set_error_code(PDFLOW_ERR_STATE, "autotuning needs two frames pushed");
    std::vector<unsigned> rows(s->mixed_rows.begin(), s->mixed_rows.begin() + n);
    for (unsigned r : rows)
        if (!r) return set_error_code(PDFLOW_ERR_STATE, "a pair of the batch has no frames");
    if (probe_iters == 0) probe_iters = 12;
    for (unsigned i = 0; i < 8; ++i) {
        s->mixed_form[i] = -1;
        s->mixed_kk[i] = 0;
    }
    std::vector<LaunchRec> plan;
    int rc = prepare_plan(s, rows, plan);
    if (rc) return rc;
    Params p{s->prm.lambda_i, s->prm.lambda_d, s->prm.mu, s->prm.fovh, s->cols};
    const State alt{s->alt_d[0], s->alt_d[1], s->alt_d[2], s->alt[0], s->alt[1], s->alt[2], s->alt[3], s->alt[4],
                    s->alt[5], s->alt[6], s->alt[7], s->alt[8], s->alt[9]};
    pdflow_tune_report rep{};
    rep.levels = kSteps;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (unsigned i = 0; i < kSteps && rc == PDFLOW_OK; ++i) {
        for (int c = 0; c < PDFLOW_TUNE_CANDIDATES; ++c) rep.level[i].ms_per_iter[c] = NAN;
        rep.level[i].form = -1;
        size_t q = 0;
        while (q < plan.size() && !(plan[q].kind == 0 && plan[q].step == i)) ++q;
        if (q == plan.size()) continue;   // no pair has this level
        unsigned cnt = 0;
        rc = enqueue_mixed(s, s->stream, plan, &cnt, q + 1, true);
        if (rc) break;
        const LevelGeom g = step_geom(s, i, plan[q].count, s->map_table + plan[q].off);
        const PyrLevel o = s->pyr[s->new_slot ^ 1][kSteps - 1 - i];
        float best = INFINITY;
        int best_form = 5;
        unsigned best_kk = 4;
        for (int idx = 0; idx < PDFLOW_TUNE_CANDIDATES; ++idx) {
                const int form = tune_candidate(idx).form;
                const unsigned kk = tune_candidate(idx).kk;
                if (form < 3) continue;                   // mixed steps run tile forms only
                if (form >= 7 && !stream_eligible(g, s->L, s->S, s->S, form)) continue;
                float t = INFINITY;
                for (int r = 0; r < 4 && rc == PDFLOW_OK; ++r) {
                    cudaEventRecord(e0, s->stream);
                    State cur = s->S, nxt = alt;
                    for (unsigned done = 0; done < probe_iters;) {
                        const unsigned k = std::min(kk, probe_iters - done);
                        const cudaError_t e = launch_step_tiles(s, g, cur, nxt, p, o, k, s->stream, form);
                        if (e != cudaSuccess) {
                            rc = set_error_code(PDFLOW_ERR_CUDA, "mixed autotune launch", e);
                            break;
                        }
                        std::swap(cur, nxt);
                        done += k;
                    }
                    cudaEventRecord(e1, s->stream);
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (r > 0 && ms < t) t = ms;
                }
                if (rc) break;
                rep.level[i].ms_per_iter[idx] = t / float(probe_iters);
                if (t < best) {
                    best = t;
                    best_form = form;
                    best_kk = kk;
                }
            }
        s->mixed_form[i] = best_form;
        s->mixed_kk[i] = best_kk;
        rep.level[i].form = best_form;
        rep.level[i].iters_per_launch = best_kk;
        rc = rc ? rc : prepare_plan(s, rows, plan);   // later steps replay with this step's choice
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    rc = check_status(s);
    if (rc) return rc;
    if (report) *report = rep;
    return PDFLOW_OK;
}

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
    const int rc0 = prepare_plan(s, rows, plan);
    if (rc0) return rc0;
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
