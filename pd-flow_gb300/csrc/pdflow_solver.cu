// Host side of the solver: one device arena per handle, the coarse-to-fine
// schedule of PD_flow_opencv::solveSceneFlowGPU (scene_flow_impair.cpp:95-168),
// CUDA-graph replay of the whole solve, and the C ABI of include/pdflow.h.
//
// Unlike the reference, which calls cudaMalloc ~60 times and cudaFree ~55
// times per pyramid level (pdflow_cudalib.cu:74-162, :290-326), every device
// buffer is carved once from a single allocation at create time, so a solve
// issues no allocation, no host synchronisation and (in graph mode) one launch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pdflow.h"
#include "pdflow_internal.h"
#include "pdflow_kernels.cuh"

using namespace pdflow;

namespace {

thread_local std::string g_last_error;

int set_error(int code, const char* what, cudaError_t e = cudaSuccess)
{
    char buf[512];
    if (e != cudaSuccess)
        std::snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    else
        std::snprintf(buf, sizeof buf, "%s", what);
    g_last_error = buf;
    return code;
}

#define CUDA_TRY(call, what)                                  \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return set_error(PDFLOW_ERR_CUDA, what, _e); \
    } while (0)

unsigned log2u(unsigned x)
{
    unsigned l = 0;
    while (x > 1) { x >>= 1; ++l; }
    return l;
}

bool valid_rows(unsigned r)
{
    return r == 15 || r == 30 || r == 60 || r == 120 || r == 240 || r == 480;
}

// Bump allocator over the arena (256-byte aligned planes).
struct Carver {
    char* base;
    size_t off;
    bool dry;
    float* plane(size_t n)
    {
        off = (off + 255) & ~size_t(255);
        float* p = dry ? nullptr : reinterpret_cast<float*>(base + off);
        off += n * sizeof(float);
        return p;
    }
    void* bytes(size_t n)
    {
        off = (off + 255) & ~size_t(255);
        void* p = dry ? nullptr : base + off;
        off += n;
        return p;
    }
};

}  // namespace

namespace pdflow {

void set_last_error(const char* text) { g_last_error = text; }

// Waits for the handle's stream and reports (then clears) a device-side
// timeout recorded by a bounded wait.
int check_status(pdflow_solver* s)
{
    unsigned st = 0;
    CUDA_TRY(cudaMemcpyAsync(&st, s->status, sizeof st, cudaMemcpyDeviceToHost, s->stream), "status read");
    CUDA_TRY(cudaStreamSynchronize(s->stream), "synchronize");
    if (st != 0) {
        CUDA_TRY(cudaMemsetAsync(s->status, 0, 4 * sizeof st, s->stream), "status reset");   // and the strip counters
        CUDA_TRY(cudaStreamSynchronize(s->stream), "synchronize");
        return set_error(PDFLOW_ERR_TIMEOUT, "a bounded device-side wait gave up (iteration neighbour sync)");
    }
    return PDFLOW_OK;
}

// Carves the arena: `batch` identical per-pair slices (pair k's buffers
// k * pair_stride bytes after pair 0's) followed by a shared region (raw-frame
// staging for every pair, progress counters, status word).
void carve_solver(pdflow_solver* s, char* base, size_t* used)
{
    Carver cv{base, 0, base == nullptr};
    const size_t Nimg = size_t(s->width) * s->height;
    for (int f = 0; f < 2; ++f)
        for (unsigned l = 0; l < s->pyr_levels; ++l) {
            const size_t n = Nimg >> (2 * l);
            s->pyr[f][l] = PyrLevel{cv.plane(n), cv.plane(n), cv.plane(n), cv.plane(n)};
        }
    s->stage_I = cv.plane(Nimg);
    s->stage_Z = cv.plane(Nimg);
    const size_t N = size_t(s->rows) * s->cols;
    LevelConsts& L = s->L;
    // The 19 planes the register-resident tiles read come first and back to
    // back (ri .. dv_prev, then the 8 step products), so that one 4D tensor
    // copy moves a region of all of them (pdflow_tmap.h).
    float** lp[] = {&L.ri,  &L.rj,      &L.dct,     &L.dcu,    &L.dcv,     &L.ddt,     &L.ddu,
                    &L.ddv, &L.mu,      &L.du_prev, &L.dv_prev, &L.qs[0],  &L.qs[1],   &L.qs[2],
                    &L.qs[3], &L.qs[4], &L.qs[5],   &L.qs[6],  &L.qs[7],  &L.ri2,     &L.rj2,
                    &L.dcu_aux, &L.dcv_aux, &L.ddu_aux, &L.ddv_aux, &L.spd, &L.spuvx, &L.spuvy,
                    &L.spwx, &L.spwy, &L.tu, &L.tv, &L.tw};
    for (float** p : lp) *p = cv.plane(N);
    State& S = s->S;
    float** sp[] = {&S.du, &S.dv, &S.dw, &S.dua, &S.dva, &S.dwa, &S.pd, &S.puu, &S.puv, &S.pvu, &S.pvv, &S.pwu,
                    &S.pwv};
    for (float** p : sp) *p = cv.plane(N);
    LevelSol& O = s->sol;
    float** op[] = {&O.du, &O.dv, &O.dw, &O.pd, &O.puu, &O.puv, &O.pvu, &O.pvv, &O.pwu, &O.pwv};
    for (float** p : op) *p = cv.plane(N);
    // the second state buffer in the order of S (du dv dw, then the rest)
    for (float*& p : s->alt_d) p = cv.plane(N);
    for (float*& p : s->alt) p = cv.plane(N);
    s->dx = cv.plane(N);
    s->dy = cv.plane(N);
    s->dz = cv.plane(N);
    cv.off = (cv.off + 255) & ~size_t(255);
    s->pair_stride = cv.off;
    cv.off = s->pair_stride * s->batch;
    s->stage_u8 = static_cast<uint8_t*>(cv.bytes(Nimg * s->batch));
    s->stage_u16 = static_cast<uint16_t*>(cv.bytes(Nimg * 2 * s->batch));
    s->flags = static_cast<unsigned*>(cv.bytes(sizeof(unsigned) * 1024));
    s->status = static_cast<unsigned*>(cv.bytes(sizeof(unsigned) * 4));
    s->map = static_cast<unsigned*>(cv.bytes(sizeof(unsigned) * s->batch));
    s->energy = static_cast<float*>(cv.bytes(sizeof(float) * 2 * s->batch));
    s->energy_part = static_cast<double*>(cv.bytes(sizeof(double) * 1024 * s->batch));
    s->seed = (s->ctf_levels > kSeedLevel) || s->rows == 60 ? cv.plane(size_t(3) * kSeedN * s->batch) : nullptr;
    *used = cv.off;
}

int set_error_code(int code, const char* what, cudaError_t e) { return set_error(code, what, e); }

int enqueue_pyramid(pdflow_solver* s, cudaStream_t st, unsigned pairs, const unsigned* map)
{
    const int f = s->new_slot;
    for (unsigned l = 1; l < s->pyr_levels; ++l) {
        const unsigned Cl = 640 / (s->cam_mode << l), Rl = 480 / (s->cam_mode << l);
        CUDA_TRY(launch_pyr_down(s->pyr[f][l - 1], Rl, Cl, s->pyr[f][l], s->prm.fovh, pairs, s->pair_stride, st,
                                 map),
                 "pyramid launch");
    }
    return PDFLOW_OK;
}

size_t level_keep_offset(const pdflow_solver* s, unsigned level)
{
    size_t off = 0;
    for (unsigned k = 0; k < level; ++k) {
        const LevelGeom g = level_geom(s, k, nullptr);
        off += 6 * size_t(g.N);
    }
    return off;
}

unsigned scaled_iters(unsigned iters, float scale)
{
    if (scale >= 1.f) return iters;
    const double v = std::ceil(double(iters) * double(scale));
    return v < 0 ? 0u : unsigned(v);
}

LevelGeom level_geom(const pdflow_solver* s, unsigned i, unsigned* level_image, unsigned pairs)
{
    const unsigned sdiv = 1u << (s->ctf_levels - (i + 1));
    const unsigned Ci = s->cols / sdiv, Ri = s->rows / sdiv;
    if (level_image) *level_image = s->ctf_levels - i + log2u(s->width / s->cols) - 1;
    LevelGeom g{Ri, Ci, Ri * Ci};
    g.pairs = pairs;
    g.pstride = s->pair_stride;
    g.slots = s->batch;
    return g;
}

// The kernel sequence of one solve (scene_flow_impair.cpp:103-167) for pairs
// [0, pairs), for the current old/new slot assignment.  A level's iterations
// run as one launch (k_iterate: one CTA, one cluster, or, for a single pair,
// the cooperative full grid) or, for a batch of pairs at a level that needs
// the full grid, as two batched kernels per iteration.
// Whether level `level`'s iterations run as shared-memory tiles (which
// recompute the step sizes in registers).  Batches: tiles at every level
// (measured faster than the cluster-persistent form from 15x20 up to 120x160
// too); a single pair: tiles above 15x20 (per iteration at 30x40 .. 120x160
// about half the time of the one-launch form; whole VGA solves 2.00 against
// 2.34 ms, QVGA 1.22 against 1.55 ms), the one-CTA launch at 15x20.
static bool level_runs_tiles(const pdflow_solver* s, const LevelGeom& g, unsigned iters, unsigned pairs,
                             unsigned level)
{
    const int forced = level < 8 ? s->level_form[level] : -1;
    if (forced >= 0) return forced >= 2 && iters > 0;
    return s->iter_form >= 2 && iters > 0 && (pairs > 1 || g.N > 300u);
}

// The level's iteration form: its autotuned or hand-set form, else the
// handle's.  By default the strips (form 10) run only where the level has a
// strip (a pair's 24-row band) for every SM; smaller levels run the streamed
// tiles (form 8), which deal fewer pixels to every SM, and levels whose 16x16
// tiles all fit in one round of CTAs the deep tiles (form 9: twice the
// iterations per launch where the launches are latency-bound, as the
// autotuner finds for a single pair's 60x80 and 120x160 levels).  Levels
// whose rows are even but not a multiple of 4 (30x40) cannot run the strips'
// tensor copies and take the same tile rule.
static int level_form(const pdflow_solver* s, const LevelGeom& g, unsigned pairs, unsigned level)
{
    const int forced = level < 8 ? s->level_form[level] : -1;
    if (forced >= 0) return forced;
    if (s->iter_form == 10 && (pairs * ((g.R + 23u) / 24u) < unsigned(s->num_sms) ||
                               !stream_eligible(g, s->L, s->S, s->S, 10)))
        return pairs * ((g.R + 15u) / 16u) * ((g.C + 15u) / 16u) <= unsigned(s->num_sms) ? 9 : 8;
    return s->iter_form;
}

// Whether level `level`'s tiles run register-resident (quad tiles, form 7, or
// streamed tiles and strips, forms 8-10): chosen for the level and possible at its size
// (rows % 4 == 0, or even rows for the streamed tiles; other levels of such a
// solve run the paired 24x24 tiles, form 5).
static bool level_runs_quads(const pdflow_solver* s, const LevelGeom& g, unsigned iters, unsigned pairs,
                             unsigned level)
{
    if (!level_runs_tiles(s, g, iters, pairs, level)) return false;
    const int form = level_form(s, g, pairs, level);
    return (form >= 7 && form <= 10) && stream_eligible(g, s->L, s->S, s->S, form);
}

// The step-size planes the level's set-up writes for its iteration form.
static int level_steps(const pdflow_solver* s, const LevelGeom& g, unsigned iters, unsigned pairs, unsigned level,
                       bool all_steps)
{
    if (all_steps) return kStepsAll;
    if (!level_runs_tiles(s, g, iters, pairs, level)) return kStepsRaw;
    return level_runs_quads(s, g, iters, pairs, level) ? kStepsQuads : kStepsNone;
}

// Enqueues `iters` iterations of level i for pairs [0, pairs) in the
// solve's launch form; returns the number of kernels launched via *count.
// The final duals' buffer is reported in *fin.
static int enqueue_iterations(pdflow_solver* s, cudaStream_t st, const LevelGeom& g, const PyrLevel& o,
                              unsigned iters, unsigned pairs, State* fin, unsigned* count, unsigned level)
{
    Params p{s->prm.lambda_i, s->prm.lambda_d, s->prm.mu, s->prm.fovh, s->cols};
    *fin = s->S;
    const IterPlan pl = plan_iterate(g, s->num_sms);
    const int forced = level < 8 ? s->level_form[level] : -1;
    const bool one_launch_ok = (pairs == 1 || pl.mode != kIterGrid) && pl.smem_bytes <= iterate_smem_limit();
    const bool tiles = level_runs_tiles(s, g, iters, pairs, level);
    const int form = level_form(s, g, pairs, level);
    const bool one_launch = forced >= 0 ? (forced == 1 && iters > 0 && one_launch_ok)
                                        : (s->iter_form >= 1 && iters > 0 && !tiles && one_launch_ok);
    const bool quads = tiles && level_runs_quads(s, g, iters, pairs, level);
    const bool paired = tiles && form >= 3;
    const int shape = form >= 7 ? 2 : form - 3;   // 40x40, 40x34, 24x24 or 24x28 tiles (forms 7-10 elsewhere: 24x24)
    if (tiles) {
        State cur = s->S;
        State nxt{s->alt_d[0], s->alt_d[1], s->alt_d[2], s->alt[0], s->alt[1], s->alt[2], s->alt[3], s->alt[4],
                  s->alt[5], s->alt[6], s->alt[7], s->alt[8], s->alt[9]};
        // iterations per launch: the level's tuned choice, else the halo width
        // (8 for the deep streamed tiles, 4 for every other tile form)
        const unsigned halo = (quads && form == 9) ? 8u : tiles_halo();
        const unsigned h = (level < 8 && s->level_kk[level] > 0 && s->level_kk[level] <= halo)
                               ? s->level_kk[level]
                               : halo;
        for (unsigned done = 0; done < iters;) {
            const unsigned kk = (iters - done < h) ? iters - done : h;
            if (quads && form >= 8)
                CUDA_TRY(launch_iterate_stream(g, s->L, cur, nxt, p, o.dep, kk, done + kk == iters, st, s->status,
                                               unsigned(s->num_sms), stream_layout(form)),
                         "streamed tile iteration launch");
            else if (quads)
                CUDA_TRY(launch_iterate_quads(g, s->L, cur, nxt, p, o.dep, kk, done + kk == iters, st, s->status),
                         "quad tile iteration launch");
            else if (paired)
                CUDA_TRY(launch_iterate_tiles2(g, s->L, cur, nxt, p, o.dep, kk, done + kk == iters, st, shape,
                                               s->status),
                         "tile iteration launch");
            else
                CUDA_TRY(launch_iterate_tiles(g, s->L, cur, nxt, p, o.dep, kk, done + kk == iters, st),
                         "tile iteration launch");
            const State t = cur;
            cur = nxt;
            nxt = t;
            done += kk;
            *count += 1;
        }
        *fin = cur;
    } else if (one_launch) {
        IterArgs a{};
        a.g = g;
        a.L = s->L;
        a.du = s->S.du;
        a.dv = s->S.dv;
        a.dw = s->S.dw;
        float* b0[10] = {s->S.dua, s->S.dva, s->S.dwa, s->S.pd, s->S.puu, s->S.puv, s->S.pvu, s->S.pvv,
                         s->S.pwu, s->S.pwv};
        for (int k = 0; k < 3; ++k) {
            a.acc[0][k] = b0[k];
            a.acc[1][k] = s->alt[k];
        }
        for (int k = 0; k < 7; ++k) {
            a.p_[0][k] = b0[3 + k];
            a.p_[1][k] = s->alt[3 + k];
        }
        a.p = p;
        a.depth_old = o.dep;
        a.iters = iters;
        a.flags = s->flags;
        a.status = s->status;
        CUDA_TRY(launch_iterate(pl, a, st), "iteration launch");
        *count += 1;
        if (iters & 1) {   // the final duals are in the second buffer
            float** fp[7] = {&fin->pd, &fin->puu, &fin->puv, &fin->pvu, &fin->pvv, &fin->pwu, &fin->pwv};
            for (int k = 0; k < 7; ++k) *fp[k] = s->alt[3 + k];
        }
    } else {
        for (unsigned it = 0; it < iters; ++it) {
            CUDA_TRY(launch_dual(g, s->L, s->S, p, st), "dual launch");
            CUDA_TRY(launch_primal(g, s->L, s->S, p, it + 1 == iters, o.dep, st), "primal launch");
        }
        *count += 2 * iters;
    }
    return PDFLOW_OK;
}

int enqueue_level_iterations(pdflow_solver* s, cudaStream_t st, unsigned pairs, unsigned level, unsigned iters)
{
    unsigned li, cnt = 0;
    const LevelGeom g = level_geom(s, level, &li, pairs);
    State fin;
    return enqueue_iterations(s, st, g, s->pyr[s->new_slot ^ 1][li], iters, pairs, &fin, &cnt, level);
}

// Energy of level `level`'s median output (the solution passed to the next
// level): warp both frames at the solution's flow, then sum the data and TV
// terms per pair into out[0..pairs).
int enqueue_energy(pdflow_solver* s, cudaStream_t st, unsigned pairs, unsigned level, float* out,
                   const unsigned* map)
{
    Params p{s->prm.lambda_i, s->prm.lambda_d, s->prm.mu, s->prm.fovh, s->cols};
    unsigned li;
    LevelGeom g = level_geom(s, level, &li, pairs);
    g.map = map;
    const PyrLevel o = s->pyr[s->new_slot ^ 1][li], n = s->pyr[s->new_slot][li];
    CUDA_TRY(launch_energy_prep(g, s->sol, s->L, st), "energy prep launch");
    CUDA_TRY(launch_im_gradients(g, n, s->L, st), "image gradients launch");
    CUDA_TRY(launch_warp_steps(g, o, n, s->L, p, st, false), "warping launch");   // the energy needs mu only
    CUDA_TRY(launch_energy(g, s->sol, s->L, p, out, s->energy_part, st), "energy launch");
    s->launches += 5;
    return PDFLOW_OK;
}

// Levels [plan.first, plan.last] of the coarse-to-fine schedule for pairs
// [0, pairs) (or the mapped slots).  The plain solve is the default plan.
int enqueue_solve(pdflow_solver* s, cudaStream_t st, unsigned pairs, const SolvePlan& plan)
{
    Params p{s->prm.lambda_i, s->prm.lambda_d, s->prm.mu, s->prm.fovh, s->cols};
    const int fn = s->new_slot, fo = fn ^ 1;
    unsigned count = 0;
    const unsigned last = plan.last < s->ctf_levels ? plan.last : s->ctf_levels - 1;
    for (unsigned i = plan.first; i <= last; ++i) {
        unsigned li;
        LevelGeom g = level_geom(s, i, &li, pairs);
        g.map = plan.map;
        const PyrLevel o = s->pyr[fo][li], n = s->pyr[fn][li];
        const float* seed = (i == plan.first) ? plan.seed : nullptr;
        static const char* const kLevelNames[8] = {"level 0", "level 1", "level 2", "level 3",
                                                   "level 4", "level 5", "level 6", "level 7"};
        const NvtxRange level_range(kLevelNames[i < 8 ? i : 7]);
        cudaEvent_t* tr = plan.trace ? plan.trace + 3 * (i - plan.first) : nullptr;
        if (tr) CUDA_TRY(cudaEventRecord(tr[0], st), "trace event");
        CUDA_TRY(launch_level_init(g, i == 0, s->sol, o, n, s->L, s->S, st, seed), "level init launch");
        const unsigned iters = scaled_iters(s->prm.num_max_iter[i], plan.iter_scale);
        const int steps = level_steps(s, g, iters, pairs, i, plan.all_steps);
        CUDA_TRY(launch_im_gradients(g, n, s->L, st), "image gradients launch");
        CUDA_TRY(launch_warp_steps(g, o, n, s->L, p, st, steps), "warping launch");
        count += 3;
        if (tr) CUDA_TRY(cudaEventRecord(tr[1], st), "trace event");
        State fin;
        int rc = enqueue_iterations(s, st, g, o, iters, pairs, &fin, &count, i);
        if (rc) return rc;
        if (iters == 0) {
            CUDA_TRY(launch_saturate(g, s->L, s->S, o.dep, st), "saturate launch");
            ++count;
        }
        if (tr) CUDA_TRY(cudaEventRecord(tr[2], st), "trace event");
        CUDA_TRY(launch_median(g, i + 1 == s->ctf_levels, o, s->L, fin, s->sol, s->dx, s->dy, s->dz, p, nullptr, st,
                               nullptr, steps_hold_ddt_sq(steps)),
                 "median launch");
        ++count;
        if (s->keep_levels && s->lvl_keep) {
            CUDA_TRY(launch_level_keep(g, s->sol, o, p, s->lvl_keep, s->lvl_keep_stride, level_keep_offset(s, i), st),
                     "level record launch");
            ++count;
        }
        if (int(i) == plan.energy_level && plan.energy) {
            s->launches = 0;
            rc = enqueue_energy(s, st, pairs, i, plan.energy, plan.map);
            if (rc) return rc;
            count += s->launches;
        }
    }
    if (plan.trace) CUDA_TRY(cudaEventRecord(plan.trace[3 * (last + 1 - plan.first)], st), "trace event");
    s->launches = count;
    return PDFLOW_OK;
}

int run_graphed(pdflow_solver* s, unsigned pairs, unsigned kind, EnqueueFn fn, const void* ctx,
                unsigned long long key)
{
    if (!s->use_graph) return fn(s, s->stream, pairs, ctx);
    cudaGraphExec_t ge = nullptr;
    for (auto& g : s->graphs)
        if (g.slot == s->new_slot && g.pairs == pairs && g.form == s->iter_form && g.kind == kind && g.key == key) {
            ge = g.exec;
            s->launches = g.launches;
        }
    if (!ge) {
        cudaStream_t cap;
        CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "capture stream");
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        int rc = PDFLOW_OK;
        if (e == cudaSuccess) {
            rc = fn(s, cap, pairs, ctx);
            cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
            if (e == cudaSuccess) e = e2;
        }
        if (e == cudaSuccess && rc == PDFLOW_OK) e = cudaGraphInstantiate(&ge, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cap);
        if (rc != PDFLOW_OK) return rc;
        if (e != cudaSuccess) return set_error(PDFLOW_ERR_CUDA, "solve graph capture", e);
        s->graphs.push_back(pdflow_solver::GraphEntry{s->new_slot, pairs, s->iter_form, kind, key, ge, s->launches});
    }
    CUDA_TRY(cudaGraphLaunch(ge, s->stream), "solve graph launch");
    return PDFLOW_OK;
}

}  // namespace pdflow

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
namespace {

int push_common(pdflow_solver* s, unsigned pairs)
{
    int rc = enqueue_pyramid(s, s->stream, pairs);
    if (rc) return rc;
    if (s->frames < 2) ++s->frames;
    return PDFLOW_OK;
}

bool bad_count(const pdflow_solver* s, unsigned n) { return n == 0 || n > s->batch; }

constexpr unsigned kKindPlain = 0, kKindSlots = 1;

int plain_solve(pdflow_solver* s, cudaStream_t st, unsigned pairs, const void*)
{
    return enqueue_solve(s, st, pairs);
}

int slots_solve(pdflow_solver* s, cudaStream_t st, unsigned pairs, const void*)
{
    SolvePlan plan;
    plan.map = s->map;
    return enqueue_solve(s, st, pairs, plan);
}

// Checks a slot list (in range, no repeats) and uploads it to the device map.
int upload_slots(pdflow_solver* s, unsigned n, const unsigned* slots)
{
    if (!slots) return set_error(PDFLOW_ERR_ARG, "null slot list");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    std::vector<unsigned char> seen(s->batch, 0);
    for (unsigned k = 0; k < n; ++k) {
        if (slots[k] >= s->batch) return set_error(PDFLOW_ERR_ARG, "slot out of range");
        if (seen[slots[k]]++) return set_error(PDFLOW_ERR_ARG, "slot listed twice");
    }
    CUDA_TRY(cudaMemcpyAsync(s->map, slots, sizeof(unsigned) * n, cudaMemcpyHostToDevice, s->stream), "H2D slots");
    return PDFLOW_OK;
}

}  // namespace

extern "C" {

int pdflow_default_params(unsigned rows, pdflow_params* p)
{
    if (!p) return set_error(PDFLOW_ERR_ARG, "null params");
    if (!valid_rows(rows)) return set_error(PDFLOW_ERR_ARG, "rows must be one of 15,30,60,120,240,480");
    const unsigned ctf = log2u(rows / 15) + 1;
    for (int i = 5; i >= 0; --i)
        p->num_max_iter[i] = (i >= int(ctf) - 1) ? 100u : p->num_max_iter[i + 1] - 15u;
    p->lambda_i = 0.04f;
    p->lambda_d = 0.35f;
    p->mu = 75.f;
    p->fovh = float(M_PI * 62.5 / 180.0);
    p->fovv = float(M_PI * 48.5 / 180.0);
    return PDFLOW_OK;
}

int pdflow_create_batch(unsigned rows, unsigned width, unsigned height, const pdflow_params* params,
                        unsigned max_pairs, pdflow_solver** out)
{
    if (!out) return set_error(PDFLOW_ERR_ARG, "null output handle");
    *out = nullptr;
    if (!valid_rows(rows)) return set_error(PDFLOW_ERR_ARG, "rows must be one of 15,30,60,120,240,480");
    if (!((width == 640 && height == 480) || (width == 320 && height == 240)))
        return set_error(PDFLOW_ERR_ARG, "image must be 640x480 or 320x240");
    const unsigned cols = rows * 320 / 240;
    if (cols > width) return set_error(PDFLOW_ERR_ARG, "rows exceed the image resolution");
    if (max_pairs == 0 || max_pairs > 65535) return set_error(PDFLOW_ERR_ARG, "batch size must be 1..65535");
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    if (!(prop.major == 10 && prop.minor == 3))
        return set_error(PDFLOW_ERR_NO_DEVICE, "this library is built for sm_103a (GB300) only");
    {
        // kernel attributes are per device: set them once per device, under a lock
        static std::mutex mu;
        static unsigned long long prepared = 0;
        std::lock_guard<std::mutex> lk(mu);
        if (dev >= 64 || !((prepared >> dev) & 1ull)) {
            CUDA_TRY(prepare_iterate(), "kernel attributes");
            CUDA_TRY(prepare_tiles(), "kernel attributes");
            CUDA_TRY(prepare_tiles2(), "kernel attributes");
            CUDA_TRY(prepare_quads(), "kernel attributes");
            CUDA_TRY(prepare_stream_tiles(), "kernel attributes");
            if (dev < 64) prepared |= 1ull << dev;
        }
    }

    pdflow_solver* s = new (std::nothrow) pdflow_solver();
    if (!s) return set_error(PDFLOW_ERR_OOM, "host allocation");
    s->device = dev;
    s->num_sms = prop.multiProcessorCount;
    s->rows = rows;
    s->cols = cols;
    s->width = width;
    s->height = height;
    s->batch = max_pairs;
    s->cam_mode = (height == 240) ? 2u : 1u;
    s->ctf_levels = log2u(rows / 15) + 1;
    s->pyr_levels = log2u(width / cols) + s->ctf_levels;
    if (params) s->prm = *params;
    else pdflow_default_params(rows, &s->prm);
    s->use_graph = 1;
    size_t bytes = 0;
    carve_solver(s, nullptr, &bytes);
    cudaError_t e = cudaMalloc(&s->arena, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return set_error(PDFLOW_ERR_OOM, "arena allocation", e);
    }
    s->arena_bytes = bytes;
    carve_solver(s, static_cast<char*>(s->arena), &bytes);
    e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->arena, 0, s->arena_bytes, s->own_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->own_stream);
    if (e != cudaSuccess) {
        cudaFree(s->arena);
        if (s->own_stream) cudaStreamDestroy(s->own_stream);
        delete s;
        return set_error(PDFLOW_ERR_CUDA, "stream / arena init", e);
    }
    s->stream = s->own_stream;
    *out = s;
    return PDFLOW_OK;
}

int pdflow_create(unsigned rows, unsigned width, unsigned height, const pdflow_params* params, pdflow_solver** out)
{
    return pdflow_create_batch(rows, width, height, params, 1, out);
}

int pdflow_destroy(pdflow_solver* s)
{
    if (!s) return PDFLOW_OK;
    cudaStreamSynchronize(s->stream);
    for (auto& g : s->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (s->mixed_graph) cudaGraphExecDestroy(s->mixed_graph);
    if (s->map_table) cudaFree(s->map_table);
    if (s->stage_rgb) cudaFree(s->stage_rgb);
    if (s->sol_keep) cudaFree(s->sol_keep);
    if (s->lvl_keep) cudaFree(s->lvl_keep);
    cudaFree(s->arena);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    delete s;
    return PDFLOW_OK;
}

size_t pdflow_device_bytes(const pdflow_solver* s)
{
    if (!s) return 0;
    size_t b = s->arena_bytes;   // plus the buffers allocated on first use
    if (s->sol_keep) b += learned_keep_bytes(s->batch);
    if (s->stage_rgb) b += size_t(s->width) * s->height * 3 * s->batch;
    if (s->lvl_keep) b += sizeof(float) * s->lvl_keep_stride * s->batch;
    return b;
}

int pdflow_push_frames(pdflow_solver* s, unsigned n, const float* I, const float* Z)
{
    const NvtxRange trace_range("pdflow_push_frames");
    if (!s || !I || !Z) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (s->mixed) return set_error(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (s->slot_mode) return set_error(PDFLOW_ERR_STATE, "frames were pushed per slot: use the slot calls");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    const size_t b = size_t(s->width) * s->height * 4;
    s->new_slot ^= 1;  // copyNewFrames pointer swap (pdflow_cudalib.cu:203-221)
    CUDA_TRY(cudaMemcpy2DAsync(s->stage_I, s->pair_stride, I, b, b, n, cudaMemcpyHostToDevice, s->stream),
             "H2D intensity");
    CUDA_TRY(cudaMemcpy2DAsync(s->stage_Z, s->pair_stride, Z, b, b, n, cudaMemcpyHostToDevice, s->stream),
             "H2D depth");
    CUDA_TRY(launch_pyr_level0(s->stage_I, s->stage_Z, s->height, s->width, s->pyr[s->new_slot][0], s->prm.fovh, n,
                               s->pair_stride, s->stream),
             "level-0 launch");
    return push_common(s, n);
}

int pdflow_push_frame(pdflow_solver* s, const float* I, const float* Z) { return pdflow_push_frames(s, 1, I, Z); }

int pdflow_push_frames_u16_device(pdflow_solver* s, unsigned n, const uint8_t* d_intensity, const uint16_t* d_depth)
{
    const NvtxRange trace_range("pdflow_push_frames_u16_device");
    if (!s || !d_intensity || !d_depth) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (s->mixed) return set_error(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (s->slot_mode) return set_error(PDFLOW_ERR_STATE, "frames were pushed per slot: use the slot calls");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    s->new_slot ^= 1;
    CUDA_TRY(launch_decode_u16(d_intensity, d_depth, s->width, s->height, s->pyr[s->new_slot][0], s->prm.fovh, n,
                               s->pair_stride, s->stream),
             "decode launch");
    return push_common(s, n);
}

int pdflow_push_frame_u16_device(pdflow_solver* s, const uint8_t* d_intensity, const uint16_t* d_depth)
{
    return pdflow_push_frames_u16_device(s, 1, d_intensity, d_depth);
}

int pdflow_push_frames_u16(pdflow_solver* s, unsigned n, const uint8_t* intensity, const uint16_t* depth)
{
    if (!s || !intensity || !depth) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    const size_t px = size_t(s->width) * s->height * n;
    CUDA_TRY(cudaMemcpyAsync(s->stage_u8, intensity, px, cudaMemcpyHostToDevice, s->stream), "H2D intensity");
    CUDA_TRY(cudaMemcpyAsync(s->stage_u16, depth, px * 2, cudaMemcpyHostToDevice, s->stream), "H2D depth");
    return pdflow_push_frames_u16_device(s, n, s->stage_u8, s->stage_u16);
}

int pdflow_push_frame_u16(pdflow_solver* s, const uint8_t* intensity, const uint16_t* depth)
{
    return pdflow_push_frames_u16(s, 1, intensity, depth);
}

int pdflow_push_frames_rgb8_mm_device(pdflow_solver* s, unsigned n, const uint8_t* d_rgb, const uint16_t* d_depth_mm,
                                      int rotate180)
{
    if (!s || !d_rgb || !d_depth_mm) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (s->mixed) return set_error(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (s->slot_mode) return set_error(PDFLOW_ERR_STATE, "frames were pushed per slot: use the slot calls");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    s->new_slot ^= 1;
    CUDA_TRY(launch_decode_rgb8_mm(d_rgb, d_depth_mm, s->width, s->height, s->pyr[s->new_slot][0], s->prm.fovh, n,
                                   s->pair_stride, s->stream, rotate180 ? 1 : 0),
             "RGB decode launch");
    return push_common(s, n);
}

int pdflow_push_frames_rgb8_mm(pdflow_solver* s, unsigned n, const uint8_t* rgb, const uint16_t* depth_mm,
                               int rotate180)
{
    if (!s || !rgb || !depth_mm) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    const size_t px = size_t(s->width) * s->height * n;
    if (!s->stage_rgb) {
        void* p = nullptr;
        if (cudaMalloc(&p, size_t(s->width) * s->height * 3 * s->batch) != cudaSuccess) {
            cudaGetLastError();
            return set_error(PDFLOW_ERR_OOM, "RGB staging buffer");
        }
        s->stage_rgb = static_cast<uint8_t*>(p);
    }
    CUDA_TRY(cudaMemcpyAsync(s->stage_rgb, rgb, px * 3, cudaMemcpyHostToDevice, s->stream), "H2D RGB");
    CUDA_TRY(cudaMemcpyAsync(s->stage_u16, depth_mm, px * 2, cudaMemcpyHostToDevice, s->stream), "H2D depth");
    return pdflow_push_frames_rgb8_mm_device(s, n, s->stage_rgb, s->stage_u16, rotate180);
}

int pdflow_push_frame_rgb8_mm(pdflow_solver* s, const uint8_t* rgb, const uint16_t* depth_mm, int rotate180)
{
    return pdflow_push_frames_rgb8_mm(s, 1, rgb, depth_mm, rotate180);
}

int pdflow_solve_batch(pdflow_solver* s, unsigned n)
{
    const NvtxRange trace_range("pdflow_solve_batch");
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    if (s->mixed) return set_error(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    if (s->slot_mode) return set_error(PDFLOW_ERR_STATE, "frames were pushed per slot: use pdflow_solve_slots");
    if (s->frames < 2) return set_error(PDFLOW_ERR_STATE, "solve needs two pushed frames");
    return run_graphed(s, n, kKindPlain, plain_solve, nullptr);
}

int pdflow_solve(pdflow_solver* s) { return pdflow_solve_batch(s, 1); }

int pdflow_read_flow_batch(pdflow_solver* s, unsigned n, float* dx, float* dy, float* dz)
{
    const NvtxRange trace_range("pdflow_read_flow_batch");
    if (!s || !dx || !dy || !dz) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (s->mixed) return set_error(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    const size_t b = size_t(s->rows) * s->cols * 4;
    CUDA_TRY(cudaMemcpy2DAsync(dx, b, s->dx, s->pair_stride, b, n, cudaMemcpyDeviceToHost, s->stream), "D2H dx");
    CUDA_TRY(cudaMemcpy2DAsync(dy, b, s->dy, s->pair_stride, b, n, cudaMemcpyDeviceToHost, s->stream), "D2H dy");
    CUDA_TRY(cudaMemcpy2DAsync(dz, b, s->dz, s->pair_stride, b, n, cudaMemcpyDeviceToHost, s->stream), "D2H dz");
    return check_status(s);
}

int pdflow_read_flow(pdflow_solver* s, float* dx, float* dy, float* dz)
{
    return pdflow_read_flow_batch(s, 1, dx, dy, dz);
}

int pdflow_flow_device(pdflow_solver* s, const float** dx, const float** dy, const float** dz)
{
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    if (dx) *dx = s->dx;
    if (dy) *dy = s->dy;
    if (dz) *dz = s->dz;
    return PDFLOW_OK;
}

int pdflow_copy_flow_device(pdflow_solver* s, unsigned n, float* d_dx, float* d_dy, float* d_dz)
{
    if (!s || !d_dx || !d_dy || !d_dz) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (s->mixed) return set_error(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    const size_t b = size_t(s->rows) * s->cols * 4;
    CUDA_TRY(cudaMemcpy2DAsync(d_dx, b, s->dx, s->pair_stride, b, n, cudaMemcpyDeviceToDevice, s->stream), "D2D dx");
    CUDA_TRY(cudaMemcpy2DAsync(d_dy, b, s->dy, s->pair_stride, b, n, cudaMemcpyDeviceToDevice, s->stream), "D2D dy");
    CUDA_TRY(cudaMemcpy2DAsync(d_dz, b, s->dz, s->pair_stride, b, n, cudaMemcpyDeviceToDevice, s->stream), "D2D dz");
    return PDFLOW_OK;
}

int pdflow_batch_info(const pdflow_solver* s, unsigned* max_pairs, size_t* pair_stride_bytes)
{
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    if (max_pairs) *max_pairs = s->batch;
    if (pair_stride_bytes) *pair_stride_bytes = s->pair_stride;
    return PDFLOW_OK;
}

int pdflow_synchronize(pdflow_solver* s)
{
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    return check_status(s);
}

int pdflow_set_stream(pdflow_solver* s, void* stream)
{
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    s->stream = stream ? static_cast<cudaStream_t>(stream) : s->own_stream;
    return PDFLOW_OK;
}

int pdflow_get_config(const pdflow_solver* s, unsigned* rows, unsigned* cols, unsigned* ctf_levels,
                      unsigned* pyr_levels, unsigned* cam_mode)
{
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    if (rows) *rows = s->rows;
    if (cols) *cols = s->cols;
    if (ctf_levels) *ctf_levels = s->ctf_levels;
    if (pyr_levels) *pyr_levels = s->pyr_levels;
    if (cam_mode) *cam_mode = s->cam_mode;
    return PDFLOW_OK;
}

int pdflow_set_graph_mode(pdflow_solver* s, int use_graph)
{
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    s->use_graph = use_graph ? 1 : 0;
    return PDFLOW_OK;
}

int pdflow_push_frames_slots_u16_device(pdflow_solver* s, unsigned n, const unsigned* slots,
                                        const uint8_t* d_intensity, const uint16_t* d_depth)
{
    if (!s || !d_intensity || !d_depth) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (s->mixed) return set_error(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (!s->slot_mode && s->frames > 0)
        return set_error(PDFLOW_ERR_STATE, "frames were pushed for the whole batch: use the batch calls");
    int rc = upload_slots(s, n, slots);
    if (rc) return rc;
    if (s->slot_frames.size() != s->batch) s->slot_frames.assign(s->batch, 0);
    s->slot_mode = 1;
    // frame t-1 := frame t for these slots, then frame t := the new frame
    const int fn = s->new_slot, fo = fn ^ 1;
    const size_t Nimg = size_t(s->width) * s->height;
    for (unsigned l = 0; l < s->pyr_levels; ++l)
        CUDA_TRY(launch_pyr_copy(s->pyr[fn][l], s->pyr[fo][l], unsigned(Nimg >> (2 * l)), n, s->pair_stride, s->map,
                                 s->stream),
                 "pyramid copy launch");
    CUDA_TRY(launch_decode_u16(d_intensity, d_depth, s->width, s->height, s->pyr[fn][0], s->prm.fovh, n,
                               s->pair_stride, s->stream, s->map),
             "decode launch");
    rc = enqueue_pyramid(s, s->stream, n, s->map);
    if (rc) return rc;
    for (unsigned k = 0; k < n; ++k)
        if (s->slot_frames[slots[k]] < 2) ++s->slot_frames[slots[k]];
    return PDFLOW_OK;
}

int pdflow_push_frames_slots_u16(pdflow_solver* s, unsigned n, const unsigned* slots, const uint8_t* intensity,
                                 const uint16_t* depth)
{
    if (!s || !intensity || !depth) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    const size_t px = size_t(s->width) * s->height * n;
    CUDA_TRY(cudaMemcpyAsync(s->stage_u8, intensity, px, cudaMemcpyHostToDevice, s->stream), "H2D intensity");
    CUDA_TRY(cudaMemcpyAsync(s->stage_u16, depth, px * 2, cudaMemcpyHostToDevice, s->stream), "H2D depth");
    return pdflow_push_frames_slots_u16_device(s, n, slots, s->stage_u8, s->stage_u16);
}

int pdflow_solve_slots(pdflow_solver* s, unsigned n, const unsigned* slots)
{
    const NvtxRange trace_range("pdflow_solve_slots");
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    if (s->mixed) return set_error(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (!s->slot_mode) return set_error(PDFLOW_ERR_STATE, "no frames were pushed per slot");
    int rc = upload_slots(s, n, slots);
    if (rc) return rc;
    for (unsigned k = 0; k < n; ++k)
        if (s->slot_frames[slots[k]] < 2) return set_error(PDFLOW_ERR_STATE, "a slot has fewer than two frames");
    return run_graphed(s, n, kKindSlots, slots_solve, nullptr);
}

int pdflow_read_flow_slots(pdflow_solver* s, unsigned n, const unsigned* slots, float* dx, float* dy, float* dz)
{
    if (!s || !slots || !dx || !dy || !dz) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    const size_t N = size_t(s->rows) * s->cols;
    for (unsigned k = 0; k < n; ++k) {
        if (slots[k] >= s->batch) return set_error(PDFLOW_ERR_ARG, "slot out of range");
        const size_t po = slots[k] * s->pair_stride;
        CUDA_TRY(cudaMemcpyAsync(dx + k * N, at(s->dx, po), N * 4, cudaMemcpyDeviceToHost, s->stream), "D2H dx");
        CUDA_TRY(cudaMemcpyAsync(dy + k * N, at(s->dy, po), N * 4, cudaMemcpyDeviceToHost, s->stream), "D2H dy");
        CUDA_TRY(cudaMemcpyAsync(dz + k * N, at(s->dz, po), N * 4, cudaMemcpyDeviceToHost, s->stream), "D2H dz");
    }
    return check_status(s);
}

int pdflow_energy_batch(pdflow_solver* s, unsigned n, float* energies)
{
    if (!s || !energies) return set_error(PDFLOW_ERR_ARG, "null argument");
    if (bad_count(s, n)) return set_error(PDFLOW_ERR_ARG, "pair count out of range");
    s->launches = 0;
    int rc = enqueue_energy(s, s->stream, n, s->ctf_levels - 1, s->energy, nullptr);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(energies, s->energy, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream),
             "D2H energies");
    return check_status(s);
}

int pdflow_image_flow_device(pdflow_solver* s, const float** du, const float** dv, const float** dw)
{
    if (!s) return set_error(PDFLOW_ERR_ARG, "null handle");
    if (du) *du = s->sol.du;
    if (dv) *dv = s->sol.dv;
    if (dw) *dw = s->sol.dw;
    return PDFLOW_OK;
}

const char* pdflow_last_error(void) { return g_last_error.c_str(); }

const char* pdflow_version(void) { return "pdflow-gb300 0.1 (sm_103a)"; }

}  // extern "C"
