// Autotuner of the per-level iteration launch form (include/pdflow.h):
// times each candidate form of every level on the handle's own batch and
// keeps the fastest.  All forms compute the same bits, so the choice only
// changes speed.
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/pdflow.h"
#include "pdflow_internal.h"

using namespace pdflow;

namespace {

constexpr TuneCandidate kCandidates[PDFLOW_TUNE_CANDIDATES] = {{0, 0}, {1, 0}, {2, 2}, {2, 3}, {2, 4}, {3, 2}, {3, 3},
                                                            {3, 4}, {4, 2}, {4, 3}, {4, 4}, {5, 2}, {5, 3}, {5, 4},
                                                            {6, 2}, {6, 3}, {6, 4}, {7, 2}, {7, 3}, {7, 4},
                                                            {8, 2}, {8, 3}, {8, 4}, {9, 4}, {9, 6}, {9, 8},
                                                               {10, 2}, {10, 3}, {10, 4}};

}  // namespace

TuneCandidate pdflow::tune_candidate(int c) { return kCandidates[c]; }

namespace {

void drop_graphs(pdflow_solver* s)
{
    cudaStreamSynchronize(s->stream);
    for (auto& g : s->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    s->graphs.clear();
}

}  // namespace

extern "C" {

int pdflow_set_level_form(pdflow_solver* s, unsigned level, int form, unsigned iters_per_launch)
{
    if (!s || level >= 8 || form < -1 || form > 10 || iters_per_launch > (form == 9 ? 8u : 4u)) {
        set_last_error("bad argument (form -1..10, level < 8, iterations per launch 0..4, 0..8 for form 9)");
        return PDFLOW_ERR_ARG;
    }
    drop_graphs(s);
    s->level_form[level] = form;
    s->level_kk[level] = iters_per_launch;
    return PDFLOW_OK;
}

int pdflow_autotune(pdflow_solver* s, unsigned n, unsigned probe_iters, pdflow_tune_report* report)
{
    if (!s || n == 0 || n > s->batch) {
        set_last_error("bad argument");
        return PDFLOW_ERR_ARG;
    }
    if (s->mixed) return mixed_autotune(s, n, probe_iters, report);
    if (s->frames < 2 || s->slot_mode) {
        set_last_error("autotuning needs two frames pushed for the whole batch");
        return PDFLOW_ERR_STATE;
    }
    if (probe_iters == 0) probe_iters = 12;   // a multiple of 2, 3 and 4 iterations per launch
    drop_graphs(s);
    const int saved_graph = s->use_graph;
    s->use_graph = 0;
    for (int i = 0; i < 8; ++i) {
        s->level_form[i] = -1;
        s->level_kk[i] = 0;
    }
    pdflow_tune_report rep{};
    rep.levels = s->ctf_levels;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = PDFLOW_OK;
    for (unsigned i = 0; i < s->ctf_levels && rc == PDFLOW_OK; ++i) {
        SolvePlan plan;
        plan.last = i;
        plan.all_steps = true;   // every candidate form finds its step sizes
        rc = enqueue_solve(s, s->stream, n, plan);   // level i's constants in place
        if (rc) break;
        unsigned li;
        const LevelGeom g = level_geom(s, i, &li, n);
        const IterPlan pl = plan_iterate(g, s->num_sms);
        const bool one_ok = (n == 1 || pl.mode != kIterGrid) && pl.smem_bytes <= iterate_smem_limit();
        float best = INFINITY;
        int best_c = 0;
        for (int c = 0; c < PDFLOW_TUNE_CANDIDATES; ++c) {
            rep.level[i].ms_per_iter[c] = NAN;
            if (kCandidates[c].form == 1 && !one_ok) continue;
            if (kCandidates[c].form >= 7 && !stream_eligible(g, s->L, s->S, s->S, kCandidates[c].form)) continue;
            s->level_form[i] = kCandidates[c].form;
            s->level_kk[i] = kCandidates[c].kk;
            float t = INFINITY;
            for (int r = 0; r < 4 && rc == PDFLOW_OK; ++r) {   // first run warms up
                cudaEventRecord(e0, s->stream);
                rc = enqueue_level_iterations(s, s->stream, n, i, probe_iters);
                cudaEventRecord(e1, s->stream);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (r > 0 && ms < t) t = ms;
            }
            if (rc) break;
            rep.level[i].ms_per_iter[c] = t / float(probe_iters);
            if (t < best) {
                best = t;
                best_c = c;
            }
        }
        s->level_form[i] = kCandidates[best_c].form;
        s->level_kk[i] = kCandidates[best_c].kk;
        rep.level[i].form = kCandidates[best_c].form;
        rep.level[i].iters_per_launch = kCandidates[best_c].kk;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->use_graph = saved_graph;
    if (rc) return rc;
    rc = check_status(s);
    if (rc) return rc;
    if (report) *report = rep;
    return PDFLOW_OK;
}

}  // extern "C"
