// Learned warm start of a batched solve (include/pdflow_net.h).
//
// A first CUDA graph per (pair count, iteration scale, slot addressing) runs
// the plain schedule to the 60x80 level with its energy, keeps that level's
// plain solution, runs the network on the level's images and the 60x80 level
// again from the network's prediction with its own energy.  The host compares
// the two energies per pair; a second graph continues the accepted pairs with
// the warm-started schedule from 120x160 on, a third puts the kept plain
// 60x80 solution back for the rejected pairs and continues them with the plain
// schedule, which makes them the plain solve bit for bit.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/pdflow_net.h"
#include "pdflow_internal.h"
#include "pdflow_net.cuh"

using namespace pdflow;

namespace {

// Block means of the finest-level solution (du, dv in finest pixels, dw) over
// s x s blocks, in 60x80-level units: [pair][3][4800].
__global__ void k_seed_labels(LevelSol sol, unsigned R, unsigned s, size_t pstride, int n, float* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * int(kSeedN)) return;
    const int b = i / int(kSeedN), q = i % int(kSeedN);
    const unsigned vq = unsigned(q) % 60u, uq = unsigned(q) / 60u;
    const size_t po = size_t(b) * pstride;
    const float* du = at(sol.du, po);
    const float* dv = at(sol.dv, po);
    const float* dw = at(sol.dw, po);
    double a = 0.0, c = 0.0, w = 0.0;
    for (unsigned du_ = 0; du_ < s; ++du_)
        for (unsigned dv_ = 0; dv_ < s; ++dv_) {
            const size_t j = size_t(vq * s + dv_) + size_t(uq * s + du_) * R;
            a += du[j];
            c += dv[j];
            w += dw[j];
        }
    const double inv = 1.0 / double(s * s);
    float* o = out + size_t(b) * 3 * kSeedN;
    o[q] = float(a * inv / s);
    o[kSeedN + q] = float(c * inv / s);
    o[2 * kSeedN + q] = float(w * inv);
}

// Saves (save = true) or restores the 10 solution planes (du, dv, dw and the
// 7 duals) of the 60x80 level of the mapped pairs to / from keep[slot][10][n].
__global__ void k_sol_keep(LevelSol sol, float* __restrict__ keep, unsigned n, size_t pstride,
                           const unsigned* __restrict__ map, bool save)
{
    const unsigned slot = map ? (__ldg(map + blockIdx.y) & kMapSlotMask) : blockIdx.y;
    sol = at(sol, pair_off(map, pstride, blockIdx.y));
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* k = keep + size_t(slot) * 10 * n;
    float* p[10] = {sol.du, sol.dv, sol.dw, sol.pd, sol.puu, sol.puv, sol.pvu, sol.pvv, sol.pwu, sol.pwv};
#pragma unroll
    for (int c = 0; c < 10; ++c) {
        if (save) k[size_t(c) * n + i] = p[c][i];
        else p[c][i] = k[size_t(c) * n + i];
    }
}

cudaError_t launch_sol_keep(pdflow_solver* s, unsigned pairs, const unsigned* map, bool save, cudaStream_t st)
{
    dim3 grid((kSeedN + 255) / 256, pairs);
    k_sol_keep<<<grid, 256, 0, st>>>(s->sol, s->sol_keep, kSeedN, s->pair_stride, map, save);
    return cudaGetLastError();
}

struct LearnedCtx {
    pdflow_net* net;
    float iter_scale;
    bool mapped;
};

int learned_enqueue(pdflow_solver* s, cudaStream_t st, unsigned pairs, const void* vctx)
{
    const LearnedCtx& c = *static_cast<const LearnedCtx*>(vctx);
    const unsigned* map = c.mapped ? s->map : nullptr;
    unsigned total = 0;
    SolvePlan plain;
    plain.last = kSeedLevel;
    plain.energy_level = int(kSeedLevel);
    plain.energy = s->energy;
    plain.map = map;
    int rc = enqueue_solve(s, st, pairs, plain);
    if (rc) return rc;
    total += s->launches;
    if (cudaError_t e = launch_sol_keep(s, pairs, map, true, st))
        return set_error_code(PDFLOW_ERR_CUDA, "keep the plain 60x80 solution", e);
    total += 1;

    unsigned li;
    level_geom(s, kSeedLevel, &li, pairs);
    const cudaStream_t net_st = net_stream(c.net);
    net_set_stream_internal(c.net, st);
    rc = net_gather_input(c.net, s->pyr[s->new_slot ^ 1][li], s->pyr[s->new_slot][li], s->pair_stride, map,
                          int(pairs), st);
    if (!rc) rc = net_seed(c.net, int(pairs), net_input_buffer(c.net), s->seed);
    net_set_stream_internal(c.net, net_st);
    if (rc) return rc;
    total += 1 + net_seed_launches(c.net, int(pairs));   // the input gather, then the network

    SolvePlan warm;
    warm.first = kSeedLevel;
    warm.last = kSeedLevel;
    warm.seed = s->seed;
    warm.iter_scale = c.iter_scale;
    warm.energy_level = int(kSeedLevel);
    warm.energy = s->energy + s->batch;
    warm.map = map;
    rc = enqueue_solve(s, st, pairs, warm);
    if (rc) return rc;
    s->launches += total;
    return PDFLOW_OK;
}

struct TailCtx {
    float iter_scale;
    bool restore;            // put the kept plain 60x80 solution back first
    const unsigned* map;
};

// The levels finer than 60x80 for the mapped pairs, from the 60x80 solution in sol.
int learned_tail(pdflow_solver* s, cudaStream_t st, unsigned pairs, const void* vctx)
{
    const TailCtx& c = *static_cast<const TailCtx*>(vctx);
    if (c.restore)
        if (cudaError_t e = launch_sol_keep(s, pairs, c.map, false, st))
            return set_error_code(PDFLOW_ERR_CUDA, "restore the plain 60x80 solution", e);
    SolvePlan tail;
    tail.first = kSeedLevel + 1;
    tail.iter_scale = c.iter_scale;
    tail.map = c.map;
    const int rc = enqueue_solve(s, st, pairs, tail);
    if (rc == PDFLOW_OK && c.restore) s->launches += 1;
    return rc;
}

unsigned scale_kind(float scale, bool mapped)
{
    uint32_t b;
    std::memcpy(&b, &scale, 4);
    return 0x10000000u ^ (b >> 4) ^ (mapped ? 0x20000000u : 0u);
}

// graph kinds of the two continuations (the head's kinds have bit 28 set)
unsigned tail_kind(float scale)
{
    uint32_t b;
    std::memcpy(&b, &scale, 4);
    return 0x40000000u ^ (b >> 4);
}
constexpr unsigned kKindFallbackTail = 2u;

int learned_solve(pdflow_solver* s, unsigned n, const unsigned* slots, pdflow_net* net,
                  const pdflow_learned_opts* opts, pdflow_learned_report* report, bool force_fallback = false)
{
    if (!s || !net) {
        set_last_error("null argument");
        return PDFLOW_ERR_ARG;
    }
    if (s->mixed) {
        set_last_error("a mixed-resolution handle: use the mixed calls");
        return PDFLOW_ERR_STATE;
    }
    if (n == 0 || n > s->batch || n > net_max_batch(net)) {
        set_last_error("pair count out of range (solver batch or network batch)");
        return PDFLOW_ERR_ARG;
    }
    if (s->ctf_levels <= kSeedLevel + 1 || !s->seed) {
        set_last_error("the learned warm start needs rows >= 120 (a level finer than 60x80)");
        return PDFLOW_ERR_ARG;
    }
    pdflow_learned_opts o{0.5f, 0.01f};
    if (opts) o = *opts;
    if (!(o.iter_scale > 0.f) || o.iter_scale > 1.f) {
        set_last_error("iter_scale must be in (0, 1]");
        return PDFLOW_ERR_ARG;
    }
    std::vector<unsigned> ids(n);
    if (slots) {
        if (!s->slot_mode) {
            set_last_error("no frames were pushed per slot");
            return PDFLOW_ERR_STATE;
        }
        for (unsigned k = 0; k < n; ++k) {
            if (slots[k] >= s->batch) {
                set_last_error("slot out of range");
                return PDFLOW_ERR_ARG;
            }
            if (s->slot_frames[slots[k]] < 2) {
                set_last_error("a slot has fewer than two frames");
                return PDFLOW_ERR_STATE;
            }
            ids[k] = slots[k];
        }
        std::vector<unsigned char> seen(s->batch, 0);
        for (unsigned k = 0; k < n; ++k)
            if (seen[ids[k]]++) {
                set_last_error("slot listed twice");
                return PDFLOW_ERR_ARG;
            }
        cudaError_t e = cudaMemcpyAsync(s->map, ids.data(), sizeof(unsigned) * n, cudaMemcpyHostToDevice, s->stream);
        if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "H2D slots", e);
    } else {
        if (s->slot_mode) {
            set_last_error("frames were pushed per slot: pass the slot list");
            return PDFLOW_ERR_STATE;
        }
        if (s->frames < 2) {
            set_last_error("solve needs two pushed frames");
            return PDFLOW_ERR_STATE;
        }
        for (unsigned k = 0; k < n; ++k) ids[k] = k;
    }

    if (!s->sol_keep) {   // outside any capture: the graphs below only use it
        void* p = nullptr;
        const size_t keep = sizeof(float) * 10 * kSeedN * s->batch;
        if (cudaMalloc(&p, learned_keep_bytes(s->batch)) != cudaSuccess) {
            cudaGetLastError();
            set_last_error("learned-path buffers");
            return PDFLOW_ERR_OOM;
        }
        s->sol_keep = static_cast<float*>(p);
        s->map2 = reinterpret_cast<unsigned*>(static_cast<char*>(p) + keep);
    }
    const NvtxRange trace_range("pdflow learned solve");
    LearnedCtx ctx{net, o.iter_scale, slots != nullptr};
    int rc;
    {
        const NvtxRange head_range("head: plain to 60x80, network, warm 60x80");
        // keyed by the network's uid, never by its address: a network created
        // where a destroyed one lived must not replay that one's graph (whose
        // launches point at the destroyed network's buffers)
        rc = run_graphed(s, n, scale_kind(o.iter_scale, slots != nullptr), learned_enqueue, &ctx, net_uid(net));
    }
    if (rc) return rc;
    unsigned launches = s->launches;
    std::vector<float> e(2 * size_t(s->batch));
    cudaError_t ce = cudaMemcpyAsync(e.data(), s->energy, sizeof(float) * 2 * s->batch, cudaMemcpyDeviceToHost,
                                     s->stream);
    if (ce != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "D2H energies", ce);
    rc = check_status(s);
    if (rc) return rc;

    std::vector<unsigned> fall, keep;
    float worst = 0.f;
    for (unsigned k = 0; k < n; ++k) {
        const float ep = e[k], el = e[s->batch + k];
        const float ratio = ep > 0.f ? el / ep : (el > 0.f ? INFINITY : 1.f);
        if (!(ratio <= worst)) worst = ratio;   // NaN propagates as "worst"
        if (force_fallback || (o.energy_margin >= 0.f && !(el <= (1.f + o.energy_margin) * ep)))
            fall.push_back(ids[k]);
        else keep.push_back(ids[k]);
    }
    // the head graph has finished (its energies were read), so both maps are free
    const NvtxRange tail_range("continuations");
    if (!keep.empty()) {
        ce = cudaMemcpyAsync(s->map, keep.data(), sizeof(unsigned) * keep.size(), cudaMemcpyHostToDevice, s->stream);
        if (ce != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "H2D accepted slots", ce);
        const TailCtx tc{o.iter_scale, false, s->map};
        rc = run_graphed(s, unsigned(keep.size()), tail_kind(o.iter_scale), learned_tail, &tc);
        if (rc) return rc;
        launches += s->launches;
    }
    if (!fall.empty()) {
        ce = cudaMemcpyAsync(s->map2, fall.data(), sizeof(unsigned) * fall.size(), cudaMemcpyHostToDevice,
                             s->stream);
        if (ce != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "H2D fallback slots", ce);
        const TailCtx tc{1.f, true, s->map2};
        rc = run_graphed(s, unsigned(fall.size()), kKindFallbackTail, learned_tail, &tc);
        if (rc) return rc;
        launches += s->launches;
    }
    s->launches = launches;   // the continuations run asynchronously, as a plain solve does
    if (report) {
        report->fallbacks = unsigned(fall.size());
        report->max_energy_ratio = worst;
    }
    return PDFLOW_OK;
}

}  // namespace

int pdflow::learned_solve_all_fallback(pdflow_solver* s, unsigned n, const unsigned* slots, pdflow_net* net,
                                       const pdflow_learned_opts* opts)
{
    return learned_solve(s, n, slots, net, opts, nullptr, true);
}

extern "C" {

int pdflow_solve_batch_learned(pdflow_solver* s, unsigned n, pdflow_net* net, const pdflow_learned_opts* opts,
                               pdflow_learned_report* report)
{
    return learned_solve(s, n, nullptr, net, opts, report);
}

int pdflow_solve_slots_learned(pdflow_solver* s, unsigned n, const unsigned* slots, pdflow_net* net,
                               const pdflow_learned_opts* opts, pdflow_learned_report* report)
{
    if (!slots) {
        set_last_error("null slot list");
        return PDFLOW_ERR_ARG;
    }
    return learned_solve(s, n, slots, net, opts, report);
}

int pdflow_seed_level_inputs(pdflow_solver* s, unsigned n, float* d_out)
{
    if (!s || !d_out || n == 0 || n > s->batch) {
        set_last_error("bad argument");
        return PDFLOW_ERR_ARG;
    }
    if (s->ctf_levels <= kSeedLevel || s->frames < 2 || s->slot_mode) {
        set_last_error("needs rows >= 60 and two frames pushed for the whole batch");
        return PDFLOW_ERR_STATE;
    }
    unsigned li;
    level_geom(s, kSeedLevel, &li, n);
    cudaError_t e = launch_gather_seed_input(s->pyr[s->new_slot ^ 1][li], s->pyr[s->new_slot][li], s->pair_stride,
                                             nullptr, int(n), d_out, s->stream);
    if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "seed input gather", e);
    return check_status(s);
}

int pdflow_seed_level_labels(pdflow_solver* s, unsigned n, float* d_out)
{
    if (!s || !d_out || n == 0 || n > s->batch) {
        set_last_error("bad argument");
        return PDFLOW_ERR_ARG;
    }
    if (s->ctf_levels <= kSeedLevel) {
        set_last_error("needs rows >= 60");
        return PDFLOW_ERR_STATE;
    }
    const unsigned blk = s->cols / 80;
    k_seed_labels<<<(n * kSeedN + 255) / 256, 256, 0, s->stream>>>(s->sol, s->rows, blk, s->pair_stride, int(n),
                                                                     d_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "seed label launch", e);
    return check_status(s);
}

int pdflow_learned_energies(const pdflow_solver* s, unsigned n, float* plain, float* learned)
{
    if (!s || n == 0 || n > s->batch) {
        set_last_error("bad argument");
        return PDFLOW_ERR_ARG;
    }
    if (plain && cudaMemcpy(plain, s->energy, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error_code(PDFLOW_ERR_CUDA, "D2H energies");
    if (learned &&
        cudaMemcpy(learned, s->energy + s->batch, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error_code(PDFLOW_ERR_CUDA, "D2H energies");
    return PDFLOW_OK;
}

}  // extern "C"
