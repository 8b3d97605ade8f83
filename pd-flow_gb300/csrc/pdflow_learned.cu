// Learned warm start of a batched solve (include/pdflow_net.h).
//
// One CUDA graph per (pair count, iteration scale, slot addressing) runs the
// plain schedule to the 60x80 level with its energy, the network on that
// level's images, and the warm-started schedule from the 60x80 level with its
// own energy; the host then compares the two energies per pair and re-solves
// the rejected pairs with the plain schedule.
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

    unsigned li;
    level_geom(s, kSeedLevel, &li, pairs);
    const cudaStream_t net_st = net_stream(c.net);
    net_set_stream_internal(c.net, st);
    rc = net_gather_input(c.net, s->pyr[s->new_slot ^ 1][li], s->pyr[s->new_slot][li], s->pair_stride, map,
                          int(pairs), st);
    if (!rc) rc = net_seed(c.net, int(pairs), net_input_buffer(c.net), s->seed);
    net_set_stream_internal(c.net, net_st);
    if (rc) return rc;
    total += 2 + 3 * 12 + 3 + 2;   // gather, input, 12 x (im2col + GEMM), 3 pools, head bias + output

    SolvePlan warm;
    warm.first = kSeedLevel;
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

int slots_plain(pdflow_solver* s, cudaStream_t st, unsigned pairs, const void*)
{
    SolvePlan plan;
    plan.map = s->map;
    return enqueue_solve(s, st, pairs, plan);
}

unsigned scale_kind(float scale, bool mapped)
{
    uint32_t b;
    std::memcpy(&b, &scale, 4);
    return 0x10000000u ^ (b >> 4) ^ (mapped ? 0x20000000u : 0u);
}

int learned_solve(pdflow_solver* s, unsigned n, const unsigned* slots, pdflow_net* net,
                  const pdflow_learned_opts* opts, pdflow_learned_report* report)
{
    if (!s || !net) {
        set_last_error("null argument");
        return PDFLOW_ERR_ARG;
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

    LearnedCtx ctx{net, o.iter_scale, slots != nullptr};
    int rc = run_graphed(s, n, scale_kind(o.iter_scale, slots != nullptr), learned_enqueue, &ctx, net);
    if (rc) return rc;
    std::vector<float> e(2 * size_t(s->batch));
    cudaError_t ce = cudaMemcpyAsync(e.data(), s->energy, sizeof(float) * 2 * s->batch, cudaMemcpyDeviceToHost,
                                     s->stream);
    if (ce != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "D2H energies", ce);
    rc = check_status(s);
    if (rc) return rc;

    std::vector<unsigned> fall;
    float worst = 0.f;
    for (unsigned k = 0; k < n; ++k) {
        const float ep = e[k], el = e[s->batch + k];
        const float ratio = ep > 0.f ? el / ep : (el > 0.f ? INFINITY : 1.f);
        if (!(ratio <= worst)) worst = ratio;   // NaN propagates as "worst"
        if (o.energy_margin >= 0.f && !(el <= (1.f + o.energy_margin) * ep)) fall.push_back(ids[k]);
    }
    if (!fall.empty()) {
        ce = cudaMemcpyAsync(s->map, fall.data(), sizeof(unsigned) * fall.size(), cudaMemcpyHostToDevice, s->stream);
        if (ce != cudaSuccess) return set_error_code(PDFLOW_ERR_CUDA, "H2D fallback slots", ce);
        const unsigned launches = s->launches;
        rc = run_graphed(s, unsigned(fall.size()), 1u, slots_plain, nullptr);
        s->launches += launches;
        if (rc) return rc;
    }
    if (report) {
        report->fallbacks = unsigned(fall.size());
        report->max_energy_ratio = worst;
    }
    return PDFLOW_OK;
}

}  // namespace

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
