// Inspection entry points (include/pdflow_debug.h) and the level-image
// readback of include/pdflow.h.  Not on the solve path.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/pdflow.h"
#include "../../include/pdflow_debug.h"
#include "pdflow_internal.h"
#include "pdflow_iterate.cuh"
#include "pdflow_kernels.cuh"
#include "pdflow_math.cuh"

using namespace pdflow;

namespace {

int fail(const char* what, cudaError_t e) { return set_error_code(PDFLOW_ERR_CUDA, what, e); }

int fail(int code, const char* what) { return set_error_code(code, what); }

struct Dumper {
    pdflow_dump_fn fn;
    void* ctx;
    cudaStream_t st;
    std::vector<float> buf;
    int operator()(const char* name, int level, const float* dev, size_t n)
    {
        buf.resize(n);
        cudaError_t e = cudaMemcpyAsync(buf.data(), dev, n * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail("dump copy", e);
        fn(ctx, name, level, buf.data(), long(n));
        return 0;
    }
};

}  // namespace

extern "C" {

int pdflow_read_level_images(pdflow_solver* s, unsigned level, int frame, float* colour, float* depth, float* xx,
                             float* yy)
{
    if (!s || level >= s->pyr_levels || (frame != 0 && frame != 1))
        return fail(PDFLOW_ERR_ARG, "level beyond the pyramid or frame not 0/1");
    const PyrLevel& P = s->pyr[frame ? s->new_slot : (s->new_slot ^ 1)][level];
    const size_t n = (size_t(s->width) >> level) * (size_t(s->height) >> level);
    const float* src[4] = {P.col, P.dep, P.xx, P.yy};
    float* dst[4] = {colour, depth, xx, yy};
    for (int a = 0; a < 4; ++a)
        if (dst[a]) {
            cudaError_t e = cudaMemcpyAsync(dst[a], src[a], n * 4, cudaMemcpyDeviceToHost, s->stream);
            if (e != cudaSuccess) return fail("level image copy", e);
        }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? PDFLOW_OK : fail("synchronize", e);
}

int pdflow_read_all_solutions(pdflow_solver* s, float* dx, float* dy, float* dz, float* depth, float* depth_old,
                              float* colour, float* colour_old, float* xx, float* xx_old, float* yy, float* yy_old)
{
    if (!s) return fail(PDFLOW_ERR_ARG, "null handle");
    unsigned li = 0;
    level_geom(s, s->ctf_levels - 1, &li);   // the image level of the finest solved level
    int rc = pdflow_read_level_images(s, li, 1, colour, depth, xx, yy);
    if (!rc) rc = pdflow_read_level_images(s, li, 0, colour_old, depth_old, xx_old, yy_old);
    if (rc) return rc;
    if (!dx && !dy && !dz) return PDFLOW_OK;
    const size_t n = size_t(s->rows) * s->cols * 4;
    float* dst[3] = {dx, dy, dz};
    const float* src[3] = {s->dx, s->dy, s->dz};
    for (int a = 0; a < 3; ++a)
        if (dst[a]) {
            cudaError_t e = cudaMemcpyAsync(dst[a], src[a], n, cudaMemcpyDeviceToHost, s->stream);
            if (e != cudaSuccess) return fail("motion field copy", e);
        }
    return check_status(s);
}

int pdflow_keep_level_solutions(pdflow_solver* s, int keep)
{
    if (!s) return fail(PDFLOW_ERR_ARG, "null handle");
    if (s->mixed) return fail(PDFLOW_ERR_STATE, "a mixed-resolution handle keeps no per-level record");
    keep = keep ? 1 : 0;
    if (keep == s->keep_levels) return PDFLOW_OK;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail("synchronize", e);
    if (keep && !s->lvl_keep) {
        const size_t stride = level_keep_offset(s, s->ctf_levels);
        void* p = nullptr;
        e = cudaMalloc(&p, sizeof(float) * stride * s->batch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error_code(PDFLOW_ERR_OOM, "per-level record allocation", e);
        }
        e = cudaMemsetAsync(p, 0, sizeof(float) * stride * s->batch, s->stream);
        if (e != cudaSuccess) {
            cudaFree(p);
            return fail("per-level record clear", e);
        }
        s->lvl_keep = static_cast<float*>(p);
        s->lvl_keep_stride = stride;
    }
    // captured solves hold the old launch sequence
    for (auto& g : s->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    s->graphs.clear();
    s->keep_levels = keep;
    return PDFLOW_OK;
}

int pdflow_read_level_flow(pdflow_solver* s, unsigned pair, unsigned level, float* du, float* dv, float* dw,
                           float* dx, float* dy, float* dz)
{
    if (!s) return fail(PDFLOW_ERR_ARG, "null handle");
    if (pair >= s->batch || level >= s->ctf_levels) return fail(PDFLOW_ERR_ARG, "pair or level out of range");
    if (!s->keep_levels || !s->lvl_keep)
        return fail(PDFLOW_ERR_STATE, "per-level record off (pdflow_keep_level_solutions)");
    const LevelGeom g = level_geom(s, level, nullptr);
    const float* base = s->lvl_keep + size_t(pair) * s->lvl_keep_stride + level_keep_offset(s, level);
    float* dst[6] = {du, dv, dw, dx, dy, dz};
    for (int a = 0; a < 6; ++a)
        if (dst[a]) {
            cudaError_t e = cudaMemcpyAsync(dst[a], base + size_t(a) * g.N, sizeof(float) * g.N,
                                            cudaMemcpyDeviceToHost, s->stream);
            if (e != cudaSuccess) return fail("level record copy", e);
        }
    return check_status(s);
}

int pdflow_read_level_solutions(pdflow_solver* s, unsigned level, float* dx, float* dy, float* dz, float* depth,
                                float* depth_old, float* colour, float* colour_old, float* xx, float* xx_old,
                                float* yy, float* yy_old)
{
    if (!s) return fail(PDFLOW_ERR_ARG, "null handle");
    if (level >= s->ctf_levels) return fail(PDFLOW_ERR_ARG, "level beyond the solved levels");
    unsigned li = 0;
    level_geom(s, level, &li);   // the pyramid level holding this solved level's images
    int rc = pdflow_read_level_images(s, li, 1, colour, depth, xx, yy);
    if (!rc) rc = pdflow_read_level_images(s, li, 0, colour_old, depth_old, xx_old, yy_old);
    if (rc) return rc;
    if (!dx && !dy && !dz) return PDFLOW_OK;
    return pdflow_read_level_flow(s, 0, level, nullptr, nullptr, nullptr, dx, dy, dz);
}

int pdflow_debug_solve(pdflow_solver* s, pdflow_dump_fn fn, void* ctx)
{
    if (!s || !fn) return fail(PDFLOW_ERR_ARG, "null argument");
    if (s->frames < 2) return fail(PDFLOW_ERR_STATE, "solve needs two pushed frames");
    cudaStream_t st = s->stream;
    Dumper dump{fn, ctx, st, {}};
    Params p{s->prm.lambda_i, s->prm.lambda_d, s->prm.mu, s->prm.fovh, s->cols};
    const int fn_ = s->new_slot, fo = fn_ ^ 1;
    const LevelConsts& L = s->L;
    const State& S = s->S;
    for (unsigned i = 0; i < s->ctf_levels; ++i) {
        unsigned li;
        const LevelGeom g = level_geom(s, i, &li);
        const PyrLevel o = s->pyr[fo][li], n = s->pyr[fn_][li];
        cudaError_t e = launch_level_init(g, i == 0, s->sol, o, n, L, S, st);
        if (e == cudaSuccess) e = launch_im_gradients(g, n, L, st);
        if (e == cudaSuccess) e = launch_warp_steps(g, o, n, L, p, st);
        if (e != cudaSuccess) return fail("set-up launch", e);
        const struct { const char* name; const float* ptr; } setup[] = {
            {"dct", L.dct}, {"dcu", L.dcu}, {"dcv", L.dcv}, {"ddt", L.ddt}, {"ddu", L.ddu}, {"ddv", L.ddv},
            {"mu", L.mu}, {"ri", L.ri}, {"rj", L.rj}, {"ri_2", L.ri2}, {"rj_2", L.rj2}, {"du_prev", L.du_prev},
            {"dv_prev", L.dv_prev}, {"sigma_pd", L.spd}, {"sigma_puvx", L.spuvx}, {"sigma_puvy", L.spuvy},
            {"sigma_pwx", L.spwx}, {"sigma_pwy", L.spwy}, {"tau_u", L.tu}, {"tau_v", L.tv}, {"tau_w", L.tw},
            {"init_dw", S.dw}, {"init_dw_acc", S.dwa}, {"init_pd", S.pd}, {"init_puu", S.puu},
            {"init_puv", S.puv}, {"init_pvu", S.pvu}, {"init_pvv", S.pvv}, {"init_pwu", S.pwu},
            {"init_pwv", S.pwv}};
        for (const auto& d : setup)
            if (dump(d.name, int(i), d.ptr, g.N)) return PDFLOW_ERR_CUDA;
        const unsigned iters = s->prm.num_max_iter[i];
        for (unsigned it = 0; it < iters; ++it) {
            e = launch_dual(g, L, S, p, st);
            if (e == cudaSuccess) e = launch_primal(g, L, S, p, false, o.dep, st);
            if (e != cudaSuccess) return fail("iteration launch", e);
        }
        const struct { const char* name; const float* ptr; } state[] = {
            {"du_new", S.du}, {"dv_new", S.dv}, {"dw_new", S.dw}, {"du_acc", S.dua}, {"dv_acc", S.dva},
            {"dw_acc", S.dwa}, {"pd", S.pd}, {"puu", S.puu}, {"puv", S.puv}, {"pvu", S.pvu}, {"pvv", S.pvv},
            {"pwu", S.pwu}, {"pwv", S.pwv}};
        for (const auto& d : state)
            if (dump(d.name, int(i), d.ptr, g.N)) return PDFLOW_ERR_CUDA;
        e = launch_saturate(g, L, S, o.dep, st);
        if (e != cudaSuccess) return fail("saturate launch", e);
        if (dump("sat_du", int(i), S.du, g.N) || dump("sat_dv", int(i), S.dv, g.N) ||
            dump("sat_dw", int(i), S.dw, g.N))
            return PDFLOW_ERR_CUDA;
        e = launch_median(g, i + 1 == s->ctf_levels, o, L, S, s->sol, s->dx, s->dy, s->dz, p, nullptr, st);
        if (e != cudaSuccess) return fail("median launch", e);
        if (dump("du_l", int(i), s->sol.du, g.N) || dump("dv_l", int(i), s->sol.dv, g.N) ||
            dump("dw_l", int(i), s->sol.dw, g.N))
            return PDFLOW_ERR_CUDA;
    }
    return PDFLOW_OK;
}

int pdflow_set_iteration_form(pdflow_solver* s, int form)
{
    if (!s || form < 0 || form > 10) return fail(PDFLOW_ERR_ARG, "iteration form must be 0..10");
    if (s->iter_form != form) {
        cudaStreamSynchronize(s->stream);
        s->iter_form = form;   // graphs are cached per iteration form
    }
    return PDFLOW_OK;
}

int pdflow_last_solve_launches(const pdflow_solver* s, unsigned* count)
{
    if (!s || !count) return fail(PDFLOW_ERR_ARG, "null argument");
    *count = s->launches;
    return PDFLOW_OK;
}

int pdflow_time_level_iterations(pdflow_solver* s, unsigned n, unsigned level, unsigned iters, float* ms)
{
    if (!s || !ms || n == 0 || n > s->batch || level >= s->ctf_levels || iters == 0)
        return fail(PDFLOW_ERR_ARG, "bad pair count, level or iteration count");
    cudaEvent_t a, b;
    cudaError_t ce = cudaEventCreate(&a);
    if (ce != cudaSuccess) return fail("event create", ce);
    ce = cudaEventCreate(&b);
    if (ce != cudaSuccess) {
        cudaEventDestroy(a);
        return fail("event create", ce);
    }
    cudaEventRecord(a, s->stream);
    int rc = enqueue_level_iterations(s, s->stream, n, level, iters);
    cudaEventRecord(b, s->stream);
    cudaError_t e = cudaEventSynchronize(b);
    if (rc == PDFLOW_OK && e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc != PDFLOW_OK) return rc;
    return e == cudaSuccess ? PDFLOW_OK : fail("timing", e);
}

}  // extern "C"

namespace {

// div_rcp against the IEEE division on random pairs of its range: a = +-2^[-60, 59]
// x mantissa (one in 1024 a signed zero), b = 2^[-40, 59] x mantissa (one in 256
// just above the shrinkage's 1e-10 floor); counts the pairs whose bits differ.
__device__ __forceinline__ unsigned mix64(unsigned long long x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return unsigned(x);
}
__device__ __forceinline__ float rand_mag(unsigned r, int lo, int hi)   // sign, exponent in [lo, hi], mantissa
{
    const int e = lo + int(r % unsigned(hi - lo + 1));
    return __uint_as_float((r & 0x80000000u) | (unsigned(e + 127) << 23) | (mix64(r) & 0x7fffffu));
}
__global__ void k_div_rcp_check(unsigned long long n, unsigned long long seed, unsigned long long* bad)
{
    unsigned long long mine = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned r1 = mix64(seed + 2 * i), r2 = mix64(seed + 2 * i + 1);
        float a = rand_mag(r1, -60, 59);
        if ((r2 & 1023u) == 0) a = (r2 & 1024u) ? -0.f : 0.f;
        float b = rand_mag(r2 & 0x7fffffffu, -40, 59);
        if ((r1 & 255u) == 3) b = __fadd_rn(__uint_as_float((mix64(r1) & 0x007fffffu) | 0x2e000000u), 1e-10f);
        if (__float_as_uint(div_rcp(a, b, __frcp_rn(b))) != __float_as_uint(__fdiv_rn(a, b))) ++mine;
    }
    if (mine) atomicAdd(bad, mine);
}

// `passes` copies a -> b, b -> a, a -> b ... in one launch; each thread moves
// the same elements every pass (no cross-thread hazard), with L2-level loads
// and stores (ld/st.global.cg) that the compiler cannot fold across passes.
__global__ void __launch_bounds__(512) k_copy4(float4* a, float4* b, size_t n, unsigned passes)
{
    for (unsigned r = 0; r < passes; ++r) {
        float4* src = (r & 1) ? b : a;
        float4* dst = (r & 1) ? a : b;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
            float4 v;
            asm volatile("ld.global.cg.v4.f32 {%0, %1, %2, %3}, [%4];"
                         : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                         : "l"(src + i));
            asm volatile("st.global.cg.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst + i), "f"(v.x), "f"(v.y), "f"(v.z),
                         "f"(v.w)
                         : "memory");
        }
    }
}

}  // namespace

extern "C" {

int pdflow_check_div_rcp(unsigned long long pairs, unsigned long long seed, unsigned long long* mismatches)
{
    if (!mismatches) return fail(PDFLOW_ERR_ARG, "null output");
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof *d) != cudaSuccess) {
        cudaGetLastError();
        return fail(PDFLOW_ERR_OOM, "counter");
    }
    cudaError_t e = cudaMemset(d, 0, sizeof *d);
    if (e == cudaSuccess) {
        k_div_rcp_check<<<1024, 256>>>(pairs, seed, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, d, sizeof *d, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? PDFLOW_OK : fail("division check", e);
}

int pdflow_strip_units(unsigned bands, unsigned cols, unsigned iters_per_launch, unsigned ctas, unsigned* whole,
                       unsigned* tier_n, unsigned* tier_p)
{
    if (!whole || !tier_n || !tier_p) return fail(PDFLOW_ERR_ARG, "null output");
    if (bands == 0 || cols == 0 || ctas == 0 || iters_per_launch == 0 || iters_per_launch > 4)
        return fail(PDFLOW_ERR_ARG, "bands, columns and CTAs must be positive, 1 <= iterations per launch <= 4");
    const pdflow::StripUnits su = pdflow::strip_units(bands, cols, iters_per_launch, ctas);
    *whole = su.whole;
    for (int i = 0; i < 3; ++i) {
        tier_n[i] = su.tier_n[i];
        tier_p[i] = su.tier_p[i];
    }
    return PDFLOW_OK;
}

int pdflow_measure_copy_gbs(size_t bytes, unsigned reps, void* stream, float* gbs)
{
    if (!gbs || bytes < 16 || reps == 0) return fail(PDFLOW_ERR_ARG, "bad size, repetitions or null output");
    bytes &= ~size_t(15);
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail("device query", e);
    void *a = nullptr, *b = nullptr;
    if (cudaMalloc(&a, bytes) != cudaSuccess || cudaMalloc(&b, bytes) != cudaSuccess) {
        cudaGetLastError();
        if (a) cudaFree(a);
        return fail(PDFLOW_ERR_OOM, "copy buffers");
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t n = bytes / 16;
    const unsigned grid = unsigned(sms) * 4u;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaMemsetAsync(a, 0, bytes, st);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        k_copy4<<<grid, 512, 0, st>>>(static_cast<float4*>(a), static_cast<float4*>(b), n, 2);   // warm-up
        e = cudaEventRecord(e0, st);
        if (e == cudaSuccess) {
            k_copy4<<<grid, 512, 0, st>>>(static_cast<float4*>(a), static_cast<float4*>(b), n, reps);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess) *gbs = float(2.0 * double(bytes) * reps / (double(ms) * 1e-3) / 1e9);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(b);
    return e == cudaSuccess ? PDFLOW_OK : fail("copy timing", e);
}

int pdflow_trace_solve(pdflow_solver* s, unsigned n, float* ms)
{
    if (!s || !ms || n == 0 || n > s->batch) return fail(PDFLOW_ERR_ARG, "bad pair count or null output");
    if (s->slot_mode) return fail(PDFLOW_ERR_STATE, "frames were pushed per slot");
    if (s->mixed) return fail(PDFLOW_ERR_STATE, "a mixed-resolution handle: use the mixed calls");
    if (s->frames < 2) return fail(PDFLOW_ERR_STATE, "solve needs two pushed frames");
    const unsigned L = s->ctf_levels, ne = 3 * L + 1;
    std::vector<cudaEvent_t> ev(ne, nullptr);
    cudaError_t e = cudaSuccess;
    for (unsigned k = 0; k < ne && e == cudaSuccess; ++k) e = cudaEventCreate(&ev[k]);
    int rc = PDFLOW_OK;
    if (e == cudaSuccess) {
        SolvePlan plan;
        plan.trace = ev.data();
        rc = enqueue_solve(s, s->stream, n, plan);
        if (rc == PDFLOW_OK) e = cudaEventSynchronize(ev[ne - 1]);
        for (unsigned k = 0; k + 1 < ne && rc == PDFLOW_OK && e == cudaSuccess; ++k)
            e = cudaEventElapsedTime(ms + k, ev[k], ev[k + 1]);
    }
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    if (rc != PDFLOW_OK) return rc;
    if (e != cudaSuccess) return fail("trace events", e);
    return pdflow::check_status(s);
}

int pdflow_stage_median(unsigned R, unsigned C, const float* depth_old, const float* ddt, const float* du,
                        const float* dv, const float* dw, float* du_l, float* dv_l, float* dw_l, int32_t* sel,
                        void* stream)
{
    if (!depth_old || !ddt || !du || !dv || !dw || !du_l || !dv_l || !dw_l || R < 2 || C < 2)
        return fail(PDFLOW_ERR_ARG, "null plane or level smaller than 2x2");
    LevelGeom g{R, C, R * C};  // one pair, no stride
    PyrLevel o{nullptr, const_cast<float*>(depth_old), nullptr, nullptr};
    LevelConsts L{};
    L.ddt = const_cast<float*>(ddt);
    State S{};
    S.du = const_cast<float*>(du);
    S.dv = const_cast<float*>(dv);
    S.dw = const_cast<float*>(dw);
    LevelSol out{};
    out.du = du_l;
    out.dv = dv_l;
    out.dw = dw_l;
    Params p{};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = launch_median(g, false, o, L, S, out, nullptr, nullptr, nullptr, p, sel, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? PDFLOW_OK : fail("stage median", e);
}

int pdflow_solve_levels(pdflow_solver* s, unsigned n, unsigned first, unsigned last, const float* d_seed,
                        float iter_scale, int energy_level, float* energies)
{
    if (!s) return fail(PDFLOW_ERR_ARG, "null handle");
    if (n == 0 || n > s->batch) return fail(PDFLOW_ERR_ARG, "pair count out of range");
    if (first >= s->ctf_levels || last < first) return fail(PDFLOW_ERR_ARG, "level range out of range");
    if (s->frames < 2) return fail(PDFLOW_ERR_STATE, "solve needs two pushed frames");
    if (!(iter_scale > 0.f)) return fail(PDFLOW_ERR_ARG, "iteration scale must be positive");
    if (first > 0 && !d_seed) return fail(PDFLOW_ERR_ARG, "a level after the coarsest starts from a seed");
    pdflow::SolvePlan plan;
    plan.first = first;
    plan.last = last;
    plan.seed = d_seed;
    plan.iter_scale = iter_scale;
    plan.energy_level = energy_level;
    plan.energy = energy_level >= 0 ? s->energy : nullptr;
    int rc = pdflow::enqueue_solve(s, s->stream, n, plan);
    if (rc) return rc;
    if (plan.energy && energies) {
        cudaError_t e = cudaMemcpyAsync(energies, s->energy, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream);
        if (e != cudaSuccess) return fail(PDFLOW_ERR_CUDA, "D2H energies");
    }
    return pdflow::check_status(s);
}

int pdflow_debug_wait_timeout(pdflow_solver* s, unsigned polls)
{
    if (!s || polls == 0 || polls > 10000000u) return fail(PDFLOW_ERR_ARG, "polls 1..1e7");
    const cudaError_t e = launch_wait_probe(s->flags, s->status, polls, s->stream);
    if (e != cudaSuccess) return fail("wait probe launch", e);
    return pdflow::check_status(s);
}

int pdflow_set_tile_copy_mode(int shape, int mode)
{
    if (shape < 0 || shape > 3 || mode < 0 || mode > 7) return fail(PDFLOW_ERR_ARG, "shape 0..3, mode 0..7");
    set_tile_copy_mode(shape, mode);
    return PDFLOW_OK;
}

int pdflow_set_quad_prefetch(unsigned ctas_ahead)
{
    if (ctas_ahead > (1u << 20)) return fail(PDFLOW_ERR_ARG, "prefetch distance above 2^20 CTAs");
    set_quad_prefetch(ctas_ahead);
    return PDFLOW_OK;
}

}  // extern "C"
