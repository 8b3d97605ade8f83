// The primal-dual iterations of one pyramid level in a single launch.
//
// Each CTA owns a slab of columns [u0, u1) of the level (column-major
// planes: a column is R contiguous floats, so a slab is one contiguous range).
// Per iteration it
//   1. computes the dual step (gradient + updateDualVariables) on its columns
//      and, redundantly, on the column u0-1 of its left neighbour, into shared
//      memory (the primal's backward divergence needs the new duals one
//      column to the left);
//   2. computes the primal step (divergence + updatePrimalVariables) on its
//      own columns.
// The over-relaxed primal (du_acc, dv_acc, dw_acc) and the duals are double
// buffered (iteration t reads buffer t&1 and writes buffer (t+1)&1), so the
// only synchronisation is one wait per iteration for the two neighbouring
// slabs to have finished the previous iteration.  The wait is
//   - nothing (one CTA owns the level),
//   - the hardware cluster barrier (the level fits one thread-block cluster), or
//   - per-CTA progress counters in global memory, spun on with a bounded
//     count (a cooperative launch keeps every CTA resident).  A wait that
//     runs out sets an error code in the status word and the kernel returns.
// Data written by another CTA is read with ld.global.cg (L2), never through a
// possibly stale L1 line.  Per-pixel arithmetic is pdflow_math.cuh, identical
// to the stage kernels, so the results are bit-for-bit the same.
#include <algorithm>
#include <atomic>

#include <cooperative_groups.h>

#include "pdflow_iterate.cuh"
#include "pdflow_math.cuh"

namespace cg = cooperative_groups;

namespace pdflow {

namespace {

constexpr unsigned kIterThreads = 1024;
// One CTA owns a whole small level (at most 1200 pixels): fewer threads, so
// that the level's plane pointers and per-pixel temporaries fit in registers.
constexpr unsigned kSingleThreads = 384;
constexpr unsigned long long kSpinLimit = 1ull << 24;   // ~seconds of polling, then give up

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 waits until both neighbouring slabs have completed `need`
// iterations, polling at most `limit` times.  Returns false (after recording
// the failure) on timeout.
__device__ bool wait_neighbours(const IterArgs& a, unsigned need, unsigned long long limit = kSpinLimit)
{
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned b = blockIdx.x;
        unsigned long long spins = 0;
        if (b > 0)
            while (ld_acquire(a.flags + b - 1) < need) {
                if (++spins > limit || ld_acquire(a.status) != 0) { ok = 0; break; }
            }
        if (ok && b + 1 < gridDim.x)
            while (ld_acquire(a.flags + b + 1) < need) {
                if (++spins > limit || ld_acquire(a.status) != 0) { ok = 0; break; }
            }
        if (!ok) atomicCAS(a.status, 0u, kStatusTimeout);
    }
    __syncthreads();
    return ok != 0;
}

// Shared-memory layout of a CTA (slab of W = u1-u0 columns, halo column h0 = u0-1):
//   13 state planes over the slab:  du dv dw | du_acc dv_acc dw_acc | pd puu puv pvu pvv pwu pwv
//    7 planes of new duals over [h0, u1)
enum { SDU, SDV, SDW, SUA, SVA, SWA, SPD, SPUU, SPUV, SPVU, SPVV, SPWU, SPWV, SNST };

// A level with at most one pixel per thread of a single CTA: each thread
// keeps its pixel's state, duals and constants in registers for all the
// iterations, and only the values its neighbours read go through shared
// memory (the over-relaxed primal for the forward differences of the right
// and lower neighbours' duals; the TV duals for the backward divergence of
// the left and upper ones).  The same per-pixel functions in the same order
// as the general loop below, so the same bits.  Two barriers per iteration
// order every exchange: a plane is rewritten only after the barrier that
// follows its readers' last read.
__device__ __forceinline__ void iterate_resident(const IterArgs& a, float* sm)
{
    const unsigned R = a.g.R, C = a.g.C, N = a.g.N;
    const LevelConsts L = a.L;
    const float li = a.p.lambda_i, ld = a.p.lambda_d;
    float* xa = sm;                  // [3][N]: du_acc, dv_acc, dw_acc
    float* xp = sm + 3 * N;          // [6][N]: puu, puv, pvu, pvv, pwu, pwv
    const unsigned i = threadIdx.x;
    const bool live = i < N;
    const unsigned v = live ? i % R : 0, u = live ? i / R : 0;
    const bool fu = (u == 0), lu = (u == C - 1), fv = (v == 0), lv = (v == R - 1);
    const unsigned iu = lu ? i : i + R, iv = lv ? i : i + 1;   // right / lower neighbour (itself at a border)
    const unsigned im = fu ? i : i - R, jm = fv ? i : i - 1;   // left / upper neighbour
    float du = 0.f, dv = 0.f, dw = 0.f, ua = 0.f, va = 0.f, wa = 0.f;
    Duals d{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float spd = 0.f, spuvx = 0.f, spuvy = 0.f, spwx = 0.f, spwy = 0.f, mu = 0.f, ddt = 0.f, ddu = 0.f, ddv = 0.f;
    float ri = 0.f, rj = 0.f, ri_m = 0.f, rj_m = 0.f, dup = 0.f, dvp = 0.f, dup_u = 0.f, dvp_u = 0.f, dup_v = 0.f,
          dvp_v = 0.f, tu = 0.f, tv = 0.f, tw = 0.f, dct = 0.f, dcu = 0.f, dcv = 0.f;
    if (live) {
        du = a.du[i];
        dv = a.dv[i];
        dw = a.dw[i];
        ua = __ldcg(a.acc[0][0] + i);
        va = __ldcg(a.acc[0][1] + i);
        wa = __ldcg(a.acc[0][2] + i);
        d = Duals{__ldcg(a.p_[0][0] + i), __ldcg(a.p_[0][1] + i), __ldcg(a.p_[0][2] + i), __ldcg(a.p_[0][3] + i),
                  __ldcg(a.p_[0][4] + i), __ldcg(a.p_[0][5] + i), __ldcg(a.p_[0][6] + i)};
        spd = __ldg(L.spd + i); spuvx = __ldg(L.spuvx + i); spuvy = __ldg(L.spuvy + i);
        spwx = __ldg(L.spwx + i); spwy = __ldg(L.spwy + i); mu = __ldg(L.mu + i); ddt = __ldg(L.ddt + i);
        ddu = __ldg(L.ddu + i); ddv = __ldg(L.ddv + i); ri = __ldg(L.ri + i); rj = __ldg(L.rj + i);
        ri_m = fu ? ri : __ldg(L.ri + i - R);
        rj_m = fv ? rj : __ldg(L.rj + i - 1);
        dup = __ldg(L.du_prev + i); dvp = __ldg(L.dv_prev + i);
        dup_u = __ldg(L.du_prev + iu); dvp_u = __ldg(L.dv_prev + iu);
        dup_v = __ldg(L.du_prev + iv); dvp_v = __ldg(L.dv_prev + iv);
        tu = __ldg(L.tu + i); tv = __ldg(L.tv + i); tw = __ldg(L.tw + i);
        dct = __ldg(L.dct + i); dcu = __ldg(L.dcu + i); dcv = __ldg(L.dcv + i);
    }
    for (unsigned t = 0; t < a.iters; ++t) {
        // ---- dual step ----
        if (live) {
            xa[i] = ua;
            xa[N + i] = va;
            xa[2 * N + i] = wa;
        }
        __syncthreads();
        if (live) {
            dual_update(d, spd, spuvx, spuvy, spwx, spwy, mu, ddt, ddu, ddv, li, ld, ri, rj, ua, va, wa, dup, dvp,
                        xa[iu], xa[N + iu], xa[2 * N + iu], dup_u, dvp_u, xa[iv], xa[N + iv], xa[2 * N + iv], dup_v,
                        dvp_v, lu, lv);
            xp[i] = d.puu;
            xp[N + i] = d.puv;
            xp[2 * N + i] = d.pvu;
            xp[3 * N + i] = d.pvv;
            xp[4 * N + i] = d.pwu;
            xp[5 * N + i] = d.pwv;
        }
        __syncthreads();
        // ---- primal step ----
        if (live) {
            const float divu = divergence(ri, ri_m, rj, rj_m, d.puu, xp[im], d.puv, xp[N + jm], fu, lu, fv, lv);
            const float divv = divergence(ri, ri_m, rj, rj_m, d.pvu, xp[2 * N + im], d.pvv, xp[3 * N + jm], fu, lu,
                                          fv, lv);
            const float divw = divergence(ri, ri_m, rj, rj_m, d.pwu, xp[4 * N + im], d.pwv, xp[5 * N + jm], fu, lu,
                                          fv, lv);
            primal_update(du, dv, dw, ua, va, wa, tu, tv, tw, mu, ddu, ddv, d.pd, li, ld, divu, divv, divw, dct, dcu,
                          dcv);
            if (t + 1 == a.iters) saturate(du, dv, dw, dup, dvp, __ldg(a.depth_old + i));
        }
    }
    // final state for the weighted median, the duals to buffer (iters & 1),
    // as the general loop leaves them
    if (live) {
        a.du[i] = du;
        a.dv[i] = dv;
        a.dw[i] = dw;
        const bool fb = a.iters & 1;
        const float pn[7] = {d.pd, d.puu, d.puv, d.pvu, d.pvv, d.pwu, d.pwv};
#pragma unroll
        for (int k = 0; k < 7; ++k) (fb ? a.p_[1][k] : a.p_[0][k])[i] = pn[k];
    }
}

template <int kMode>
__global__ void __launch_bounds__(kMode == kIterSingle ? kSingleThreads : kIterThreads, 1) k_iterate(IterArgs a)
{
    extern __shared__ float sm[];
    if (a.g.map || (kMode != kIterGrid && blockIdx.y > 0)) {
        // batch: the pair of grid row y (the grid form solves one pair) of a strided arena
        const size_t po = pair_off(a.g.map, a.g.pstride, kMode == kIterGrid ? 0u : blockIdx.y);
        a.L = at(a.L, po);
        a.du = at(a.du, po);
        a.dv = at(a.dv, po);
        a.dw = at(a.dw, po);
        for (int q = 0; q < 2; ++q) {
            for (int k = 0; k < 3; ++k) a.acc[q][k] = at(a.acc[q][k], po);
            for (int k = 0; k < 7; ++k) a.p_[q][k] = at(a.p_[q][k], po);
        }
        a.depth_old = at(a.depth_old, po);
    }
    const unsigned R = a.g.R, C = a.g.C;
    const unsigned nb = gridDim.x, b = blockIdx.x;
    const unsigned u0 = (unsigned)((unsigned long long)b * C / nb);
    const unsigned u1 = (unsigned)((unsigned long long)(b + 1) * C / nb);
    const unsigned h0 = (u0 > 0) ? u0 - 1 : 0;
    const unsigned nown = (u1 - u0) * R;          // own pixels
    const unsigned nsp = (u1 - h0) * R;           // pixels with a dual in this CTA
    const unsigned off = (u0 - h0) * R;           // index of the first own pixel in the dual planes
    const unsigned ps = a.smem_state_plane;       // floats per state plane (>= nown)
    const unsigned pq = a.smem_plane;             // floats per dual plane (>= nsp)
    float* st = sm;                               // SNST planes, own pixels at [0, nown)
    float* np = sm + SNST * ps;                   // 7 planes of new duals, [0, nsp)
    const LevelConsts& L = a.L;
    const float li = a.p.lambda_i, ld = a.p.lambda_d;
    // one CTA (kIterSingle) owns every column: no halo column, no neighbours
    constexpr bool kOne = kMode == kIterSingle;
    const bool has_left = !kOne && (u0 > 0), has_right = !kOne && (u1 < C);
    if (kOne && nsp <= blockDim.x) {
        iterate_resident(a, sm);
        return;
    }

    // initial state of the level (written by the set-up kernel into buffer 0)
    for (unsigned j = threadIdx.x; j < nown; j += blockDim.x) {
        const unsigned i = u0 * R + j;
        st[SDU * ps + j] = a.du[i];
        st[SDV * ps + j] = a.dv[i];
        st[SDW * ps + j] = a.dw[i];
#pragma unroll
        for (int k = 0; k < 3; ++k) st[(SUA + k) * ps + j] = __ldcg(a.acc[0][k] + i);
#pragma unroll
        for (int k = 0; k < 7; ++k) st[(SPD + k) * ps + j] = __ldcg(a.p_[0][k] + i);
    }
    __syncthreads();

    for (unsigned t = 0; t < a.iters; ++t) {
        const int cur = t & 1, nxt = cur ^ 1;
        if (t > 0) {
            if (kMode == kIterGrid) {
                if (!wait_neighbours(a, t)) return;
            } else if (kMode == kIterCluster) {
                cg::this_cluster().sync();
            }
        }
        // ---- dual step over [h0, u1) ----
        for (unsigned j = threadIdx.x; j < nsp; j += blockDim.x) {
            const unsigned v = j % R, u = h0 + j / R, i = v + u * R;
            const bool own = kOne || (u >= u0);
            const unsigned jo = j - off;          // own-slab index (valid when own)
            const bool lu = (u == C - 1), lv = (v == R - 1);
            float dua, dva, dwa, dua_u, dva_u, dwa_u, dua_v, dva_v, dwa_v;
            Duals d;
            if (own) {
                dua = st[SUA * ps + jo]; dva = st[SVA * ps + jo]; dwa = st[SWA * ps + jo];
                d = Duals{st[SPD * ps + jo], st[SPUU * ps + jo], st[SPUV * ps + jo], st[SPVU * ps + jo],
                          st[SPVV * ps + jo], st[SPWU * ps + jo], st[SPWV * ps + jo]};
                const unsigned jv = lv ? jo : jo + 1;
                dua_v = st[SUA * ps + jv]; dva_v = st[SVA * ps + jv]; dwa_v = st[SWA * ps + jv];
            } else {
                // halo column u0-1: the left neighbour's state of this iteration
                dua = __ldcg(a.acc[cur][0] + i); dva = __ldcg(a.acc[cur][1] + i); dwa = __ldcg(a.acc[cur][2] + i);
                d = Duals{__ldcg(a.p_[cur][0] + i), __ldcg(a.p_[cur][1] + i), __ldcg(a.p_[cur][2] + i),
                          __ldcg(a.p_[cur][3] + i), __ldcg(a.p_[cur][4] + i), __ldcg(a.p_[cur][5] + i),
                          __ldcg(a.p_[cur][6] + i)};
                const unsigned iv = lv ? i : i + 1;
                dua_v = __ldcg(a.acc[cur][0] + iv); dva_v = __ldcg(a.acc[cur][1] + iv);
                dwa_v = __ldcg(a.acc[cur][2] + iv);
            }
            if (lu) {
                dua_u = dua; dva_u = dva; dwa_u = dwa;
            } else if (kOne || u + 1 < u1) {
                const unsigned ju = (u + 1 - u0) * R + v;   // own column to the right
                dua_u = st[SUA * ps + ju]; dva_u = st[SVA * ps + ju]; dwa_u = st[SWA * ps + ju];
            } else {
                // column u1: the right neighbour's first column
                dua_u = __ldcg(a.acc[cur][0] + i + R); dva_u = __ldcg(a.acc[cur][1] + i + R);
                dwa_u = __ldcg(a.acc[cur][2] + i + R);
            }
            const unsigned iu = lu ? i : i + R, iv = lv ? i : i + 1;
            dual_update(d, __ldg(L.spd + i), __ldg(L.spuvx + i), __ldg(L.spuvy + i), __ldg(L.spwx + i),
                        __ldg(L.spwy + i), __ldg(L.mu + i), __ldg(L.ddt + i), __ldg(L.ddu + i), __ldg(L.ddv + i), li,
                        ld, __ldg(L.ri + i), __ldg(L.rj + i), dua, dva, dwa, __ldg(L.du_prev + i),
                        __ldg(L.dv_prev + i), dua_u, dva_u, dwa_u, __ldg(L.du_prev + iu), __ldg(L.dv_prev + iu), dua_v,
                        dva_v, dwa_v, __ldg(L.du_prev + iv), __ldg(L.dv_prev + iv), lu, lv);
            np[0 * pq + j] = d.pd;
            np[1 * pq + j] = d.puu;
            np[2 * pq + j] = d.puv;
            np[3 * pq + j] = d.pvu;
            np[4 * pq + j] = d.pvv;
            np[5 * pq + j] = d.pwu;
            np[6 * pq + j] = d.pwv;
        }
        __syncthreads();
        // ---- primal step over [u0, u1) ----
        const bool last = (t + 1 == a.iters);
        for (unsigned j = threadIdx.x; j < nown; j += blockDim.x) {
            const unsigned v = j % R, u = u0 + j / R, i = v + u * R;
            const unsigned jl = off + j;                   // index in the dual planes
            const bool fu = (u == 0), lu = (u == C - 1), fv = (v == 0), lv = (v == R - 1);
            const unsigned jum = fu ? jl : jl - R, jvm = fv ? jl : jl - 1;
            const float ri = __ldg(L.ri + i), rj = __ldg(L.rj + i);
            const float ri_m = fu ? ri : __ldg(L.ri + i - R), rj_m = fv ? rj : __ldg(L.rj + i - 1);
            float pn[7];
#pragma unroll
            for (int k = 0; k < 7; ++k) pn[k] = np[k * pq + jl];
            const float divu = divergence(ri, ri_m, rj, rj_m, pn[1], np[1 * pq + jum], pn[2], np[2 * pq + jvm], fu, lu,
                                          fv, lv);
            const float divv = divergence(ri, ri_m, rj, rj_m, pn[3], np[3 * pq + jum], pn[4], np[4 * pq + jvm], fu, lu,
                                          fv, lv);
            const float divw = divergence(ri, ri_m, rj, rj_m, pn[5], np[5 * pq + jum], pn[6], np[6 * pq + jvm], fu, lu,
                                          fv, lv);
            float du = st[SDU * ps + j], dv = st[SDV * ps + j], dw = st[SDW * ps + j], nua, nva, nwa;
            primal_update(du, dv, dw, nua, nva, nwa, __ldg(L.tu + i), __ldg(L.tv + i), __ldg(L.tw + i),
                          __ldg(L.mu + i), __ldg(L.ddu + i), __ldg(L.ddv + i), pn[0], li, ld, divu, divv, divw,
                          __ldg(L.dct + i), __ldg(L.dcu + i), __ldg(L.dcv + i));
            if (last) saturate(du, dv, dw, __ldg(L.du_prev + i), __ldg(L.dv_prev + i), __ldg(a.depth_old + i));
            st[SDU * ps + j] = du;
            st[SDV * ps + j] = dv;
            st[SDW * ps + j] = dw;
            st[SUA * ps + j] = nua;
            st[SVA * ps + j] = nva;
            st[SWA * ps + j] = nwa;
#pragma unroll
            for (int k = 0; k < 7; ++k) st[(SPD + k) * ps + j] = pn[k];
            if (!last) {
                // publish the columns the neighbours read in the next iteration
                if (has_left && u == u0) {
                    __stcg(a.acc[nxt][0] + i, nua);
                    __stcg(a.acc[nxt][1] + i, nva);
                    __stcg(a.acc[nxt][2] + i, nwa);
                }
                if (has_right && u == u1 - 1) {
                    __stcg(a.acc[nxt][0] + i, nua);
                    __stcg(a.acc[nxt][1] + i, nva);
                    __stcg(a.acc[nxt][2] + i, nwa);
#pragma unroll
                    for (int k = 0; k < 7; ++k) __stcg(a.p_[nxt][k] + i, pn[k]);
                }
            }
        }
        __syncthreads();
        if (kMode == kIterGrid && !last) {
            if (threadIdx.x == 0) {
                __threadfence();
                st_release(a.flags + b, t + 1);
            }
        }
    }
    // Final state for the weighted median: saturated (du, dv, dw) and the duals.
    // The duals go to buffer (iters & 1): the neighbours may still be reading
    // buffer ((iters - 1) & 1) in their last iteration, and nobody reads the
    // other one any more.
    const bool fb = a.iters & 1;
    for (unsigned j = threadIdx.x; j < nown; j += blockDim.x) {
        const unsigned i = u0 * R + j;
        a.du[i] = st[SDU * ps + j];
        a.dv[i] = st[SDV * ps + j];
        a.dw[i] = st[SDW * ps + j];
#pragma unroll
        for (int k = 0; k < 7; ++k) (fb ? a.p_[1][k] : a.p_[0][k])[i] = st[(SPD + k) * ps + j];
    }
}

// Failure-detection probe: CTA 1 waits, through wait_neighbours with `limit`
// polls, for CTA 0 to complete an iteration, and CTA 0 never publishes one
// (its counter is a flag nothing sets), so the wait runs out and records
// kStatusTimeout; both CTAs return.
__global__ void k_wait_probe(IterArgs a, unsigned limit)
{
    if (blockIdx.x == 0) return;
    wait_neighbours(a, 1u, limit);
}

// Written by prepare_iterate (once per device, under the caller's lock), read by
// planning threads: atomics, so concurrent handles never race on them.
std::atomic<unsigned> g_max_cluster{8};    // largest cluster the GPU places with this kernel's resources
std::atomic<unsigned> g_max_dyn_smem{0};   // dynamic shared memory available to the iteration kernels

}  // namespace

unsigned iterate_smem_limit() { return g_max_dyn_smem; }

IterPlan plan_iterate(LevelGeom g, int num_sms)
{
    IterPlan pl;
    if (g.N <= 1200 || g.C < 8) {
        pl.mode = kIterSingle;
        pl.ctas = 1;
    } else if (g.N <= 19200) {
        pl.mode = kIterCluster;
        pl.ctas = (g.C >= 160) ? g_max_cluster.load() : 8u;
    } else {
        pl.mode = kIterGrid;
        unsigned s = g.C / 2;
        if (s > (unsigned)num_sms) s = (unsigned)num_sms;
        pl.ctas = s;
    }
    unsigned maxcols = 0, maxown = 0;
    for (unsigned b = 0; b < pl.ctas; ++b) {
        const unsigned u0 = (unsigned)((unsigned long long)b * g.C / pl.ctas);
        const unsigned u1 = (unsigned)((unsigned long long)(b + 1) * g.C / pl.ctas);
        const unsigned h0 = u0 > 0 ? u0 - 1 : 0;
        if (u1 - h0 > maxcols) maxcols = u1 - h0;
        if (u1 - u0 > maxown) maxown = u1 - u0;
    }
    pl.smem_plane = maxcols * g.R;
    pl.smem_state_plane = maxown * g.R;
    pl.smem_bytes = (size_t(13) * pl.smem_state_plane + size_t(7) * pl.smem_plane) * sizeof(float);
    return pl;
}

template <int kMode>
static cudaError_t allow_smem(int optin)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k_iterate<kMode>);
    if (e != cudaSuccess) return e;
    const int dyn = optin - (int)fa.sharedSizeBytes;
    const unsigned cur = g_max_dyn_smem.load();
    if (cur == 0 || (unsigned)dyn < cur) g_max_dyn_smem.store((unsigned)dyn);
    return cudaFuncSetAttribute(k_iterate<kMode>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
}

cudaError_t prepare_iterate()
{
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_iterate<kIterCluster>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess) e = allow_smem<kIterCluster>(optin);
    if (e == cudaSuccess) e = allow_smem<kIterGrid>(optin);
    if (e == cudaSuccess) e = allow_smem<kIterSingle>(optin);
    if (e != cudaSuccess) return e;
    // Is a 16-CTA cluster of this kernel placeable (shared memory of the largest clustered level)?
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kIterThreads);
    cfg.dynamicSmemBytes = 100 * 1024;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = 16;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_iterate<kIterCluster>, &cfg) == cudaSuccess && nclusters > 0)
        g_max_cluster = 16;
    else
        cudaGetLastError();
    return cudaSuccess;
}

cudaError_t launch_wait_probe(unsigned* flags, unsigned* status, unsigned polls, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(flags, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    IterArgs a{};
    a.flags = flags;
    a.status = status;
    k_wait_probe<<<2, 32, 0, st>>>(a, polls);
    return cudaGetLastError();
}

cudaError_t launch_iterate(const IterPlan& pl, IterArgs a, cudaStream_t st)
{
    a.smem_plane = pl.smem_plane;
    a.smem_state_plane = pl.smem_state_plane;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(pl.ctas, pl.mode == kIterGrid ? 1 : a.g.pairs);
    const unsigned single = std::min(kSingleThreads, (a.g.N + 31u) / 32u * 32u);
    cfg.blockDim = dim3(pl.mode == kIterSingle ? single : kIterThreads);
    cfg.dynamicSmemBytes = pl.smem_bytes;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    cfg.attrs = attr;
    cfg.numAttrs = 0;
    if (pl.mode == kIterGrid) {
        cudaError_t e = cudaMemsetAsync(a.flags, 0, sizeof(unsigned) * pl.ctas, st);
        if (e != cudaSuccess) return e;
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_iterate<kIterGrid>, a);
    }
    if (pl.mode == kIterCluster) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = pl.ctas;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_iterate<kIterCluster>, a);
    }
    return cudaLaunchKernelEx(&cfg, k_iterate<kIterSingle>, a);
}

}  // namespace pdflow
