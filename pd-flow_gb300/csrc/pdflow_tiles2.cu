// Temporally blocked primal-dual iterations, paired form.
//
// Same tiling as pdflow_tiles.cu (40x40 interior, 4-pixel halo, 48x48 region
// of 24 planes in shared memory, kk <= 4 iterations per launch, alternating
// state buffers), but each of the 576 threads owns two vertically adjacent
// pixel pairs (v, v+1) in each of two region columns (or, in the narrower
// shapes, 40x34 interiors and 1008 threads, or 24x24 interiors and 512
// threads, each thread owning one pair).  A pair's arithmetic
// runs as packed FP32x2 instructions (fma/add/sub/mul.rn.f32x2: each lane
// rounds exactly as the scalar __f*_rn operation, so the results are the
// same bits as the scalar kernels, as long as no packed product feeds only a
// packed sum, see the dw update), its own and horizontally neighbouring
// values are read with 8-byte shared loads, and only the vertical neighbour
// beyond the pair needs a scalar load.  Work that depends on a lane's branch
// (clamping, disc projection with rhypotf, the shrinkage cases) stays scalar.
//
// A pixel pair is updated in iteration j while at least one of its pixels is
// j or more from a non-border region edge; the other pixel of such a pair and
// pixels further out compute garbage from stale neighbours, exactly as they
// would hold stale values if skipped, and no exact pixel ever reads them.  Reads beyond a region edge are redirected into the
// region's own storage, so every shared access stays in bounds.
//
// Region loads (levels with rows % 4 == 0): each plane's whole region as one
// TMA tensor copy (3D tensor map over rows, columns and arena slots), issued by
// one thread and completing on two mbarriers (the step-size set-up's five
// planes first); or one TMA bulk copy per plane column; or plain loads.
#include <cuda.h>

#include <atomic>

#include "pdflow_iterate.cuh"
#include "pdflow_math.cuh"

namespace pdflow {

namespace {

constexpr int kH = 4;

// Four shapes (interior rows TV x columns TU): 40x40 with 576 threads owning
// two pairs each; 40x34 with 1008 threads owning one pair each (more warps
// per SM, slightly more halo); 24x24 with 512 threads owning one pair each,
// small enough (96 KB) for two CTAs per SM, so that one CTA's region load and
// store overlap the other's iterations at the price of more halo; 24x28 with
// 288 threads owning two pairs each, two CTAs per SM (108 KB each).
template <int TV, int TU>
struct Shape {
    static constexpr int kTV = TV, kRV = TV + 2 * kH, kPV = kRV / 2;   // region rows, pairs per region column
    static constexpr int kTU = TU, kRU = TU + 2 * kH, kPlane = kRV * kRU;
    static constexpr int kCols = (TU == 40 || TU == 28) ? 2 : 1;   // region columns per thread
    static constexpr int kTY = kRU / kCols;             // columns per sweep
    static constexpr int kThreads = kPV * kTY;
    static constexpr int kBlocksPerSM = TV == 24 ? 2 : 1;           // CTAs per SM the registers allow
    static_assert(kTY * kCols == kRU && kThreads <= 1024 && kRV % 2 == 0, "paired tile layout");
};

enum { T_DU, T_DV, T_DW, T_UA, T_VA, T_WA, T_PD, T_PUU, T_PUV, T_PVU, T_PVV, T_PWU, T_PWV,
       T_MU, T_DDT, T_DDU, T_DDV, T_DCT, T_DCU, T_DCV, T_RI, T_RJ, T_DUP, T_DVP, T_NPLANES };

struct Tile2Args {
    LevelGeom g;
    LevelConsts L;
    State src, dst;
    Params p;
    const float* depth_old;
    unsigned kk;
    bool last;
    unsigned tiles_v;
    bool bulk;            // region columns load by TMA bulk copies (16-byte aligned: R % 4 == 0)
    bool bulk_store;      // interior columns store by TMA bulk copies
    unsigned* status;     // device word: kTileBulkTimeout when the bounded wait for the region gives up
    bool tensor;          // each plane's kRV x kRU region by one TMA tensor copy (maps below)
};

// Tensor maps of the 24 region planes (3D: rows, columns, arena slots), for
// the tensor-copy region load (box = one whole region).
struct Tile2Maps {
    CUtensorMap m[T_NPLANES];
};

constexpr unsigned kTileBulkTimeout = 0x54494C45u;
constexpr unsigned kBulkWaitLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- packed FP32x2 arithmetic (per-lane IEEE round-to-nearest) ----
__device__ __forceinline__ unsigned long long pk(float2 a)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 upk(unsigned long long v)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ float2 fm2(float2 a, float2 b, float2 c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pk(a)), "l"(pk(b)), "l"(pk(c)));
    return upk(r);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk(a)), "l"(pk(b)));
    return upk(r);
}
__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk(a)), "l"(pk(b)));
    return upk(r);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk(a)), "l"(pk(b)));
    return upk(r);
}
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }

// pair flags
enum : unsigned { F_V0 = 1, F_V1 = 2, F_FU = 4, F_LU = 8, F_FV0 = 16, F_LV0 = 32, F_LV1 = 64 };

__device__ __forceinline__ void clamp_pd(float& pd)
{
    if (fabsf(pd) > 1.f) pd = (pd > 1.f) ? 1.f : -1.f;
}

template <int TV, int TU>
__global__ void __launch_bounds__(Shape<TV, TU>::kThreads, Shape<TV, TU>::kBlocksPerSM)
    k_iterate_tiles2(Tile2Args a, const __grid_constant__ Tile2Maps tm)
{
    using S = Shape<TV, TU>;
    constexpr int kTV = S::kTV, kRV = S::kRV, kPV = S::kPV;
    constexpr int kTU = S::kTU, kRU = S::kRU, kPlane = S::kPlane, kCols = S::kCols, kTY = S::kTY;
    extern __shared__ __align__(128) float sm[];   // TMA tensor copies land on 128-byte boundaries
    const size_t po = pair_off(a.g.map, a.g.pstride, blockIdx.y);
    const LevelConsts L = at(a.L, po);
    const State src = at(a.src, po), dst = at(a.dst, po);
    const float* depth_old = at(a.depth_old, po);
    const int R = (int)a.g.R, C = (int)a.g.C;
    const int tv = (int)(blockIdx.x % a.tiles_v), tu = (int)(blockIdx.x / a.tiles_v);
    const int iv0 = tv * kTV, iu0 = tu * kTU;
    const int iv1 = min(iv0 + kTV, R), iu1 = min(iu0 + kTU, C);
    const int rv0 = max(iv0 - kH, 0), ru0 = max(iu0 - kH, 0);
    const int rv1 = min(iv1 + kH, R), ru1 = min(iu1 + kH, C);
    const int RV = rv1 - rv0, RU = ru1 - ru0;
    const int tx = threadIdx.x % kPV, ty = threadIdx.x / kPV;
    const int rv = 2 * tx;                      // the pair's first row in the region
    const bool even_rows = (R & 1) == 0;        // global pair loads are 8-byte aligned
    float* P[T_NPLANES];
#pragma unroll
    for (int k = 0; k < T_NPLANES; ++k) P[k] = sm + k * kPlane;

    // ---- load the region ----
    const float* gs[T_NPLANES] = {src.du, src.dv, src.dw, src.dua, src.dva, src.dwa, src.pd, src.puu, src.puv,
                                  src.pvu, src.pvv, src.pwu, src.pwv, L.mu, L.ddt, L.ddu, L.ddv, L.dct, L.dcu,
                                  L.dcv, L.ri, L.rj, L.du_prev, L.dv_prev};
    // bar[0]: the whole region, or with tensor copies only the five planes the
    // step-size set-up reads (mu, ddu, ddv, ri, rj); bar[1]: with tensor copies
    // the other 19 planes, awaited after the set-up so that it overlaps them
    __shared__ __align__(8) unsigned long long bar[2];
    __shared__ const float* s_gs[T_NPLANES];
    __shared__ float* s_gd[13];
    // plane tables of the bulk copies; the barrier after the load publishes them
    // to the store phase whichever way the region is loaded
    if ((a.bulk || a.bulk_store) && threadIdx.x == 0) {
        float* gd[13] = {dst.du, dst.dv, dst.dw, dst.dua, dst.dva, dst.dwa, dst.pd, dst.puu, dst.puv, dst.pvu,
                         dst.pvv, dst.pwu, dst.pwv};
#pragma unroll
        for (int k = 0; k < T_NPLANES; ++k) s_gs[k] = gs[k];
#pragma unroll
        for (int k = 0; k < 13; ++k) s_gd[k] = gd[k];
    }
    // bounded wait for phase 0 of an mbarrier; on timeout the status word is set
    auto wait_region = [&](uint32_t b) {
        bool done = false;
        for (uint32_t i = 0; i < kBulkWaitLimit && !done; ++i) {
            uint32_t ok;
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(ok)
                : "r"(b)
                : "memory");
            done = ok != 0;
        }
        if (!done && a.status) atomicExch(a.status, kTileBulkTimeout);
    };
    const bool tensor = a.bulk && a.tensor;
    if (a.bulk) {
        // one bulk copy per (plane, region column): RV contiguous floats, all
        // addresses and sizes multiples of 16 bytes (checked by the launcher)
        const uint32_t b = smem_addr(&bar[0]), b1 = smem_addr(&bar[1]);
        // tensor copies move whole kRV x kRU boxes (rows or columns past the level's
        // edge arrive as zeros and, like rows beyond the region, are never read)
        constexpr uint32_t kBox = (uint32_t)kPlane * 4u;
        const uint32_t bytes = tensor ? 5u * kBox : (uint32_t)(T_NPLANES * RU * RV) * 4u;
        if (threadIdx.x == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b));
            if (tensor) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b1));
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
            if (tensor) {
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b1),
                             "r"((uint32_t)(T_NPLANES - 5) * kBox)
                             : "memory");
                // one copy per plane: box (kRV rows, kRU columns, 1 slot) at (rv0, ru0, slot);
                // rv0 is a multiple of 4 floats (16 bytes), as tensor copies require.
                // The set-up's planes go first.
                const int slot = (int)(a.g.map ? (__ldg(a.g.map + blockIdx.y) & kMapSlotMask) : blockIdx.y);
                constexpr int kOrder[T_NPLANES] = {T_MU,  T_DDU, T_DDV, T_RI,  T_RJ,  T_DU,  T_DV,  T_DW,
                                                   T_UA,  T_VA,  T_WA,  T_PD,  T_PUU, T_PUV, T_PVU, T_PVV,
                                                   T_PWU, T_PWV, T_DDT, T_DCT, T_DCU, T_DCV, T_DUP, T_DVP};
#pragma unroll
                for (int o = 0; o < T_NPLANES; ++o) {
                    const int k = kOrder[o];
                    asm volatile(
                        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(sm + k * kPlane)),
                        "l"(reinterpret_cast<uint64_t>(&tm.m[k])), "r"(rv0), "r"(ru0), "r"(slot),
                        "r"(o < 5 ? b : b1)
                        : "memory");
                }
            }
        }
        __syncthreads();
        for (int c = threadIdx.x; !tensor && c < T_NPLANES * RU; c += blockDim.x) {
            const int k = c / RU, ru = c % RU;
            const float* g = s_gs[k] + (size_t)rv0 + (size_t)(ru0 + ru) * R;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_addr(sm + k * kPlane + ru * kRV)),
                "l"(g), "r"((uint32_t)RV * 4u), "r"(b)
                : "memory");
        }
        wait_region(b);
    } else {
#pragma unroll
        for (int c = 0; c < kCols; ++c) {
            const int ru = ty + kTY * c;
            if (ru >= RU || rv >= RV) continue;
            const int q = rv + ru * kRV;
            const size_t gi = (size_t)(rv0 + rv) + (size_t)(ru0 + ru) * R;
            if (even_rows) {
#pragma unroll
                for (int k = 0; k < T_NPLANES; ++k) st2(P[k] + q, __ldg(reinterpret_cast<const float2*>(gs[k] + gi)));
            } else {
                const bool v1 = rv + 1 < RV;
#pragma unroll
                for (int k = 0; k < T_NPLANES; ++k) {
                    P[k][q] = __ldg(gs[k] + gi);
                    if (v1) P[k][q + 1] = __ldg(gs[k] + gi + 1);
                }
            }
        }
    }
    // plain loads need a barrier before any thread reads its neighbours; TMA copies
    // are visible to every thread once its own wait on their mbarrier has returned
    if (!a.bulk) __syncthreads();

    const float li = a.p.lambda_i, ld = a.p.lambda_d;
    unsigned flags[kCols];
    int ring[kCols];       // the pair's larger distance to a non-border region edge
    float2 sg[kCols][8];   // spd*mu, spuvx*li, spuvy*li, spwx*ld, spwy*ld, tau_u, tau_v, tau_w
#pragma unroll
    for (int c = 0; c < kCols; ++c) {
        const int ru = ty + kTY * c;
        const int u = ru0 + ru, v0 = rv0 + rv;
        unsigned f = 0;
        if (ru < RU) {
            if (rv < RV) f |= F_V0;
            if (rv + 1 < RV) f |= F_V1;
        }
        if (u == 0) f |= F_FU;
        if (u == C - 1) f |= F_LU;
        if (v0 == 0) f |= F_FV0;
        if (v0 == R - 1) f |= F_LV0;
        if (v0 + 1 == R - 1) f |= F_LV1;
        flags[c] = f;
        {
            // after j iterations only pixels at least j from a non-border region edge
            // are exact; a pair whose both pixels are closer is skipped from then on
            int du_ = 1 << 20;
            if (ru0 > 0) du_ = min(du_, ru);
            if (ru1 < C) du_ = min(du_, RU - 1 - ru);
            int d0 = du_, d1 = du_;
            if (rv0 > 0) { d0 = min(d0, rv); d1 = min(d1, rv + 1); }
            if (rv1 < R) { d0 = min(d0, RV - 1 - rv); d1 = min(d1, RV - 2 - rv); }
            ring[c] = (f & F_V1) ? max(d0, d1) : d0;
        }
        const int q = rv + ru * kRV;
        float s[2][8];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const bool valid = l == 0 ? (f & F_V0) : (f & F_V1);
            if (!valid) {
#pragma unroll
                for (int m = 0; m < 8; ++m) s[l][m] = 0.f;
                continue;
            }
            const int ql = q + l, rvl = rv + l;
            const bool fu = f & F_FU, fv = (l == 0) && (f & F_FV0);
            const float mu = P[T_MU][ql], ddu = P[T_DDU][ql], ddv = P[T_DDV][ql], ri = P[T_RI][ql], rj = P[T_RJ][ql];
            // the set-up kernel's expressions (mu_and_steps); at a region edge that is not an
            // image border the left/top neighbour is missing: that pixel is stale anyway
            const float ri_m = (fu || ru == 0) ? ri : P[T_RI][ql - kRV];
            const float rj_m = (fv || rvl == 0) ? rj : P[T_RJ][ql - 1];
            const float spd = fdividef(1.f, fm(mu, add(add(1.f, fabsf(ddu)), fabsf(ddv)), 1e-10f));
            s[l][0] = mul(spd, mu);
            s[l][1] = mul(fdividef(0.5f, fm(li, ri, 1e-10f)), li);
            s[l][2] = mul(fdividef(0.5f, fm(li, rj, 1e-10f)), li);
            s[l][3] = mul(fdividef(0.5f, fm(ri, ld, 1e-10f)), ld);
            s[l][4] = mul(fdividef(0.5f, fm(rj, ld, 1e-10f)), ld);
            float acu_r = add(ri, rj);
            if (!fu) acu_r = add(acu_r, ri_m);
            if (!fv) acu_r = add(acu_r, rj_m);
            s[l][5] = fdividef(1.f, add(fm(li, acu_r, mul(mu, fabsf(ddu))), 1e-10f));
            s[l][6] = fdividef(1.f, add(fm(li, acu_r, mul(mu, fabsf(ddv))), 1e-10f));
            s[l][7] = fdividef(1.f, add(fm(ld, acu_r, mu), 1e-10f));
        }
#pragma unroll
        for (int m = 0; m < 8; ++m) sg[c][m] = make_float2(s[0][m], s[1][m]);
    }
    if (tensor) wait_region(smem_addr(&bar[1]));   // the state and the other constant planes
    const float2 li2 = make_float2(li, li), ld2v = make_float2(ld, ld), two = make_float2(2.f, 2.f);
    const float2 zero = make_float2(0.f, 0.f);

    const bool last_launch = a.last || (pair_flags(a.g.map, blockIdx.y) & kMapLast);
    for (unsigned j = 0; j < a.kk; ++j) {
        const bool last_iter = last_launch && (j + 1 == a.kk);
        // ---- dual step (in place: each pixel reads only its own duals) ----
#pragma unroll
        for (int c = 0; c < kCols; ++c) {
            const unsigned f = flags[c];
            if (!(f & F_V0) || ring[c] < (int)j) continue;
            const int ru = ty + kTY * c, q = rv + ru * kRV;
            const int qu = (ru + 1 < kRU) ? q + kRV : q;           // beyond the region: own storage
            const int qv = (rv + 2 < kRV) ? q + 2 : q + 1;
            const float2 ua = ld2(P[T_UA] + q), va = ld2(P[T_VA] + q), wa = ld2(P[T_WA] + q);
            const float2 dup = ld2(P[T_DUP] + q), dvp = ld2(P[T_DVP] + q);
            const float2 ri = ld2(P[T_RI] + q), rj = ld2(P[T_RJ] + q);
            float2 gu1 = zero, gv1 = zero, gw1 = zero;
            if (!(f & F_LU)) {
                const float2 ua1 = ld2(P[T_UA] + qu), va1 = ld2(P[T_VA] + qu), wa1 = ld2(P[T_WA] + qu);
                const float2 dup1 = ld2(P[T_DUP] + qu), dvp1 = ld2(P[T_DVP] + qu);
                gu1 = mul2(ri, sub2(add2(ua1, dup1), add2(ua, dup)));
                gv1 = mul2(ri, sub2(add2(va1, dvp1), add2(va, dvp)));
                gw1 = mul2(ri, sub2(wa1, wa));
            }
            const float2 uav = make_float2(ua.y, P[T_UA][qv]), vav = make_float2(va.y, P[T_VA][qv]);
            const float2 wav = make_float2(wa.y, P[T_WA][qv]);
            const float2 dupv = make_float2(dup.y, P[T_DUP][qv]), dvpv = make_float2(dvp.y, P[T_DVP][qv]);
            float2 gu2 = mul2(rj, sub2(add2(uav, dupv), add2(ua, dup)));
            float2 gv2 = mul2(rj, sub2(add2(vav, dvpv), add2(va, dvp)));
            float2 gw2 = mul2(rj, sub2(wav, wa));
            if (f & F_LV0) { gu2.x = 0.f; gv2.x = 0.f; gw2.x = 0.f; }
            if (f & F_LV1) { gu2.y = 0.f; gv2.y = 0.f; gw2.y = 0.f; }
            const float2 X = fm2(ld2(P[T_DDV] + q), va, fm2(ld2(P[T_DDU] + q), ua, sub2(ld2(P[T_DDT] + q), wa)));
            float2 pd = fm2(sg[c][0], X, ld2(P[T_PD] + q));
            float2 puu = fm2(sg[c][1], gu1, ld2(P[T_PUU] + q)), puv = fm2(sg[c][2], gu2, ld2(P[T_PUV] + q));
            float2 pvu = fm2(sg[c][1], gv1, ld2(P[T_PVU] + q)), pvv = fm2(sg[c][2], gv2, ld2(P[T_PVV] + q));
            float2 pwu = fm2(sg[c][3], gw1, ld2(P[T_PWU] + q)), pwv = fm2(sg[c][4], gw2, ld2(P[T_PWV] + q));
            clamp_pd(pd.x);
            clamp_pd(pd.y);
            project_disc(puu.x, puv.x);
            project_disc(puu.y, puv.y);
            project_disc(pvu.x, pvv.x);
            project_disc(pvu.y, pvv.y);
            project_disc(pwu.x, pwv.x);
            project_disc(pwu.y, pwv.y);
            st2(P[T_PD] + q, pd);
            st2(P[T_PUU] + q, puu);
            st2(P[T_PUV] + q, puv);
            st2(P[T_PVU] + q, pvu);
            st2(P[T_PVV] + q, pvv);
            st2(P[T_PWU] + q, pwu);
            st2(P[T_PWV] + q, pwv);
        }
        __syncthreads();
        // ---- primal step (in place: each pixel writes only its own primal) ----
#pragma unroll
        for (int c = 0; c < kCols; ++c) {
            const unsigned f = flags[c];
            if (!(f & F_V0) || ring[c] < (int)j) continue;
            const int ru = ty + kTY * c, q = rv + ru * kRV;
            const int qm = ru > 0 ? q - kRV : q;                   // beyond the region: own storage
            const int qvm = rv > 0 ? q - 1 : q;
            const bool fu = f & F_FU, lu = f & F_LU;
            const float2 ri = ld2(P[T_RI] + q), rj = ld2(P[T_RJ] + q);
            const float2 rim = ld2(P[T_RI] + qm);
            const float2 rjm = make_float2(P[T_RJ][qvm], rj.x);
            const float2 puu = ld2(P[T_PUU] + q), puv = ld2(P[T_PUV] + q);
            const float2 pvu = ld2(P[T_PVU] + q), pvv = ld2(P[T_PVV] + q);
            const float2 pwu = ld2(P[T_PWU] + q), pwv = ld2(P[T_PWV] + q);
            const float2 puum = ld2(P[T_PUU] + qm), pvum = ld2(P[T_PVU] + qm), pwum = ld2(P[T_PWU] + qm);
            const float2 puvm = make_float2(P[T_PUV][qvm], puv.x), pvvm = make_float2(P[T_PVV][qvm], pvv.x);
            const float2 pwvm = make_float2(P[T_PWV][qvm], pwv.x);
            float2 div[3];
            const float2 pu_[3] = {puu, pvu, pwu}, pv_[3] = {puv, pvv, pwv};
            const float2 pum_[3] = {puum, pvum, pwum}, pvm_[3] = {puvm, pvvm, pwvm};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                float2 d;
                if (fu) d = mul2(ri, pu_[k]);
                else if (lu) d = mul2(neg2(rim), pum_[k]);
                else d = fm2(ri, pu_[k], neg2(mul2(rim, pum_[k])));
                float2 g = add2(d, fm2(rj, pv_[k], neg2(mul2(rjm, pvm_[k]))));
                if (f & F_FV0) g.x = fm(rj.x, pv_[k].x, d.x);
                else if (f & F_LV0) g.x = fm(-rjm.x, pvm_[k].x, d.x);
                if (f & F_LV1) g.y = fm(-rjm.y, pvm_[k].y, d.y);
                div[k] = g;
            }
            const float2 mu = ld2(P[T_MU] + q), pd = ld2(P[T_PD] + q);
            const float2 dcu = ld2(P[T_DCU] + q), dcv = ld2(P[T_DCV] + q), dct = ld2(P[T_DCT] + q);
            float2 du = ld2(P[T_DU] + q), dv = ld2(P[T_DV] + q), dw = ld2(P[T_DW] + q);
            const float2 du_old = du, dv_old = dv, dw_old = dw;
            const float2 tu = sg[c][5], tv = sg[c][6], tw = sg[c][7];
            du = fm2(neg2(tu), fm2(mul2(mu, ld2(P[T_DDU] + q)), pd, neg2(mul2(li2, div[0]))), du);
            dv = fm2(neg2(tv), fm2(mul2(mu, ld2(P[T_DDV] + q)), pd, neg2(mul2(li2, div[1]))), dv);
            // Per lane: a packed multiply whose only use is a packed add may be contracted
            // into one fused multiply-add by the assembler, which changes the rounding of
            // add(dw, mul(-tw, .)); the scalar intrinsics are never contracted.
            {
                const float2 t = fm2(neg2(mu), pd, neg2(mul2(ld2v, div[2])));
                dw.x = add(dw.x, mul(-tw.x, t.x));
                dw.y = add(dw.y, mul(-tw.y, t.y));
            }
            const float2 of = fm2(dcv, dv, fm2(dcu, du, dct));
            const float2 a1 = mul2(tu, dcu), b1 = mul2(tv, dcv);
            const float2 th = fm2(a1, dcu, mul2(b1, dcv));
            // L1 shrinkage, per lane (pdflow_cudalib.cu:906-923)
            {
                if (of.x < -th.x) { du.x = add(du.x, a1.x); dv.x = add(dv.x, b1.x); }
                else if (of.x > th.x) { du.x = sub(du.x, a1.x); dv.x = sub(dv.x, b1.x); }
                else {
                    const float den = add(th.x, 1e-10f);
                    du.x = sub(du.x, qt(mul(a1.x, of.x), den));
                    dv.x = sub(dv.x, qt(mul(b1.x, of.x), den));
                }
                if (of.y < -th.y) { du.y = add(du.y, a1.y); dv.y = add(dv.y, b1.y); }
                else if (of.y > th.y) { du.y = sub(du.y, a1.y); dv.y = sub(dv.y, b1.y); }
                else {
                    const float den = add(th.y, 1e-10f);
                    du.y = sub(du.y, qt(mul(a1.y, of.y), den));
                    dv.y = sub(dv.y, qt(mul(b1.y, of.y), den));
                }
            }
            const float2 nua = fm2(two, du, neg2(du_old)), nva = fm2(two, dv, neg2(dv_old));
            const float2 nwa = fm2(two, dw, neg2(dw_old));
            if (last_iter) {
                const size_t gi = (size_t)(rv0 + rv) + (size_t)(ru0 + ru) * R;
                const float2 dup = ld2(P[T_DUP] + q), dvp = ld2(P[T_DVP] + q);
                saturate(du.x, dv.x, dw.x, dup.x, dvp.x, __ldg(depth_old + gi));
                if (f & F_V1) saturate(du.y, dv.y, dw.y, dup.y, dvp.y, __ldg(depth_old + gi + 1));
            }
            st2(P[T_DU] + q, du);
            st2(P[T_DV] + q, dv);
            st2(P[T_DW] + q, dw);
            st2(P[T_UA] + q, nua);
            st2(P[T_VA] + q, nva);
            st2(P[T_WA] + q, nwa);
        }
        __syncthreads();
    }

    // ---- write the interior ----
    if (a.bulk_store) {
        // one bulk store per (state plane, interior column)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        const int IU = iu1 - iu0, IV = iv1 - iv0;
        for (int c = threadIdx.x; c < 13 * IU; c += blockDim.x) {
            const int k = c / IU, ru = iu0 - ru0 + c % IU;
            float* g = s_gd[k] + (size_t)iv0 + (size_t)(ru0 + ru) * R;
            asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(g),
                         "r"(smem_addr(sm + k * kPlane + (iv0 - rv0) + ru * kRV)), "r"((uint32_t)IV * 4u)
                         : "memory");
        }
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        return;
    }
    float* gd[13] = {dst.du, dst.dv, dst.dw, dst.dua, dst.dva, dst.dwa, dst.pd, dst.puu, dst.puv, dst.pvu, dst.pvv,
                     dst.pwu, dst.pwv};
    const int v0 = rv0 + rv;
    const bool in0 = v0 >= iv0 && v0 < iv1 && rv < RV, in1 = v0 + 1 >= iv0 && v0 + 1 < iv1 && rv + 1 < RV;
#pragma unroll
    for (int c = 0; c < kCols; ++c) {
        const int ru = ty + kTY * c, u = ru0 + ru;
        if (ru >= RU || u < iu0 || u >= iu1 || !(in0 || in1)) continue;
        const int q = rv + ru * kRV;
        const size_t gi = (size_t)v0 + (size_t)u * R;
        if (even_rows && in0 && in1) {
#pragma unroll
            for (int k = 0; k < 13; ++k) st2(gd[k] + gi, ld2(P[k] + q));
        } else {
#pragma unroll
            for (int k = 0; k < 13; ++k) {
                if (in0) gd[k][gi] = P[k][q];
                if (in1) gd[k][gi + 1] = P[k][q + 1];
            }
        }
    }
}

}  // namespace

template <int TV, int TU>
static cudaError_t prepare_shape()
{
    cudaError_t e = cudaFuncSetAttribute(k_iterate_tiles2<TV, TU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(float) * T_NPLANES * Shape<TV, TU>::kPlane));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_iterate_tiles2<TV, TU>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    return e;
}

cudaError_t prepare_tiles2()
{
    cudaError_t e = prepare_shape<40, 40>();
    if (e == cudaSuccess) e = prepare_shape<40, 34>();
    if (e == cudaSuccess) e = prepare_shape<24, 24>();
    if (e == cudaSuccess) e = prepare_shape<24, 28>();
    return e;
}

// cuTensorMapEncodeTiled through the runtime's driver entry-point query, so
// that the library does not link the driver library itself (it then loads,
// for symbol checks, on machines without a GPU driver); null: not available.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled()
{
    static const EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

template <int TV, int TU>
static cudaError_t launch_shape(Tile2Args a, const LevelGeom& g, cudaStream_t st, bool want_tensor)
{
    using S = Shape<TV, TU>;
    Tile2Maps maps{};   // a launch parameter: copied at launch (and into a graph node when captured)
    a.tensor = false;
    const EncodeTiledFn encode = want_tensor ? encode_tiled() : nullptr;
    if (encode) {
        // 3D maps (rows, columns, arena slots) of the 24 region planes, box = the whole region
        const float* tp[T_NPLANES] = {a.src.du,  a.src.dv,  a.src.dw,  a.src.dua, a.src.dva, a.src.dwa,
                                      a.src.pd,  a.src.puu, a.src.puv, a.src.pvu, a.src.pvv, a.src.pwu,
                                      a.src.pwv, a.L.mu,    a.L.ddt,   a.L.ddu,   a.L.ddv,   a.L.dct,
                                      a.L.dcu,   a.L.dcv,   a.L.ri,    a.L.rj,    a.L.du_prev, a.L.dv_prev};
        const cuuint64_t dims[3] = {g.R, g.C, g.slots};
        const cuuint64_t strides[2] = {cuuint64_t(g.R) * 4u, g.pstride};
        const cuuint32_t box[3] = {S::kRV, S::kRU, 1}, estr[3] = {1, 1, 1};
        bool enc = true;
        for (int k = 0; k < T_NPLANES && enc; ++k)
            enc = encode(&maps.m[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(tp[k]), dims, strides,
                         box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        a.tensor = enc;   // else the per-column bulk copies
    }
    a.tiles_v = (g.R + TV - 1) / TV;
    dim3 grid(a.tiles_v * ((g.C + TU - 1) / TU), g.pairs);
    k_iterate_tiles2<TV, TU><<<grid, S::kThreads, sizeof(float) * T_NPLANES * S::kPlane, st>>>(a, maps);
    return cudaGetLastError();
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Which region copies use TMA bulk copies, per shape: bit 0 = load, bit 1 =
// store, bit 2 (with bit 0) = the load as one tensor copy per plane
// instead of one bulk copy per plane column; index 0 = 40x40 tiles,
// 1 = 40x34 tiles, 2 = 24x24, 3 = 24x28.  Measured
// on 64 VGA pairs (whole batched solves, one GB300): bulk loads make the
// 24x24 shape 9.4 % faster (73.6 -> 66.7 ms), the 40x34 shape 6 % faster
// (77.3 -> 72.5 ms) and the 40x40 shape 10 % faster per iteration; bulk
// stores gain nothing on top; tensor loads make every shape another 8-10 %
// faster than its bulk loads (24x24: 66.42 -> 61.25 ms, 40x40: 68.7 ->
// 63.7 ms, 40x34: 71.0 -> 65.7 ms, 24x28: 68.4 -> 62.3 ms).
static std::atomic<int> g_copy_mode[4] = {{5}, {5}, {5}, {5}};   // set by a debug call, read by launchers

void set_tile_copy_mode(int shape, int mode)
{
    if (shape >= 0 && shape < 4) g_copy_mode[shape] = mode & 7;
}

cudaError_t launch_iterate_tiles2(LevelGeom g, LevelConsts L, State src, State dst, Params p, const float* depth_old,
                                  unsigned kk, bool last, cudaStream_t st, int shape, unsigned* status)
{
    Tile2Args a;
    a.g = g;
    a.L = L;
    a.src = src;
    a.dst = dst;
    a.p = p;
    a.depth_old = depth_old;
    a.kk = kk;
    a.last = last;
    a.tiles_v = 0;   // set per shape
    // bulk copies need every region column start, the region height and the
    // interior height to be multiples of 16 bytes: rows % 4 == 0 (tile and
    // halo sizes are multiples of 4) and 16-byte aligned planes and pair stride
    const void* planes[] = {src.du, src.dv, src.dw, src.dua, src.dva, src.dwa, src.pd, src.puu, src.puv, src.pvu,
                            src.pvv, src.pwu, src.pwv, dst.du, dst.dv, dst.dw, dst.dua, dst.dva, dst.dwa, dst.pd,
                            dst.puu, dst.puv, dst.pvu, dst.pvv, dst.pwu, dst.pwv, L.mu, L.ddt, L.ddu, L.ddv,
                            L.dct, L.dcu, L.dcv, L.ri, L.rj, L.du_prev, L.dv_prev};
    bool ok = (g.R % 4u) == 0 && (g.pstride % 16u) == 0 && status != nullptr;
    for (const void* q : planes) ok = ok && aligned16(q);
    const int mode = g_copy_mode[shape];
    a.bulk = ok && (mode & 1);
    a.bulk_store = ok && (mode & 2);
    a.status = status;
    // tensor copies: one per plane, the region as one box; its first row
    // (a multiple of 4) and the row stride (R % 4 == 0) are 16-byte aligned,
    // and every shape's plane size in shared memory is a multiple of 128 bytes
    const bool want_tensor = a.bulk && (mode & 4) && g.slots > 0;
    switch (shape) {
    case 0: return launch_shape<40, 40>(a, g, st, want_tensor);
    case 1: return launch_shape<40, 34>(a, g, st, want_tensor);
    case 2: return launch_shape<24, 24>(a, g, st, want_tensor);
    case 3: return launch_shape<24, 28>(a, g, st, want_tensor);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pdflow
