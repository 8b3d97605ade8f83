// Temporally blocked primal-dual iterations with the state in registers
// ("quad tiles", iteration form 7).
//
// A CTA of 256 threads owns a 32 x 32 region of the level (a 24 x 24 interior
// plus a 4-pixel halo, the same tiling as pdflow_tiles2.cu) for kk <= 4
// iterations.  Thread t owns the four vertically adjacent pixels (a quad) at
// region rows 4q .. 4q+3 of region column c (q = t % 8, c = t / 8); a warp is
// four region columns of eight quads.  The quad's 13 state values live in
// registers for the whole launch (loaded with 16-byte global loads, stored the
// same way), and every per-pixel operation runs on the quad's two row pairs as
// packed FP32x2 instructions (each lane rounds as the scalar __f*_rn
// operation).  Neighbours:
//   - within the quad: registers;
//   - the row below the quad (dual step) and the row above (primal step):
//     warp shuffles inside the column's eight lanes;
//   - the column to the right (dual step) and to the left (primal step): each
//     thread publishes the values its neighbours read (U = du_acc + du_prev,
//     V = dv_acc + dv_prev, W = dw_acc for the dual; ri * the u-component of
//     each TV dual for the primal) in shared memory, one 16-byte store per
//     value, and reads its neighbour's with one 16-byte load.
// A neighbour's published value is the same rounded expression the reference
// evaluates at that pixel (computeGradient and computeDivergence,
// pdflow_cudalib.cu:935-1013), so the results are bit-identical to the other
// iteration forms.  The 19 level constants (11 set-up planes plus the 8 step
// products the warping kernel stores for this form), which the arena keeps
// back to back, arrive in shared memory by one 4D TMA tensor copy
// (pdflow_tmap.h).
//
// Every pixel of the region is updated in every iteration; after j
// iterations the ring of width j at a non-border region edge holds values
// computed from stale neighbours, which no exact pixel reads, and only the
// interior is stored.  Needs rows % 4 == 0 (quads never straddle the image's
// last row, and every quad starts on a 16-byte boundary).
#include <cuda.h>

#include <atomic>

#include "pdflow_iterate.cuh"
#include "pdflow_math.cuh"
#include "pdflow_tmap.h"

namespace pdflow {

namespace {

constexpr int kQH = 4;                         // halo (iterations per launch at most)
constexpr int kQT = 24;                        // interior rows and columns
constexpr int kQR = kQT + 2 * kQH;             // region rows and columns (32)
constexpr int kQPlane = kQR * kQR;             // floats per shared plane
constexpr int kQThreads = kQR * kQR / 4;       // one thread per quad (256)

// shared planes: the 19 constants (one tensor copy; the arena's order), then
// the six exchange planes
enum { C_RI, C_RJ, C_DCT, C_DCU, C_DCV, C_DDT, C_DDU, C_DDV, C_MU, C_DUP, C_DVP,
       C_S0, C_S1, C_S2, C_S3, C_S4, C_TU, C_TV, C_TW,
       C_NCONST,
       X_U = C_NCONST, X_V, X_W, Y_U, Y_V, Y_W, Q_NPLANES };

struct QuadArgs {
    LevelGeom g;
    const float* src[13];      // du dv dw du_acc dv_acc dw_acc pd puu puv pvu pvv pwu pwv (read)
    float* dst[13];            // the same planes of the other buffer (written: interior only)
    const float* depth_old;
    Params p;
    unsigned kk;
    bool last;
    unsigned tiles_v;
    unsigned tiles;            // tiles per pair
    unsigned ahead;            // L2 prefetch of the region of the CTA `ahead` launch slots later (0: none)
    unsigned* status;          // device word: kQuadTimeout when the bounded wait for the region gives up
};

// 4D tensor maps: the 19 constant planes (region loads) and the 13 source
// state planes (L2 prefetches only; the state is loaded with 16-byte loads).
struct QuadMaps {
    CUtensorMap consts, state;
};

constexpr unsigned kQuadTimeout = 0x51554144u;
constexpr unsigned kQuadWaitLimit = 1u << 20;

__device__ __forceinline__ uint32_t sm_addr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

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

// A quad: rows 0,1 in lo, rows 2,3 in hi.
struct Q {
    float2 lo, hi;
};
__device__ __forceinline__ Q lds(const float* p)
{
    const float4 v = *reinterpret_cast<const float4*>(p);
    return Q{make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
__device__ __forceinline__ void sts(float* p, const Q& q)
{
    *reinterpret_cast<float4*>(p) = make_float4(q.lo.x, q.lo.y, q.hi.x, q.hi.y);
}
__device__ __forceinline__ Q ldg_q(const float* p)
{
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    return Q{make_float2(v.x, v.y), make_float2(v.z, v.w)};
}
__device__ __forceinline__ void stg_q(float* p, const Q& q)
{
    *reinterpret_cast<float4*>(p) = make_float4(q.lo.x, q.lo.y, q.hi.x, q.hi.y);
}
__device__ __forceinline__ Q qadd(const Q& a, const Q& b) { return Q{add2(a.lo, b.lo), add2(a.hi, b.hi)}; }
__device__ __forceinline__ Q qsub(const Q& a, const Q& b) { return Q{sub2(a.lo, b.lo), sub2(a.hi, b.hi)}; }
__device__ __forceinline__ Q qmul(const Q& a, const Q& b) { return Q{mul2(a.lo, b.lo), mul2(a.hi, b.hi)}; }
__device__ __forceinline__ Q qfm(const Q& a, const Q& b, const Q& c) { return Q{fm2(a.lo, b.lo, c.lo), fm2(a.hi, b.hi, c.hi)}; }
__device__ __forceinline__ Q qneg(const Q& a) { return Q{neg2(a.lo), neg2(a.hi)}; }

// The quad shifted down by one row: rows (-1, 0, 1, 2) with `above` as row -1.
__device__ __forceinline__ Q shift_down(const Q& a, float above)
{
    return Q{make_float2(above, a.lo.x), make_float2(a.lo.y, a.hi.x)};
}
// The quad shifted up by one row: rows (1, 2, 3, 4) with `below` as row 4.
__device__ __forceinline__ Q shift_up(const Q& a, float below)
{
    return Q{make_float2(a.lo.y, a.hi.x), make_float2(a.hi.y, below)};
}

__device__ __forceinline__ float clamp1(float pd) { return (fabsf(pd) > 1.f) ? ((pd > 1.f) ? 1.f : -1.f) : pd; }

// Projection onto the unit disc (updateDualVariables, pdflow_cudalib.cu:813-887).
// Branch-free: outside the projection the factor is 1 and x * 1 == x exactly,
// so the bits are those of the reference's conditional update.
__device__ __forceinline__ void disc(float& a, float& b)
{
    const float m = rhypotf(a, b);
    const float f = (m < 1.f) ? m : 1.f;
    a = mul(a, f);
    b = mul(b, f);
}

__global__ void __launch_bounds__(kQThreads, 2) k_iterate_quads(QuadArgs a, const __grid_constant__ QuadMaps tm)
{
    extern __shared__ __align__(128) float sm[];   // TMA tensor copies land on 128-byte boundaries
    __shared__ __align__(8) unsigned long long bar[1];
    const unsigned y = blockIdx.y;
    const size_t po = pair_off(a.g.map, a.g.pstride, y);
    const int R = (int)a.g.R, C = (int)a.g.C;
    const int tv = (int)(blockIdx.x % a.tiles_v), tu = (int)(blockIdx.x / a.tiles_v);
    const int iv0 = tv * kQT, iu0 = tu * kQT;
    const int iv1 = min(iv0 + kQT, R), iu1 = min(iu0 + kQT, C);
    const int rv0 = max(iv0 - kQH, 0), ru0 = max(iu0 - kQH, 0);
    const int t = threadIdx.x;
    const int c = t >> 3, q = t & 7;                // region column, quad
    const int u = ru0 + c, v0 = rv0 + 4 * q;        // the quad's image column and first row
    const bool live = u < C && v0 < R;              // v0 < R implies v0 + 3 < R (R % 4 == 0)

    // ---- region load: constants by one TMA tensor copy, state by 16-byte loads ----
    const uint32_t b0 = sm_addr(&bar[0]);
    constexpr uint32_t kBox = (uint32_t)kQPlane * 4u;
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b0));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b0),
                     "r"((uint32_t)C_NCONST * kBox)
                     : "memory");
        // box (32 rows, 32 columns, 19 planes, 1 slot) at (rv0, ru0, 0, slot): rv0
        // is a multiple of 4 floats (16 bytes); rows and columns past the level
        // arrive as zeros
        const int slot = (int)(a.g.map ? (__ldg(a.g.map + y) & kMapSlotMask) : y);
        asm volatile(
            "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(sm_addr(sm)),
            "l"(reinterpret_cast<uint64_t>(&tm.consts)), "r"(rv0), "r"(ru0), "r"(0), "r"(slot), "r"(b0)
            : "memory");
    }
    if (t == 32 && a.ahead) {
        // Warm L2 with the region of the CTA that takes over this launch slot:
        // CTAs start in launch order, so the one `ahead` positions later starts
        // about when this one finishes.  One tensor prefetch per plane group.
        const unsigned n = blockIdx.x + a.tiles * y + a.ahead;
        if (n < a.tiles * gridDim.y) {
            const unsigned ny = n / a.tiles, nx = n % a.tiles;
            const int ntv = (int)(nx % a.tiles_v), ntu = (int)(nx / a.tiles_v);
            const int nrv0 = max(ntv * kQT - kQH, 0), nru0 = max(ntu * kQT - kQH, 0);
            const int nslot = (int)(a.g.map ? (__ldg(a.g.map + ny) & kMapSlotMask) : ny);
            asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(
                             reinterpret_cast<uint64_t>(&tm.consts)),
                         "r"(nrv0), "r"(nru0), "r"(0), "r"(nslot)
                         : "memory");
            asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(
                             reinterpret_cast<uint64_t>(&tm.state)),
                         "r"(nrv0), "r"(nru0), "r"(0), "r"(nslot)
                         : "memory");
        }
    }
    Q du{}, dv{}, dw{}, ua{}, va{}, wa{}, pd{}, puu{}, puv{}, pvu{}, pvv{}, pwu{}, pwv{};
    const size_t gi = (size_t)v0 + (size_t)u * (size_t)R;   // the quad's first pixel
    if (live) {
        Q* st[13] = {&du, &dv, &dw, &ua, &va, &wa, &pd, &puu, &puv, &pvu, &pvv, &pwu, &pwv};
#pragma unroll
        for (int k = 0; k < 13; ++k) *st[k] = ldg_q(at(a.src[k], po) + gi);
    }
    // the barrier makes thread 0's mbarrier initialisation visible before anyone waits on it
    __syncthreads();
    auto wait_group = [&](uint32_t b) {
        bool done = false;
        for (uint32_t i = 0; i < kQuadWaitLimit && !done; ++i) {
            uint32_t ok;
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(ok)
                : "r"(b)
                : "memory");
            done = ok != 0;
        }
        if (!done && a.status) atomicExch(a.status, kQuadTimeout);
    };

    // ---- per-thread geometry ----
    const bool fu = (u == 0), lu = (u == C - 1);
    const bool fv = (v0 == 0), lv = (v0 + 3 == R - 1);   // row 0 of the quad is v = 0 / row 3 is v = R - 1
    const int me = c * kQR + 4 * q;                       // the quad's offset in a shared plane
    const int right = (c + 1 < kQR ? c + 1 : c) * kQR + 4 * q;   // beyond the region: own storage
    const int left = (c > 0 ? c - 1 : c) * kQR + 4 * q;
    const float li = a.p.lambda_i, ld = a.p.lambda_d;
    const float2 li2 = make_float2(li, li), ld2 = make_float2(ld, ld), two = make_float2(2.f, 2.f);
    const Q zero{};
    const bool last_launch = a.last || (pair_flags(a.g.map, y) & kMapLast);
    const float* P = sm;
    float* XU = sm + X_U * kQPlane;
    float* XV = sm + X_V * kQPlane;
    float* XW = sm + X_W * kQPlane;
    float* YU = sm + Y_U * kQPlane;
    float* YV = sm + Y_V * kQPlane;
    float* YW = sm + Y_W * kQPlane;
    const unsigned lane = t & 31u;

    wait_group(b0);
    for (unsigned j = 0; j < a.kk; ++j) {
        // ---------------- dual step (computeGradient + updateDualVariables) ----------------
        {
            const Q U = qadd(ua, lds(P + C_DUP * kQPlane + me));
            const Q V = qadd(va, lds(P + C_DVP * kQPlane + me));
            sts(XU + me, U);
            sts(XV + me, V);
            sts(XW + me, wa);
            // row 4 (the first row of the quad below, same column)
            const float Ub = __shfl_down_sync(0xffffffffu, U.lo.x, 1, 8);
            const float Vb = __shfl_down_sync(0xffffffffu, V.lo.x, 1, 8);
            const float Wb = __shfl_down_sync(0xffffffffu, wa.lo.x, 1, 8);
            __syncthreads();
            const Q ri = lds(P + C_RI * kQPlane + me), rj = lds(P + C_RJ * kQPlane + me);
            // borders by selects, not branches (the neighbour slot at the region's
            // right edge is the thread's own: read, then dropped)
            Q gu1 = qmul(ri, qsub(lds(XU + right), U));
            Q gv1 = qmul(ri, qsub(lds(XV + right), V));
            Q gw1 = qmul(ri, qsub(lds(XW + right), wa));
            if (lu) {
                gu1 = zero;
                gv1 = zero;
                gw1 = zero;
            }
            Q gu2 = qmul(rj, qsub(shift_up(U, Ub), U));
            Q gv2 = qmul(rj, qsub(shift_up(V, Vb), V));
            Q gw2 = qmul(rj, qsub(shift_up(wa, Wb), wa));
            if (lv) {
                gu2.hi.y = 0.f;
                gv2.hi.y = 0.f;
                gw2.hi.y = 0.f;
            }
            const Q X = qfm(lds(P + C_DDV * kQPlane + me), va,
                            qfm(lds(P + C_DDU * kQPlane + me), ua, qsub(lds(P + C_DDT * kQPlane + me), wa)));
            const Q s1 = lds(P + C_S1 * kQPlane + me), s2 = lds(P + C_S2 * kQPlane + me);
            pd = qfm(lds(P + C_S0 * kQPlane + me), X, pd);
            puu = qfm(s1, gu1, puu);
            puv = qfm(s2, gu2, puv);
            pvu = qfm(s1, gv1, pvu);
            pvv = qfm(s2, gv2, pvv);
            pwu = qfm(lds(P + C_S3 * kQPlane + me), gw1, pwu);
            pwv = qfm(lds(P + C_S4 * kQPlane + me), gw2, pwv);
            pd.lo.x = clamp1(pd.lo.x);
            pd.lo.y = clamp1(pd.lo.y);
            pd.hi.x = clamp1(pd.hi.x);
            pd.hi.y = clamp1(pd.hi.y);
            disc(puu.lo.x, puv.lo.x);
            disc(puu.lo.y, puv.lo.y);
            disc(puu.hi.x, puv.hi.x);
            disc(puu.hi.y, puv.hi.y);
            disc(pvu.lo.x, pvv.lo.x);
            disc(pvu.lo.y, pvv.lo.y);
            disc(pvu.hi.x, pvv.hi.x);
            disc(pvu.hi.y, pvv.hi.y);
            disc(pwu.lo.x, pwv.lo.x);
            disc(pwu.lo.y, pwv.lo.y);
            disc(pwu.hi.x, pwv.hi.x);
            disc(pwu.hi.y, pwv.hi.y);
        }
        // ---------------- primal step (computeDivergence + updatePrimalVariables) ----------------
        {
            const Q ri = lds(P + C_RI * kQPlane + me), rj = lds(P + C_RJ * kQPlane + me);
            // products the neighbours read: ri * p_u to the right, rj * p_v to the row below
            const Q yu = qmul(ri, puu), yv = qmul(ri, pvu), yw = qmul(ri, pwu);
            sts(YU + me, yu);
            sts(YV + me, yv);
            sts(YW + me, yw);
            const Q zu = qmul(rj, puv), zv = qmul(rj, pvv), zw = qmul(rj, pwv);
            const float zua = __shfl_up_sync(0xffffffffu, zu.hi.y, 1, 8);   // row -1 (the quad above)
            const float zva = __shfl_up_sync(0xffffffffu, zv.hi.y, 1, 8);
            const float zwa = __shfl_up_sync(0xffffffffu, zw.hi.y, 1, 8);
            __syncthreads();
            const Q pu_[3] = {puu, pvu, pwu}, pv_[3] = {puv, pvv, pwv};
            const Q z_[3] = {shift_down(zu, zua), shift_down(zv, zva), shift_down(zw, zwa)};
            const float* Yp[3] = {YU, YV, YW};
            Q div[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const Q ym = qneg(lds(Yp[k] + left));
                const Q dm = qfm(ri, pu_[k], ym), df = qmul(ri, pu_[k]);
                const Q d = fu ? df : (lu ? ym : dm);   // first / last / inner column
                Q g = qadd(d, qfm(rj, pv_[k], qneg(z_[k])));
                if (fv) g.lo.x = fm(rj.lo.x, pv_[k].lo.x, d.lo.x);
                if (lv) g.hi.y = fm(-rj.hi.x, pv_[k].hi.x, d.hi.y);
                div[k] = g;
            }
            const Q mu = lds(P + C_MU * kQPlane + me);
            const Q ddu = lds(P + C_DDU * kQPlane + me), ddv = lds(P + C_DDV * kQPlane + me);
            const Q tu_ = lds(P + C_TU * kQPlane + me), tv_ = lds(P + C_TV * kQPlane + me);
            const Q tw_ = lds(P + C_TW * kQPlane + me);
            const Q du_old = du, dv_old = dv, dw_old = dw;
            du = qfm(qneg(tu_), qfm(qmul(mu, ddu), pd, qneg(Q{mul2(li2, div[0].lo), mul2(li2, div[0].hi)})), du);
            dv = qfm(qneg(tv_), qfm(qmul(mu, ddv), pd, qneg(Q{mul2(li2, div[1].lo), mul2(li2, div[1].hi)})), dv);
            {
                // per lane: a packed product whose only use is a packed sum may be
                // contracted into one fused multiply-add, which would change the
                // rounding of add(dw, mul(-tw, .)); the scalar intrinsics never are
                const Q tq = qfm(qneg(mu), pd, qneg(Q{mul2(ld2, div[2].lo), mul2(ld2, div[2].hi)}));
                dw.lo.x = add(dw.lo.x, mul(-tw_.lo.x, tq.lo.x));
                dw.lo.y = add(dw.lo.y, mul(-tw_.lo.y, tq.lo.y));
                dw.hi.x = add(dw.hi.x, mul(-tw_.hi.x, tq.hi.x));
                dw.hi.y = add(dw.hi.y, mul(-tw_.hi.y, tq.hi.y));
            }
            const Q dcu = lds(P + C_DCU * kQPlane + me), dcv = lds(P + C_DCV * kQPlane + me);
            const Q of = qfm(dcv, dv, qfm(dcu, du, lds(P + C_DCT * kQPlane + me)));
            const Q a1 = qmul(tu_, dcu), b1 = qmul(tv_, dcv);
            const Q th = qfm(a1, dcu, qmul(b1, dcv));
            shrink(du.lo.x, dv.lo.x, of.lo.x, th.lo.x, a1.lo.x, b1.lo.x);
            shrink(du.lo.y, dv.lo.y, of.lo.y, th.lo.y, a1.lo.y, b1.lo.y);
            shrink(du.hi.x, dv.hi.x, of.hi.x, th.hi.x, a1.hi.x, b1.hi.x);
            shrink(du.hi.y, dv.hi.y, of.hi.y, th.hi.y, a1.hi.y, b1.hi.y);
            ua = Q{fm2(two, du.lo, neg2(du_old.lo)), fm2(two, du.hi, neg2(du_old.hi))};
            va = Q{fm2(two, dv.lo, neg2(dv_old.lo)), fm2(two, dv.hi, neg2(dv_old.hi))};
            wa = Q{fm2(two, dw.lo, neg2(dw_old.lo)), fm2(two, dw.hi, neg2(dw_old.hi))};
            if (last_launch && j + 1 == a.kk && live) {
                // saturateVariables (pdflow_cudalib.cu:1018-1038) after the level's last iteration
                const Q dup = lds(P + C_DUP * kQPlane + me), dvp = lds(P + C_DVP * kQPlane + me);
                const Q z = ldg_q(at(a.depth_old, po) + gi);
                saturate(du.lo.x, dv.lo.x, dw.lo.x, dup.lo.x, dvp.lo.x, z.lo.x);
                saturate(du.lo.y, dv.lo.y, dw.lo.y, dup.lo.y, dvp.lo.y, z.lo.y);
                saturate(du.hi.x, dv.hi.x, dw.hi.x, dup.hi.x, dvp.hi.x, z.hi.x);
                saturate(du.hi.y, dv.hi.y, dw.hi.y, dup.hi.y, dvp.hi.y, z.hi.y);
            }
        }
        // no barrier here: this iteration's exchange reads all happen before the
        // next one's first barrier, and the next stores to the same planes after it
        // (X planes: written before the dual's barrier, read after it; Y planes the same
        // around the primal's barrier)
    }

    // ---- write the interior ----
    if (live && v0 >= iv0 && v0 < iv1 && u >= iu0 && u < iu1) {
        const Q* st[13] = {&du, &dv, &dw, &ua, &va, &wa, &pd, &puu, &puv, &pvu, &pvv, &pwu, &pwv};
#pragma unroll
        for (int k = 0; k < 13; ++k) stg_q(at(a.dst[k], po) + gi, *st[k]);
    }
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

std::atomic<unsigned> g_quad_ahead{0};   // CTAs ahead for the L2 prefetch (0: off)

}  // namespace

void set_quad_prefetch(unsigned ctas_ahead) { g_quad_ahead = ctas_ahead; }

size_t quads_smem_bytes() { return sizeof(float) * Q_NPLANES * kQPlane; }

cudaError_t prepare_quads()
{
    cudaError_t e = cudaFuncSetAttribute(k_iterate_quads, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)quads_smem_bytes());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_iterate_quads, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    return e;
}

// The constant planes of the register-resident tiles, in their arena (and
// shared-memory) order, and the state planes in State order.
static void const_group(const LevelConsts& L, const float* out[19])
{
    const float* c[19] = {L.ri, L.rj, L.dct, L.dcu, L.dcv, L.ddt, L.ddu, L.ddv, L.mu, L.du_prev, L.dv_prev,
                          L.qs[0], L.qs[1], L.qs[2], L.qs[3], L.qs[4], L.qs[5], L.qs[6], L.qs[7]};
    for (int k = 0; k < 19; ++k) out[k] = c[k];
}
static void state_group(const State& S, const float* out[13])
{
    const float* c[13] = {S.du, S.dv, S.dw, S.dua, S.dva, S.dwa, S.pd, S.puu, S.puv, S.pvu, S.pvv, S.pwu, S.pwv};
    for (int k = 0; k < 13; ++k) out[k] = c[k];
}

bool quads_eligible(const LevelGeom& g, const LevelConsts& L, const State& src, const State& dst)
{
    if (g.R % 4u != 0 || g.pstride % 16u != 0 || g.slots == 0 || !tensor_map_encoder()) return false;
    // the constants and both state buffers are runs of planes at one stride
    const float* cg[19];
    const float* sg[13];
    const float* dg[13];
    const_group(L, cg);
    state_group(src, sg);
    state_group(dst, dg);
    size_t a = 0, b = 0, c = 0;
    if (!equally_spaced(cg, 19, &a) || !equally_spaced(sg, 13, &b) || !equally_spaced(dg, 13, &c)) return false;
    return aligned16(cg[0]) && aligned16(sg[0]) && aligned16(dg[0]);
}

cudaError_t launch_iterate_quads(LevelGeom g, LevelConsts L, State src, State dst, Params p, const float* depth_old,
                                 unsigned kk, bool last, cudaStream_t st, unsigned* status)
{
    if (kk > (unsigned)kQH || !quads_eligible(g, L, src, dst) || !status || !aligned16(depth_old))
        return cudaErrorInvalidValue;
    QuadArgs a;
    a.g = g;
    const float* s13[13] = {src.du, src.dv, src.dw, src.dua, src.dva, src.dwa, src.pd,
                            src.puu, src.puv, src.pvu, src.pvv, src.pwu, src.pwv};
    float* d13[13] = {dst.du, dst.dv, dst.dw, dst.dua, dst.dva, dst.dwa, dst.pd,
                      dst.puu, dst.puv, dst.pvu, dst.pvv, dst.pwu, dst.pwv};
    for (int k = 0; k < 13; ++k) {
        a.src[k] = s13[k];
        a.dst[k] = d13[k];
    }
    a.depth_old = depth_old;
    a.p = p;
    a.kk = kk;
    a.last = last;
    a.status = status;
    a.tiles_v = (g.R + kQT - 1) / kQT;
    a.tiles = a.tiles_v * ((g.C + kQT - 1) / kQT);
    a.ahead = g_quad_ahead.load();
    // 4D maps (rows, columns, planes, arena slots): the 19 constant planes and the
    // 13 source state planes, box = the whole region of every plane of the group
    QuadMaps maps{};
    const float* cg[19];
    const float* sg[13];
    const_group(L, cg);
    state_group(src, sg);
    size_t cs = 0, ss = 0;
    equally_spaced(cg, 19, &cs);
    equally_spaced(sg, 13, &ss);
    if (!encode_plane_group(&maps.consts, cg[0], 19, cs, g.R, g.C, g.slots, g.pstride, kQR, kQR) ||
        !encode_plane_group(&maps.state, sg[0], 13, ss, g.R, g.C, g.slots, g.pstride, kQR, kQR))
        return cudaErrorInvalidValue;
    dim3 grid(a.tiles, g.pairs);
    k_iterate_quads<<<grid, kQThreads, quads_smem_bytes(), st>>>(a, maps);
    return cudaGetLastError();
}

}  // namespace pdflow
