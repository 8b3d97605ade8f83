// Persistent, register-resident tile iterations ("streamed tiles", iteration
// forms 8 and 9; the strips of form 10 below).
//
// One CTA per SM walks a list of tiles (every 24 x 24 interior of every pair
// of the launch, 4-pixel halo: 32 x 32 regions, as in pdflow_tiles2.cu).  A
// tile's 13 state planes and 19 level constants (11 set-up planes and the 8
// step products) live in registers while its kk <= 4 iterations run: each of
// the 512 threads owns a vertical pixel pair (rows 2p, 2p+1 of region column
// c) and computes it with packed FP32x2 instructions.  Meanwhile the TMA unit
// copies the next tile's 32 planes into a shared-memory staging buffer (two 4D
// tensor copies, one per run of planes the arena keeps back to back: the 13
// state planes and the 19 constants, pdflow_tmap.h; completing on an
// mbarrier), so the region loads run behind the arithmetic.
//
// Neighbours: the row below the pair (dual step) and above it (primal step)
// by warp shuffles inside the column's 16 lanes; the column to the right
// (dual) and to the left (primal) through six shared exchange planes, into
// which each thread publishes what its neighbours read (U = du_acc + du_prev,
// V = dv_acc + dv_prev, W = dw_acc; ri * the u-component of each TV dual).
// These are the same rounded expressions the reference evaluates
// (computeGradient, computeDivergence: pdflow_cudalib.cu:935-1013), so the
// results are bit-identical to every other iteration form.  Every pixel of
// the region is updated in every iteration; the stale ring at non-border
// region edges is never read by an exact pixel and only the interior is
// stored.  Needs rows % 4 == 0 (16-byte aligned tensor-copy rows); levels
// with an even row count otherwise (a VGA solve's 30x40) run the tiles with
// each thread loading its pixel pair's 32 values directly (8-byte loads, no
// staging: such levels have about one region per CTA, nothing to stream).
//
// Strips (iteration form 10).  Of an iteration's column neighbours only the
// primal step's backward difference looks left (ri * the dual's u-component
// at column u - 1), and only the dual step's forward difference looks right.
// A CTA that walks a row of regions left to right can therefore hand the
// next region the left neighbour's exchange values of every iteration (a
// carry of 3 x 32 floats per iteration, in shared memory) instead of
// recomputing a left halo: after kk iterations columns [x, x + 32 - kk) of a
// region at column x are exact, 28 of 32 at kk = 4 instead of 24.  The
// units of work are whole strips (a pair's 24-row bands) and, for the last
// strips of the launch, column pieces of them, smaller towards the end (each
// starting with a region that recomputes a left halo of kk columns).  CTAs take units in order from
// a device counter as they finish the previous one: they walk vertically
// adjacent bands side by side (their row halos meet in L2 and their reads
// fill DRAM pages, as the tiles' do), and a CTA whose strips converge faster
// (the disc projection's work depends on the data) takes more of them; the
// pieces keep the last units short.  The last CTA to finish resets the
// counter for the next launch.
#include <cuda.h>

#include <algorithm>
#include <type_traits>

#include "pdflow_iterate.cuh"
#include "pdflow_math.cuh"
#include "pdflow_pack.cuh"
#include "pdflow_tmap.h"

namespace pdflow {

namespace {

using namespace pack;

constexpr int kSR = 32;                        // region rows and columns
// Interior and halo (= iterations per launch at most) are launch parameters:
// 24 + 2 x 4 (form 8) or 16 + 2 x 8 (form 9: twice the iterations per launch
// for levels whose launches are latency-bound, at four times the halo work).
constexpr int kSPlane = kSR * kSR;             // floats per shared plane
constexpr int kSThreads = kSR * kSR / 2;       // one thread per pixel pair (512)

// staging planes (TMA destinations, in the arena's order): 13 state, 19
// constants; then the six exchange planes
enum { S_DU, S_DV, S_DW, S_UA, S_VA, S_WA, S_PD, S_PUU, S_PUV, S_PVU, S_PVV, S_PWU, S_PWV,
       K_RI, K_RJ, K_DCT, K_DCU, K_DCV, K_DDT, K_DDU, K_DDV, K_MU, K_DUP, K_DVP,
       K_S0, K_S1, K_S2, K_S3, K_S4, K_TU, K_TV, K_TW,
       N_STAGE,
       X_U = N_STAGE, X_V, X_W, Y_U, Y_V, Y_W, N_PLANES };

struct StreamArgs {
    LevelGeom g;
    const float* planes[32];   // direct loads: the 13 source state and 19 constant planes, in the staging order
    unsigned whole;            // strips: units 0 .. whole-1 are strips 0 .. whole-1
    unsigned tier_n[3], tier_p[3];   // strips: then tier i: tier_p[i] pieces of each of the next tier_n[i] strips
    unsigned* work;            // strips: [next unit - grid, CTAs finished], zero between launches
    float* dst[13];            // du dv dw du_acc dv_acc dw_acc pd puu puv pvu pvv pwu pwv (interior written)
    const float* depth_old;
    Params p;
    unsigned kk;
    bool last;
    int tile, halo;            // interior rows and columns, halo width (tile + 2 halo = kSR)
    unsigned tiles_v;          // tiles per column of tiles
    unsigned tiles;            // tiles per pair
    unsigned total;            // tiles of the launch (tiles * pairs)
    unsigned* status;          // device word: kStreamTimeout when a bounded wait gives up
};

// 4D maps (rows, columns, planes, arena slots) of the 13 source state planes
// and of the 19 constant planes, box = one region of every plane of the group.
struct StreamMaps {
    CUtensorMap state, consts;
};

constexpr unsigned kStreamTimeout = 0x5354524Du;
constexpr uint32_t kStreamWaitLimit = 1u << 22;

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

// Both pixels of a pair.  Inside the disc of radius sqrt(0.999) rhypotf
// (maximum error 2 ulp) returns more than 1, the factor is 1 and the values
// stay as they are: a warp whose 64 pixels are all there skips the
// reciprocal norms (NaN and infinite inputs fail the test and take them).
__device__ __forceinline__ void disc2(float2& a, float2& b)
{
    const float2 s = fm2(a, a, mul2(b, b));
    if (__all_sync(0xffffffffu, s.x < 0.999f && s.y < 0.999f)) return;
    disc(a.x, b.x);
    disc(a.y, b.y);
}

// shrink_rcp (pdflow_math.cuh) for both pixels of a pair: the quotients'
// Markstein corrections and the three cases' values in packed FP32x2 (each
// lane the same correctly rounded operations), the case chosen per lane.
__device__ __forceinline__ float2 div_rcp2(float2 a, float2 b, float2 y)
{
    const float2 q0 = mul2(a, y);
    const float2 q1 = fm2(fm2(neg2(q0), b, a), y, q0);
    const float2 q2 = fm2(fm2(neg2(q1), b, a), y, q1);
    return make_float2(a.x == 0.f ? a.x : q2.x, a.y == 0.f ? a.y : q2.y);
}
__device__ __forceinline__ void shrink_rcp2(float2& du, float2& dv, float2 of, float2 th, float2 den, float2 rden,
                                            float2 a1, float2 b1)
{
    const float2 mu_ = sub2(du, div_rcp2(mul2(a1, of), den, rden));
    const float2 mv_ = sub2(dv, div_rcp2(mul2(b1, of), den, rden));
    const float2 pu = add2(du, a1), pv = add2(dv, b1), su = sub2(du, a1), sv = sub2(dv, b1);
    const bool lox = of.x < -th.x, hix = of.x > th.x, loy = of.y < -th.y, hiy = of.y > th.y;
    du = make_float2(lox ? pu.x : (hix ? su.x : mu_.x), loy ? pu.y : (hiy ? su.y : mu_.y));
    dv = make_float2(lox ? pv.x : (hix ? sv.x : mv_.x), loy ? pv.y : (hiy ? sv.y : mv_.y));
}

// One region of a CTA's walk: its origin, the rows and columns it stores,
// and (strips) where the walk goes next.
struct Tile {
    unsigned y;                  // grid pair index
    int rv0, ru0, iv0, iv1, iu0, iu1;
    bool more;                   // a region to process
    bool carry_in, carry_out;    // strips: reads / writes the column carry
    unsigned k;                  // strips: the unit; tiles: the tile index
    int c1;                      // strips: the unit's end column
};

// Tiles: the launch's tile n (regions of every pair, dealt round-robin).
__device__ __forceinline__ Tile tile_at(const StreamArgs& a, unsigned n)
{
    Tile t;
    t.more = n < a.total;
    t.k = n;
    t.c1 = 0;
    t.carry_in = t.carry_out = false;
    t.y = n / a.tiles;
    const unsigned x = n % a.tiles;
    const int R = (int)a.g.R, C = (int)a.g.C;
    const int tv = (int)(x % a.tiles_v), tu = (int)(x / a.tiles_v);
    t.iv0 = tv * a.tile;
    t.iu0 = tu * a.tile;
    t.iv1 = min(t.iv0 + a.tile, R);
    t.iu1 = min(t.iu0 + a.tile, C);
    t.rv0 = max(t.iv0 - a.halo, 0);
    t.ru0 = max(t.iu0 - a.halo, 0);
    return t;
}

// Strips: unit k, columns [c0, c1) of strip `strip` (strip s is row band
// s % tiles_v of pair s / tiles_v): a whole strip, or piece i of a strip of
// one of the tiers that follow (within a tier, pieces in order of i, then of
// the strip).
struct Segment {
    bool ok;
    unsigned strip;
    int c0, c1;
};
__device__ __forceinline__ Segment segment(const StreamArgs& a, unsigned k)
{
    const int C = (int)a.g.C;
    if (k < a.whole) return {true, k, 0, C};
    unsigned x = k - a.whole, base = a.whole;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const unsigned n = a.tier_n[i], m = a.tier_p[i];
        if (x < n * m) {
            const int piece = (int)(x / n);
            return {true, base + x % n, C * piece / (int)m, C * (piece + 1) / (int)m};
        }
        x -= n * m;
        base += n;
    }
    return {false, 0, 0, 0};
}

// Strips: the region of unit k whose stored columns start at `col`.  With
// the carry the region starts at that column; without it, kk columns further
// left (their values go stale from the left, one column per iteration) or at
// the image's first column.  Columns up to 32 - kk past the origin are exact
// (all of them when the region reaches the image's last column).
__device__ __forceinline__ Tile strip_at(const StreamArgs& a, unsigned k, int col, bool carry)
{
    Tile t;
    const Segment sg = segment(a, k);
    t.more = sg.ok;
    t.k = k;
    t.c1 = sg.c1;
    const int R = (int)a.g.R, C = (int)a.g.C, K = (int)a.kk;
    if (col < 0) col = sg.c0;
    t.y = sg.strip / a.tiles_v;
    const int tv = (int)(sg.strip - t.y * a.tiles_v);
    t.iv0 = tv * a.tile;
    t.iv1 = min(t.iv0 + a.tile, R);
    t.rv0 = max(t.iv0 - a.halo, 0);
    t.ru0 = carry ? col : max(col - K, 0);
    const int exact = (t.ru0 + kSR >= C) ? C : t.ru0 + kSR - K;
    t.iu0 = col;
    t.iu1 = min(exact, sg.c1);
    t.carry_in = carry;
    t.carry_out = t.iu1 == exact && t.iu1 < sg.c1;   // the next region continues the unit
    return t;
}

// The region after t: the rest of t's unit, else unit `unit` (strips); the
// CTA's next tile (tiles).
template <bool kStrips>
__device__ __forceinline__ Tile next_tile(const StreamArgs& a, const Tile& t, unsigned unit)
{
    if constexpr (kStrips)
        return t.iu1 < t.c1 ? strip_at(a, t.k, t.iu1, true) : strip_at(a, unit, -1, false);
    else
        return tile_at(a, t.k + gridDim.x);
}

// Thread 0: the tensor copies of region t into the staging planes,
// completing on `bar` (the caller's threads have finished reading staging).
__device__ __forceinline__ void issue_region(const StreamArgs& a, const StreamMaps& tm, float* sm, uint32_t bar,
                                             const Tile& t)
{
    const int slot = (int)(a.g.map ? (__ldg(a.g.map + t.y) & kMapSlotMask) : t.y);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // earlier generic reads before async writes
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"((uint32_t)N_STAGE * (uint32_t)kSPlane * 4u)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(sm + S_DU * kSPlane)),
        "l"(reinterpret_cast<uint64_t>(&tm.state)), "r"(t.rv0), "r"(t.ru0), "r"(0), "r"(slot), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(sm + K_RI * kSPlane)),
        "l"(reinterpret_cast<uint64_t>(&tm.consts)), "r"(t.rv0), "r"(t.ru0), "r"(0), "r"(slot), "r"(bar)
        : "memory");
}

// carry (strips): [buffer][iteration][u, v, w][region row] of the column
// that the next region of the strip sees on its left
constexpr int kCarryFloats = 2 * 4 * 3 * kSR;

template <bool kStrips, bool kTma = true>
__global__ void __launch_bounds__(kSThreads, 1) k_iterate_stream(StreamArgs a, const __grid_constant__ StreamMaps tm)
{
    static_assert(kTma || !kStrips, "the strips stream their regions");
    extern __shared__ __align__(128) float sm[];
    __shared__ __align__(8) unsigned long long bar_mem;
    __shared__ unsigned next_unit;   // strips: the unit thread 0 took for after the current one
    const int t = threadIdx.x;
    const int c = t >> 4, p = t & 15;              // region column, pixel pair
    const int me = c * kSR + 2 * p;                 // the pair's offset in a shared plane
    const int right = (c + 1 < kSR ? c + 1 : c) * kSR + 2 * p;   // beyond the region: own storage
    const int left = (c > 0 ? c - 1 : c) * kSR + 2 * p;
    const uint32_t bar = smem_u32(&bar_mem);
    const int R = (int)a.g.R, C = (int)a.g.C;
    const float li = a.p.lambda_i, ld = a.p.lambda_d;
    const float2 li2 = make_float2(li, li), ld2 = make_float2(ld, ld), two = make_float2(2.f, 2.f);
    const float2 zero = make_float2(0.f, 0.f);
    float* XU = sm + X_U * kSPlane;
    float* XV = sm + X_V * kSPlane;
    float* XW = sm + X_W * kSPlane;
    float* YU = sm + Y_U * kSPlane;
    float* YV = sm + Y_V * kSPlane;
    float* YW = sm + Y_W * kSPlane;

    float* carry = sm + N_PLANES * kSPlane;
    const int cc = kSR - 1 - (int)a.kk;              // strips: the column the next region needs
    // this CTA's walk: tiles blockIdx.x, + gridDim.x, ...; or (strips) unit
    // blockIdx.x, then the units it takes from the counter
    Tile tl;
    if constexpr (kStrips)
        tl = strip_at(a, blockIdx.x, -1, false);
    else
        tl = tile_at(a, blockIdx.x);
    if (kTma && t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (tl.more) issue_region(a, tm, sm, bar, tl);
    }
    __syncthreads();   // the mbarrier's initialisation before anyone waits on it
    uint32_t phase = 0;
    for (unsigned n = 0; tl.more; ++n) {
        const size_t po = pair_off(a.g.map, a.g.pstride, tl.y);
        const int u = tl.ru0 + c, v0 = tl.rv0 + 2 * p;
        const bool live = u < C && v0 < R;           // v0 < R implies v0 + 1 < R (R even)
        const bool fu = (u == 0), lu = (u == C - 1);
        const bool fv = (v0 == 0), lv = (v0 + 1 == R - 1);
        const bool last_launch = a.last || (pair_flags(a.g.map, tl.y) & kMapLast);

        const bool ok = kTma ? mbar_wait(bar, phase, kStreamWaitLimit) : true;
        // the pair's value of plane k: from the staging copy, or loaded
        // directly (zero outside the image, as the tensor copy fills)
        auto ld2s = [&](int k) {
            if constexpr (kTma) return *reinterpret_cast<const float2*>(sm + k * kSPlane + me);
            return live ? __ldg(reinterpret_cast<const float2*>(at(a.planes[k], po) + v0 + (size_t)u * (size_t)R))
                        : zero;
        };
        float2 du = ld2s(S_DU), dv = ld2s(S_DV), dw = ld2s(S_DW), ua = ld2s(S_UA), va = ld2s(S_VA),
               wa = ld2s(S_WA), pd = ld2s(S_PD), puu = ld2s(S_PUU), puv = ld2s(S_PUV), pvu = ld2s(S_PVU),
               pvv = ld2s(S_PVV), pwu = ld2s(S_PWU), pwv = ld2s(S_PWV);
        const float2 dup = ld2s(K_DUP), dvp = ld2s(K_DVP), ri = ld2s(K_RI), rj = ld2s(K_RJ), ddt = ld2s(K_DDT),
                     ddu = ld2s(K_DDU), ddv = ld2s(K_DDV), s0 = ld2s(K_S0), s1 = ld2s(K_S1), s2 = ld2s(K_S2),
                     s3 = ld2s(K_S3), s4 = ld2s(K_S4), mu = ld2s(K_MU), dct = ld2s(K_DCT), dcu = ld2s(K_DCU),
                     dcv = ld2s(K_DCV), tu = ld2s(K_TU), tv = ld2s(K_TV), tw = ld2s(K_TW);
        // staging read by every thread: the next region may land.  A wait that ran
        // out anywhere ends the whole CTA (values read above are then unused)
        if (__syncthreads_or(!ok)) {
            if (t == 0) {
                if (a.status) atomicExch(a.status, kStreamTimeout);
                mbar_wait(bar, phase, kStreamWaitLimit);   // bounded: the copies still in flight
            }
            break;
        }
        phase ^= 1u;
        if (kTma && t == 0) {
            // the unit after this one (read by every thread after this tile's
            // iteration barriers; rewritten only after the next tile's first)
            unsigned unit = 0;
            if (kStrips && tl.iu1 >= tl.c1) {
                unit = gridDim.x + atomicAdd(a.work, 1u);
                next_unit = unit;
            }
            const Tile nx = next_tile<kStrips>(a, tl, unit);
            if (nx.more) issue_region(a, tm, sm, bar, nx);
        }
        // the left neighbour's exchange values: the carry of the previous
        // region (strips, first column) or the exchange planes; j advances
        // the carry by one iteration
        const bool from_carry = kStrips && tl.carry_in && c == 0;
        const float* yl = from_carry ? carry + ((n + 1) & 1) * (4 * 3 * kSR) + 2 * p : sm + Y_U * kSPlane + left;
        const int yl_k = from_carry ? kSR : kSPlane, yl_j = from_carry ? 3 * kSR : 0;
        float* yc = carry + (n & 1) * (4 * 3 * kSR) + 2 * p;
        const bool to_carry = kStrips && tl.carry_out && c == cc;

        const float2 mudu = mul2(mu, ddu), mudv = mul2(mu, ddv);
        const float2 a1 = mul2(tu, dcu), b1 = mul2(tv, dcv);
        const float2 th = fm2(a1, dcu, mul2(b1, dcv));
        // the shrinkage's denominators and their reciprocals, fixed for the level
        const float2 den = make_float2(add(th.x, 1e-10f), add(th.y, 1e-10f));
        const float2 rden = make_float2(__frcp_rn(den.x), __frcp_rn(den.y));
        const bool rcp_ok = shrink_rcp_level_ok(a1.x, b1.x, den.x) && shrink_rcp_level_ok(a1.y, b1.y, den.y);
        // the iterations, with the image-border cases (kBorder) or, for a region
        // that touches no image border, without them (the same expressions)
        auto iterate = [&](auto border) {
            constexpr bool kBorder = decltype(border)::value;
            for (unsigned j = 0; j < a.kk; ++j) {
                // ---------------- dual step (computeGradient + updateDualVariables) ----------------
                {
                    const float2 U = add2(ua, dup), V = add2(va, dvp);
                    *reinterpret_cast<float2*>(XU + me) = U;
                    *reinterpret_cast<float2*>(XV + me) = V;
                    *reinterpret_cast<float2*>(XW + me) = wa;
                    const float Ub = __shfl_down_sync(0xffffffffu, U.x, 1, 16);   // the next pair's first row
                    const float Vb = __shfl_down_sync(0xffffffffu, V.x, 1, 16);
                    const float Wb = __shfl_down_sync(0xffffffffu, wa.x, 1, 16);
                    __syncthreads();
                    // borders by selects, not branches (the neighbour slot at the
                    // region's right edge is the thread's own: read, then dropped)
                    float2 gu1 = mul2(ri, sub2(*reinterpret_cast<const float2*>(XU + right), U));
                    float2 gv1 = mul2(ri, sub2(*reinterpret_cast<const float2*>(XV + right), V));
                    float2 gw1 = mul2(ri, sub2(*reinterpret_cast<const float2*>(XW + right), wa));
                    if (kBorder && lu) {
                        gu1 = zero;
                        gv1 = zero;
                        gw1 = zero;
                    }
                    float2 gu2 = mul2(rj, sub2(make_float2(U.y, Ub), U));
                    float2 gv2 = mul2(rj, sub2(make_float2(V.y, Vb), V));
                    float2 gw2 = mul2(rj, sub2(make_float2(wa.y, Wb), wa));
                    if (kBorder && lv) {
                        gu2.y = 0.f;
                        gv2.y = 0.f;
                        gw2.y = 0.f;
                    }
                    const float2 X = fm2(ddv, va, fm2(ddu, ua, sub2(ddt, wa)));
                    pd = fm2(s0, X, pd);
                    puu = fm2(s1, gu1, puu);
                    puv = fm2(s2, gu2, puv);
                    pvu = fm2(s1, gv1, pvu);
                    pvv = fm2(s2, gv2, pvv);
                    pwu = fm2(s3, gw1, pwu);
                    pwv = fm2(s4, gw2, pwv);
                    pd.x = clamp1(pd.x);
                    pd.y = clamp1(pd.y);
                    disc2(puu, puv);
                    disc2(pvu, pvv);
                    disc2(pwu, pwv);
                }
                // ---------------- primal step (computeDivergence + updatePrimalVariables) ----------------
                {
                    const float2 yu = mul2(ri, puu), yv = mul2(ri, pvu), yw = mul2(ri, pwu);
                    *reinterpret_cast<float2*>(YU + me) = yu;
                    *reinterpret_cast<float2*>(YV + me) = yv;
                    *reinterpret_cast<float2*>(YW + me) = yw;
                    if (to_carry) {
                        float* y = yc + j * (3 * kSR);
                        *reinterpret_cast<float2*>(y) = yu;
                        *reinterpret_cast<float2*>(y + kSR) = yv;
                        *reinterpret_cast<float2*>(y + 2 * kSR) = yw;
                    }
                    const float2 zu = mul2(rj, puv), zv = mul2(rj, pvv), zw = mul2(rj, pwv);
                    const float zua = __shfl_up_sync(0xffffffffu, zu.y, 1, 16);   // the previous pair's second row
                    const float zva = __shfl_up_sync(0xffffffffu, zv.y, 1, 16);
                    const float zwa = __shfl_up_sync(0xffffffffu, zw.y, 1, 16);
                    __syncthreads();
                    const float2 pu_[3] = {puu, pvu, pwu}, pv_[3] = {puv, pvv, pwv};
                    const float2 zm_[3] = {make_float2(zua, zu.x), make_float2(zva, zv.x), make_float2(zwa, zw.x)};
                    float2 div[3];
    #pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const float2 ym = neg2(*reinterpret_cast<const float2*>(yl + k * yl_k + (int)j * yl_j));
                        float2 d = fm2(ri, pu_[k], ym);
                        // first / last / inner column
                        if constexpr (kBorder) d = fu ? mul2(ri, pu_[k]) : (lu ? ym : d);
                        float2 g = add2(d, fm2(rj, pv_[k], neg2(zm_[k])));
                        if constexpr (kBorder) {
                            if (fv) g.x = fm(rj.x, pv_[k].x, d.x);
                            if (lv) g.y = fm(-rj.x, pv_[k].x, d.y);
                        }
                        div[k] = g;
                    }
                    const float2 du_old = du, dv_old = dv, dw_old = dw;
                    du = fm2(neg2(tu), fm2(mudu, pd, neg2(mul2(li2, div[0]))), du);
                    dv = fm2(neg2(tv), fm2(mudv, pd, neg2(mul2(li2, div[1]))), dv);
                    {
                        // per lane: see pdflow_pack.cuh on contraction of packed products
                        const float2 tq = fm2(neg2(mu), pd, neg2(mul2(ld2, div[2])));
                        dw.x = add(dw.x, mul(-tw.x, tq.x));
                        dw.y = add(dw.y, mul(-tw.y, tq.y));
                    }
                    const float2 of = fm2(dcv, dv, fm2(dcu, du, dct));
                    // quotients by the reciprocal when the whole warp is in its range
                    if (__all_sync(0xffffffffu, rcp_ok && shrink_rcp_ok(of.x) && shrink_rcp_ok(of.y))) {
                        shrink_rcp2(du, dv, of, th, den, rden, a1, b1);
                    } else {
                        shrink(du.x, dv.x, of.x, th.x, a1.x, b1.x);
                        shrink(du.y, dv.y, of.y, th.y, a1.y, b1.y);
                    }
                    ua = fm2(two, du, neg2(du_old));
                    va = fm2(two, dv, neg2(dv_old));
                    wa = fm2(two, dw, neg2(dw_old));
                    if (last_launch && j + 1 == a.kk && live) {
                        // saturateVariables (pdflow_cudalib.cu:1018-1038) after the level's last iteration
                        const float2 z = __ldg(reinterpret_cast<const float2*>(at(a.depth_old, po) + v0 +
                                                                                (size_t)u * (size_t)R));
                        saturate(du.x, dv.x, dw.x, dup.x, dvp.x, z.x);
                        saturate(du.y, dv.y, dw.y, dup.y, dvp.y, z.y);
                    }
                }
                // no barrier here: this iteration's exchange reads happen before the next
                // one's first barrier, and the next stores to the same planes after it
            }
        };
        if (tl.ru0 > 0 && tl.ru0 + kSR < C && tl.rv0 > 0 && tl.rv0 + kSR < R)   // the same for the whole CTA
            iterate(std::false_type{});
        else
            iterate(std::true_type{});

        // ---- the interior to the destination buffer ----
        if (live && v0 >= tl.iv0 && v0 < tl.iv1 && u >= tl.iu0 && u < tl.iu1) {
            const size_t gi = (size_t)v0 + (size_t)u * (size_t)R;
            const float2 st[13] = {du, dv, dw, ua, va, wa, pd, puu, puv, pvu, pvv, pwu, pwv};
#pragma unroll
            for (int k = 0; k < 13; ++k) *reinterpret_cast<float2*>(at(a.dst[k], po) + gi) = st[k];
        }
        // the next tile's staging wait is followed by a barrier before its first
        // exchange store, so the exchange planes (and the carry) need none here
        tl = next_tile<kStrips>(a, tl, kStrips ? next_unit : 0u);
    }
    // strips: the last CTA to finish (every CTA has taken its last unit)
    // clears the counter for the next launch
    if (kStrips && t == 0 && atomicAdd(a.work + 1, 1u) == gridDim.x - 1) {
        atomicExch(a.work, 0u);
        atomicExch(a.work + 1, 0u);
    }
}

}  // namespace

size_t stream_smem_bytes() { return sizeof(float) * (N_PLANES * kSPlane + kCarryFloats); }

// Strip units: the last grid / 8 strips in 8 pieces (grid / 4 for strips
// of 16 regions or more), the grid / 8 before them in 4, the grid / 8 before
// those in 2, the rest whole; no more strips than CTAs: every strip in as
// many pieces as CTAs allow.  Pieces are at least one restart region's
// 32 - 2 kk exact columns wide.  Each piece recomputes a left halo, so the
// tail is kept short: on 64-pair VGA solves (1 280 strips of 23 regions at
// 480x640, 640 of 12 at 240x320) the last grid / 4, grid / 2 and grid strips
// in 8, 4 and 2 pieces took 38.06 ms, these tiers 37.3 ms.
StripUnits strip_units(unsigned strips_n, unsigned C, unsigned kk, unsigned grid)
{
    StripUnits su{};
    if (strips_n == 0 || C == 0 || kk == 0 || 2 * kk >= (unsigned)kSR || grid == 0) return su;
    const unsigned most = (C + (kSR - 2 * kk) - 1) / (kSR - 2 * kk);
    const unsigned regions = (C + (kSR - kk) - 1) / (kSR - kk);   // of a whole strip walked with the carry
    unsigned left = strips_n;
    const unsigned tn[3] = {grid / 8, grid / 8, regions >= 16 ? grid / 4 : grid / 8}, tp[3] = {2, 4, 8};
    for (int i = 2; i >= 0; --i) {
        su.tier_n[i] = strips_n > grid ? std::min(tn[i], left) : 0u;
        su.tier_p[i] = std::min(tp[i], most);
        left -= su.tier_n[i];
    }
    if (strips_n <= grid) {
        su.tier_n[0] = strips_n;
        su.tier_p[0] = std::max(1u, std::min(grid / strips_n, most));
        left = 0;
    }
    su.whole = left;
    return su;
}

// The direct loads and stores move a pixel pair as one float2: even rows and
// pair spacing, 8-byte aligned planes.
bool stream_direct_eligible(const LevelGeom& g, const LevelConsts& L, const State& src, const State& dst)
{
    if (g.R % 2 != 0 || g.slots == 0 || g.pstride % 2 != 0) return false;
    const float* cg[19] = {L.ri, L.rj, L.dct, L.dcu, L.dcv, L.ddt, L.ddu, L.ddv, L.mu, L.du_prev, L.dv_prev,
                           L.qs[0], L.qs[1], L.qs[2], L.qs[3], L.qs[4], L.qs[5], L.qs[6], L.qs[7]};
    const float* sd[26] = {src.du, src.dv, src.dw, src.dua, src.dva, src.dwa, src.pd, src.puu, src.puv,
                           src.pvu, src.pvv, src.pwu, src.pwv, dst.du, dst.dv, dst.dw, dst.dua, dst.dva,
                           dst.dwa, dst.pd, dst.puu, dst.puv, dst.pvu, dst.pvv, dst.pwu, dst.pwv};
    for (const float* q : cg)
        if (!q || reinterpret_cast<uintptr_t>(q) % 8u != 0) return false;
    for (const float* q : sd)
        if (!q || reinterpret_cast<uintptr_t>(q) % 8u != 0) return false;
    return true;
}

bool stream_eligible(const LevelGeom& g, const LevelConsts& L, const State& src, const State& dst, int form)
{
    if (quads_eligible(g, L, src, dst)) return true;
    return (form == 8 || form == 9) && stream_direct_eligible(g, L, src, dst);
}

cudaError_t prepare_stream_tiles()
{
    cudaError_t e = cudaSuccess;
    for (const void* k : {(const void*)k_iterate_stream<false>, (const void*)k_iterate_stream<true>,
                          (const void*)k_iterate_stream<false, false>}) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stream_smem_bytes());
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    }
    return e;
}

cudaError_t launch_iterate_stream(LevelGeom g, LevelConsts L, State src, State dst, Params p, const float* depth_old,
                                  unsigned kk, bool last, cudaStream_t st, unsigned* status, unsigned ctas,
                                  StreamLayout layout)
{
    // the region stays 32 x 32; rows of region origins stay multiples of 4
    // (16-byte tensor-copy coordinates): halo 4 (interior 24) or 8 (interior 16)
    const bool strips = layout == StreamLayout::Strips;
    const int kSH = layout == StreamLayout::Tiles16 ? 8 : 4, kST = kSR - 2 * kSH;
    // the tensor copies need the quad tiles' preconditions (16-byte aligned
    // planes at one spacing, rows % 4 == 0); the tiles also run on direct loads
    // where the rows are even
    const bool tma = quads_eligible(g, L, src, dst);
    if (kk == 0 || kk > (unsigned)kSH || !status || ctas == 0 || reinterpret_cast<uintptr_t>(depth_old) % 8u != 0 ||
        !(tma || (!strips && stream_direct_eligible(g, L, src, dst))))
        return cudaErrorInvalidValue;
    StreamArgs a;
    a.g = g;
    float* d13[13] = {dst.du, dst.dv, dst.dw, dst.dua, dst.dva, dst.dwa, dst.pd,
                      dst.puu, dst.puv, dst.pvu, dst.pvv, dst.pwu, dst.pwv};
    for (int k = 0; k < 13; ++k) a.dst[k] = d13[k];
    a.depth_old = depth_old;
    a.p = p;
    a.kk = kk;
    a.last = last;
    a.status = status;
    a.tile = kST;
    a.halo = kSH;
    a.tiles_v = (g.R + kST - 1) / kST;
    a.tiles = a.tiles_v * ((g.C + kST - 1) / kST);
    a.total = a.tiles * g.pairs;
    const unsigned grid = ctas < a.total ? ctas : a.total;
    const StripUnits su = strip_units(g.pairs * a.tiles_v, g.C, kk, grid);
    a.whole = su.whole;
    for (int i = 0; i < 3; ++i) {
        a.tier_n[i] = su.tier_n[i];
        a.tier_p[i] = su.tier_p[i];
    }
    a.work = status + 2;
    // the runs of planes (quads_eligible checked that each is equally spaced)
    const float* sg[13] = {src.du, src.dv, src.dw, src.dua, src.dva, src.dwa, src.pd,
                           src.puu, src.puv, src.pvu, src.pvv, src.pwu, src.pwv};
    const float* cg[19] = {L.ri, L.rj, L.dct, L.dcu, L.dcv, L.ddt, L.ddu, L.ddv, L.mu, L.du_prev, L.dv_prev,
                           L.qs[0], L.qs[1], L.qs[2], L.qs[3], L.qs[4], L.qs[5], L.qs[6], L.qs[7]};
    for (int k = 0; k < 13; ++k) a.planes[k] = sg[k];
    for (int k = 0; k < 19; ++k) a.planes[13 + k] = cg[k];
    StreamMaps maps{};
    if (!tma) {
        k_iterate_stream<false, false><<<grid, kSThreads, stream_smem_bytes(), st>>>(a, maps);
        return cudaGetLastError();
    }
    size_t ss = 0, cs = 0;
    if (!equally_spaced(sg, 13, &ss) || !equally_spaced(cg, 19, &cs) ||
        !encode_plane_group(&maps.state, sg[0], 13, ss, g.R, g.C, g.slots, g.pstride, kSR, kSR) ||
        !encode_plane_group(&maps.consts, cg[0], 19, cs, g.R, g.C, g.slots, g.pstride, kSR, kSR))
        return cudaErrorInvalidValue;
    if (strips)
        k_iterate_stream<true><<<grid, kSThreads, stream_smem_bytes(), st>>>(a, maps);
    else
        k_iterate_stream<false><<<grid, kSThreads, stream_smem_bytes(), st>>>(a, maps);
    return cudaGetLastError();
}

}  // namespace pdflow
