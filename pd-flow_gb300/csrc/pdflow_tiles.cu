// Temporally blocked primal-dual iterations: several iterations per launch
// on tiles held in shared memory.
//
// A CTA owns an interior tile of TV x TU pixels of one pair's level and loads
// the tile plus a halo of H pixels on every side that is not an image border
// (the "region") into shared memory: the 13 state values and the 11 level
// constants the iteration reads (mu, ddt, ddu, ddv, dct, dcu, dcv, ri, rj,
// du_prev, dv_prev; the 8 step sizes are recomputed from them with the same
// function as the set-up kernel, so they are the same bits).  One iteration's
// dual step reads the over-relaxed primal one pixel forward and its primal
// step the duals one pixel back, so after j iterations only the pixels at
// least j from a non-border region edge are still exact; after `kk` <= H
// iterations the interior is exact and is written back.  Reads come from one
// copy of the state and writes go to the other (neighbouring tiles read the
// halo from the same copy), so launches alternate the two buffers.
//
// Shared memory: 24 floats per region pixel; with TV = TU = 40 and H = 4 the
// region is 48 x 48 (221 KB).  Per launch the region is read once (24 floats
// per pixel) and the interior's state written once (13 floats), for kk
// iterations: with kk = 4 about 48 B of DRAM traffic per pixel-iteration,
// against 148 B for one iteration through memory.
#include "pdflow_iterate.cuh"
#include "pdflow_math.cuh"

namespace pdflow {

namespace {

constexpr int kTV = 40, kTU = 40, kH = 4;
constexpr int kRV = kTV + 2 * kH, kRU = kTU + 2 * kH;
constexpr int kPlane = kRV * kRU;          // floats per shared plane
constexpr int kTileThreads = 768;

// shared planes
enum { T_DU, T_DV, T_DW, T_UA, T_VA, T_WA, T_PD, T_PUU, T_PUV, T_PVU, T_PVV, T_PWU, T_PWV,   // state
       T_MU, T_DDT, T_DDU, T_DDV, T_DCT, T_DCU, T_DCV, T_RI, T_RJ, T_DUP, T_DVP, T_NPLANES };

struct TileArgs {
    LevelGeom g;
    LevelConsts L;
    State src, dst;
    Params p;
    const float* depth_old;
    unsigned kk;          // iterations in this launch (<= kH)
    bool last;            // the level's last iteration is in this launch (saturate)
    unsigned tiles_v;     // tiles along v
};

// Thread layout: 48 x 16 threads; thread (tx, ty) owns region pixels
// (rv = tx, ru = ty + 16 k), k = 0..2, for the whole launch, so the pixel
// bookkeeping and the step sizes are computed once per launch.
constexpr int kTX = kRV, kTY = kTileThreads / kRV, kPerThread = kRU / kTY;
static_assert(kTX * kTY == kTileThreads && kTY * kPerThread == kRU, "tile thread layout");

__global__ void __launch_bounds__(kTileThreads, 1) k_iterate_tiles(TileArgs a)
{
    extern __shared__ float sm[];
    const size_t po = pair_off(a.g.map, a.g.pstride, blockIdx.y);
    const LevelConsts L = at(a.L, po);
    const State src = at(a.src, po), dst = at(a.dst, po);
    const float* depth_old = at(a.depth_old, po);
    const int R = (int)a.g.R, C = (int)a.g.C;
    const int tv = (int)(blockIdx.x % a.tiles_v), tu = (int)(blockIdx.x / a.tiles_v);
    // interior [iv0, iv1) x [iu0, iu1), region [rv0, rv1) x [ru0, ru1)
    const int iv0 = tv * kTV, iu0 = tu * kTU;
    const int iv1 = min(iv0 + kTV, R), iu1 = min(iu0 + kTU, C);
    const int rv0 = max(iv0 - kH, 0), ru0 = max(iu0 - kH, 0);
    const int rv1 = min(iv1 + kH, R), ru1 = min(iu1 + kH, C);
    const int RV = rv1 - rv0, RU = ru1 - ru0;
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    float* P[T_NPLANES];
#pragma unroll
    for (int k = 0; k < T_NPLANES; ++k) P[k] = sm + k * kPlane;

    // ---- load the region (plane index q = rv + ru * kRV) ----
    {
        const float* gs[T_NPLANES] = {src.du, src.dv, src.dw, src.dua, src.dva, src.dwa, src.pd, src.puu, src.puv,
                                      src.pvu, src.pvv, src.pwu, src.pwv, L.mu, L.ddt, L.ddu, L.ddv, L.dct, L.dcu,
                                      L.dcv, L.ri, L.rj, L.du_prev, L.dv_prev};
        if (tx < RV)
            for (int ru = ty; ru < RU; ru += kTY) {
                const int q = tx + ru * kRV;
                const size_t gi = (size_t)(rv0 + tx) + (size_t)(ru0 + ru) * R;
#pragma unroll
                for (int k = 0; k < T_NPLANES; ++k) P[k][q] = __ldg(gs[k] + gi);
            }
    }
    __syncthreads();

    const float li = a.p.lambda_i, ld = a.p.lambda_d;
    // per owned pixel: flags (bit 0 valid, 1 fu, 2 lu, 3 fv, 4 lv), halo-ring distance, step sizes
    unsigned flags[kPerThread];
    int ringd[kPerThread];
    float sg[kPerThread][8];
#pragma unroll
    for (int k = 0; k < kPerThread; ++k) {
        const int rv = tx, ru = ty + kTY * k;
        const bool valid = rv < RV && ru < RU;
        const int v = rv0 + rv, u = ru0 + ru;
        flags[k] = valid ? (1u | (u == 0 ? 2u : 0u) | (u == C - 1 ? 4u : 0u) | (v == 0 ? 8u : 0u) |
                            (v == R - 1 ? 16u : 0u))
                         : 0u;
        int d = 1 << 20;
        if (rv0 > 0) d = min(d, rv);
        if (rv1 < R) d = min(d, RV - 1 - rv);
        if (ru0 > 0) d = min(d, ru);
        if (ru1 < C) d = min(d, RU - 1 - ru);
        ringd[k] = d;
        if (valid) {
            const int q = rv + ru * kRV;
            const bool fu = (flags[k] & 2u), fv = (flags[k] & 8u);
            const float mu = P[T_MU][q], ddu = P[T_DDU][q], ddv = P[T_DDV][q], ri = P[T_RI][q], rj = P[T_RJ][q];
            // the set-up kernel's expressions (mu_and_steps); at a region edge that is
            // not an image border the left/top neighbour is missing: that pixel is stale anyway
            const float ri_m = (fu || ru == 0) ? ri : P[T_RI][q - kRV];
            const float rj_m = (fv || rv == 0) ? rj : P[T_RJ][q - 1];
            sg[k][0] = fdividef(1.f, fm(mu, add(add(1.f, fabsf(ddu)), fabsf(ddv)), 1e-10f));
            sg[k][1] = fdividef(0.5f, fm(li, ri, 1e-10f));
            sg[k][2] = fdividef(0.5f, fm(li, rj, 1e-10f));
            sg[k][3] = fdividef(0.5f, fm(ri, ld, 1e-10f));
            sg[k][4] = fdividef(0.5f, fm(rj, ld, 1e-10f));
            float acu_r = add(ri, rj);
            if (!fu) acu_r = add(acu_r, ri_m);
            if (!fv) acu_r = add(acu_r, rj_m);
            sg[k][5] = fdividef(1.f, add(fm(li, acu_r, mul(mu, fabsf(ddu))), 1e-10f));
            sg[k][6] = fdividef(1.f, add(fm(li, acu_r, mul(mu, fabsf(ddv))), 1e-10f));
            sg[k][7] = fdividef(1.f, add(fm(ld, acu_r, mu), 1e-10f));
        } else {
#pragma unroll
            for (int m = 0; m < 8; ++m) sg[k][m] = 0.f;
        }
    }

    for (unsigned j = 0; j < a.kk; ++j) {
        const bool last_iter = a.last && (j + 1 == a.kk);
        // ---- dual step (in place: each pixel reads only its own duals) ----
#pragma unroll
        for (int k = 0; k < kPerThread; ++k) {
            if (!(flags[k] & 1u) || ringd[k] < (int)j) continue;
            const int rv = tx, ru = ty + kTY * k, q = rv + ru * kRV;
            const bool lu = flags[k] & 4u, lv = flags[k] & 16u;
            const int qu = (lu || ru + 1 >= RU) ? q : q + kRV;    // beyond the region: stale, unused
            const int qv = (lv || rv + 1 >= RV) ? q : q + 1;
            Duals d{P[T_PD][q], P[T_PUU][q], P[T_PUV][q], P[T_PVU][q], P[T_PVV][q], P[T_PWU][q], P[T_PWV][q]};
            dual_update(d, sg[k][0], sg[k][1], sg[k][2], sg[k][3], sg[k][4], P[T_MU][q], P[T_DDT][q], P[T_DDU][q],
                        P[T_DDV][q], li, ld, P[T_RI][q], P[T_RJ][q], P[T_UA][q], P[T_VA][q], P[T_WA][q], P[T_DUP][q],
                        P[T_DVP][q], P[T_UA][qu], P[T_VA][qu], P[T_WA][qu], P[T_DUP][qu], P[T_DVP][qu], P[T_UA][qv],
                        P[T_VA][qv], P[T_WA][qv], P[T_DUP][qv], P[T_DVP][qv], lu, lv);
            P[T_PD][q] = d.pd;
            P[T_PUU][q] = d.puu;
            P[T_PUV][q] = d.puv;
            P[T_PVU][q] = d.pvu;
            P[T_PVV][q] = d.pvv;
            P[T_PWU][q] = d.pwu;
            P[T_PWV][q] = d.pwv;
        }
        __syncthreads();
        // ---- primal step (in place: each pixel writes only its own primal) ----
#pragma unroll
        for (int k = 0; k < kPerThread; ++k) {
            if (!(flags[k] & 1u) || ringd[k] < (int)j) continue;
            const int rv = tx, ru = ty + kTY * k, q = rv + ru * kRV;
            const bool fu = flags[k] & 2u, lu = flags[k] & 4u, fv = flags[k] & 8u, lv = flags[k] & 16u;
            const int qum = (fu || ru == 0) ? q : q - kRV;         // beyond the region: stale, unused
            const int qvm = (fv || rv == 0) ? q : q - 1;
            const float ri = P[T_RI][q], rj = P[T_RJ][q], ri_m = P[T_RI][qum], rj_m = P[T_RJ][qvm];
            const float divu = divergence(ri, ri_m, rj, rj_m, P[T_PUU][q], P[T_PUU][qum], P[T_PUV][q], P[T_PUV][qvm],
                                          fu, lu, fv, lv);
            const float divv = divergence(ri, ri_m, rj, rj_m, P[T_PVU][q], P[T_PVU][qum], P[T_PVV][q], P[T_PVV][qvm],
                                          fu, lu, fv, lv);
            const float divw = divergence(ri, ri_m, rj, rj_m, P[T_PWU][q], P[T_PWU][qum], P[T_PWV][q], P[T_PWV][qvm],
                                          fu, lu, fv, lv);
            float du = P[T_DU][q], dv = P[T_DV][q], dw = P[T_DW][q], nua, nva, nwa;
            primal_update(du, dv, dw, nua, nva, nwa, sg[k][5], sg[k][6], sg[k][7], P[T_MU][q], P[T_DDU][q],
                          P[T_DDV][q], P[T_PD][q], li, ld, divu, divv, divw, P[T_DCT][q], P[T_DCU][q], P[T_DCV][q]);
            if (last_iter) {
                const size_t gi = (size_t)(rv0 + rv) + (size_t)(ru0 + ru) * R;
                saturate(du, dv, dw, P[T_DUP][q], P[T_DVP][q], __ldg(depth_old + gi));
            }
            P[T_DU][q] = du;
            P[T_DV][q] = dv;
            P[T_DW][q] = dw;
            P[T_UA][q] = nua;
            P[T_VA][q] = nva;
            P[T_WA][q] = nwa;
        }
        __syncthreads();
    }

    // ---- write the interior ----
    float* gd[13] = {dst.du, dst.dv, dst.dw, dst.dua, dst.dva, dst.dwa, dst.pd, dst.puu, dst.puv, dst.pvu, dst.pvv,
                     dst.pwu, dst.pwv};
    const int v = rv0 + tx;
    if (v >= iv0 && v < iv1)
        for (int ru = ty; ru < RU; ru += kTY) {
            const int u = ru0 + ru;
            if (u < iu0 || u >= iu1) continue;
            const int q = tx + ru * kRV;
            const size_t gi = (size_t)v + (size_t)u * R;
#pragma unroll
            for (int k = 0; k < 13; ++k) gd[k][gi] = P[k][q];
        }
}

}  // namespace

unsigned tiles_per_level(LevelGeom g)
{
    return ((g.R + kTV - 1) / kTV) * ((g.C + kTU - 1) / kTU);
}

cudaError_t prepare_tiles()
{
    return cudaFuncSetAttribute(k_iterate_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(float) * T_NPLANES * kPlane));
}

size_t tiles_smem_bytes() { return sizeof(float) * T_NPLANES * kPlane; }

unsigned tiles_halo() { return kH; }

cudaError_t launch_iterate_tiles(LevelGeom g, LevelConsts L, State src, State dst, Params p, const float* depth_old,
                                 unsigned kk, bool last, cudaStream_t st)
{
    TileArgs a;
    a.g = g;
    a.L = L;
    a.src = src;
    a.dst = dst;
    a.p = p;
    a.depth_old = depth_old;
    a.kk = kk;
    a.last = last;
    a.tiles_v = (g.R + kTV - 1) / kTV;
    dim3 grid(tiles_per_level(g), g.pairs);
    k_iterate_tiles<<<grid, kTileThreads, tiles_smem_bytes(), st>>>(a);
    return cudaGetLastError();
}

}  // namespace pdflow
