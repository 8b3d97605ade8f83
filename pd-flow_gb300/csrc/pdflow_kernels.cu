// Stage kernels of the PD-Flow solver on sm_103a.
//
// One thread per pixel, column-major planes (idx = v + u*R, rows contiguous,
// so a warp reads 32 consecutive rows of one column: coalesced).  The per-level
// set-up is fused into three kernels (init = zero/upsample + connectivity,
// image gradients, warp + step sizes), an iteration is two kernels
// (gradient+dual, divergence+primal; the reference uses four) and the last
// primal kernel of a level also saturates; the weighted median and the motion
// field are one kernel.  All per-pixel arithmetic lives in pdflow_math.cuh.
#include "pdflow_kernels.cuh"
#include "pdflow_math.cuh"

namespace pdflow {

namespace {

constexpr unsigned kBlock = 256;

__host__ __device__ inline unsigned blocks_for(unsigned n) { return (n + kBlock - 1) / kBlock; }

// ---------------------------------------------------------------------------
// Pyramid (computePyramidLevel, pdflow_cudalib.cu:331-434)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void write_xy(PyrLevel out, unsigned R, unsigned C, unsigned v, unsigned u,
                                         unsigned idx, float depth, float fovh)
{
    const float inv_f_i = inv_focal(fovh, C);
    out.xx[idx] = backproject(u, C, depth, inv_f_i);
    out.yy[idx] = backproject(v, R, depth, inv_f_i);
}

// Row-major uint8/uint16 camera images -> column-major level 0 (decode +
// transpose through a 32x33 shared tile so that both sides are coalesced).
__global__ void __launch_bounds__(1024) k_decode_u16(const uint8_t* __restrict__ img,
                                                     const uint16_t* __restrict__ depth, unsigned W, unsigned H,
                                                     PyrLevel out, float fovh, size_t pstride,
                                                     const unsigned* __restrict__ map)
{
    img += (size_t)blockIdx.z * W * H;
    depth += (size_t)blockIdx.z * W * H;
    out = at(out, pair_off(map, pstride, blockIdx.z));
    __shared__ float sc[32][33];
    __shared__ float sz[32][33];
    const unsigned x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    {
        const unsigned x = x0 + threadIdx.x, y = y0 + threadIdx.y;
        if (x < W && y < H) {
            const size_t i = (size_t)y * W + x;
            sc[threadIdx.y][threadIdx.x] = float(img[i]);
            sz[threadIdx.y][threadIdx.x] = decode_depth(depth[i]);
        }
    }
    __syncthreads();
    const unsigned v = y0 + threadIdx.x, u = x0 + threadIdx.y;  // writes walk along v
    if (u < W && v < H) {
        const unsigned idx = v + u * H;
        const float z = sz[threadIdx.x][threadIdx.y];
        out.col[idx] = sc[threadIdx.x][threadIdx.y];
        out.dep[idx] = z;
        write_xy(out, H, W, v, u, idx, z, fovh);
    }
}

// Row-major RGB888 + uint16 millimetre depth -> column-major level 0 with the
// live application's conversion (gray_rgb, decode_depth_mm).  rotate180: its
// camera loop (scene_flow_visualization.cpp:313-323) stores camera pixel
// (y, x) at row H-1-y, column W-1-x.
__global__ void __launch_bounds__(1024) k_decode_rgb8_mm(const uint8_t* __restrict__ rgb,
                                                         const uint16_t* __restrict__ depth, unsigned W, unsigned H,
                                                         PyrLevel out, float fovh, size_t pstride,
                                                         const unsigned* __restrict__ map, int rotate180)
{
    rgb += (size_t)blockIdx.z * W * H * 3;
    depth += (size_t)blockIdx.z * W * H;
    out = at(out, pair_off(map, pstride, blockIdx.z));
    __shared__ float sc[32][33];
    __shared__ float sz[32][33];
    const unsigned x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    {
        const unsigned x = x0 + threadIdx.x, y = y0 + threadIdx.y;   // stored (row y, column x)
        if (x < W && y < H) {
            const size_t i = rotate180 ? (size_t)(H - 1 - y) * W + (W - 1 - x) : (size_t)y * W + x;
            sc[threadIdx.y][threadIdx.x] = gray_rgb(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
            sz[threadIdx.y][threadIdx.x] = decode_depth_mm(depth[i]);
        }
    }
    __syncthreads();
    const unsigned v = y0 + threadIdx.x, u = x0 + threadIdx.y;  // writes walk along v
    if (u < W && v < H) {
        const unsigned idx = v + u * H;
        const float z = sz[threadIdx.x][threadIdx.y];
        out.col[idx] = sc[threadIdx.x][threadIdx.y];
        out.dep[idx] = z;
        write_xy(out, H, W, v, u, idx, z, fovh);
    }
}

__global__ void k_pyr_level0(const float* __restrict__ I, const float* __restrict__ Z, unsigned R, unsigned C,
                             PyrLevel out, float fovh, size_t pstride, const unsigned* __restrict__ map)
{
    const size_t po = pair_off(map, pstride, blockIdx.y);
    I = at(I, po);
    Z = at(Z, po);
    out = at(out, po);
    const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= R * C) return;
    const unsigned v = idx % R, u = idx / R;
    out.col[idx] = I[idx];
    const float z = Z[idx];
    out.dep[idx] = z;
    write_xy(out, R, C, v, u, idx, z, fovh);
}

__global__ void k_pyr_down(PyrLevel prev, unsigned R, unsigned C, PyrLevel out, float fovh, size_t pstride,
                           const unsigned* __restrict__ map)
{
    const size_t po = pair_off(map, pstride, blockIdx.y);
    prev = at(prev, po);
    out = at(out, po);
    const unsigned index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= R * C) return;
    const unsigned v = index % R, u = index / R;
    const float max_depth_dif = 0.1f;
    const float* __restrict__ cp = prev.col;
    const float* __restrict__ dp = prev.dep;
    float sumd = 0.f, sumc = 0.f, acu_weights_d = 0.f, acu_weights_c = 0.f;
    const unsigned ind_cent_prev = 2 * v + 4 * u * R;
    const float dcenter = dp[ind_cent_prev];
    float dres, cres;
    // sumc and sumd fuse their products; the depth weight is added after
    // rounding (acu_weights_d += aux_w), as in the reference build.
    if ((v > 0) && (v < R - 1) && (u > 0) && (u < C - 1)) {
#pragma unroll
        for (int k = -2; k < 3; k++)
#pragma unroll
            for (int l = -2; l < 3; l++) {
                const unsigned ind_loop_prev = 2 * v + k + 2 * (2 * u + l) * R;
                const float gm = gmask(k, l);
                sumc = fm(gm, cp[ind_loop_prev], sumc);
                const float d = dp[ind_loop_prev];
                const float ad = fabsf(sub(d, dcenter));
                if ((d > 0.f) && (ad < max_depth_dif)) {
                    const float aux_w = mul(gm, sub(max_depth_dif, ad));
                    acu_weights_d = add(acu_weights_d, aux_w);
                    sumd = fm(aux_w, d, sumd);
                }
            }
        dres = (sumd > 0.f) ? qt(sumd, acu_weights_d) : 0.f;
        cres = sumc;
    } else {
        for (int k = -2; k < 3; k++)
            for (int l = -2; l < 3; l++) {
                const int indv = 2 * (int)v + k, indu = 2 * (int)u + l;
                if ((indv >= 0) && (indv < 2 * (int)R) && (indu >= 0) && (indu < 2 * (int)C)) {
                    const unsigned ind_loop_prev = 2 * v + k + 2 * (2 * u + l) * R;
                    const float gm = gmask(k, l);
                    sumc = fm(gm, cp[ind_loop_prev], sumc);
                    acu_weights_c = add(acu_weights_c, gm);
                    const float d = dp[ind_loop_prev];
                    const float ad = fabsf(sub(d, dcenter));
                    if ((d > 0.f) && (ad < max_depth_dif)) {
                        const float aux_w = mul(gm, sub(max_depth_dif, ad));
                        acu_weights_d = add(acu_weights_d, aux_w);
                        sumd = fm(aux_w, d, sumd);
                    }
                }
            }
        cres = qt(sumc, acu_weights_c);
        dres = (sumd > 0.f) ? qt(sumd, acu_weights_d) : 0.f;
    }
    out.col[index] = cres;
    out.dep[index] = dres;
    write_xy(out, R, C, v, u, index, dres, fovh);
}

// ---------------------------------------------------------------------------
// Level set-up
// ---------------------------------------------------------------------------

// upsampleCopy + upsampleFilterPrevSolution (pdflow_cudalib.cu:460-569) at one
// pixel, as a gather over the coarse solution (the zero-inserted taps
// contribute exactly zero and are skipped): acc = du dv dw pd puu puv pvu pvv
// pwu pwv, the taps in the reference's order (row offset, then column).
__device__ __forceinline__ void upsample_px(const LevelSol& cs, unsigned v, unsigned u, unsigned R, unsigned C,
                                            float (&acc)[10])
{
    const unsigned Rc = R / 2;
    const bool inner = (v > 1) && (v < R - 2) && (u > 1) && (u < C - 2);
#pragma unroll
    for (int q = 0; q < 10; ++q) acc[q] = 0.f;
    float acu_weight = 1.f;
#pragma unroll
    for (int k = -2; k < 3; k++)
#pragma unroll
        for (int l = -2; l < 3; l++) {
            const int indv = (int)v + k, indu = (int)u + l;
            const float gm4 = mul(4.f, gmask(k, l));
            if ((indv < 0) || (indv >= (int)R) || (indu < 0) || (indu >= (int)C)) {
                acu_weight = sub(acu_weight, mul(0.25f, gm4));
                continue;
            }
            if ((indv & 1) || (indu & 1)) continue;  // zero-inserted tap
            const unsigned ci = (unsigned)(indv >> 1) + (unsigned)(indu >> 1) * Rc;
            acc[0] = fm(gm4, mul(2.f, cs.du[ci]), acc[0]);
            acc[1] = fm(gm4, mul(2.f, cs.dv[ci]), acc[1]);
            acc[2] = fm(gm4, cs.dw[ci], acc[2]);
            acc[3] = fm(gm4, cs.pd[ci], acc[3]);
            acc[4] = fm(gm4, cs.puu[ci], acc[4]);
            acc[5] = fm(gm4, cs.puv[ci], acc[5]);
            acc[6] = fm(gm4, cs.pvu[ci], acc[6]);
            acc[7] = fm(gm4, cs.pvv[ci], acc[7]);
            acc[8] = fm(gm4, cs.pwu[ci], acc[8]);
            acc[9] = fm(gm4, cs.pwv[ci], acc[9]);
        }
    if (!inner) {
        const float inv_acu_weight = fdividef(1.f, acu_weight);
#pragma unroll
        for (int q = 0; q < 10; ++q) acc[q] = mul(acc[q], inv_acu_weight);
    }
}

// assignZeros (pdflow_cudalib.cu:439-455) with the upsampled solution acc
// (du dv dw pd puu puv pvu pvv pwu pwv, zero at the coarsest level), then
// computeRij (:725-779), at one pixel.
__device__ __forceinline__ void level_init_store(unsigned index, unsigned v, unsigned u, unsigned R, unsigned C,
                                                 const PyrLevel& o, const PyrLevel& n, const LevelConsts& L,
                                                 const State& S, const float (&acc)[10])
{
    L.du_prev[index] = acc[0];
    L.dv_prev[index] = acc[1];
    S.du[index] = 0.f;
    S.dv[index] = 0.f;
    S.dw[index] = acc[2];
    S.dua[index] = 0.f;
    S.dva[index] = 0.f;
    S.dwa[index] = acc[2];
    S.pd[index] = acc[3];
    S.puu[index] = acc[4];
    S.puv[index] = acc[5];
    S.pvu[index] = acc[6];
    S.pvv[index] = acc[7];
    S.pwu[index] = acc[8];
    S.pwv[index] = acc[9];

    // computeRij
    float dxu = 0.f, dzu = 0.f, dxu_2 = 0.f, dzu_2 = 0.f, dyv = 0.f, dzv = 0.f, dyv_2 = 0.f, dzv_2 = 0.f;
    if (u != C - 1) {
        dxu = sub(o.xx[index + R], o.xx[index]);
        dzu = sub(o.dep[index + R], o.dep[index]);
        dxu_2 = sub(n.xx[index + R], n.xx[index]);
        dzu_2 = sub(n.dep[index + R], n.dep[index]);
    }
    if (v != R - 1) {
        dyv = sub(o.yy[index + 1], o.yy[index]);
        dzv = sub(o.dep[index + 1], o.dep[index]);
        dyv_2 = sub(n.yy[index + 1], n.yy[index]);
        dzv_2 = sub(n.dep[index + 1], n.dep[index]);
    }
    L.ri[index] = rfac(dxu, dzu);
    L.rj[index] = rfac(dyv, dzv);
    L.ri2[index] = rfac(dxu_2, dzu_2);
    L.rj2[index] = rfac(dyv_2, dzv_2);
}

// Level set-up, one pixel per thread: the coarsest level (zeros), a warm
// start's seed (its flow, duals from zero), or the upsampled coarse solution.
__global__ void k_level_init(LevelGeom g, bool first, LevelSol cs, PyrLevel o, PyrLevel n, LevelConsts L, State S,
                             const float* __restrict__ seed)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    cs = at(cs, po);
    o = at(o, po);
    n = at(n, po);
    L = at(L, po);
    S = at(S, po);
    const unsigned index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= g.N) return;
    const unsigned R = g.R, C = g.C;
    const unsigned v = index % R, u = index / R;
    float acc[10] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (seed) {   // warm start: a predicted solution of this level, duals from zero
        const float* sp = seed + (size_t)blockIdx.y * 3 * g.N;
        acc[0] = sp[index];
        acc[1] = sp[g.N + index];
        acc[2] = sp[2 * g.N + index];
    } else if (!first) {
        upsample_px(cs, v, u, R, C, acc);
    }
    level_init_store(index, v, u, R, C, o, n, L, S, acc);
}

// Level set-up with the upsampled coarse solution, one vertical pixel pair
// (rows 2a, 2a+1 of column u) per thread.  In a pair whose pixels are both
// inner, the even row's taps with a coarse sample are rows -2, 0, +2 and the
// odd row's -1, +1, and the column's parity fixes the columns (-2, 0, +2 or
// -1, +1): both pixels read the same 3 x 3 (or 3 x 2) coarse neighbourhood,
// loaded once per plane, and accumulate their taps in the reference's order.
// Border pairs take the per-pixel gather.  Same bits as k_level_init.
__global__ void k_level_init_pairs(LevelGeom g, LevelSol cs, PyrLevel o, PyrLevel n, LevelConsts L, State S)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    cs = at(cs, po);
    o = at(o, po);
    n = at(n, po);
    L = at(L, po);
    S = at(S, po);
    const unsigned R = g.R, C = g.C, Rc = R / 2;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Rc * C) return;
    const unsigned a = t % Rc, u = t / Rc, v0 = 2 * a, index0 = v0 + u * R;
    float acc0[10], acc1[10];
    if (a >= 1 && v0 + 3 < R && u > 1 && u + 2 < C) {
        const unsigned b = u >> 1;
        const float* planes[10] = {cs.du, cs.dv, cs.dw, cs.pd, cs.puu, cs.puv, cs.pvu, cs.pvv, cs.pwu, cs.pwv};
        if ((u & 1u) == 0) {   // column taps -2, 0, +2: coarse columns b-1, b, b+1
#pragma unroll
            for (int q = 0; q < 10; ++q) {
                float c[3][3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int e = 0; e < 3; ++e) {
                        const float x = planes[q][(a - 1 + r) + (b - 1 + e) * Rc];
                        c[r][e] = q < 2 ? mul(2.f, x) : x;
                    }
                float x0 = 0.f, x1 = 0.f;
#pragma unroll
                for (int r = 0; r < 3; ++r)   // even row: row taps -2, 0, +2 = coarse rows a-1, a, a+1
#pragma unroll
                    for (int e = 0; e < 3; ++e) x0 = fm(mul(4.f, gmask(2 * r - 2, 2 * e - 2)), c[r][e], x0);
#pragma unroll
                for (int r = 1; r < 3; ++r)   // odd row: row taps -1, +1 = coarse rows a, a+1
#pragma unroll
                    for (int e = 0; e < 3; ++e) x1 = fm(mul(4.f, gmask(2 * r - 3, 2 * e - 2)), c[r][e], x1);
                acc0[q] = x0;
                acc1[q] = x1;
            }
        } else {   // column taps -1, +1: coarse columns b, b+1
#pragma unroll
            for (int q = 0; q < 10; ++q) {
                float c[3][2];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const float x = planes[q][(a - 1 + r) + (b + e) * Rc];
                        c[r][e] = q < 2 ? mul(2.f, x) : x;
                    }
                float x0 = 0.f, x1 = 0.f;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int e = 0; e < 2; ++e) x0 = fm(mul(4.f, gmask(2 * r - 2, 2 * e - 1)), c[r][e], x0);
#pragma unroll
                for (int r = 1; r < 3; ++r)
#pragma unroll
                    for (int e = 0; e < 2; ++e) x1 = fm(mul(4.f, gmask(2 * r - 3, 2 * e - 1)), c[r][e], x1);
                acc0[q] = x0;
                acc1[q] = x1;
            }
        }
    } else {
        upsample_px(cs, v0, u, R, C, acc0);
        upsample_px(cs, v0 + 1, u, R, C, acc1);
    }
    level_init_store(index0, v0, u, R, C, o, n, L, S, acc0);
    level_init_store(index0 + 1, v0 + 1, u, R, C, o, n, L, S, acc1);
}

// computeImGradients (pdflow_cudalib.cu:574-627) on the new frame.
__global__ void k_im_gradients(LevelGeom g, PyrLevel n, LevelConsts L)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    n = at(n, po);
    L = at(L, po);
    const unsigned index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= g.N) return;
    const unsigned R = g.R, C = g.C;
    const unsigned v = index % R, u = index / R;
    const float* __restrict__ c = n.col;
    const float* __restrict__ d = n.dep;
    const float* __restrict__ ri2 = L.ri2;
    const float* __restrict__ rj2 = L.rj2;
    if (u == 0) {
        L.dcu_aux[index] = sub(c[index + R], c[index]);
        L.ddu_aux[index] = sub(d[index + R], d[index]);
    } else if (u == C - 1) {
        L.dcu_aux[index] = sub(c[index], c[index - R]);
        L.ddu_aux[index] = sub(d[index], d[index - R]);
    } else {
        L.dcu_aux[index] = wgrad(ri2[index], ri2[index - R], c[index + R], c[index], c[index - R]);
        L.ddu_aux[index] = (d[index] > 0.f) ? wgrad(ri2[index], ri2[index - R], d[index + R], d[index], d[index - R])
                                            : 0.f;
    }
    if (v == 0) {
        L.dcv_aux[index] = sub(c[index + 1], c[index]);
        L.ddv_aux[index] = sub(d[index + 1], d[index]);
    } else if (v == R - 1) {
        L.dcv_aux[index] = sub(c[index], c[index - 1]);
        L.ddv_aux[index] = sub(d[index], d[index - 1]);
    } else {
        L.dcv_aux[index] = wgrad(rj2[index], rj2[index - 1], c[index + 1], c[index], c[index - 1]);
        L.ddv_aux[index] = (d[index] > 0.f) ? wgrad(rj2[index], rj2[index - 1], d[index + 1], d[index], d[index - 1])
                                            : 0.f;
    }
}

// performWarping (pdflow_cudalib.cu:629-652) + computeMu/computeStepSizes (:781-808).
// steps = false: only mu of the step fields (the tile kernels recompute the
// step sizes from mu, ri, rj, ddu, ddv in registers); the free spd plane then
// holds powf(ddt, 2) for the level's median, so each pixel's square is taken
// once instead of once per neighbour.
__global__ void k_warp_steps(LevelGeom g, PyrLevel o, PyrLevel n, LevelConsts L, Params p, int steps)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    o = at(o, po);
    n = at(n, po);
    L = at(L, po);
    const unsigned index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= g.N) return;
    const unsigned R = g.R, C = g.C;
    const unsigned v = index % R, u = index / R;
    const float ind_uf = add(float(u), L.du_prev[index]);
    const float ind_vf = add(float(v), L.dv_prev[index]);
    // the five plain interpolations at one position share their case analysis
    const Bilin b = bilin(R, C, ind_uf, ind_vf);
    const float* const mats[5] = {n.col, L.dcu_aux, L.dcv_aux, L.ddu_aux, L.ddv_aux};
    float w5[5];
    bilin_blend_n<5>(mats, R, b, w5);
    const float dct = sub(w5[0], o.col[index]);
    const float dcu = w5[1], dcv = w5[2], ddu = w5[3], ddv = w5[4];
    const float wz = interp_depth_at(n.dep, R, b);
    const float ddt = (wz > 0.f) ? sub(wz, o.dep[index]) : 0.f;
    L.dct[index] = dct;
    L.dcu[index] = dcu;
    L.dcv[index] = dcv;
    L.ddt[index] = ddt;
    L.ddu[index] = ddu;
    L.ddv[index] = ddv;
    if (steps == kStepsNone) {
        L.mu[index] = data_weight(p.mu, ddu, ddv, ddt);
        L.spd[index] = powf(ddt, 2.f);
        return;
    }
    const float ri = L.ri[index], rj = L.rj[index];
    const float ri_m = (u > 0) ? L.ri[index - R] : 0.f;
    const float rj_m = (v > 0) ? L.rj[index - 1] : 0.f;
    const Steps s = mu_and_steps(p.mu, p.lambda_i, p.lambda_d, ddu, ddv, ddt, ri, rj, ri_m, rj_m, u > 0, v > 0);
    L.mu[index] = s.mu;
    if (steps == kStepsRaw || steps == kStepsAll) {
        L.spd[index] = s.spd;
        L.spuvx[index] = s.spuvx;
        L.spuvy[index] = s.spuvy;
        L.spwx[index] = s.spwx;
        L.spwy[index] = s.spwy;
        L.tu[index] = s.tu;
        L.tv[index] = s.tv;
        L.tw[index] = s.tw;
    } else {
        L.spd[index] = powf(ddt, 2.f);   // the median's depth-change weight
    }
    if (steps == kStepsQuads || steps == kStepsAll) {
        // the products the dual update forms (dual_update: mul(spd, mu), mul(spuvx, li), ...)
        L.qs[0][index] = mul(s.spd, s.mu);
        L.qs[1][index] = mul(s.spuvx, p.lambda_i);
        L.qs[2][index] = mul(s.spuvy, p.lambda_i);
        L.qs[3][index] = mul(s.spwx, p.lambda_d);
        L.qs[4][index] = mul(s.spwy, p.lambda_d);
        L.qs[5][index] = s.tu;
        L.qs[6][index] = s.tv;
        L.qs[7][index] = s.tw;
    }
}

// ---------------------------------------------------------------------------
// Iteration kernels
// ---------------------------------------------------------------------------
__global__ void k_dual(LevelGeom g, LevelConsts L, State S, Params p)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    L = at(L, po);
    S = at(S, po);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    const unsigned R = g.R, C = g.C;
    const unsigned v = i % R, u = i / R;
    const bool lu = (u == C - 1), lv = (v == R - 1);
    const unsigned iu = lu ? i : i + R, iv = lv ? i : i + 1;
    Duals d{S.pd[i], S.puu[i], S.puv[i], S.pvu[i], S.pvv[i], S.pwu[i], S.pwv[i]};
    dual_update(d, L.spd[i], L.spuvx[i], L.spuvy[i], L.spwx[i], L.spwy[i], L.mu[i], L.ddt[i], L.ddu[i], L.ddv[i],
                p.lambda_i, p.lambda_d, L.ri[i], L.rj[i], S.dua[i], S.dva[i], S.dwa[i], L.du_prev[i], L.dv_prev[i],
                S.dua[iu], S.dva[iu], S.dwa[iu], L.du_prev[iu], L.dv_prev[iu], S.dua[iv], S.dva[iv], S.dwa[iv],
                L.du_prev[iv], L.dv_prev[iv], lu, lv);
    S.pd[i] = d.pd;
    S.puu[i] = d.puu;
    S.puv[i] = d.puv;
    S.pvu[i] = d.pvu;
    S.pvv[i] = d.pvv;
    S.pwu[i] = d.pwu;
    S.pwv[i] = d.pwv;
}

__global__ void k_primal(LevelGeom g, LevelConsts L, State S, Params p, bool last, const float* depth_old)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    L = at(L, po);
    S = at(S, po);
    depth_old = at(depth_old, po);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    const unsigned R = g.R, C = g.C;
    const unsigned v = i % R, u = i / R;
    const bool fu = (u == 0), lu = (u == C - 1), fv = (v == 0), lv = (v == R - 1);
    const unsigned im = fu ? i : i - R, jm = fv ? i : i - 1;
    const float ri = L.ri[i], rj = L.rj[i], ri_m = L.ri[im], rj_m = L.rj[jm];
    const float divu = divergence(ri, ri_m, rj, rj_m, S.puu[i], S.puu[im], S.puv[i], S.puv[jm], fu, lu, fv, lv);
    const float divv = divergence(ri, ri_m, rj, rj_m, S.pvu[i], S.pvu[im], S.pvv[i], S.pvv[jm], fu, lu, fv, lv);
    const float divw = divergence(ri, ri_m, rj, rj_m, S.pwu[i], S.pwu[im], S.pwv[i], S.pwv[jm], fu, lu, fv, lv);
    float du = S.du[i], dv = S.dv[i], dw = S.dw[i], dua, dva, dwa;
    primal_update(du, dv, dw, dua, dva, dwa, L.tu[i], L.tv[i], L.tw[i], L.mu[i], L.ddu[i], L.ddv[i], S.pd[i],
                  p.lambda_i, p.lambda_d, divu, divv, divw, L.dct[i], L.dcu[i], L.dcv[i]);
    if (last) {
        saturate(du, dv, dw, L.du_prev[i], L.dv_prev[i], depth_old[i]);
    } else {
        S.dua[i] = dua;
        S.dva[i] = dva;
        S.dwa[i] = dwa;
    }
    S.du[i] = du;
    S.dv[i] = dv;
    S.dw[i] = dw;
}

// saturateVariables alone, for a level scheduled with zero iterations.
__global__ void k_saturate(LevelGeom g, LevelConsts L, State S, const float* depth_old)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    L = at(L, po);
    S = at(S, po);
    depth_old = at(depth_old, po);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    float du = S.du[i], dv = S.dv[i], dw = S.dw[i];
    saturate(du, dv, dw, L.du_prev[i], L.dv_prev[i], depth_old[i]);
    S.du[i] = du;
    S.dv[i] = dv;
    S.dw[i] = dw;
}

// ---------------------------------------------------------------------------
// filterSolution (pdflow_cudalib.cu:1040-1148) + computeMotionField (:1150-1167)
// ---------------------------------------------------------------------------
// Weighted median of up to 9 samples, register resident (the reference
// accumulates the weights in sorted order and walks to the first cumulative
// weight >= med, pdflow_cudalib.cu:1083-1132).
//
// Stable sort of up to 9 samples (the reference's bubbleSortDev,
// pdflow_cudalib.cu:1457-1473, swaps only on a strict '>', so equal values
// keep their input order) as an odd-even transposition network: 9 rounds of
// exchanges between neighbours (i, i+1), i of the round's parity, each on a
// strict '<'.  It sorts every 0/1 input and hence every input, and equal
// values never pass each other, so the order is the stable one.  Missing
// samples (n < 9) enter as (+inf, weight 0) after the present ones and stay
// there.  Then the cumulative weights are summed in sorted order, as the
// reference does, and the bracketing samples are interpolated; the result and
// the selected index are the reference's bit for bit.  Every index is a
// compile-time constant: nothing spills.
__device__ __forceinline__ float median9(const float (&f)[9], const float (&w)[9], unsigned present,
                                         float med_or_neg, float* total, int32_t* cont_out)
{
    // the samples in tap order, a missing one (bit clear in `present`) as +inf
    // of weight 0: the stable sort keeps the present samples in their order
    // and puts the missing ones after them, so its first n entries are those
    // of the reference's sort of the n present samples
    float sf[9], sw[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const bool in = (present >> i) & 1u;
        sf[i] = in ? f[i] : INFINITY;
        sw[i] = in ? w[i] : 0.f;
    }
    // odd-even transposition sort: 9 rounds of adjacent exchanges on a strict
    // '<', so equal values never pass each other and the order is the stable
    // one of the reference's bubble sort, without carrying input indices
#pragma unroll
    for (int r = 0; r < 9; ++r)
#pragma unroll
        for (int a = r & 1; a + 1 < 9; a += 2) {
            const bool sw_ = sf[a + 1] < sf[a];
            const float tf = sf[a], tw = sw[a];
            sf[a] = sw_ ? sf[a + 1] : sf[a];
            sw[a] = sw_ ? sw[a + 1] : sw[a];
            sf[a + 1] = sw_ ? tf : sf[a + 1];
            sw[a + 1] = sw_ ? tw : sw[a + 1];
        }
    // cumulative weights; the missing samples (weight +0, sorted last) leave
    // the sum as it is (x + 0 == x for the non-negative sums), so cum[8] is
    // the reference's cum[n - 1]
    float cum[9];
    cum[0] = sw[0];
#pragma unroll
    for (int r = 1; r < 9; ++r) cum[r] = add(cum[r - 1], sw[r]);
    *total = cum[8];
    const float med = (med_or_neg < 0.f) ? mul(0.5f, cum[8]) : med_or_neg;
    // the reference counts the samples with med > cum (among the present
    // ones: a missing one's cum is the total, never below med) and
    // interpolates between that sample and the one before; cum does not
    // decrease, so the counted samples are a prefix and one pass finds both
    int cont = 0;
    float cr = 0.f, cl = 0.f, fr = 0.f, fl = 0.f;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const bool t = med > cum[r];
        cont = t ? r + 1 : cont;
        cl = t ? cum[r] : cl;
        fl = t ? sf[r] : fl;
        cr = t ? cum[r + 1] : cr;
        fr = t ? sf[r + 1] : fr;
    }
    if (med > cum[8]) {   // past every sample: the reference finds no bracket
        cont = 9;
        cr = cl = fr = fl = 0.f;
    }
    *cont_out = cont;
    if (cont == 0) return sf[0];
    return median_lerp(cr, cl, med, fl, fr);
}

// The median's pixels in tiles of kMedRows x kMedCols (rows along
// threadIdx.x, so a warp's loads are one column's consecutive rows): the
// block first stages its tile and a one-pixel halo of the five planes the
// taps read, then every pixel takes its nine taps from shared memory at
// fixed offsets (outside the image the halo holds zeros; those taps are
// missing in `present` and never reach the median).
constexpr int kMedRows = 32, kMedCols = 8;
constexpr int kMedHR = kMedRows + 2, kMedHC = kMedCols + 2;

template <bool kDdtSq>   // L.spd holds powf(ddt, 2) (levels run as tiles)
__global__ void __launch_bounds__(kMedRows * kMedCols) k_median(LevelGeom g, bool finest, PyrLevel o, LevelConsts L,
                                                               State S, State Salt, LevelSol out, float* dx,
                                                               float* dy, float* dz, Params p, int32_t* sel)
{
    __shared__ float t_dep[kMedHC][kMedHR], t_sq[kMedHC][kMedHR], t_du[kMedHC][kMedHR], t_dv[kMedHC][kMedHR],
        t_dw[kMedHC][kMedHR];
    const size_t po = pair_off(g.map, g.pstride, blockIdx.z);
    const unsigned pf = pair_flags(g.map, blockIdx.z);
    finest = finest || (pf & kMapFinest);
    o = at(o, po);
    L = at(L, po);
    S = at((pf & kMapAlt) ? Salt : S, po);
    out = at(out, po);
    dx = at(dx, po);
    dy = at(dy, po);
    dz = at(dz, po);
    const int R = (int)g.R, C = (int)g.C;
    const int v0 = (int)blockIdx.x * kMedRows, u0 = (int)blockIdx.y * kMedCols;
    // the tile and its halo: rows v0-1 .. v0+kMedRows, columns u0-1 .. u0+kMedCols
    for (int e = threadIdx.y * kMedRows + threadIdx.x; e < kMedHR * kMedHC; e += kMedRows * kMedCols) {
        const int hr = e % kMedHR, hc = e / kMedHR, gv = v0 - 1 + hr, gu = u0 - 1 + hc;
        float z = 0.f, q = 0.f, a = 0.f, b = 0.f, c = 0.f;
        if (gv >= 0 && gv < R && gu >= 0 && gu < C) {
            const int j = gv + gu * R;
            z = o.dep[j];
            q = kDdtSq ? L.spd[j] : powf(L.ddt[j], 2.f);
            a = S.du[j];
            b = S.dv[j];
            c = S.dw[j];
        }
        t_dep[hc][hr] = z;
        t_sq[hc][hr] = q;
        t_du[hc][hr] = a;
        t_dv[hc][hr] = b;
        t_dw[hc][hr] = c;
    }
    __syncthreads();
    const int tv = (int)threadIdx.x, tu = (int)threadIdx.y;
    const int v = v0 + tv, u = u0 + tu;
    if (v >= R || u >= C) return;
    const unsigned index = (unsigned)(v + u * R);
    const float depth_old = t_dep[tu + 1][tv + 1];
    float ru, rv, rw;
    if (depth_old > 0.f) {
        // the nine taps in the reference's order (row offset, then column);
        // taps outside the image are marked missing (median9)
        unsigned present = 0x1ffu;
        if (v == 0) present &= ~0x007u;       // row offset -1: taps 0, 1, 2
        if (v == R - 1) present &= ~0x1c0u;   // row offset +1: taps 6, 7, 8
        if (u == 0) present &= ~0x049u;       // column offset -1: taps 0, 3, 6
        if (u == C - 1) present &= ~0x124u;   // column offset +1: taps 2, 5, 8
        float fu[9], fv[9], fw[9], wt[9];
#pragma unroll
        for (int k = -1; k < 2; k++)
#pragma unroll
            for (int l = -1; l < 2; l++) {
                const int q = 3 * (k + 1) + (l + 1);
                const int hc = tu + 1 + l, hr = tv + 1 + k;
                const float dz2 = (q == 4) ? pow2_diff_voted(depth_old, t_dep[hc][hr])   // the centre: z0 - z0
                                           : powf(sub(depth_old, t_dep[hc][hr]), 2.f);
                wt[q] = __frcp_rn(fm(10.f, t_sq[hc][hr], fm(5.f, dz2, 1.f)));
                fu[q] = t_du[hc][hr];
                fv[q] = t_dv[hc][hr];
                fw[q] = t_dw[hc][hr];
            }
        float tot;
        int32_t c0, c1, c2;
        ru = median9(fu, wt, present, -1.f, &tot, &c0);
        const float pres_med = mul(0.5f, tot);   // half of u's total, for all three (:1097)
        rv = median9(fv, wt, present, pres_med, &tot, &c1);
        rw = median9(fw, wt, present, pres_med, &tot, &c2);
        if (sel) { sel[index] = c0; sel[g.N + index] = c1; sel[2 * g.N + index] = c2; }
    } else {
        ru = t_du[tu + 1][tv + 1];
        rv = t_dv[tu + 1][tv + 1];
        rw = t_dw[tu + 1][tv + 1];
        if (sel) { sel[index] = -1; sel[g.N + index] = -1; sel[2 * g.N + index] = -1; }
    }
    out.du[index] = ru;
    out.dv[index] = rv;
    out.dw[index] = rw;
    if (!out.pd) return;  // stage form: no duals to carry
    out.pd[index] = S.pd[index];
    out.puu[index] = S.puu[index];
    out.puv[index] = S.puv[index];
    out.pvu[index] = S.pvu[index];
    out.pvv[index] = S.pvv[index];
    out.pwu[index] = S.pwu[index];
    out.pwv[index] = S.pwv[index];
    if (finest) {
        if (depth_old > 0) {
            // the finest level is cols wide (g.C == p.cols), also for a mixed batch's smaller pairs
            motion_field(depth_old, ru, rv, rw, o.xx[index], o.yy[index], inv_focal(p.fovh, g.C), dx[index],
                         dy[index], dz[index]);
        } else {
            dx[index] = 0.f;
            dy[index] = 0.f;
            dz[index] = 0.f;
        }
    }
}

// Per-level record of a solve (copyAllSolutions of the live application,
// called after every level: scene_flow_visualization.cpp:194-199).
__global__ void k_level_keep(LevelGeom g, LevelSol sol, PyrLevel o, Params p, float* __restrict__ keep,
                             size_t stride, size_t off)
{
    const unsigned y = blockIdx.y;
    const size_t po = pair_off(g.map, g.pstride, y);
    const unsigned slot = g.map ? (__ldg(g.map + y) & kMapSlotMask) : y;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    sol = at(sol, po);
    o = at(o, po);
    float* k = keep + (size_t)slot * stride + off;
    const float du = sol.du[i], dv = sol.dv[i], dw = sol.dw[i];
    k[i] = du;
    k[g.N + i] = dv;
    k[2 * g.N + i] = dw;
    const float z = o.dep[i];
    float dx = 0.f, dy = 0.f, dz = 0.f;
    if (z > 0.f) motion_field(z, du, dv, dw, o.xx[i], o.yy[i], inv_focal(p.fovh, p.cols), dx, dy, dz);
    k[3 * g.N + i] = dx;
    k[4 * g.N + i] = dy;
    k[5 * g.N + i] = dz;
}

// Frame t's pyramid level becomes frame t-1's, for the mapped slots (float4
// copies; level planes are 16-byte aligned and padded to whole float4s).
__global__ void k_pyr_copy(PyrLevel src, PyrLevel dst, unsigned n, size_t pstride, const unsigned* __restrict__ map)
{
    const size_t po = pair_off(map, pstride, blockIdx.y);
    src = at(src, po);
    dst = at(dst, po);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (4 * i >= n) return;
    if (4 * i + 4 <= n) {
        reinterpret_cast<float4*>(dst.col)[i] = reinterpret_cast<const float4*>(src.col)[i];
        reinterpret_cast<float4*>(dst.dep)[i] = reinterpret_cast<const float4*>(src.dep)[i];
        reinterpret_cast<float4*>(dst.xx)[i] = reinterpret_cast<const float4*>(src.xx)[i];
        reinterpret_cast<float4*>(dst.yy)[i] = reinterpret_cast<const float4*>(src.yy)[i];
    } else {
        for (unsigned k = 4 * i; k < n; ++k) {
            dst.col[k] = src.col[k];
            dst.dep[k] = src.dep[k];
            dst.xx[k] = src.xx[k];
            dst.yy[k] = src.yy[k];
        }
    }
}

// The warp point of the energy: the solution's total image-plane flow.
__global__ void k_energy_prep(LevelGeom g, LevelSol sol, LevelConsts L)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    at(L.du_prev, po)[i] = at(sol.du, po)[i];
    at(L.dv_prev, po)[i] = at(sol.dv, po)[i];
}

// 1024 accumulators per pair: accumulator t sums pixels t, t + 1024, ... in
// that order (32 one-warp CTAs per pair, so the FP64 work of one pair spreads
// over 32 SMs); k_energy_sum then adds the 1024 partial sums of a pair in a
// fixed tree, so the energy is deterministic and independent of the batch.
// With du = dv = 0 increments at the warp point the linearised data terms
// equal the warped residuals.
constexpr unsigned kEnergyAcc = 1024;

__global__ void __launch_bounds__(32) k_energy(LevelGeom g, LevelSol sol, LevelConsts L, Params p,
                                               double* __restrict__ part)
{
    const size_t po = pair_off(g.map, g.pstride, blockIdx.y);
    sol = at(sol, po);
    L = at(L, po);
    const unsigned R = g.R, C = g.C;
    const unsigned t = blockIdx.x * 32 + threadIdx.x;
    double acc = 0.0;
    for (unsigned i = t; i < g.N; i += kEnergyAcc) {
        const unsigned v = i % R, u = i / R;
        const float U = sol.du[i], V = sol.dv[i], W = sol.dw[i], ri = L.ri[i], rj = L.rj[i];
        const bool lu = u == C - 1, lv = v == R - 1;
        const float gu1 = lu ? 0.f : mul(ri, sub(sol.du[i + R], U)), gu2 = lv ? 0.f : mul(rj, sub(sol.du[i + 1], U));
        const float gv1 = lu ? 0.f : mul(ri, sub(sol.dv[i + R], V)), gv2 = lv ? 0.f : mul(rj, sub(sol.dv[i + 1], V));
        const float gw1 = lu ? 0.f : mul(ri, sub(sol.dw[i + R], W)), gw2 = lv ? 0.f : mul(rj, sub(sol.dw[i + 1], W));
        double e = fabs((double)L.dct[i]) + (double)L.mu[i] * fabs((double)L.ddt[i] - (double)W);
        e += (double)p.lambda_i * (hypot((double)gu1, (double)gu2) + hypot((double)gv1, (double)gv2));
        e += (double)p.lambda_d * hypot((double)gw1, (double)gw2);
        acc += e;
    }
    part[(size_t)blockIdx.y * kEnergyAcc + t] = acc;
}

__global__ void __launch_bounds__(kEnergyAcc) k_energy_sum(const double* __restrict__ part,
                                                           float* __restrict__ energies)
{
    __shared__ double red[kEnergyAcc];
    red[threadIdx.x] = part[(size_t)blockIdx.y * kEnergyAcc + threadIdx.x];
    __syncthreads();
    for (unsigned w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) energies[blockIdx.y] = (float)red[0];
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
cudaError_t launch_decode_u16(const uint8_t* img, const uint16_t* depth, unsigned W, unsigned H, PyrLevel out,
                              float fovh, unsigned pairs, size_t pstride, cudaStream_t st, const unsigned* map)
{
    dim3 grid((W + 31) / 32, (H + 31) / 32, pairs), block(32, 32);
    k_decode_u16<<<grid, block, 0, st>>>(img, depth, W, H, out, fovh, pstride, map);
    return cudaGetLastError();
}

cudaError_t launch_decode_rgb8_mm(const uint8_t* rgb, const uint16_t* depth, unsigned W, unsigned H, PyrLevel out,
                                  float fovh, unsigned pairs, size_t pstride, cudaStream_t st, int rotate180)
{
    dim3 grid((W + 31) / 32, (H + 31) / 32, pairs), block(32, 32);
    k_decode_rgb8_mm<<<grid, block, 0, st>>>(rgb, depth, W, H, out, fovh, pstride, nullptr, rotate180);
    return cudaGetLastError();
}

cudaError_t launch_pyr_level0(const float* I, const float* Z, unsigned R, unsigned C, PyrLevel out, float fovh,
                              unsigned pairs, size_t pstride, cudaStream_t st, const unsigned* map)
{
    k_pyr_level0<<<dim3(blocks_for(R * C), pairs), kBlock, 0, st>>>(I, Z, R, C, out, fovh, pstride, map);
    return cudaGetLastError();
}

cudaError_t launch_pyr_down(PyrLevel prev, unsigned R, unsigned C, PyrLevel out, float fovh, unsigned pairs,
                            size_t pstride, cudaStream_t st, const unsigned* map)
{
    k_pyr_down<<<dim3(blocks_for(R * C), pairs), kBlock, 0, st>>>(prev, R, C, out, fovh, pstride, map);
    return cudaGetLastError();
}

cudaError_t launch_pyr_copy(PyrLevel src, PyrLevel dst, unsigned n, unsigned pairs, size_t pstride,
                            const unsigned* map, cudaStream_t st)
{
    k_pyr_copy<<<dim3(blocks_for((n + 3) / 4), pairs), kBlock, 0, st>>>(src, dst, n, pstride, map);
    return cudaGetLastError();
}

static dim3 level_grid(const LevelGeom& g) { return dim3(blocks_for(g.N), g.pairs); }

cudaError_t launch_level_init(LevelGeom g, bool first, LevelSol coarse, PyrLevel old_l, PyrLevel new_l,
                              LevelConsts L, State S, cudaStream_t st, const float* seed)
{
    if (!first && !seed && g.R % 2 == 0)
        k_level_init_pairs<<<dim3(blocks_for(g.N / 2), g.pairs), kBlock, 0, st>>>(g, coarse, old_l, new_l, L, S);
    else
        k_level_init<<<level_grid(g), kBlock, 0, st>>>(g, first, coarse, old_l, new_l, L, S, seed);
    return cudaGetLastError();
}

cudaError_t launch_im_gradients(LevelGeom g, PyrLevel new_l, LevelConsts L, cudaStream_t st)
{
    k_im_gradients<<<level_grid(g), kBlock, 0, st>>>(g, new_l, L);
    return cudaGetLastError();
}

cudaError_t launch_warp_steps(LevelGeom g, PyrLevel old_l, PyrLevel new_l, LevelConsts L, Params p, cudaStream_t st,
                              int steps)
{
    k_warp_steps<<<level_grid(g), kBlock, 0, st>>>(g, old_l, new_l, L, p, steps);
    return cudaGetLastError();
}

cudaError_t launch_dual(LevelGeom g, LevelConsts L, State S, Params p, cudaStream_t st)
{
    k_dual<<<level_grid(g), kBlock, 0, st>>>(g, L, S, p);
    return cudaGetLastError();
}

cudaError_t launch_primal(LevelGeom g, LevelConsts L, State S, Params p, bool last, const float* depth_old,
                          cudaStream_t st)
{
    k_primal<<<level_grid(g), kBlock, 0, st>>>(g, L, S, p, last, depth_old);
    return cudaGetLastError();
}

cudaError_t launch_saturate(LevelGeom g, LevelConsts L, State S, const float* depth_old, cudaStream_t st)
{
    k_saturate<<<level_grid(g), kBlock, 0, st>>>(g, L, S, depth_old);
    return cudaGetLastError();
}

cudaError_t launch_level_keep(LevelGeom g, LevelSol sol, PyrLevel old_l, Params p, float* keep, size_t stride,
                              size_t off, cudaStream_t st)
{
    k_level_keep<<<level_grid(g), kBlock, 0, st>>>(g, sol, old_l, p, keep, stride, off);
    return cudaGetLastError();
}

cudaError_t launch_median(LevelGeom g, bool finest, PyrLevel old_l, LevelConsts L, State S, LevelSol out, float* dx,
                          float* dy, float* dz, Params p, int32_t* sel, cudaStream_t st, const State* alt,
                          bool ddt_sq)
{
    const dim3 grid((g.R + kMedRows - 1) / kMedRows, (g.C + kMedCols - 1) / kMedCols, g.pairs);
    const dim3 block(kMedRows, kMedCols);
    if (ddt_sq)
        k_median<true><<<grid, block, 0, st>>>(g, finest, old_l, L, S, alt ? *alt : S, out, dx, dy, dz, p, sel);
    else
        k_median<false><<<grid, block, 0, st>>>(g, finest, old_l, L, S, alt ? *alt : S, out, dx, dy, dz, p, sel);
    return cudaGetLastError();
}

cudaError_t launch_energy_prep(LevelGeom g, LevelSol sol, LevelConsts L, cudaStream_t st)
{
    k_energy_prep<<<level_grid(g), kBlock, 0, st>>>(g, sol, L);
    return cudaGetLastError();
}

cudaError_t launch_energy(LevelGeom g, LevelSol sol, LevelConsts L, Params p, float* energies, double* part,
                          cudaStream_t st)
{
    k_energy<<<dim3(kEnergyAcc / 32, g.pairs), 32, 0, st>>>(g, sol, L, p, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_energy_sum<<<dim3(1, g.pairs), kEnergyAcc, 0, st>>>(part, energies);
    return cudaGetLastError();
}

}  // namespace pdflow
