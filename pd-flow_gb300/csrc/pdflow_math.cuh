// Per-pixel arithmetic of the PD-Flow solver, shared by every kernel form.
//
// Each function restates one per-pixel step of the reference
// (pdflow_cudalib.cu) as a pure function of the values it reads, so that the
// kernels are free to stage those values in registers, shared memory or L2.
// Expressions keep the reference's operand order and call the same device
// intrinsics (fdividef, rhypotf, powf, __float2int_r*), so that nvcc forms the
// same fused multiply-adds and the results track the reference's own CUDA
// path, not just the mathematics.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace pdflow {

// 5x5 binomial mask (1,4,6,4,1)x(1,4,6,4,1)/256 (scene_flow_impair.cpp:55-58),
// indexed [2+k + 5*(2+l)] for row offset k and column offset l.
__device__ __forceinline__ float gmask(int k, int l)
{
    const int a = (k == 0) ? 6 : ((k == 1 || k == -1) ? 4 : 1);
    const int b = (l == 0) ? 6 : ((l == 1 || l == -1) ? 4 : 1);
    return float(a * b) / 256.f;
}

// Depth decode of the reference's loader: uint16 * (float)(1/5000)
// (scene_flow_impair.cpp:242, :269 via OpenCV convertTo). Exact product, rounded once.
__device__ __forceinline__ float decode_depth(unsigned short d)
{
    return __fmul_rn(float(d), 0.0002f);
}

// Connectivity weight of computeRij (pdflow_cudalib.cu:760-778).
__device__ __forceinline__ float rfac(float a, float b)
{
    return (fabsf(a) + fabsf(b) > 0.f) ? 2.f * rhypotf(a, b) : 1.f;
}

// interpolatePixel (pdflow_cudalib.cu:654-682) over a column-major plane.
__device__ __forceinline__ float interp(const float* __restrict__ mat, unsigned R, unsigned C, float ind_u,
                                        float ind_v)
{
    if (ind_u < 0.f) ind_u = 0.f;
    else if (ind_u > C - 1.f) ind_u = C - 1.f;
    if (ind_v < 0.f) ind_v = 0.f;
    else if (ind_v > R - 1.f) ind_v = R - 1.f;
    const unsigned sup_u = __float2int_ru(ind_u);
    const unsigned inf_u = __float2int_rd(ind_u);
    const unsigned sup_v = __float2int_ru(ind_v);
    const unsigned inf_v = __float2int_rd(ind_v);
    if ((sup_u == inf_u) && (sup_v == inf_v)) return mat[lrintf(ind_v + R * ind_u)];
    if (sup_u == inf_u)
        return (sup_v - ind_v) * mat[inf_v + R * lrintf(ind_u)] + (ind_v - inf_v) * mat[sup_v + R * lrintf(ind_u)];
    if (sup_v == inf_v)
        return (sup_u - ind_u) * mat[lrintf(ind_v) + R * inf_u] + (ind_u - inf_u) * mat[lrintf(ind_v) + R * sup_u];
    const float val_sup_v = (sup_u - ind_u) * mat[sup_v + R * inf_u] + (ind_u - inf_u) * mat[sup_v + R * sup_u];
    const float val_inf_v = (sup_u - ind_u) * mat[inf_v + R * inf_u] + (ind_u - inf_u) * mat[inf_v + R * sup_u];
    return (sup_v - ind_v) * val_inf_v + (ind_v - inf_v) * val_sup_v;
}

// interpolatePixelDepth (pdflow_cudalib.cu:684-721): nearest sample when any
// of the four taps is a hole.
__device__ __forceinline__ float interp_depth(const float* __restrict__ mat, unsigned R, unsigned C, float ind_u,
                                              float ind_v)
{
    if (ind_u < 0.f) ind_u = 0.f;
    else if (ind_u > C - 1.f) ind_u = C - 1.f;
    if (ind_v < 0.f) ind_v = 0.f;
    else if (ind_v > R - 1.f) ind_v = R - 1.f;
    const unsigned sup_u = __float2int_ru(ind_u);
    const unsigned inf_u = __float2int_rd(ind_u);
    const unsigned sup_v = __float2int_ru(ind_v);
    const unsigned inf_v = __float2int_rd(ind_v);
    if ((mat[sup_v + R * sup_u] == 0.f) || (mat[sup_v + R * inf_u] == 0.f) || (mat[inf_v + R * sup_u] == 0.f) ||
        (mat[inf_v + R * inf_u] == 0.f)) {
        const unsigned rind_u = __float2int_rn(ind_u);
        const unsigned rind_v = __float2int_rn(ind_v);
        return mat[rind_v + R * rind_u];
    }
    if ((sup_u == inf_u) && (sup_v == inf_v)) return mat[lrintf(ind_v + R * ind_u)];
    if (sup_u == inf_u)
        return (sup_v - ind_v) * mat[inf_v + R * lroundf(ind_u)] + (ind_v - inf_v) * mat[sup_v + R * lroundf(ind_u)];
    if (sup_v == inf_v)
        return (sup_u - ind_u) * mat[lroundf(ind_v) + R * inf_u] + (ind_u - inf_u) * mat[lroundf(ind_v) + R * sup_u];
    const float val_sup_v = (sup_u - ind_u) * mat[sup_v + R * inf_u] + (ind_u - inf_u) * mat[sup_v + R * sup_u];
    const float val_inf_v = (sup_u - ind_u) * mat[inf_v + R * inf_u] + (ind_u - inf_u) * mat[inf_v + R * sup_u];
    return (sup_v - ind_v) * val_inf_v + (ind_v - inf_v) * val_sup_v;
}

// Step sizes of computeMu + computeStepSizes (pdflow_cudalib.cu:781-808).
struct Steps {
    float mu, spd, spuvx, spuvy, spwx, spwy, tu, tv, tw;
};

__device__ __forceinline__ Steps mu_and_steps(float mu_p, float li, float ld, float ddu, float ddv, float ddt, float ri,
                                              float rj, float ri_um1, float rj_vm1, bool has_um1, bool has_vm1)
{
    Steps s;
    s.mu = fdividef(mu_p, 1.f + 1000.f * (ddu * ddu + ddv * ddv + ddt * ddt));
    s.spd = fdividef(1.f, s.mu * (1.f + fabsf(ddu) + fabsf(ddv)) + 1e-10f);
    s.spuvx = fdividef(0.5f, li * ri + 1e-10f);
    s.spuvy = fdividef(0.5f, li * rj + 1e-10f);
    s.spwx = fdividef(0.5f, ri * ld + 1e-10f);
    s.spwy = fdividef(0.5f, rj * ld + 1e-10f);
    float acu_r = ri + rj;
    if (has_um1) acu_r += ri_um1;
    if (has_vm1) acu_r += rj_vm1;
    s.tu = fdividef(1.f, s.mu * fabsf(ddu) + li * acu_r + 1e-10f);
    s.tv = fdividef(1.f, s.mu * fabsf(ddv) + li * acu_r + 1e-10f);
    s.tw = fdividef(1.f, s.mu + ld * acu_r + 1e-10f);
    return s;
}

// Dual step: computeGradient (pdflow_cudalib.cu:982-1013) then
// updateDualVariables (:813-887) at one pixel.  `*_u1` are the values at
// (v, u+1), `*_v1` at (v+1, u); last_u / last_v mark the far borders where
// the forward difference is zero.
struct Duals {
    float pd, puu, puv, pvu, pvv, pwu, pwv;
};

__device__ __forceinline__ void dual_update(Duals& p, float spd, float spuvx, float spuvy, float spwx, float spwy,
                                            float mu, float ddt, float ddu, float ddv, float li, float ld, float ri,
                                            float rj, float dua, float dva, float dwa, float dup, float dvp,
                                            float dua_u1, float dva_u1, float dwa_u1, float dup_u1, float dvp_u1,
                                            float dua_v1, float dva_v1, float dwa_v1, float dup_v1, float dvp_v1,
                                            bool last_u, bool last_v)
{
    float gu1, gv1, gw1, gu2, gv2, gw2;
    if (last_u) {
        gu1 = 0.f; gv1 = 0.f; gw1 = 0.f;
    } else {
        gu1 = ri * ((dua_u1 + dup_u1) - (dua + dup));
        gv1 = ri * ((dva_u1 + dvp_u1) - (dva + dvp));
        gw1 = ri * (dwa_u1 - dwa);
    }
    if (last_v) {
        gu2 = 0.f; gv2 = 0.f; gw2 = 0.f;
    } else {
        gu2 = rj * ((dua_v1 + dup_v1) - (dua + dup));
        gv2 = rj * ((dva_v1 + dvp_v1) - (dva + dvp));
        gw2 = rj * (dwa_v1 - dwa);
    }
    float pd = p.pd, puu = p.puu, puv = p.puv, pvu = p.pvu, pvv = p.pvv, pwu = p.pwu, pwv = p.pwv;
    pd += spd * mu * (-dwa + ddt + ddu * dua + ddv * dva);
    puu += spuvx * li * gu1;
    puv += spuvy * li * gu2;
    pvu += spuvx * li * gv1;
    pvv += spuvy * li * gv2;
    pwu += spwx * ld * gw1;
    pwv += spwy * ld * gw2;
    float m = fabsf(pd);
    if (m > 1.f) p.pd = (pd > 1.f) ? 1.f : -1.f;
    else p.pd = pd;
    m = rhypotf(puu, puv);
    if (m < 1.f) { p.puu = puu * m; p.puv = puv * m; }
    else { p.puu = puu; p.puv = puv; }
    m = rhypotf(pvu, pvv);
    if (m < 1.f) { p.pvu = pvu * m; p.pvv = pvv * m; }
    else { p.pvu = pvu; p.pvv = pvv; }
    m = rhypotf(pwu, pwv);
    if (m < 1.f) { p.pwu = pwu * m; p.pwv = pwv * m; }
    else { p.pwu = pwu; p.pwv = pwv; }
}

// Divergence term of computeDivergence (pdflow_cudalib.cu:935-980) for one
// component: (pu, pv) at the pixel, pu_um1 at (v, u-1), pv_vm1 at (v-1, u).
__device__ __forceinline__ float divergence(float ri, float ri_um1, float rj, float rj_vm1, float pu, float pu_um1,
                                            float pv, float pv_vm1, bool first_u, bool last_u, bool first_v,
                                            bool last_v)
{
    float d;
    if (first_u) d = ri * pu;
    else if (last_u) d = -ri_um1 * pu_um1;
    else d = ri * pu - ri_um1 * pu_um1;
    if (first_v) d += rj * pv;
    else if (last_v) d += -rj_vm1 * pv_vm1;
    else d += rj * pv - rj_vm1 * pv_vm1;
    return d;
}

// Primal step updatePrimalVariables (pdflow_cudalib.cu:889-933): explicit step,
// L1 photometric shrinkage and over-relaxation.  du/dv/dw are updated in
// place; the over-relaxed values are returned in dua/dva/dwa.
__device__ __forceinline__ void primal_update(float& du, float& dv, float& dw, float& dua, float& dva, float& dwa,
                                              float tu, float tv, float tw, float mu, float ddu, float ddv, float pd,
                                              float li, float ld, float divu, float divv, float divw, float dct,
                                              float dcu, float dcv)
{
    const float du_old = du, dv_old = dv, dw_old = dw;
    du += -tu * (mu * ddu * pd - li * divu);
    dv += -tv * (mu * ddv * pd - li * divv);
    dw += -tw * (-mu * pd - ld * divw);
    const float optflow = dct + dcu * du + dcv * dv;
    const float of_threshold = tu * dcu * dcu + tv * dcv * dcv;
    if (optflow < -of_threshold) {
        du += tu * dcu;
        dv += tv * dcv;
    } else if (optflow > of_threshold) {
        du -= tu * dcu;
        dv -= tv * dcv;
    } else {
        const float den = tu * dcu * dcu + tv * dcv * dcv + 1e-10f;
        du -= tu * dcu * optflow / den;
        dv -= tv * dcv * optflow / den;
    }
    dua = 2.f * du - du_old;
    dva = 2.f * dv - dv_old;
    dwa = 2.f * dw - dw_old;
}

// saturateVariables (pdflow_cudalib.cu:1018-1038).
__device__ __forceinline__ void saturate(float& du, float& dv, float& dw, float du_prev, float dv_prev,
                                         float depth_old)
{
    if (du > 1.f) du = 1.f;
    else if (du < -1.f) du = -1.f;
    if (dv > 1.f) dv = 1.f;
    else if (dv < -1.f) dv = -1.f;
    if (depth_old == 0.f) dw = 0.f;
    du = du + du_prev;
    dv = dv + dv_prev;
}

}  // namespace pdflow
