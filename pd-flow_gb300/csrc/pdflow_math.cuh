// Per-pixel arithmetic of the PD-Flow solver, shared by every kernel form.
//
// Each function restates one per-pixel step of the reference
// (pdflow_cudalib.cu) as a pure function of the values it reads, so that the
// kernels are free to stage those values in registers, shared memory or L2.
//
// Bit-exactness.  The reference's kernels are plain C++ expressions that nvcc
// contracts into fused multiply-adds as it sees fit; where an expression adds
// two products (a*b + c*d) or a product with several uses, the contraction it
// picks decides the last bit, and over hundreds of non-smooth iterations the
// last bit decides branch outcomes.  Every operation below is therefore
// written with an explicit rounding intrinsic (__fmaf_rn, __fmul_rn,
// __fadd_rn, ...; nvcc never re-associates or fuses these), in the form the
// reference's own build (nvcc 13.0, sm_103a) produces for that expression.
// Those forms were identified by replaying the reference's per-level and
// per-iteration state; with them the solver reproduces the reference's output
// bit for bit (tests/test_gpu_parity.py).  Where the reference calls a device
// intrinsic (fdividef, rhypotf, powf, tanf, __float2int_r*) it is called
// here too.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace pdflow {

__device__ __forceinline__ float fm(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float qt(float a, float b) { return __fdiv_rn(a, b); }

// 5x5 binomial mask (1,4,6,4,1)x(1,4,6,4,1)/256 (scene_flow_impair.cpp:55-58),
// for row offset k and column offset l in [-2, 2].
__device__ __forceinline__ float gmask(int k, int l)
{
    const int a = (k == 0) ? 6 : ((k == 1 || k == -1) ? 4 : 1);
    const int b = (l == 0) ? 6 : ((l == 1 || l == -1) ? 4 : 1);
    return float(a * b) / 256.f;   // exact
}

// Depth decode of the reference's loader: uint16 * (float)(1/5000)
// (scene_flow_impair.cpp:242, :269 via OpenCV convertTo). One rounding.
__device__ __forceinline__ float decode_depth(unsigned short d) { return __fmul_rn(float(d), 0.0002f); }

// The live application's conversion of an RGB-D camera's frames
// (scene_flow_visualization.cpp:320-321): gray = 0.299 r + 0.587 g + 0.114 b
// evaluated in double, each product and sum rounded once, then rounded to
// float; depth = 0.001f * millimetres in float.
__device__ __forceinline__ float gray_rgb(unsigned r, unsigned g, unsigned b)
{
    const double s = __dadd_rn(__dadd_rn(__dmul_rn(0.299, double(r)), __dmul_rn(0.587, double(g))),
                               __dmul_rn(0.114, double(b)));
    return __double2float_rn(s);
}
__device__ __forceinline__ float decode_depth_mm(unsigned short d) { return __fmul_rn(0.001f, float(d)); }

// Focal factor 2*tan(fovh/2)/cols of computePyramidLevel (pdflow_cudalib.cu:428)
// and computeMotionField (:1152).
__device__ __forceinline__ float inv_focal(float fovh, unsigned cols)
{
    return qt(mul(2.f, tanf(mul(0.5f, fovh))), float(cols));
}

// Back-projection (pdflow_cudalib.cu:428-433): ((u - (C-1)/2) * z) * inv_f.
__device__ __forceinline__ float backproject(unsigned u, unsigned C, float z, float inv_f)
{
    return mul(mul(sub(float(u), mul(0.5f, float(C - 1))), z), inv_f);
}

// Connectivity weight of computeRij (pdflow_cudalib.cu:760-778).
__device__ __forceinline__ float rfac(float a, float b)
{
    return (add(fabsf(a), fabsf(b)) > 0.f) ? mul(2.f, rhypotf(a, b)) : 1.f;
}

// Interpolation weights / taps of interpolatePixel (pdflow_cudalib.cu:654-682).
struct Bilin {
    float iu, iv;
    unsigned su, fu, sv, fv;
};

__device__ __forceinline__ Bilin bilin(unsigned R, unsigned C, float ind_u, float ind_v)
{
    if (ind_u < 0.f) ind_u = 0.f;
    else if (ind_u > sub(float(C), 1.f)) ind_u = sub(float(C), 1.f);
    if (ind_v < 0.f) ind_v = 0.f;
    else if (ind_v > sub(float(R), 1.f)) ind_v = sub(float(R), 1.f);
    Bilin b;
    b.iu = ind_u;
    b.iv = ind_v;
    b.su = __float2int_ru(ind_u);
    b.fu = __float2int_rd(ind_u);
    b.sv = __float2int_ru(ind_v);
    b.fv = __float2int_rd(ind_v);
    return b;
}

// Blend of the four taps (identical for interpolatePixel and the non-hole
// branch of interpolatePixelDepth; lrintf and lroundf coincide on the
// integral positions they are applied to).
__device__ __forceinline__ float bilin_blend(const float* __restrict__ mat, unsigned R, const Bilin& b)
{
    if ((b.su == b.fu) && (b.sv == b.fv)) return mat[lrintf(fm(float(R), b.iu, b.iv))];
    if (b.su == b.fu) {
        const long cu = lrintf(b.iu);
        return fm(sub(float(b.sv), b.iv), mat[b.fv + R * cu], mul(sub(b.iv, float(b.fv)), mat[b.sv + R * cu]));
    }
    if (b.sv == b.fv) {
        const long cv = lrintf(b.iv);
        return fm(sub(float(b.su), b.iu), mat[cv + R * b.fu], mul(sub(b.iu, float(b.fu)), mat[cv + R * b.su]));
    }
    const float A = sub(float(b.su), b.iu), B = sub(b.iu, float(b.fu));
    const float val_sup_v = fm(A, mat[b.sv + R * b.fu], mul(B, mat[b.sv + R * b.su]));
    const float val_inf_v = fm(A, mat[b.fv + R * b.fu], mul(B, mat[b.fv + R * b.su]));
    return fm(sub(b.iv, float(b.fv)), val_sup_v, mul(sub(float(b.sv), b.iv), val_inf_v));
}

// bilin_blend of N matrices at the same position: one case analysis, each
// matrix blended with the same expressions (the same bits as N calls).
template <int N>
__device__ __forceinline__ void bilin_blend_n(const float* const (&mat)[N], unsigned R, const Bilin& b, float (&out)[N])
{
    if ((b.su == b.fu) && (b.sv == b.fv)) {
        const long i = lrintf(fm(float(R), b.iu, b.iv));
#pragma unroll
        for (int m = 0; m < N; ++m) out[m] = mat[m][i];
    } else if (b.su == b.fu) {
        const long cu = lrintf(b.iu);
        const float wl = sub(float(b.sv), b.iv), wr = sub(b.iv, float(b.fv));
#pragma unroll
        for (int m = 0; m < N; ++m) out[m] = fm(wl, mat[m][b.fv + R * cu], mul(wr, mat[m][b.sv + R * cu]));
    } else if (b.sv == b.fv) {
        const long cv = lrintf(b.iv);
        const float wl = sub(float(b.su), b.iu), wr = sub(b.iu, float(b.fu));
#pragma unroll
        for (int m = 0; m < N; ++m) out[m] = fm(wl, mat[m][cv + R * b.fu], mul(wr, mat[m][cv + R * b.su]));
    } else {
        const float A = sub(float(b.su), b.iu), B = sub(b.iu, float(b.fu));
        const float wv = sub(b.iv, float(b.fv)), wf = sub(float(b.sv), b.iv);
#pragma unroll
        for (int m = 0; m < N; ++m) {
            const float val_sup_v = fm(A, mat[m][b.sv + R * b.fu], mul(B, mat[m][b.sv + R * b.su]));
            const float val_inf_v = fm(A, mat[m][b.fv + R * b.fu], mul(B, mat[m][b.fv + R * b.su]));
            out[m] = fm(wv, val_sup_v, mul(wf, val_inf_v));
        }
    }
}

// interpolatePixelDepth (pdflow_cudalib.cu:684-721): nearest sample
// (round-half-even) when any of the four taps is a hole.
__device__ __forceinline__ float interp_depth_at(const float* __restrict__ mat, unsigned R, const Bilin& b)
{
    if ((mat[b.sv + R * b.su] == 0.f) || (mat[b.sv + R * b.fu] == 0.f) || (mat[b.fv + R * b.su] == 0.f) ||
        (mat[b.fv + R * b.fu] == 0.f)) {
        const unsigned rind_u = __float2int_rn(b.iu);
        const unsigned rind_v = __float2int_rn(b.iv);
        return mat[rind_v + R * rind_u];
    }
    return bilin_blend(mat, R, b);
}

// Gradient of computeImGradients (pdflow_cudalib.cu:593-599): weighted
// central difference (w*(f1-f0) + wm*(f0-fm)) / (w + wm).
__device__ __forceinline__ float wgrad(float w, float wm, float f1, float f0, float fm_)
{
    return qt(fm(w, sub(f1, f0), mul(wm, sub(f0, fm_))), add(w, wm));
}

// Step sizes of computeMu + computeStepSizes (pdflow_cudalib.cu:781-808).
struct Steps {
    float mu, spd, spuvx, spuvy, spwx, spwy, tu, tv, tw;
};

__device__ __forceinline__ float data_weight(float mu_p, float ddu, float ddv, float ddt)
{
    const float s = fm(ddt, ddt, fm(ddu, ddu, mul(ddv, ddv)));
    return fdividef(mu_p, fm(1000.f, s, 1.f));
}

__device__ __forceinline__ Steps mu_and_steps(float mu_p, float li, float ld, float ddu, float ddv, float ddt, float ri,
                                              float rj, float ri_um1, float rj_vm1, bool has_um1, bool has_vm1)
{
    Steps s;
    s.mu = data_weight(mu_p, ddu, ddv, ddt);
    s.spd = fdividef(1.f, fm(s.mu, add(add(1.f, fabsf(ddu)), fabsf(ddv)), 1e-10f));
    s.spuvx = fdividef(0.5f, fm(li, ri, 1e-10f));
    s.spuvy = fdividef(0.5f, fm(li, rj, 1e-10f));
    s.spwx = fdividef(0.5f, fm(ri, ld, 1e-10f));
    s.spwy = fdividef(0.5f, fm(rj, ld, 1e-10f));
    float acu_r = add(ri, rj);
    if (has_um1) acu_r = add(acu_r, ri_um1);
    if (has_vm1) acu_r = add(acu_r, rj_vm1);
    s.tu = fdividef(1.f, add(fm(li, acu_r, mul(s.mu, fabsf(ddu))), 1e-10f));
    s.tv = fdividef(1.f, add(fm(li, acu_r, mul(s.mu, fabsf(ddv))), 1e-10f));
    s.tw = fdividef(1.f, add(fm(ld, acu_r, s.mu), 1e-10f));
    return s;
}

// Dual step: computeGradient (pdflow_cudalib.cu:982-1013) then
// updateDualVariables (:813-887) at one pixel.  `*_u1` are the values at
// (v, u+1), `*_v1` at (v+1, u); last_u / last_v mark the far borders where
// the forward difference is zero.
struct Duals {
    float pd, puu, puv, pvu, pvv, pwu, pwv;
};

__device__ __forceinline__ float fwd_diff(float r, float a1, float p1, float a0, float p0)
{
    return mul(r, sub(add(a1, p1), add(a0, p0)));
}

__device__ __forceinline__ void project_disc(float& a, float& b)
{
    const float m = rhypotf(a, b);
    if (m < 1.f) {
        a = mul(a, m);
        b = mul(b, m);
    }
}

__device__ __forceinline__ void dual_update(Duals& p, float spd, float spuvx, float spuvy, float spwx, float spwy,
                                            float mu, float ddt, float ddu, float ddv, float li, float ld, float ri,
                                            float rj, float dua, float dva, float dwa, float dup, float dvp,
                                            float dua_u1, float dva_u1, float dwa_u1, float dup_u1, float dvp_u1,
                                            float dua_v1, float dva_v1, float dwa_v1, float dup_v1, float dvp_v1,
                                            bool last_u, bool last_v)
{
    const float gu1 = last_u ? 0.f : fwd_diff(ri, dua_u1, dup_u1, dua, dup);
    const float gv1 = last_u ? 0.f : fwd_diff(ri, dva_u1, dvp_u1, dva, dvp);
    const float gw1 = last_u ? 0.f : mul(ri, sub(dwa_u1, dwa));
    const float gu2 = last_v ? 0.f : fwd_diff(rj, dua_v1, dup_v1, dua, dup);
    const float gv2 = last_v ? 0.f : fwd_diff(rj, dva_v1, dvp_v1, dva, dvp);
    const float gw2 = last_v ? 0.f : mul(rj, sub(dwa_v1, dwa));
    const float X = fm(ddv, dva, fm(ddu, dua, add(-dwa, ddt)));
    float pd = fm(mul(spd, mu), X, p.pd);
    const float sx = mul(spuvx, li), sy = mul(spuvy, li), wx = mul(spwx, ld), wy = mul(spwy, ld);
    float puu = fm(sx, gu1, p.puu), puv = fm(sy, gu2, p.puv);
    float pvu = fm(sx, gv1, p.pvu), pvv = fm(sy, gv2, p.pvv);
    float pwu = fm(wx, gw1, p.pwu), pwv = fm(wy, gw2, p.pwv);
    if (fabsf(pd) > 1.f) pd = (pd > 1.f) ? 1.f : -1.f;
    project_disc(puu, puv);
    project_disc(pvu, pvv);
    project_disc(pwu, pwv);
    p.pd = pd;
    p.puu = puu; p.puv = puv;
    p.pvu = pvu; p.pvv = pvv;
    p.pwu = pwu; p.pwv = pwv;
}

// Divergence term of computeDivergence (pdflow_cudalib.cu:935-980) for one
// component: (pu, pv) at the pixel, pu_um1 at (v, u-1), pv_vm1 at (v-1, u).
__device__ __forceinline__ float divergence(float ri, float ri_um1, float rj, float rj_vm1, float pu, float pu_um1,
                                            float pv, float pv_vm1, bool first_u, bool last_u, bool first_v,
                                            bool last_v)
{
    float d;
    if (first_u) d = mul(ri, pu);
    else if (last_u) d = mul(-ri_um1, pu_um1);
    else d = fm(ri, pu, -mul(ri_um1, pu_um1));
    if (first_v) d = fm(rj, pv, d);
    else if (last_v) d = fm(-rj_vm1, pv_vm1, d);
    else d = add(d, fm(rj, pv, -mul(rj_vm1, pv_vm1)));
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
    du = fm(-tu, fm(mul(mu, ddu), pd, -mul(li, divu)), du);
    dv = fm(-tv, fm(mul(mu, ddv), pd, -mul(li, divv)), dv);
    dw = add(dw, mul(-tw, fm(-mu, pd, -mul(ld, divw))));
    const float optflow = fm(dcv, dv, fm(dcu, du, dct));
    const float a1 = mul(tu, dcu), b1 = mul(tv, dcv);
    const float of_threshold = fm(a1, dcu, mul(b1, dcv));
    if (optflow < -of_threshold) {
        du = add(du, a1);
        dv = add(dv, b1);
    } else if (optflow > of_threshold) {
        du = sub(du, a1);
        dv = sub(dv, b1);
    } else {
        const float den = add(fm(a1, dcu, mul(b1, dcv)), 1e-10f);
        du = sub(du, qt(mul(a1, optflow), den));
        dv = sub(dv, qt(mul(b1, optflow), den));
    }
    dua = fm(2.f, du, -du_old);
    dva = fm(2.f, dv, -dv_old);
    dwa = fm(2.f, dw, -dw_old);
}

// Whether x is 0 or 2^lo <= |x| < 2^(hi + 1) (from its exponent field).
__device__ __forceinline__ bool mag_in(float x, int lo, int hi)
{
    const unsigned b = __float_as_uint(x), e = (b >> 23) & 0xffu;
    return (b << 1) == 0u || e - (unsigned)(127 + lo) <= (unsigned)(hi - lo);
}

// a / b correctly rounded, from y = RN(1/b) (__frcp_rn): q0 = RN(a y) is
// within 2 ulp of a/b, one correction q1 = RN(q0 + RN(a - b q0) y) makes it
// faithful, and by Markstein's theorem (P. Markstein, IBM J. Res. Dev.
// 34(1), 1990; J.-M. Muller et al., Handbook of Floating-Point Arithmetic,
// 2nd ed., sec. 4.7) the second, whose remainder a - b q1 the FMA forms
// exactly, rounds it correctly: the bits of an IEEE division, in five
// instructions once y is known.  Valid for a == 0 or 2^-60 <= |a| < 2^60 and
// 2^-40 <= b < 2^60 (no intermediate leaves the normal range); a zero
// numerator is returned as is (the sign of a / b).  Checked bit for bit
// against __fdiv_rn on 1.7e10 random pairs of that range.
__device__ __forceinline__ float div_rcp(float a, float b, float y)
{
    const float q0 = mul(a, y);
    const float q1 = fm(fm(-q0, b, a), y, q0);
    const float q2 = fm(fm(-q1, b, a), y, q1);
    return a == 0.f ? a : q2;
}

// L1 photometric shrinkage of one pixel (pdflow_cudalib.cu:906-923) in the
// register tiles.  All three cases are evaluated and one is selected: a
// warp's lanes fall in different cases, so the branches cost more than the
// two quotients (same bits: each case's value is the reference's expression).
__device__ __forceinline__ void shrink(float& du, float& dv, float of, float th, float a1, float b1)
{
    const float den = add(th, 1e-10f);
    const float mu_ = sub(du, qt(mul(a1, of), den)), mv_ = sub(dv, qt(mul(b1, of), den));
    const bool lo = of < -th, hi = of > th;
    du = lo ? add(du, a1) : (hi ? sub(du, a1) : mu_);
    dv = lo ? add(dv, b1) : (hi ? sub(dv, b1) : mv_);
}

// The same with the quotients by div_rcp: den = th + 1e-10 and rden =
// RN(1 / den) are the pixel's, fixed for the level (shrink_rcp_ok says when
// the quotients are in div_rcp's range).
__device__ __forceinline__ void shrink_rcp(float& du, float& dv, float of, float th, float den, float rden, float a1,
                                           float b1)
{
    const float mu_ = sub(du, div_rcp(mul(a1, of), den, rden)), mv_ = sub(dv, div_rcp(mul(b1, of), den, rden));
    const bool lo = of < -th, hi = of > th;
    du = lo ? add(du, a1) : (hi ? sub(du, a1) : mu_);
    dv = lo ? add(dv, b1) : (hi ? sub(dv, b1) : mv_);
}

// Whether a pixel's shrinkage quotients a1 * of / den and b1 * of / den are
// in div_rcp's range: |a1|, |b1| and |of| zero or in [2^-30, 2^30) (so the
// numerators are zero or in [2^-60, 2^60)) and den in [2^-40, 2^60).
__device__ __forceinline__ bool shrink_rcp_level_ok(float a1, float b1, float den)
{
    return mag_in(a1, -30, 29) && mag_in(b1, -30, 29) && den >= 0x1p-40f && den < 0x1p60f;
}
__device__ __forceinline__ bool shrink_rcp_ok(float of) { return mag_in(of, -30, 29); }

// saturateVariables (pdflow_cudalib.cu:1018-1038).
__device__ __forceinline__ void saturate(float& du, float& dv, float& dw, float du_prev, float dv_prev,
                                         float depth_old)
{
    if (du > 1.f) du = 1.f;
    else if (du < -1.f) du = -1.f;
    if (dv > 1.f) dv = 1.f;
    else if (dv < -1.f) dv = -1.f;
    if (depth_old == 0.f) dw = 0.f;
    du = add(du, du_prev);
    dv = add(dv, dv_prev);
}

// Weight of a neighbour in filterSolution (pdflow_cudalib.cu:1075):
// 1 / (1 + 5 (z0 - z)^2 + 10 ddt^2).
__device__ __forceinline__ float median_weight(float z0, float z, float ddt)
{
    return __frcp_rn(fm(10.f, powf(ddt, 2.f), fm(5.f, powf(sub(z0, z), 2.f), 1.f)));   // 1 / x, IEEE rounded
}

// The same weight from a precomputed ddt_sq = powf(ddt, 2.f).
__device__ __forceinline__ float median_weight_sq(float z0, float z, float ddt_sq)
{
    return __frcp_rn(fm(10.f, ddt_sq, fm(5.f, powf(sub(z0, z), 2.f), 1.f)));
}

// powf(z0 - z, 2.f) without the call where the difference is zero in every
// active lane of the warp (the centre tap): powf(+-0, 2) is +0.
__device__ __forceinline__ float pow2_diff_voted(float z0, float z)
{
    const float d = sub(z0, z);
    if (__all_sync(__activemask(), d == 0.f)) return 0.f;
    return powf(d, 2.f);
}

// Linear interpolation between the samples bracketing the weighted median
// (pdflow_cudalib.cu:1109).
__device__ __forceinline__ float median_lerp(float cum_r, float cum_l, float med, float f_l, float f_r)
{
    return qt(fm(sub(cum_r, med), f_l, mul(sub(med, cum_l), f_r)), sub(cum_r, cum_l));
}

// computeMotionField (pdflow_cudalib.cu:1155-1160) at a pixel with depth z > 0.
__device__ __forceinline__ void motion_field(float z, float du, float dv_, float dw, float xx, float yy, float inv_f,
                                             float& dx, float& dy, float& dz)
{
    dx = dw;
    dy = fm(mul(z, du), inv_f, qt(mul(dw, xx), z));
    dz = fm(mul(z, dv_), inv_f, qt(mul(dw, yy), z));
}

}  // namespace pdflow
