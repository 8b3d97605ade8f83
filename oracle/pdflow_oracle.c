/*
 * CPU restatement of PD-Flow's coarse-to-fine primal-dual scene-flow solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark link it as the
 * checker.  The product (the CUDA library under pd-flow_gb300/) never calls
 * it and has no CPU fallback.
 *
 * One source, compiled twice:
 *   -DOR_REAL_DOUBLE  -> symbols *_f64 : FP64 transcription, the error oracle
 *   (default)         -> symbols *_f32 : FP32 transcription; built with
 *                        -fopenmp it is the timed host-core baseline
 * Both builds use -ffp-contract=off so x86-64 and aarch64 produce the same
 * bits (aarch64 gcc would otherwise fuse a*b+c).
 *
 * Every step cites the reference function it restates (file:line within the
 * PD-Flow project).  Device intrinsics map to IEEE host operations:
 *   fdividef(a,b) -> a/b          rhypotf(a,b) -> 1/hypot(a,b)
 *   __float2int_ru/rd/rn -> ceil/floor/nearbyint   lrintf/lroundf -> lrint/lround
 *   powf(x,2.f)  -> x*x           tan/tanf      -> tan
 * The FP64 build promotes every float literal and parameter of the reference
 * (0.04f, 1e-10f, ...) to double, so it isolates arithmetic rounding only.
 *
 * Layout follows the reference: column-major, rows contiguous, idx = v + u*R
 * (pdflow_cudalib.cu:343-344, scene_flow_impair.cpp:230-232).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef OR_REAL_DOUBLE
typedef double real;
#define SFX(n) n##_f64
#define RFABS fabs
#define RHYPOT hypot
#define RTAN tan
#define RCEIL ceil
#define RFLOOR floor
#define RNEAR nearbyint
#define RLRINT lrint
#define RLROUND lround
#else
typedef float real;
#define SFX(n) n##_f32
#define RFABS fabsf
#define RHYPOT hypotf
#define RTAN tanf
#define RCEIL ceilf
#define RFLOOR floorf
#define RNEAR nearbyintf
#define RLRINT lrintf
#define RLROUND lroundf
#endif

/* A float literal of the reference, promoted to `real`. */
#define K(x) ((real)(x##f))

#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

#define OR_MAX_LEVELS 8

/* ------------------------------------------------------------------------- */
/* Parameters: PD_flow_opencv ctor, scene_flow_impair.cpp:31-69, and         */
/* initializeCUDA, scene_flow_impair.cpp:175-193.                            */
/* ------------------------------------------------------------------------- */
typedef struct {
    unsigned rows, cols, width, height, cam_mode, ctf_levels, pyr_levels;
    unsigned num_max_iter[6];
    real lambda_i, lambda_d, mu, fovh;
    real g_mask[25];
} or_cfg;

static unsigned or_log2u(unsigned x) { unsigned l = 0; while (x > 1) { x >>= 1; ++l; } return l; }

/* Returns 0 on success, -1 on an unsupported size. */
static int or_make_cfg(or_cfg* c, unsigned rows, unsigned width, unsigned height,
                       const unsigned* iters_override)
{
    memset(c, 0, sizeof(*c));
    if (!(rows == 15 || rows == 30 || rows == 60 || rows == 120 || rows == 240 || rows == 480)) return -1;
    if (!((width == 640 && height == 480) || (width == 320 && height == 240))) return -1;
    c->rows = rows;
    c->cols = rows * 320 / 240;                       /* scene_flow_impair.cpp:39 */
    if (c->cols > width) return -1;
    c->width = width; c->height = height;
    c->cam_mode = (height == 240) ? 2u : 1u;          /* scene_flow_impair.cpp:182-183 */
    c->ctf_levels = or_log2u(rows / 15) + 1;          /* scene_flow_impair.cpp:40 */
    c->pyr_levels = or_log2u(width / c->cols) + c->ctf_levels; /* scene_flow_impair.cpp:88 */
    /* scene_flow_impair.cpp:46-52: 100 at the finest level, -15 per coarser level */
    for (int i = 5; i >= 0; --i) {
        if (i >= (int)c->ctf_levels - 1) c->num_max_iter[i] = 100;
        else c->num_max_iter[i] = c->num_max_iter[i + 1] - 15;
    }
    if (iters_override)
        for (int i = 0; i < 6; ++i) c->num_max_iter[i] = iters_override[i];
    /* fovh = M_PI*62.5f/180.f evaluated in double, stored as float (:41) */
    c->fovh = (real)(float)(3.14159265358979323846 * 62.5 / 180.0);
    c->lambda_i = K(0.04); c->lambda_d = K(0.35); c->mu = K(75.0);   /* :67-69 */
    static const int vm[5] = {1, 4, 6, 4, 1};                         /* :55-58 */
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j)
            c->g_mask[i + 5 * j] = (real)((float)(vm[i] * vm[j]) / 256.f);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Pyramid: computePyramidLevel, pdflow_cudalib.cu:331-434.                  */
/* `level0` copies the input; otherwise 5x5 depth-weighted decimation of the */
/* previous level (2R x 2C).                                                  */
/* ------------------------------------------------------------------------- */
void SFX(or_pyramid_level)(unsigned R, unsigned C, int level0,
                           const real* cin, const real* din,       /* level 0 input (R*C) */
                           const real* cprev, const real* dprev,   /* previous level (4*R*C) */
                           const real* g, real fovh,
                           real* col, real* dep, real* xx, real* yy)
{
    const real max_depth_dif = K(0.1);
    const real inv_f_i = K(2.0) * RTAN(K(0.5) * fovh) / (real)C;
    const real disp_u_i = K(0.5) * (real)(C - 1);
    const real disp_v_i = K(0.5) * (real)(R - 1);
    const long N = (long)R * C;
    OMP_FOR
    for (long index = 0; index < N; ++index) {
        const unsigned v = (unsigned)(index % R), u = (unsigned)(index / R);
        if (level0) {
            col[index] = cin[index];
            dep[index] = din[index];
        } else {
            real sumd = 0, sumc = 0, acu_d = 0, acu_c = 0;
            const unsigned ind_cent = 2 * v + 4 * u * R;
            const real dcenter = dprev[ind_cent];
            if (v > 0 && v < R - 1 && u > 0 && u < C - 1) {
                for (int k = -2; k < 3; ++k)
                    for (int l = -2; l < 3; ++l) {
                        const unsigned ip = 2 * v + k + 2 * (2 * u + l) * R;
                        const real gm = g[12 + k + 5 * l];
                        sumc += gm * cprev[ip];
                        const real d = dprev[ip];
                        if (d > 0 && RFABS(d - dcenter) < max_depth_dif) {
                            const real w = gm * (max_depth_dif - RFABS(d - dcenter));
                            acu_d += w;
                            sumd += w * d;
                        }
                    }
                dep[index] = (sumd > 0) ? sumd / acu_d : 0;
                col[index] = sumc;
            } else {
                for (int k = -2; k < 3; ++k)
                    for (int l = -2; l < 3; ++l) {
                        const int iv = 2 * (int)v + k, iu = 2 * (int)u + l;
                        if (iv >= 0 && iv < 2 * (int)R && iu >= 0 && iu < 2 * (int)C) {
                            const unsigned ip = (unsigned)iv + 2 * (unsigned)iu * R;
                            const real gm = g[12 + k + 5 * l];
                            sumc += gm * cprev[ip];
                            acu_c += gm;
                            const real d = dprev[ip];
                            if (d > 0 && RFABS(d - dcenter) < max_depth_dif) {
                                const real w = gm * (max_depth_dif - RFABS(d - dcenter));
                                acu_d += w;
                                sumd += w * d;
                            }
                        }
                    }
                col[index] = sumc / acu_c;
                dep[index] = (sumd > 0) ? sumd / acu_d : 0;
            }
        }
        xx[index] = ((real)u - disp_u_i) * dep[index] * inv_f_i;
        yy[index] = ((real)v - disp_v_i) * dep[index] * inv_f_i;
    }
}

/* ------------------------------------------------------------------------- */
/* Upsampling of the previous level's solution: assignZeros (:439-455),      */
/* upsampleCopyPrevSolution (:460-477), upsampleFilterPrevSolution           */
/* (:479-569).  `lc` holds the 10 coarse fields (du,dv,dw,pd,puu,puv,pvu,pvv,*/
/* pwu,pwv) of size (R/2)*(C/2); `up` is 10 scratch planes of R*C.  Outputs: */
/* du_prev, dv_prev, dw_new(=dw_acc) and the 7 duals.                         */
/* ------------------------------------------------------------------------- */
void SFX(or_upsample)(unsigned R, unsigned C, const real* const lc[10], real* const up[10],
                      const real* g, real* du_prev, real* dv_prev, real* const out8[8])
{
    const long N = (long)R * C;
    for (int f = 0; f < 10; ++f) memset(up[f], 0, sizeof(real) * (size_t)N);
    const long Nc = N / 4;
    for (long index = 0; index < Nc; ++index) {
        const unsigned v = (unsigned)(index % (R / 2));
        const unsigned u = (unsigned)(2 * index / R);
        const unsigned ib = 2 * (v + u * R);
        up[0][ib] = K(2.0) * lc[0][index];
        up[1][ib] = K(2.0) * lc[1][index];
        for (int f = 2; f < 10; ++f) up[f][ib] = lc[f][index];
    }
    real m4[25];
    for (int i = 0; i < 25; ++i) m4[i] = K(4.0) * g[i];
    OMP_FOR
    for (long index = 0; index < N; ++index) {
        const unsigned v = (unsigned)(index % R), u = (unsigned)(index / R);
        real acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (v > 1 && v < R - 2 && u > 1 && u < C - 2) {
            for (int k = -2; k < 3; ++k)
                for (int l = -2; l < 3; ++l) {
                    const unsigned ii = v + k + (u + l) * R;
                    const real gm = m4[12 + k + 5 * l];
                    for (int f = 0; f < 10; ++f) acc[f] += gm * up[f][ii];
                }
        } else {
            real acu = 1;
            for (int k = -2; k < 3; ++k)
                for (int l = -2; l < 3; ++l) {
                    const int iv = (int)v + k, iu = (int)u + l;
                    if (iv < 0 || iv >= (int)R || iu < 0 || iu >= (int)C) {
                        acu -= K(0.25) * m4[12 + k + 5 * l];
                        continue;
                    }
                    const unsigned ii = (unsigned)iv + (unsigned)iu * R;
                    const real gm = m4[12 + k + 5 * l];
                    for (int f = 0; f < 10; ++f) acc[f] += gm * up[f][ii];
                }
            const real inv = K(1.0) / acu;
            for (int f = 0; f < 10; ++f) acc[f] *= inv;
        }
        du_prev[index] = acc[0];
        dv_prev[index] = acc[1];
        for (int f = 0; f < 8; ++f) out8[f][index] = acc[2 + f];  /* dw, pd, puu..pwv */
    }
}

/* ------------------------------------------------------------------------- */
/* computeRij, pdflow_cudalib.cu:725-779.                                    */
/* ------------------------------------------------------------------------- */
static inline real or_rfac(real a, real b)
{
    if (RFABS(a) + RFABS(b) > 0) return K(2.0) * (K(1.0) / RHYPOT(a, b));
    return K(1.0);
}

void SFX(or_rij)(unsigned R, unsigned C,
                 const real* xx_old, const real* yy_old, const real* d_old,
                 const real* xx_new, const real* yy_new, const real* d_new,
                 real* ri, real* rj, real* ri2, real* rj2)
{
    const long N = (long)R * C;
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        const unsigned v = (unsigned)(i % R), u = (unsigned)(i / R);
        real dxu = 0, dzu = 0, dxu2 = 0, dzu2 = 0, dyv = 0, dzv = 0, dyv2 = 0, dzv2 = 0;
        if (u != C - 1) {
            dxu = xx_old[i + R] - xx_old[i];  dzu = d_old[i + R] - d_old[i];
            dxu2 = xx_new[i + R] - xx_new[i]; dzu2 = d_new[i + R] - d_new[i];
        }
        if (v != R - 1) {
            dyv = yy_old[i + 1] - yy_old[i];  dzv = d_old[i + 1] - d_old[i];
            dyv2 = yy_new[i + 1] - yy_new[i]; dzv2 = d_new[i + 1] - d_new[i];
        }
        ri[i] = or_rfac(dxu, dzu);
        rj[i] = or_rfac(dyv, dzv);
        ri2[i] = or_rfac(dxu2, dzu2);
        rj2[i] = or_rfac(dyv2, dzv2);
    }
}

/* ------------------------------------------------------------------------- */
/* computeImGradients, pdflow_cudalib.cu:574-627 (new frame).                */
/* ------------------------------------------------------------------------- */
void SFX(or_im_gradients)(unsigned R, unsigned C, const real* c, const real* d,
                          const real* ri2, const real* rj2,
                          real* dcu, real* dcv, real* ddu, real* ddv)
{
    const long N = (long)R * C;
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        const unsigned v = (unsigned)(i % R), u = (unsigned)(i / R);
        if (u == 0) {
            dcu[i] = c[i + R] - c[i];
            ddu[i] = d[i + R] - d[i];
        } else if (u == C - 1) {
            dcu[i] = c[i] - c[i - R];
            ddu[i] = d[i] - d[i - R];
        } else {
            dcu[i] = (ri2[i] * (c[i + R] - c[i]) + ri2[i - R] * (c[i] - c[i - R])) / (ri2[i] + ri2[i - R]);
            if (d[i] > 0)
                ddu[i] = (ri2[i] * (d[i + R] - d[i]) + ri2[i - R] * (d[i] - d[i - R])) / (ri2[i] + ri2[i - R]);
            else
                ddu[i] = 0;
        }
        if (v == 0) {
            dcv[i] = c[i + 1] - c[i];
            ddv[i] = d[i + 1] - d[i];
        } else if (v == R - 1) {
            dcv[i] = c[i] - c[i - 1];
            ddv[i] = d[i] - d[i - 1];
        } else {
            dcv[i] = (rj2[i] * (c[i + 1] - c[i]) + rj2[i - 1] * (c[i] - c[i - 1])) / (rj2[i] + rj2[i - 1]);
            if (d[i] > 0)
                ddv[i] = (rj2[i] * (d[i + 1] - d[i]) + rj2[i - 1] * (d[i] - d[i - 1])) / (rj2[i] + rj2[i - 1]);
            else
                ddv[i] = 0;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* interpolatePixel (:654-682) and interpolatePixelDepth (:684-721).         */
/* ------------------------------------------------------------------------- */
static inline real or_interp(const real* m, unsigned R, unsigned C, real iu, real iv)
{
    if (iu < 0) iu = 0; else if (iu > (real)C - K(1.0)) iu = (real)C - K(1.0);
    if (iv < 0) iv = 0; else if (iv > (real)R - K(1.0)) iv = (real)R - K(1.0);
    const unsigned su = (unsigned)RCEIL(iu), fu = (unsigned)RFLOOR(iu);
    const unsigned sv = (unsigned)RCEIL(iv), fv = (unsigned)RFLOOR(iv);
    if (su == fu && sv == fv) return m[RLRINT(iv + (real)R * iu)];
    if (su == fu) {
        const long cu = RLRINT(iu);
        return ((real)sv - iv) * m[fv + R * cu] + (iv - (real)fv) * m[sv + R * cu];
    }
    if (sv == fv) {
        const long cv = RLRINT(iv);
        return ((real)su - iu) * m[cv + R * fu] + (iu - (real)fu) * m[cv + R * su];
    }
    const real vs = ((real)su - iu) * m[sv + R * fu] + (iu - (real)fu) * m[sv + R * su];
    const real vi = ((real)su - iu) * m[fv + R * fu] + (iu - (real)fu) * m[fv + R * su];
    return ((real)sv - iv) * vi + (iv - (real)fv) * vs;
}

static inline real or_interp_depth(const real* m, unsigned R, unsigned C, real iu, real iv)
{
    if (iu < 0) iu = 0; else if (iu > (real)C - K(1.0)) iu = (real)C - K(1.0);
    if (iv < 0) iv = 0; else if (iv > (real)R - K(1.0)) iv = (real)R - K(1.0);
    const unsigned su = (unsigned)RCEIL(iu), fu = (unsigned)RFLOOR(iu);
    const unsigned sv = (unsigned)RCEIL(iv), fv = (unsigned)RFLOOR(iv);
    if (m[sv + R * su] == 0 || m[sv + R * fu] == 0 || m[fv + R * su] == 0 || m[fv + R * fu] == 0) {
        const unsigned ru = (unsigned)RNEAR(iu), rv = (unsigned)RNEAR(iv);
        return m[rv + R * ru];
    }
    if (su == fu && sv == fv) return m[RLRINT(iv + (real)R * iu)];
    if (su == fu) {
        const long cu = RLROUND(iu);
        return ((real)sv - iv) * m[fv + R * cu] + (iv - (real)fv) * m[sv + R * cu];
    }
    if (sv == fv) {
        const long cv = RLROUND(iv);
        return ((real)su - iu) * m[cv + R * fu] + (iu - (real)fu) * m[cv + R * su];
    }
    const real vs = ((real)su - iu) * m[sv + R * fu] + (iu - (real)fu) * m[sv + R * su];
    const real vi = ((real)su - iu) * m[fv + R * fu] + (iu - (real)fu) * m[fv + R * su];
    return ((real)sv - iv) * vi + (iv - (real)fv) * vs;
}

/* performWarping, pdflow_cudalib.cu:629-652. */
void SFX(or_warping)(unsigned R, unsigned C,
                     const real* c_new, const real* c_old, const real* d_new, const real* d_old,
                     const real* dcu_aux, const real* dcv_aux, const real* ddu_aux, const real* ddv_aux,
                     const real* du_prev, const real* dv_prev,
                     real* dct, real* dcu, real* dcv, real* ddt, real* ddu, real* ddv)
{
    const long N = (long)R * C;
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        const unsigned v = (unsigned)(i % R), u = (unsigned)(i / R);
        const real iu = (real)u + du_prev[i];
        const real iv = (real)v + dv_prev[i];
        dct[i] = or_interp(c_new, R, C, iu, iv) - c_old[i];
        dcu[i] = or_interp(dcu_aux, R, C, iu, iv);
        dcv[i] = or_interp(dcv_aux, R, C, iu, iv);
        const real wz = or_interp_depth(d_new, R, C, iu, iv);
        ddt[i] = (wz > 0) ? wz - d_old[i] : 0;
        ddu[i] = or_interp(ddu_aux, R, C, iu, iv);
        ddv[i] = or_interp(ddv_aux, R, C, iu, iv);
    }
}

/* computeMu (:781-784) and computeStepSizes (:786-808).
 * steps[0..7] = sigma_pd, sigma_puvx, sigma_puvy, sigma_pwx, sigma_pwy, tau_u, tau_v, tau_w */
void SFX(or_mu_steps)(unsigned R, unsigned C, real mu_p, real li, real ld,
                      const real* ddu, const real* ddv, const real* ddt,
                      const real* ri, const real* rj, real* mu, real* const st[8])
{
    const long N = (long)R * C;
    const real eps = K(1e-10);
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        const unsigned v = (unsigned)(i % R), u = (unsigned)(i / R);
        const real m = mu_p / (K(1.0) + K(1000.0) * (ddu[i] * ddu[i] + ddv[i] * ddv[i] + ddt[i] * ddt[i]));
        mu[i] = m;
        st[0][i] = K(1.0) / (m * (K(1.0) + RFABS(ddu[i]) + RFABS(ddv[i])) + eps);
        st[1][i] = K(0.5) / (li * ri[i] + eps);
        st[2][i] = K(0.5) / (li * rj[i] + eps);
        st[3][i] = K(0.5) / (ri[i] * ld + eps);
        st[4][i] = K(0.5) / (rj[i] * ld + eps);
        real acu_r = ri[i] + rj[i];
        if (u > 0) acu_r += ri[i - R];
        if (v > 0) acu_r += rj[i - 1];
        st[5][i] = K(1.0) / (m * RFABS(ddu[i]) + li * acu_r + eps);
        st[6][i] = K(1.0) / (m * RFABS(ddv[i]) + li * acu_r + eps);
        st[7][i] = K(1.0) / (m + ld * acu_r + eps);
    }
}

/* ------------------------------------------------------------------------- */
/* Primal-dual state.  Index names follow the reference arrays.              */
/* ------------------------------------------------------------------------- */
enum { S_DU, S_DV, S_DW, S_DUA, S_DVA, S_DWA, S_PD, S_PUU, S_PUV, S_PVU, S_PVV, S_PWU, S_PWV, S_N };
enum { L_DCT, L_DCU, L_DCV, L_DDT, L_DDU, L_DDV, L_MU, L_RI, L_RJ, L_DUP, L_DVP,
       L_SPD, L_SPUVX, L_SPUVY, L_SPWX, L_SPWY, L_TU, L_TV, L_TW, L_N };

/* computeGradient (:982-1013) followed by updateDualVariables (:813-887).
 * `gr` is 6 planes of scratch (gradu1, gradu2, gradv1, gradv2, gradw1, gradw2). */
void SFX(or_dual_step)(unsigned R, unsigned C, real li, real ld,
                       real* const s[S_N], const real* const L[L_N], real* const gr[6])
{
    const long N = (long)R * C;
    const real* ri = L[L_RI]; const real* rj = L[L_RJ];
    const real* dup = L[L_DUP]; const real* dvp = L[L_DVP];
    const real* dua = s[S_DUA]; const real* dva = s[S_DVA]; const real* dwa = s[S_DWA];
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        const unsigned v = (unsigned)(i % R), u = (unsigned)(i / R);
        if (u == C - 1) { gr[0][i] = 0; gr[2][i] = 0; gr[4][i] = 0; }
        else {
            gr[0][i] = ri[i] * ((dua[i + R] + dup[i + R]) - (dua[i] + dup[i]));
            gr[2][i] = ri[i] * ((dva[i + R] + dvp[i + R]) - (dva[i] + dvp[i]));
            gr[4][i] = ri[i] * (dwa[i + R] - dwa[i]);
        }
        if (v == R - 1) { gr[1][i] = 0; gr[3][i] = 0; gr[5][i] = 0; }
        else {
            gr[1][i] = rj[i] * ((dua[i + 1] + dup[i + 1]) - (dua[i] + dup[i]));
            gr[3][i] = rj[i] * ((dva[i + 1] + dvp[i + 1]) - (dva[i] + dvp[i]));
            gr[5][i] = rj[i] * (dwa[i + 1] - dwa[i]);
        }
    }
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        real pd = s[S_PD][i], puu = s[S_PUU][i], puv = s[S_PUV][i];
        real pvu = s[S_PVU][i], pvv = s[S_PVV][i], pwu = s[S_PWU][i], pwv = s[S_PWV][i];
        pd += L[L_SPD][i] * L[L_MU][i] * (-dwa[i] + L[L_DDT][i] + L[L_DDU][i] * dua[i] + L[L_DDV][i] * dva[i]);
        puu += L[L_SPUVX][i] * li * gr[0][i];
        puv += L[L_SPUVY][i] * li * gr[1][i];
        pvu += L[L_SPUVX][i] * li * gr[2][i];
        pvv += L[L_SPUVY][i] * li * gr[3][i];
        pwu += L[L_SPWX][i] * ld * gr[4][i];
        pwv += L[L_SPWY][i] * ld * gr[5][i];
        if (RFABS(pd) > K(1.0)) pd = (pd > K(1.0)) ? K(1.0) : K(-1.0);
        s[S_PD][i] = pd;
        real m = K(1.0) / RHYPOT(puu, puv);
        if (m < K(1.0)) { puu *= m; puv *= m; }
        m = K(1.0) / RHYPOT(pvu, pvv);
        if (m < K(1.0)) { pvu *= m; pvv *= m; }
        m = K(1.0) / RHYPOT(pwu, pwv);
        if (m < K(1.0)) { pwu *= m; pwv *= m; }
        s[S_PUU][i] = puu; s[S_PUV][i] = puv;
        s[S_PVU][i] = pvu; s[S_PVV][i] = pvv;
        s[S_PWU][i] = pwu; s[S_PWV][i] = pwv;
    }
}

/* computeDivergence (:935-980) followed by updatePrimalVariables (:889-933).
 * `dv3` is 3 planes of scratch (divpu, divpv, divpw). */
void SFX(or_primal_step)(unsigned R, unsigned C, real li, real ld,
                         real* const s[S_N], const real* const L[L_N], real* const dv3[3])
{
    const long N = (long)R * C;
    const real* ri = L[L_RI]; const real* rj = L[L_RJ];
    const real* const P[6] = {s[S_PUU], s[S_PVU], s[S_PWU], s[S_PUV], s[S_PVV], s[S_PWV]};
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        const unsigned v = (unsigned)(i % R), u = (unsigned)(i / R);
        for (int f = 0; f < 3; ++f) {
            const real* pu = P[f]; const real* pv = P[3 + f];
            real dd;
            if (u == 0) dd = ri[i] * pu[i];
            else if (u == C - 1) dd = -ri[i - R] * pu[i - R];
            else dd = ri[i] * pu[i] - ri[i - R] * pu[i - R];
            if (v == 0) dd += rj[i] * pv[i];
            else if (v == R - 1) dd += -rj[i - 1] * pv[i - 1];
            else dd += rj[i] * pv[i] - rj[i - 1] * pv[i - 1];
            dv3[f][i] = dd;
        }
    }
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        real du = s[S_DU][i], dv = s[S_DV][i], dw = s[S_DW][i];
        const real du0 = du, dv0 = dv, dw0 = dw;
        const real mu = L[L_MU][i], pd = s[S_PD][i];
        const real tu = L[L_TU][i], tv = L[L_TV][i], tw = L[L_TW][i];
        const real dcu = L[L_DCU][i], dcv = L[L_DCV][i];
        du += -tu * (mu * L[L_DDU][i] * pd - li * dv3[0][i]);
        dv += -tv * (mu * L[L_DDV][i] * pd - li * dv3[1][i]);
        dw += -tw * (-mu * pd - ld * dv3[2][i]);
        const real of = L[L_DCT][i] + dcu * du + dcv * dv;
        const real th = tu * dcu * dcu + tv * dcv * dcv;
        if (of < -th) { du += tu * dcu; dv += tv * dcv; }
        else if (of > th) { du -= tu * dcu; dv -= tv * dcv; }
        else {
            const real den = tu * dcu * dcu + tv * dcv * dcv + K(1e-10);
            du -= tu * dcu * of / den;
            dv -= tv * dcv * of / den;
        }
        s[S_DUA][i] = K(2.0) * du - du0;
        s[S_DVA][i] = K(2.0) * dv - dv0;
        s[S_DWA][i] = K(2.0) * dw - dw0;
        s[S_DU][i] = du; s[S_DV][i] = dv; s[S_DW][i] = dw;
    }
}

/* saturateVariables, pdflow_cudalib.cu:1018-1038 (in place). */
void SFX(or_saturate)(long N, real* du, real* dv, real* dw, const real* du_prev,
                      const real* dv_prev, const real* d_old)
{
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        real a = du[i], b = dv[i], w = dw[i];
        if (a > K(1.0)) a = K(1.0); else if (a < K(-1.0)) a = K(-1.0);
        if (b > K(1.0)) b = K(1.0); else if (b < K(-1.0)) b = K(-1.0);
        if (d_old[i] == 0) w = 0;
        du[i] = a + du_prev[i];
        dv[i] = b + dv_prev[i];
        dw[i] = w;
    }
}

/* Stable bubble sort of (field, weight) pairs on field: bubbleSortDev,
 * pdflow_cudalib.cu:1457-1473. */
static void or_bubble(real* f, real* w, unsigned n)
{
    int go = 1;
    while (go) {
        go = 0;
        for (unsigned i = 1; i < n; ++i)
            if (f[i - 1] > f[i]) {
                real t = f[i - 1]; f[i - 1] = f[i]; f[i] = t;
                t = w[i - 1]; w[i - 1] = w[i]; w[i] = t;
                go = 1;
            }
    }
}

/* filterSolution, pdflow_cudalib.cu:1040-1148: 3x3 weighted median of the
 * saturated (du,dv,dw).  `sel` (optional, 3*N ints) receives the bracketing
 * index `cont` chosen for each component, for selection-parity tests. */
void SFX(or_median)(unsigned R, unsigned C, const real* d_old, const real* ddt,
                    const real* du, const real* dv, const real* dw,
                    real* du_l, real* dv_l, real* dw_l, int32_t* sel)
{
    const long N = (long)R * C;
    const real kd = K(5.0), kddt = K(10.0);
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        const unsigned v = (unsigned)(i % R), u = (unsigned)(i / R);
        const real dz0 = d_old[i];
        if (dz0 > 0) {
            real fu[9], fv[9], fw[9], wu[9], wv[9], ww[9], cu[9], cv[9], cw[9];
            unsigned n = 0;
            for (int k = -1; k < 2; ++k)
                for (int l = -1; l < 2; ++l) {
                    const int ir = (int)v + k, ic = (int)u + l;
                    if (ir < 0 || ir >= (int)R || ic < 0 || ic >= (int)C) continue;
                    const long j = i + (long)l * R + k;
                    const real a = dz0 - d_old[j];
                    const real pres = K(1.0) / (K(1.0) + kd * (a * a) + kddt * (ddt[j] * ddt[j]));
                    fu[n] = du[j]; fv[n] = dv[j]; fw[n] = dw[j];
                    wu[n] = pres; wv[n] = pres; ww[n] = pres;
                    ++n;
                }
            or_bubble(fu, wu, n); or_bubble(fv, wv, n); or_bubble(fw, ww, n);
            cu[0] = wu[0]; cv[0] = wv[0]; cw[0] = ww[0];
            for (unsigned q = 1; q < n; ++q) {
                cu[q] = cu[q - 1] + wu[q];
                cv[q] = cv[q - 1] + wv[q];
                cw[q] = cw[q - 1] + ww[q];
            }
            const real med = K(0.5) * cu[n - 1];   /* half of u's total for all three (:1097) */
            const real* F[3] = {fu, fv, fw};
            const real* Cm[3] = {cu, cv, cw};
            real* O[3] = {du_l, dv_l, dw_l};
            for (int c = 0; c < 3; ++c) {
                unsigned cont = 0;
                while (med > Cm[c][cont]) ++cont;
                if (cont == 0) O[c][i] = F[c][0];
                else {
                    const unsigned r = cont, l = cont - 1;
                    O[c][i] = ((Cm[c][r] - med) * F[c][l] + (med - Cm[c][l]) * F[c][r]) / (Cm[c][r] - Cm[c][l]);
                }
                if (sel) sel[(long)c * N + i] = (int32_t)cont;
            }
        } else {
            du_l[i] = du[i]; dv_l[i] = dv[i]; dw_l[i] = dw[i];
            if (sel) { sel[i] = -1; sel[N + i] = -1; sel[2 * N + i] = -1; }
        }
    }
}

/* computeMotionField, pdflow_cudalib.cu:1150-1167.  `cols` is the finest
 * solved width (the reference uses `cols`, not `cols_i`, at :1152). */
void SFX(or_motion_field)(long N, unsigned cols, real fovh, const real* d_old,
                          const real* xx_old, const real* yy_old,
                          const real* du_l, const real* dv_l, const real* dw_l,
                          real* dx, real* dy, real* dz)
{
    const real inv_f = K(2.0) * RTAN(K(0.5) * fovh) / (real)cols;
    OMP_FOR
    for (long i = 0; i < N; ++i) {
        const real z = d_old[i];
        if (z > 0) {
            dx[i] = dw_l[i];
            dy[i] = z * du_l[i] * inv_f + dw_l[i] * xx_old[i] / z;
            dz[i] = z * dv_l[i] * inv_f + dw_l[i] * yy_old[i] / z;
        } else {
            dx[i] = 0; dy[i] = 0; dz[i] = 0;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Energy of a level solution (du, dv total image-plane flow in level pixels, */
/* dw in metres): the data and TV terms the iterations minimise, with the     */
/* warped residuals and data weight of the solver's own set-up at that flow:  */
/* Rij (:725-779), image gradients (:574-627), warping (:629-721), computeMu  */
/* (:781-784); forward differences as computeGradient (:982-1013).  The       */
/* reference has no energy; the GPU library's pdflow_energy_batch evaluates   */
/* the same functional.  Level images: [0] = old frame, [1] = new frame.      */
/* ------------------------------------------------------------------------- */
static real* or_alloc(size_t n);

double SFX(or_energy)(unsigned R, unsigned C, real mu_p, real li, real ld,
                      const real* const col[2], const real* const dep[2],
                      const real* const xx[2], const real* const yy[2],
                      const real* du, const real* dv, const real* dw)
{
    const long N = (long)R * C;
    real* w[14];
    for (int q = 0; q < 14; ++q) w[q] = or_alloc((size_t)N);
    real *ri = w[0], *rj = w[1], *ri2 = w[2], *rj2 = w[3], *dcu_a = w[4], *dcv_a = w[5], *ddu_a = w[6],
         *ddv_a = w[7], *dct = w[8], *dcu = w[9], *dcv = w[10], *ddt = w[11], *ddu = w[12], *ddv = w[13];
    SFX(or_rij)(R, C, xx[0], yy[0], dep[0], xx[1], yy[1], dep[1], ri, rj, ri2, rj2);
    SFX(or_im_gradients)(R, C, col[1], dep[1], ri2, rj2, dcu_a, dcv_a, ddu_a, ddv_a);
    SFX(or_warping)(R, C, col[1], col[0], dep[1], dep[0], dcu_a, dcv_a, ddu_a, ddv_a, du, dv,
                    dct, dcu, dcv, ddt, ddu, ddv);
    double e = 0.0;
    for (long i = 0; i < N; ++i) {
        const unsigned v = (unsigned)(i % R), u = (unsigned)(i / R);
        const int lu = (u == C - 1), lv = (v == R - 1);
        const real m = mu_p / (K(1.0) + K(1000.0) * (ddu[i] * ddu[i] + ddv[i] * ddv[i] + ddt[i] * ddt[i]));
        const double gu1 = lu ? 0.0 : (double)(ri[i] * (du[i + R] - du[i]));
        const double gu2 = lv ? 0.0 : (double)(rj[i] * (du[i + 1] - du[i]));
        const double gv1 = lu ? 0.0 : (double)(ri[i] * (dv[i + R] - dv[i]));
        const double gv2 = lv ? 0.0 : (double)(rj[i] * (dv[i + 1] - dv[i]));
        const double gw1 = lu ? 0.0 : (double)(ri[i] * (dw[i + R] - dw[i]));
        const double gw2 = lv ? 0.0 : (double)(rj[i] * (dw[i + 1] - dw[i]));
        e += fabs((double)dct[i]) + (double)m * fabs((double)ddt[i] - (double)dw[i]);
        e += (double)li * (hypot(gu1, gu2) + hypot(gv1, gv2)) + (double)ld * hypot(gw1, gw2);
    }
    for (int q = 0; q < 14; ++q) free(w[q]);
    return e;
}

/* ------------------------------------------------------------------------- */
/* Whole solve: PD_flow_opencv::createImagePyramidGPU (scene_flow_impair.cpp: */
/* 80-93) for two frames, then solveSceneFlowGPU (:95-168).                   */
/* Inputs are float column-major (R_img = height rows), the staging buffers  */
/* `I`, `Z` of the reference.  Outputs dx,dy,dz are rows*cols.               */
/* `dump` (optional) receives named intermediates per level for tests.       */
/* ------------------------------------------------------------------------- */
typedef void (*or_dump_fn)(void* ctx, const char* name, int level, const real* data, long n);

static real* or_alloc(size_t n) { return (real*)calloc(n ? n : 1, sizeof(real)); }

/* `first` > 0 starts at that level from `seed` ([3][N_first] floats: du, dv
 * in level pixels, dw in metres) instead of the upsampled coarser solution,
 * with zero duals (the GPU library's warm start); every solved level then
 * runs ceil(num_max_iter * iter_scale) iterations when iter_scale < 1. */
static int SFX(or_solve_impl)(unsigned rows, unsigned width, unsigned height,
                              const float* I1, const float* Z1, const float* I2, const float* Z2,
                              const unsigned* iters_override,
                              float* dx_out, float* dy_out, float* dz_out,
                              or_dump_fn dump, void* ctx,
                              unsigned first, const float* seed, double iter_scale)
{
    or_cfg c;
    if (or_make_cfg(&c, rows, width, height, iters_override) != 0) return -1;
    const long Nimg = (long)width * height;
    const unsigned P = c.pyr_levels;
    /* pyramid storage: [frame 0 = old, 1 = new][level] */
    real *col[2][OR_MAX_LEVELS], *dep[2][OR_MAX_LEVELS], *xx[2][OR_MAX_LEVELS], *yy[2][OR_MAX_LEVELS];
    for (int f = 0; f < 2; ++f)
        for (unsigned l = 0; l < P; ++l) {
            const long n = Nimg >> (2 * l);
            col[f][l] = or_alloc(n); dep[f][l] = or_alloc(n); xx[f][l] = or_alloc(n); yy[f][l] = or_alloc(n);
        }
    real* cin = or_alloc(Nimg); real* din = or_alloc(Nimg);
    for (int f = 0; f < 2; ++f) {
        const float* I = f ? I2 : I1; const float* Z = f ? Z2 : Z1;
        for (long i = 0; i < Nimg; ++i) { cin[i] = (real)I[i]; din[i] = (real)Z[i]; }
        /* GaussianPyramidBridge, pdflow_cudalib.cu:1172-1184 */
        for (unsigned l = 0; l < P; ++l) {
            const unsigned Ci = 640 / (c.cam_mode << l), Ri = 480 / (c.cam_mode << l);
            SFX(or_pyramid_level)(Ri, Ci, l == 0, cin, din, l ? col[f][l - 1] : 0, l ? dep[f][l - 1] : 0,
                                  c.g_mask, c.fovh, col[f][l], dep[f][l], xx[f][l], yy[f][l]);
            if (dump) {
                char nm[32];
                const long n = (long)Ri * Ci;
                memcpy(nm, f ? "pyr_new_" : "pyr_old_", 9);
                memcpy(nm + 8, "colour", 7); dump(ctx, nm, (int)l, col[f][l], n);
                memcpy(nm + 8, "depth", 6); dump(ctx, nm, (int)l, dep[f][l], n);
                memcpy(nm + 8, "xx", 3); dump(ctx, nm, (int)l, xx[f][l], n);
                memcpy(nm + 8, "yy", 3); dump(ctx, nm, (int)l, yy[f][l], n);
            }
        }
    }
    free(cin); free(din);

    const long Nmax = (long)c.rows * c.cols;
    real* s[S_N]; real* L[L_N]; real* aux[4]; real* gr[6]; real* dv3[3]; real* up[10]; real* lsol[10];
    for (int q = 0; q < S_N; ++q) s[q] = or_alloc(Nmax);
    for (int q = 0; q < L_N; ++q) L[q] = or_alloc(Nmax);
    for (int q = 0; q < 4; ++q) aux[q] = or_alloc(Nmax);
    for (int q = 0; q < 6; ++q) gr[q] = or_alloc(Nmax);
    for (int q = 0; q < 3; ++q) dv3[q] = or_alloc(Nmax);
    for (int q = 0; q < 10; ++q) { up[q] = or_alloc(Nmax); lsol[q] = or_alloc(Nmax); }
    real* ri2 = or_alloc(Nmax); real* rj2 = or_alloc(Nmax);
    real* dx = or_alloc(Nmax); real* dy = or_alloc(Nmax); real* dz = or_alloc(Nmax);
    const unsigned lw = or_log2u(width / c.cols);

    for (unsigned i = first; i < c.ctf_levels; ++i) {
        const unsigned sdiv = 1u << (c.ctf_levels - (i + 1));
        const unsigned Ci = c.cols / sdiv, Ri = c.rows / sdiv;
        const unsigned li = c.ctf_levels - i + lw - 1;    /* level_image, :108 */
        const long N = (long)Ri * Ci;
        /* assignZeros (:439-455) */
        for (int q = 0; q < S_N; ++q) memset(s[q], 0, sizeof(real) * (size_t)N);
        memset(L[L_DUP], 0, sizeof(real) * (size_t)N);
        memset(L[L_DVP], 0, sizeof(real) * (size_t)N);
        if (i == first && seed) {
            for (long k = 0; k < N; ++k) {
                L[L_DUP][k] = (real)seed[k];
                L[L_DVP][k] = (real)seed[N + k];
                s[S_DW][k] = (real)seed[2 * N + k];
                s[S_DWA][k] = (real)seed[2 * N + k];
            }
        } else if (i > 0) {
            const real* lc[10];
            for (int q = 0; q < 10; ++q) lc[q] = lsol[q];
            real* out8[8] = {s[S_DW], s[S_PD], s[S_PUU], s[S_PUV], s[S_PVU], s[S_PVV], s[S_PWU], s[S_PWV]};
            SFX(or_upsample)(Ri, Ci, lc, up, c.g_mask, L[L_DUP], L[L_DVP], out8);
            memcpy(s[S_DWA], s[S_DW], sizeof(real) * (size_t)N);   /* dw_acc = dw (:568) */
        }
        SFX(or_rij)(Ri, Ci, xx[0][li], yy[0][li], dep[0][li], xx[1][li], yy[1][li], dep[1][li],
                    L[L_RI], L[L_RJ], ri2, rj2);
        SFX(or_im_gradients)(Ri, Ci, col[1][li], dep[1][li], ri2, rj2, aux[0], aux[1], aux[2], aux[3]);
        SFX(or_warping)(Ri, Ci, col[1][li], col[0][li], dep[1][li], dep[0][li], aux[0], aux[1], aux[2], aux[3],
                        L[L_DUP], L[L_DVP], L[L_DCT], L[L_DCU], L[L_DCV], L[L_DDT], L[L_DDU], L[L_DDV]);
        real* st[8] = {L[L_SPD], L[L_SPUVX], L[L_SPUVY], L[L_SPWX], L[L_SPWY], L[L_TU], L[L_TV], L[L_TW]};
        SFX(or_mu_steps)(Ri, Ci, c.mu, c.lambda_i, c.lambda_d, L[L_DDU], L[L_DDV], L[L_DDT], L[L_RI], L[L_RJ],
                         L[L_MU], st);
        if (dump) {
            static const char* ln[L_N] = {"dct", "dcu", "dcv", "ddt", "ddu", "ddv", "mu", "ri", "rj", "du_prev",
                                          "dv_prev", "sigma_pd", "sigma_puvx", "sigma_puvy", "sigma_pwx",
                                          "sigma_pwy", "tau_u", "tau_v", "tau_w"};
            for (int q = 0; q < L_N; ++q) dump(ctx, ln[q], (int)i, L[q], N);
            dump(ctx, "ri_2", (int)i, ri2, N); dump(ctx, "rj_2", (int)i, rj2, N);
            static const char* sn0[S_N] = {"init_du", "init_dv", "init_dw", "init_du_acc", "init_dv_acc",
                                           "init_dw_acc", "init_pd", "init_puu", "init_puv", "init_pvu",
                                           "init_pvv", "init_pwu", "init_pwv"};
            for (int q = 0; q < S_N; ++q) dump(ctx, sn0[q], (int)i, s[q], N);
        }
        const real* Lc[L_N];
        for (int q = 0; q < L_N; ++q) Lc[q] = L[q];
        unsigned iters = c.num_max_iter[i];
        if (iter_scale < 1.0) iters = (unsigned)ceil((double)iters * iter_scale);
        for (unsigned it = 0; it < iters; ++it) {
            SFX(or_dual_step)(Ri, Ci, c.lambda_i, c.lambda_d, s, Lc, gr);
            SFX(or_primal_step)(Ri, Ci, c.lambda_i, c.lambda_d, s, Lc, dv3);
        }
        if (dump) {
            static const char* sn[S_N] = {"du_new", "dv_new", "dw_new", "du_acc", "dv_acc", "dw_acc", "pd",
                                          "puu", "puv", "pvu", "pvv", "pwu", "pwv"};
            for (int q = 0; q < S_N; ++q) dump(ctx, sn[q], (int)i, s[q], N);
        }
        SFX(or_saturate)(N, s[S_DU], s[S_DV], s[S_DW], L[L_DUP], L[L_DVP], dep[0][li]);
        if (dump) {
            dump(ctx, "sat_du", (int)i, s[S_DU], N); dump(ctx, "sat_dv", (int)i, s[S_DV], N);
            dump(ctx, "sat_dw", (int)i, s[S_DW], N);
        }
        SFX(or_median)(Ri, Ci, dep[0][li], L[L_DDT], s[S_DU], s[S_DV], s[S_DW], lsol[0], lsol[1], lsol[2], 0);
        for (int q = 0; q < 7; ++q) memcpy(lsol[3 + q], s[S_PD + q], sizeof(real) * (size_t)N);
        SFX(or_motion_field)(N, c.cols, c.fovh, dep[0][li], xx[0][li], yy[0][li], lsol[0], lsol[1], lsol[2],
                             dx, dy, dz);
        if (dump) {
            dump(ctx, "du_l", (int)i, lsol[0], N); dump(ctx, "dv_l", (int)i, lsol[1], N);
            dump(ctx, "dw_l", (int)i, lsol[2], N);
            dump(ctx, "dx", (int)i, dx, N); dump(ctx, "dy", (int)i, dy, N); dump(ctx, "dz", (int)i, dz, N);
        }
    }
    for (long i = 0; i < Nmax; ++i) {
        dx_out[i] = (float)dx[i]; dy_out[i] = (float)dy[i]; dz_out[i] = (float)dz[i];
    }
    for (int f = 0; f < 2; ++f)
        for (unsigned l = 0; l < P; ++l) { free(col[f][l]); free(dep[f][l]); free(xx[f][l]); free(yy[f][l]); }
    for (int q = 0; q < S_N; ++q) free(s[q]);
    for (int q = 0; q < L_N; ++q) free(L[q]);
    for (int q = 0; q < 4; ++q) free(aux[q]);
    for (int q = 0; q < 6; ++q) free(gr[q]);
    for (int q = 0; q < 3; ++q) free(dv3[q]);
    for (int q = 0; q < 10; ++q) { free(up[q]); free(lsol[q]); }
    free(ri2); free(rj2); free(dx); free(dy); free(dz);
    return 0;
}

/* Configuration query for tests: fills ctf_levels, pyr_levels, cols, cam_mode
 * and the 6-entry iteration schedule. */
int SFX(or_solve)(unsigned rows, unsigned width, unsigned height,
                  const float* I1, const float* Z1, const float* I2, const float* Z2,
                  const unsigned* iters_override,
                  float* dx_out, float* dy_out, float* dz_out,
                  or_dump_fn dump, void* ctx)
{
    return SFX(or_solve_impl)(rows, width, height, I1, Z1, I2, Z2, iters_override, dx_out, dy_out, dz_out, dump,
                              ctx, 0, 0, 1.0);
}

int SFX(or_solve_seeded)(unsigned rows, unsigned width, unsigned height,
                         const float* I1, const float* Z1, const float* I2, const float* Z2,
                         unsigned first, const float* seed, double iter_scale,
                         float* dx_out, float* dy_out, float* dz_out,
                         or_dump_fn dump, void* ctx)
{
    if (!seed || first == 0) return -1;
    return SFX(or_solve_impl)(rows, width, height, I1, Z1, I2, Z2, 0, dx_out, dy_out, dz_out, dump, ctx, first,
                              seed, iter_scale);
}

int SFX(or_config)(unsigned rows, unsigned width, unsigned height, unsigned* out10)
{
    or_cfg c;
    if (or_make_cfg(&c, rows, width, height, 0) != 0) return -1;
    out10[0] = c.cols; out10[1] = c.cam_mode; out10[2] = c.ctf_levels; out10[3] = c.pyr_levels;
    for (int i = 0; i < 6; ++i) out10[4 + i] = c.num_max_iter[i];
    return 0;
}

#ifndef OR_REAL_DOUBLE
/* Depth decode shared by every path: uint16 * (float)(1/5000), the value
 * OpenCV convertTo(CV_32FC1, 1.0/5000.0) produces for 16U input
 * (scene_flow_impair.cpp:242, :269), and the row-major -> column-major
 * packing of scene_flow_impair.cpp:230-245. */
void or_decode_frame(unsigned width, unsigned height, const uint8_t* img_rowmajor,
                     const uint16_t* depth_rowmajor, float* I_colmajor, float* Z_colmajor)
{
    const float scale = (float)(1.0 / 5000.0);
    for (unsigned u = 0; u < width; ++u)
        for (unsigned v = 0; v < height; ++v) {
            I_colmajor[v + u * height] = (float)img_rowmajor[(size_t)v * width + u];
            Z_colmajor[v + u * height] = (float)depth_rowmajor[(size_t)v * width + u] * scale;
        }
}

/* The live application's frame conversion (PD_flow_mrpt::CaptureFrame,
 * scene_flow_visualization.cpp:313-323): camera pixel (y, x) of a row-major
 * RGB888 + millimetre depth frame becomes
 *   colour(yc, xc) = (float)(0.299*r + 0.587*g + 0.114*b)   (double arithmetic)
 *   depth(yc, xc)  = 0.001f * mm                              (float)
 * at yc = height-1-y, xc = width-1-x (its loops walk the camera rows and
 * columns forward while counting yc and xc down; rotate180 = 0 stores (y, x)
 * in place), packed column-major as Eigen's MatrixXf::data() hands it to
 * copyNewFrames (scene_flow_visualization.cpp:115). */
void or_decode_frame_rgb8_mm(unsigned width, unsigned height, const uint8_t* rgb_rowmajor,
                             const uint16_t* depth_mm_rowmajor, int rotate180, float* I_colmajor, float* Z_colmajor)
{
    for (unsigned y = 0; y < height; ++y)
        for (unsigned x = 0; x < width; ++x) {
            const size_t i = (size_t)y * width + x;
            const unsigned yc = rotate180 ? height - 1 - y : y, xc = rotate180 ? width - 1 - x : x;
            const uint8_t* p = rgb_rowmajor + 3 * i;
            const double gray = 0.299 * p[0] + 0.587 * p[1] + 0.114 * p[2];
            I_colmajor[yc + xc * height] = (float)gray;
            Z_colmajor[yc + xc * height] = 0.001f * (float)depth_mm_rowmajor[i];
        }
}
#endif
