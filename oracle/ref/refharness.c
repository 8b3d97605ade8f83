/*
 * Host-side replay of the reference's solver driver over the reference's own
 * device code (TEST INFRASTRUCTURE ONLY: it produces the golden vectors that
 * pin the CPU oracle, and times the reference CUDA path for comparison).
 *
 * The reference's kernels come unmodified from oracle/_ref/pdflow_ref.cubin
 * (built from pdflow_cudalib.cu by oracle/ref/Makefile).  The reference's host
 * half cannot be built here (it needs OpenCV), so this file re-issues the
 * same host steps through the CUDA driver API, in the same order:
 *
 *   ctor + initializeCUDA       scene_flow_impair.cpp:31-69, :175-193
 *   readParameters              pdflow_cudalib.cu:176-193
 *   allocateDevMemory           pdflow_cudalib.cu:29-72
 *   createImagePyramidGPU       scene_flow_impair.cpp:80-93
 *     copyNewFrames             pdflow_cudalib.cu:195-222
 *     ObjectToDevice/BridgeBack pdflow_cudalib.cu:166-172, :1254-1258
 *     GaussianPyramidBridge     pdflow_cudalib.cu:1172-1184
 *   solveSceneFlowGPU           scene_flow_impair.cpp:95-168
 *     allocateMemoryNewLevel    pdflow_cudalib.cu:74-162
 *     freeLevelVariables        pdflow_cudalib.cu:290-326
 *     copyMotionField           pdflow_cudalib.cu:239-244
 *
 * including the per-level allocation churn, the fixed <<<256,128>>> launch
 * shape (pdflow_cudalib.h:28-29) and the whole-object copies, so that its
 * timing is the reference's.  Unlike the reference, every driver call is
 * checked and reported.
 */
#define _POSIX_C_SOURCE 199309L
#include <cuda.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "csf_layout.h"

#define NB 256u
#define NT 128u

typedef void (*refh_dump_fn)(void* ctx, const char* name, int level, const float* data, long n);

enum {
    K_PYR, K_ZERO, K_UPC, K_UPF, K_RIJ, K_GRAD, K_WARP, K_MUST, K_DUAL, K_PRIM, K_DIV, K_GRADIENT,
    K_SAT, K_FILT, K_MOTION, K_COUNT
};
static const char* kernel_names[K_COUNT] = {
    "ComputePyramidLevelKernel", "AssignZerosKernel", "UpsampleCopyKernel", "UpsampleFilterKernel",
    "RijKernel", "ComputeImGradients", "PerformWarping", "MuAndStepSizesKernel", "DualIteration",
    "PrimalIteration", "DivergenceComputation", "GradientComputation", "SaturateSolution",
    "FilterSolution", "MotionFieldKernel"};

/* Per-level arrays allocated by allocateMemoryNewLevel (pdflow_cudalib.cu:82-155), in order. */
static const unsigned level_fields[] = {
    CSF_OFF_dct_dev, CSF_OFF_dcu_dev, CSF_OFF_dcv_dev, CSF_OFF_ddt_dev, CSF_OFF_ddu_dev, CSF_OFF_ddv_dev,
    CSF_OFF_dcu_aux_dev, CSF_OFF_dcv_aux_dev, CSF_OFF_ddu_aux_dev, CSF_OFF_ddv_aux_dev,
    CSF_OFF_gradu1_dev, CSF_OFF_gradu2_dev, CSF_OFF_gradv1_dev, CSF_OFF_gradv2_dev, CSF_OFF_gradw1_dev,
    CSF_OFF_gradw2_dev, CSF_OFF_divpu_dev, CSF_OFF_divpv_dev, CSF_OFF_divpw_dev,
    CSF_OFF_sigma_pd_dev, CSF_OFF_sigma_puvx_dev, CSF_OFF_sigma_puvy_dev, CSF_OFF_sigma_pwx_dev,
    CSF_OFF_sigma_pwy_dev, CSF_OFF_tau_u_dev, CSF_OFF_tau_v_dev, CSF_OFF_tau_w_dev, CSF_OFF_mu_uv_dev,
    CSF_OFF_du_acc_dev, CSF_OFF_dv_acc_dev, CSF_OFF_dw_acc_dev,
    CSF_OFF_ri_dev, CSF_OFF_rj_dev, CSF_OFF_ri_2_dev, CSF_OFF_rj_2_dev, CSF_OFF_du_prev_dev, CSF_OFF_dv_prev_dev,
    CSF_OFF_du_new_dev, CSF_OFF_dv_new_dev, CSF_OFF_dw_new_dev, CSF_OFF_pd_dev, CSF_OFF_puu_dev, CSF_OFF_puv_dev,
    CSF_OFF_pvu_dev, CSF_OFF_pvv_dev, CSF_OFF_pwu_dev, CSF_OFF_pwv_dev,
    CSF_OFF_du_upsamp_dev, CSF_OFF_dv_upsamp_dev, CSF_OFF_dw_upsamp_dev, CSF_OFF_pd_upsamp_dev,
    CSF_OFF_puu_upsamp_dev, CSF_OFF_puv_upsamp_dev, CSF_OFF_pvu_upsamp_dev, CSF_OFF_pvv_upsamp_dev,
    CSF_OFF_pwu_upsamp_dev, CSF_OFF_pwv_upsamp_dev};
#define N_LEVEL_FIELDS (sizeof(level_fields) / sizeof(level_fields[0]))

/* Full-resolution solution arrays of allocateDevMemory (pdflow_cudalib.cu:62-71). */
static const unsigned sol_fields[] = {
    CSF_OFF_du_l_dev, CSF_OFF_dv_l_dev, CSF_OFF_dw_l_dev, CSF_OFF_pd_l_dev, CSF_OFF_puu_l_dev,
    CSF_OFF_puv_l_dev, CSF_OFF_pvu_l_dev, CSF_OFF_pvv_l_dev, CSF_OFF_pwu_l_dev, CSF_OFF_pwv_l_dev};
#define N_SOL_FIELDS (sizeof(sol_fields) / sizeof(sol_fields[0]))

typedef struct {
    CUcontext ctx;
    CUdevice dev;
    CUmodule mod;
    CUfunction k[K_COUNT];
    unsigned char obj[CSF_SIZEOF];       /* host image of the CSF_cuda object */
    unsigned rows, cols, width, height, cam_mode, ctf_levels, pyr_levels;
    unsigned num_max_iter[6];
    float g_mask[25];
    unsigned long long iter_dump_mask;   /* bit k: dump level-0 state after iteration k+1 */
    char err[256];
} refh;

static int fail(refh* h, const char* what, CUresult r)
{
    const char* s = 0;
    cuGetErrorString(r, &s);
    snprintf(h->err, sizeof h->err, "%s: %s (%d)", what, s ? s : "?", (int)r);
    return -(int)r - 1000;
}
#define CK(call) do { CUresult _r = (call); if (_r != CUDA_SUCCESS) return fail(h, #call, _r); } while (0)

static void set_u32(refh* h, unsigned off, unsigned v) { memcpy(h->obj + off, &v, 4); }
static void set_f32(refh* h, unsigned off, float v) { memcpy(h->obj + off, &v, 4); }
static void set_ptr(refh* h, unsigned off, CUdeviceptr p) { memcpy(h->obj + off, &p, 8); }
static CUdeviceptr get_ptr(const refh* h, unsigned off) { CUdeviceptr p; memcpy(&p, h->obj + off, 8); return p; }
static unsigned get_u32(const refh* h, unsigned off) { unsigned v; memcpy(&v, h->obj + off, 4); return v; }

static unsigned log2u(unsigned x) { unsigned l = 0; while (x > 1) { x >>= 1; ++l; } return l; }

const char* refh_error(refh* h) { return h ? h->err : "null handle"; }

void refh_set_iter_dump_mask(refh* h, unsigned long long mask) { if (h) h->iter_dump_mask = mask; }

static int launch(refh* h, int which, CUdeviceptr dobj, const unsigned* level)
{
    void* args[2] = {&dobj, (void*)level};
    CK(cuLaunchKernel(h->k[which], NB, 1, 1, NT, 1, 1, 0, 0, args, 0));
    return 0;
}

static int object_to_device(refh* h, CUdeviceptr* d)
{
    CK(cuMemAlloc(d, CSF_SIZEOF));
    CK(cuMemcpyHtoD(*d, h->obj, CSF_SIZEOF));
    return 0;
}

static int bridge_back(refh* h, CUdeviceptr d)
{
    CK(cuMemcpyDtoH(h->obj, d, CSF_SIZEOF));
    CK(cuMemFree(d));
    return 0;
}

/* Create: ctor, initializeCUDA, readParameters, allocateDevMemory. */
int refh_create(const char* cubin, unsigned rows, unsigned width, unsigned height, refh** out)
{
    *out = 0;
    refh* h = (refh*)calloc(1, sizeof(refh));
    if (!h) return -1;
    *out = h;
    if (!(rows == 15 || rows == 30 || rows == 60 || rows == 120 || rows == 240 || rows == 480)) {
        snprintf(h->err, sizeof h->err, "bad rows %u", rows);
        return -2;
    }
    h->rows = rows;
    h->cols = rows * 320 / 240;
    h->width = width; h->height = height;
    h->cam_mode = (height == 240) ? 2 : 1;
    h->ctf_levels = log2u(rows / 15) + 1;
    h->pyr_levels = log2u(width / h->cols) + h->ctf_levels;
    for (int i = 5; i >= 0; --i)
        h->num_max_iter[i] = (i >= (int)h->ctf_levels - 1) ? 100u : h->num_max_iter[i + 1] - 15u;
    static const int vm[5] = {1, 4, 6, 4, 1};
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) h->g_mask[i + 5 * j] = (float)(vm[i] * vm[j]) / 256.f;

    CK(cuInit(0));
    CK(cuDeviceGet(&h->dev, 0));
    CK(cuDevicePrimaryCtxRetain(&h->ctx, h->dev));
    CK(cuCtxSetCurrent(h->ctx));
    CK(cuModuleLoad(&h->mod, cubin));
    for (int k = 0; k < K_COUNT; ++k) {
        char mangled[96];
        snprintf(mangled, sizeof mangled, "_Z%zu%sP8CSF_cuda%s", strlen(kernel_names[k]), kernel_names[k],
                 k == K_PYR ? "j" : "");
        CK(cuModuleGetFunction(&h->k[k], h->mod, mangled));
    }
    /* readParameters */
    set_u32(h, CSF_OFF_rows, h->rows);
    set_u32(h, CSF_OFF_cols, h->cols);
    set_f32(h, CSF_OFF_lambda_i, 0.04f);
    set_f32(h, CSF_OFF_lambda_d, 0.35f);
    set_f32(h, CSF_OFF_mu, 75.f);
    set_u32(h, CSF_OFF_ctf_levels, h->ctf_levels);
    set_u32(h, CSF_OFF_cam_mode, h->cam_mode);
    set_f32(h, CSF_OFF_fovh, (float)(3.14159265358979323846 * 62.5 / 180.0));
    set_f32(h, CSF_OFF_fovv, (float)(3.14159265358979323846 * 48.5 / 180.0));
    CUdeviceptr p;
    CK(cuMemAlloc(&p, 25 * sizeof(float)));
    CK(cuMemcpyHtoD(p, h->g_mask, 25 * sizeof(float)));
    set_ptr(h, CSF_OFF_g_mask_dev, p);
    /* allocateDevMemory */
    const unsigned W = 640 / h->cam_mode, H = 480 / h->cam_mode;
    CK(cuMemAlloc(&p, (size_t)W * H * 4)); set_ptr(h, CSF_OFF_depth_wf_dev, p);
    CK(cuMemAlloc(&p, (size_t)W * H * 4)); set_ptr(h, CSF_OFF_colour_wf_dev, p);
    static const unsigned pyr[8] = {CSF_OFF_colour_dev, CSF_OFF_colour_old_dev, CSF_OFF_depth_dev, CSF_OFF_depth_old_dev,
                                    CSF_OFF_xx_dev, CSF_OFF_xx_old_dev, CSF_OFF_yy_dev, CSF_OFF_yy_old_dev};
    for (unsigned i = 0; i < h->pyr_levels; ++i) {
        const unsigned s = 1u << i;
        for (int a = 0; a < 8; ++a) {
            CK(cuMemAlloc(&p, (size_t)W * H * 4 / (s * s)));
            set_ptr(h, pyr[a] + 8 * i, p);
        }
    }
    CK(cuMemAlloc(&p, 4)); set_ptr(h, CSF_OFF_dx_dev, p);
    CK(cuMemAlloc(&p, 4)); set_ptr(h, CSF_OFF_dy_dev, p);
    CK(cuMemAlloc(&p, 4)); set_ptr(h, CSF_OFF_dz_dev, p);
    for (unsigned f = 0; f < N_SOL_FIELDS; ++f) {
        CK(cuMemAlloc(&p, (size_t)W * H * 4));
        set_ptr(h, sol_fields[f], p);
    }
    return 0;
}

static int dump_dev(refh* h, refh_dump_fn fn, void* ctx, const char* name, int level, CUdeviceptr src, long n)
{
    float* buf = (float*)malloc(sizeof(float) * (size_t)n);
    if (!buf) return -1;
    CUresult r = cuMemcpyDtoH(buf, src, sizeof(float) * (size_t)n);
    if (r != CUDA_SUCCESS) { free(buf); return fail(h, "dump", r); }
    fn(ctx, name, level, buf, n);
    free(buf);
    return 0;
}

/* createImagePyramidGPU (scene_flow_impair.cpp:80-93): copyNewFrames, then
 * the Gaussian pyramid of the new frame. */
int refh_push(refh* h, const float* I, const float* Z, refh_dump_fn dump, void* ctx)
{
    const unsigned W = 640 / h->cam_mode, H = 480 / h->cam_mode;
    CK(cuMemcpyHtoD(get_ptr(h, CSF_OFF_depth_wf_dev), Z, (size_t)W * H * 4));
    CK(cuMemcpyHtoD(get_ptr(h, CSF_OFF_colour_wf_dev), I, (size_t)W * H * 4));
    static const unsigned pairs[4][2] = {{CSF_OFF_colour_old_dev, CSF_OFF_colour_dev},
                                         {CSF_OFF_depth_old_dev, CSF_OFF_depth_dev},
                                         {CSF_OFF_xx_old_dev, CSF_OFF_xx_dev},
                                         {CSF_OFF_yy_old_dev, CSF_OFF_yy_dev}};
    for (unsigned i = 0; i < 8; ++i)
        for (int a = 0; a < 4; ++a) {
            CUdeviceptr o = get_ptr(h, pairs[a][0] + 8 * i), n = get_ptr(h, pairs[a][1] + 8 * i);
            set_ptr(h, pairs[a][0] + 8 * i, n);
            set_ptr(h, pairs[a][1] + 8 * i, o);
        }
    CUdeviceptr d;
    int rc = object_to_device(h, &d);
    if (rc) return rc;
    for (unsigned i = 0; i < h->pyr_levels; ++i) {
        const unsigned ci = 640 / (h->cam_mode << i), ri = 480 / (h->cam_mode << i);
        CK(cuMemcpyHtoD(d + CSF_OFF_rows_i, &ri, 4));
        CK(cuMemcpyHtoD(d + CSF_OFF_cols_i, &ci, 4));
        if ((rc = launch(h, K_PYR, d, &i))) return rc;
    }
    rc = bridge_back(h, d);
    if (rc) return rc;
    if (dump) {
        static const char* nm[4] = {"colour", "depth", "xx", "yy"};
        static const unsigned offs[4] = {CSF_OFF_colour_dev, CSF_OFF_depth_dev, CSF_OFF_xx_dev, CSF_OFF_yy_dev};
        for (unsigned i = 0; i < h->pyr_levels; ++i)
            for (int a = 0; a < 4; ++a) {
                char name[32];
                snprintf(name, sizeof name, "push_%s", nm[a]);
                const long n = (long)(W >> i) * (H >> i);
                if ((rc = dump_dev(h, dump, ctx, name, (int)i, get_ptr(h, offs[a] + 8 * i), n))) return rc;
            }
    }
    return 0;
}

/* solveSceneFlowGPU (scene_flow_impair.cpp:95-168). */
int refh_solve(refh* h, float* dxp, float* dyp, float* dzp, refh_dump_fn dump, void* ctx)
{
    const unsigned lw = log2u(h->width / h->cols);
    int rc;
    for (unsigned i = 0; i < h->ctf_levels; ++i) {
        const unsigned s = 1u << (h->ctf_levels - (i + 1));
        const unsigned ci = h->cols / s, ri = h->rows / s;
        const unsigned li = h->ctf_levels - i + lw - 1;
        const size_t bytes = (size_t)ri * ci * 4;
        const long n = (long)ri * ci;
        /* allocateMemoryNewLevel */
        set_u32(h, CSF_OFF_local_level, i);
        set_u32(h, CSF_OFF_level_image, li);
        set_u32(h, CSF_OFF_rows_i, ri);
        set_u32(h, CSF_OFF_cols_i, ci);
        CUdeviceptr p;
        for (unsigned f = 0; f < N_LEVEL_FIELDS; ++f) {
            CK(cuMemAlloc(&p, bytes));
            set_ptr(h, level_fields[f], p);
        }
        CK(cuMemFree(get_ptr(h, CSF_OFF_dx_dev)));
        CK(cuMemFree(get_ptr(h, CSF_OFF_dy_dev)));
        CK(cuMemFree(get_ptr(h, CSF_OFF_dz_dev)));
        CK(cuMemAlloc(&p, bytes)); set_ptr(h, CSF_OFF_dx_dev, p);
        CK(cuMemAlloc(&p, bytes)); set_ptr(h, CSF_OFF_dy_dev, p);
        CK(cuMemAlloc(&p, bytes)); set_ptr(h, CSF_OFF_dz_dev, p);

        CUdeviceptr d;
        if ((rc = object_to_device(h, &d))) return rc;
        if ((rc = launch(h, K_ZERO, d, 0))) return rc;
        if (i > 0) {
            if ((rc = launch(h, K_UPC, d, 0))) return rc;
            if ((rc = launch(h, K_UPF, d, 0))) return rc;
        }
        if ((rc = launch(h, K_RIJ, d, 0))) return rc;
        if ((rc = launch(h, K_GRAD, d, 0))) return rc;
        if ((rc = launch(h, K_WARP, d, 0))) return rc;
        if ((rc = launch(h, K_MUST, d, 0))) return rc;
        if (dump) {
            static const char* nm[] = {"dct", "dcu", "dcv", "ddt", "ddu", "ddv", "mu", "ri", "rj", "ri_2", "rj_2",
                                       "du_prev", "dv_prev", "sigma_pd", "sigma_puvx", "sigma_puvy", "sigma_pwx",
                                       "sigma_pwy", "tau_u", "tau_v", "tau_w", "init_dw", "init_dw_acc", "init_pd",
                                       "init_puu", "init_puv", "init_pvu", "init_pvv", "init_pwu", "init_pwv"};
            const unsigned offs[] = {CSF_OFF_dct_dev, CSF_OFF_dcu_dev, CSF_OFF_dcv_dev, CSF_OFF_ddt_dev,
                                     CSF_OFF_ddu_dev, CSF_OFF_ddv_dev, CSF_OFF_mu_uv_dev, CSF_OFF_ri_dev,
                                     CSF_OFF_rj_dev, CSF_OFF_ri_2_dev, CSF_OFF_rj_2_dev, CSF_OFF_du_prev_dev,
                                     CSF_OFF_dv_prev_dev, CSF_OFF_sigma_pd_dev, CSF_OFF_sigma_puvx_dev,
                                     CSF_OFF_sigma_puvy_dev, CSF_OFF_sigma_pwx_dev, CSF_OFF_sigma_pwy_dev,
                                     CSF_OFF_tau_u_dev, CSF_OFF_tau_v_dev, CSF_OFF_tau_w_dev, CSF_OFF_dw_new_dev,
                                     CSF_OFF_dw_acc_dev, CSF_OFF_pd_dev, CSF_OFF_puu_dev, CSF_OFF_puv_dev,
                                     CSF_OFF_pvu_dev, CSF_OFF_pvv_dev, CSF_OFF_pwu_dev, CSF_OFF_pwv_dev};
            for (unsigned q = 0; q < sizeof(offs) / sizeof(offs[0]); ++q)
                if ((rc = dump_dev(h, dump, ctx, nm[q], (int)i, get_ptr(h, offs[q]), n))) return rc;
        }
        for (unsigned it = 0; it < h->num_max_iter[i]; ++it) {
            if ((rc = launch(h, K_GRADIENT, d, 0))) return rc;
            if ((rc = launch(h, K_DUAL, d, 0))) return rc;
            if ((rc = launch(h, K_DIV, d, 0))) return rc;
            if ((rc = launch(h, K_PRIM, d, 0))) return rc;
            /* optional per-iteration snapshots of the coarsest level's state */
            if (dump && i == 0 && it + 1 < h->num_max_iter[i] && it < 64 && ((h->iter_dump_mask >> it) & 1ull)) {
                static const char* nm[] = {"du_new", "dv_new", "dw_new", "du_acc", "dv_acc", "dw_acc", "pd", "puu",
                                           "puv", "pvu", "pvv", "pwu", "pwv"};
                const unsigned offs[] = {CSF_OFF_du_new_dev, CSF_OFF_dv_new_dev, CSF_OFF_dw_new_dev,
                                         CSF_OFF_du_acc_dev, CSF_OFF_dv_acc_dev, CSF_OFF_dw_acc_dev, CSF_OFF_pd_dev,
                                         CSF_OFF_puu_dev, CSF_OFF_puv_dev, CSF_OFF_pvu_dev, CSF_OFF_pvv_dev,
                                         CSF_OFF_pwu_dev, CSF_OFF_pwv_dev};
                for (unsigned q = 0; q < sizeof(offs) / sizeof(offs[0]); ++q) {
                    char name[48];
                    snprintf(name, sizeof name, "it%u_%s", it + 1, nm[q]);
                    if ((rc = dump_dev(h, dump, ctx, name, (int)i, get_ptr(h, offs[q]), n))) return rc;
                }
            }
        }
        if (dump) {
            static const char* nm[] = {"du_new", "dv_new", "dw_new", "du_acc", "dv_acc", "dw_acc", "pd", "puu",
                                       "puv", "pvu", "pvv", "pwu", "pwv"};
            const unsigned offs[] = {CSF_OFF_du_new_dev, CSF_OFF_dv_new_dev, CSF_OFF_dw_new_dev, CSF_OFF_du_acc_dev,
                                     CSF_OFF_dv_acc_dev, CSF_OFF_dw_acc_dev, CSF_OFF_pd_dev, CSF_OFF_puu_dev,
                                     CSF_OFF_puv_dev, CSF_OFF_pvu_dev, CSF_OFF_pvv_dev, CSF_OFF_pwu_dev,
                                     CSF_OFF_pwv_dev};
            for (unsigned q = 0; q < sizeof(offs) / sizeof(offs[0]); ++q)
                if ((rc = dump_dev(h, dump, ctx, nm[q], (int)i, get_ptr(h, offs[q]), n))) return rc;
        }
        if ((rc = launch(h, K_SAT, d, 0))) return rc;
        if (dump) {
            if ((rc = dump_dev(h, dump, ctx, "sat_du", (int)i, get_ptr(h, CSF_OFF_du_new_dev), n))) return rc;
            if ((rc = dump_dev(h, dump, ctx, "sat_dv", (int)i, get_ptr(h, CSF_OFF_dv_new_dev), n))) return rc;
            if ((rc = dump_dev(h, dump, ctx, "sat_dw", (int)i, get_ptr(h, CSF_OFF_dw_new_dev), n))) return rc;
        }
        if ((rc = launch(h, K_FILT, d, 0))) return rc;
        if ((rc = launch(h, K_MOTION, d, 0))) return rc;
        if ((rc = bridge_back(h, d))) return rc;
        if (dump) {
            if ((rc = dump_dev(h, dump, ctx, "du_l", (int)i, get_ptr(h, CSF_OFF_du_l_dev), n))) return rc;
            if ((rc = dump_dev(h, dump, ctx, "dv_l", (int)i, get_ptr(h, CSF_OFF_dv_l_dev), n))) return rc;
            if ((rc = dump_dev(h, dump, ctx, "dw_l", (int)i, get_ptr(h, CSF_OFF_dw_l_dev), n))) return rc;
        }
        /* freeLevelVariables */
        for (unsigned f = 0; f < N_LEVEL_FIELDS; ++f) CK(cuMemFree(get_ptr(h, level_fields[f])));
        /* copyMotionField */
        CK(cuMemcpyDtoH(dxp, get_ptr(h, CSF_OFF_dx_dev), bytes));
        CK(cuMemcpyDtoH(dyp, get_ptr(h, CSF_OFF_dy_dev), bytes));
        CK(cuMemcpyDtoH(dzp, get_ptr(h, CSF_OFF_dz_dev), bytes));
        (void)get_u32;
    }
    return 0;
}

/* Wall-clock milliseconds of `reps` x (push frame 1, push frame 2, solve),
 * the offline evaluator's per-pair sequence (main_scene_flow_impair.cpp:169-175). */
int refh_time_pairs(refh* h, const float* I1, const float* Z1, const float* I2, const float* Z2,
                    float* dxp, float* dyp, float* dzp, int reps, double* ms_out)
{
    struct timespec a, b;
    int rc;
    CK(cuCtxSynchronize());
    clock_gettime(CLOCK_MONOTONIC, &a);
    for (int r = 0; r < reps; ++r) {
        if ((rc = refh_push(h, I1, Z1, 0, 0))) return rc;
        if ((rc = refh_push(h, I2, Z2, 0, 0))) return rc;
        if ((rc = refh_solve(h, dxp, dyp, dzp, 0, 0))) return rc;
    }
    CK(cuCtxSynchronize());
    clock_gettime(CLOCK_MONOTONIC, &b);
    *ms_out = ((double)(b.tv_sec - a.tv_sec) * 1e3 + (double)(b.tv_nsec - a.tv_nsec) * 1e-6) / reps;
    return 0;
}

/* freeDeviceMemory (pdflow_cudalib.cu:249-288) plus the context release. */
int refh_destroy(refh* h)
{
    if (!h) return 0;
    if (h->ctx) {
        cuCtxSetCurrent(h->ctx);
        cuMemFree(get_ptr(h, CSF_OFF_g_mask_dev));
        static const unsigned pyr[8] = {CSF_OFF_colour_dev, CSF_OFF_colour_old_dev, CSF_OFF_depth_dev,
                                        CSF_OFF_depth_old_dev, CSF_OFF_xx_dev, CSF_OFF_xx_old_dev, CSF_OFF_yy_dev,
                                        CSF_OFF_yy_old_dev};
        for (unsigned i = 0; i < h->pyr_levels; ++i)
            for (int a = 0; a < 8; ++a) cuMemFree(get_ptr(h, pyr[a] + 8 * i));
        for (unsigned f = 0; f < N_SOL_FIELDS; ++f) cuMemFree(get_ptr(h, sol_fields[f]));
        cuMemFree(get_ptr(h, CSF_OFF_colour_wf_dev));
        cuMemFree(get_ptr(h, CSF_OFF_depth_wf_dev));
        cuMemFree(get_ptr(h, CSF_OFF_dx_dev));
        cuMemFree(get_ptr(h, CSF_OFF_dy_dev));
        cuMemFree(get_ptr(h, CSF_OFF_dz_dev));
        if (h->mod) cuModuleUnload(h->mod);
        cuDevicePrimaryCtxRelease(h->dev);
    }
    free(h);
    return 0;
}
