// Kernel declarations and the device-side views of the solver's arena.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pdflow {

// One pyramid level of one frame (column-major planes of R*C floats).
struct PyrLevel {
    float* col;
    float* dep;
    float* xx;
    float* yy;
};

// Per-level constants produced by the set-up kernels (planes of N floats).
struct LevelConsts {
    float *ri, *rj, *ri2, *rj2;
    float *dcu_aux, *dcv_aux, *ddu_aux, *ddv_aux;
    float *dct, *dcu, *dcv, *ddt, *ddu, *ddv;
    float *mu, *du_prev, *dv_prev;
    float *spd, *spuvx, *spuvy, *spwx, *spwy, *tu, *tv, *tw;
};

// Primal-dual state (planes of N floats).
struct State {
    float *du, *dv, *dw, *dua, *dva, *dwa;
    float *pd, *puu, *puv, *pvu, *pvv, *pwu, *pwv;
};

// Previous level's solution: median-filtered (du,dv,dw) + the 7 duals
// (the reference's *_l arrays, pdflow_cudalib.h:109-113).
struct LevelSol {
    float *du, *dv, *dw, *pd, *puu, *puv, *pvu, *pvv, *pwu, *pwv;
};

struct LevelGeom {
    unsigned R, C, N;
};

struct Params {
    float lambda_i, lambda_d, mu, fovh;
    unsigned cols;  // finest solved width (motion-field focal length, pdflow_cudalib.cu:1152)
};

// ---- launchers (each returns the launch error) ----
cudaError_t launch_decode_u16(const uint8_t* img, const uint16_t* depth, unsigned W, unsigned H, PyrLevel out,
                              float fovh, cudaStream_t st);
cudaError_t launch_pyr_level0(const float* I, const float* Z, unsigned R, unsigned C, PyrLevel out, float fovh,
                              cudaStream_t st);
cudaError_t launch_pyr_down(PyrLevel prev, unsigned R, unsigned C, PyrLevel out, float fovh, cudaStream_t st);
cudaError_t launch_level_init(LevelGeom g, bool first, LevelSol coarse, PyrLevel old_l, PyrLevel new_l,
                              LevelConsts L, State S, cudaStream_t st);
cudaError_t launch_im_gradients(LevelGeom g, PyrLevel new_l, LevelConsts L, cudaStream_t st);
cudaError_t launch_warp_steps(LevelGeom g, PyrLevel old_l, PyrLevel new_l, LevelConsts L, Params p,
                              cudaStream_t st);
cudaError_t launch_dual(LevelGeom g, LevelConsts L, State S, Params p, cudaStream_t st);
cudaError_t launch_primal(LevelGeom g, LevelConsts L, State S, Params p, bool last, const float* depth_old,
                          cudaStream_t st);
cudaError_t launch_saturate(LevelGeom g, LevelConsts L, State S, const float* depth_old, cudaStream_t st);
cudaError_t launch_median(LevelGeom g, bool finest, PyrLevel old_l, LevelConsts L, State S, LevelSol out,
                          float* dx, float* dy, float* dz, Params p, int32_t* sel, cudaStream_t st);

}  // namespace pdflow
