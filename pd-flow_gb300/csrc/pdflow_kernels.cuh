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
    // The step sizes as the iterations use them (levels run by the quad tiles):
    // spd*mu, spuvx*lambda_i, spuvy*lambda_i, spwx*lambda_d, spwy*lambda_d, tu, tv, tw.
    float* qs[8];
};

// Which step-size planes the warping kernel writes (launch_warp_steps).
enum StepPlanes : int {
    kStepsNone = 0,     // mu, and powf(ddt, 2) in spd for the median (tile levels that recompute their steps)
    kStepsRaw = 1,      // mu and the eight raw step-size planes (spd .. tw)
    kStepsQuads = 2,    // mu, powf(ddt, 2) in spd, and the eight iteration products in qs
    kStepsAll = 3,      // mu, the raw planes and the products (every iteration form can run)
};
// Whether the median reads powf(ddt, 2) from spd after a set-up of this kind.
inline bool steps_hold_ddt_sq(int mode) { return mode == kStepsNone || mode == kStepsQuads; }

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

// Level size plus the batch view: `pairs` solves share one arena, pair k's
// buffers sit k * pstride bytes after pair 0's (every pointer handed to a
// kernel is pair 0's; kernels take the pair from their grid's y index).
struct LevelGeom {
    unsigned R, C, N;
    unsigned pairs = 1;
    size_t pstride = 0;
    const unsigned* map = nullptr;   // device [pairs]: arena slot of grid index y (null: slot y)
    unsigned slots = 0;              // arena slots behind pstride (0: unknown)
};

// A map entry is an arena slot in its low 28 bits plus per-pair flags used by
// mixed-resolution batches, whose pairs end their levels at different steps.
constexpr unsigned kMapSlotMask = 0x0FFFFFFFu;
constexpr unsigned kMapLast = 1u << 31;     // tile launch: it ends the pair's level (saturate)
constexpr unsigned kMapFinest = 1u << 30;   // median: the pair's finest level (motion field)
constexpr unsigned kMapAlt = 1u << 29;      // median: the pair's final state is in the second buffers

#ifdef __CUDACC__
// Byte offset of the arena slot that grid index y works on.
__device__ __forceinline__ size_t pair_off(const unsigned* map, size_t pstride, unsigned y)
{
    return (size_t)(map ? (__ldg(map + y) & kMapSlotMask) : y) * pstride;
}
__device__ __forceinline__ unsigned pair_flags(const unsigned* map, unsigned y)
{
    return map ? (__ldg(map + y) & ~kMapSlotMask) : 0u;
}
#endif

template <class T>
__host__ __device__ __forceinline__ T* at(T* p, size_t off)
{
    return p ? reinterpret_cast<T*>(reinterpret_cast<uintptr_t>(p) + off) : p;
}
__host__ __device__ __forceinline__ PyrLevel at(PyrLevel a, size_t o)
{
    return PyrLevel{at(a.col, o), at(a.dep, o), at(a.xx, o), at(a.yy, o)};
}
__host__ __device__ __forceinline__ LevelConsts at(LevelConsts L, size_t o)
{
    LevelConsts r;
    r.ri = at(L.ri, o); r.rj = at(L.rj, o); r.ri2 = at(L.ri2, o); r.rj2 = at(L.rj2, o);
    r.dcu_aux = at(L.dcu_aux, o); r.dcv_aux = at(L.dcv_aux, o); r.ddu_aux = at(L.ddu_aux, o);
    r.ddv_aux = at(L.ddv_aux, o);
    r.dct = at(L.dct, o); r.dcu = at(L.dcu, o); r.dcv = at(L.dcv, o); r.ddt = at(L.ddt, o); r.ddu = at(L.ddu, o);
    r.ddv = at(L.ddv, o);
    r.mu = at(L.mu, o); r.du_prev = at(L.du_prev, o); r.dv_prev = at(L.dv_prev, o);
    r.spd = at(L.spd, o); r.spuvx = at(L.spuvx, o); r.spuvy = at(L.spuvy, o); r.spwx = at(L.spwx, o);
    r.spwy = at(L.spwy, o); r.tu = at(L.tu, o); r.tv = at(L.tv, o); r.tw = at(L.tw, o);
    for (int k = 0; k < 8; ++k) r.qs[k] = at(L.qs[k], o);
    return r;
}
__host__ __device__ __forceinline__ State at(State S, size_t o)
{
    return State{at(S.du, o), at(S.dv, o), at(S.dw, o), at(S.dua, o), at(S.dva, o), at(S.dwa, o), at(S.pd, o),
                 at(S.puu, o), at(S.puv, o), at(S.pvu, o), at(S.pvv, o), at(S.pwu, o), at(S.pwv, o)};
}
__host__ __device__ __forceinline__ LevelSol at(LevelSol s, size_t o)
{
    return LevelSol{at(s.du, o), at(s.dv, o), at(s.dw, o), at(s.pd, o), at(s.puu, o), at(s.puv, o), at(s.pvu, o),
                    at(s.pvv, o), at(s.pwu, o), at(s.pwv, o)};
}

struct Params {
    float lambda_i, lambda_d, mu, fovh;
    unsigned cols;  // finest solved width (motion-field focal length, pdflow_cudalib.cu:1152)
};

// ---- launchers (each returns the launch error) ----
// Pyramid launchers: `pairs` frames, pair k's arena buffers k * pstride bytes
// after pair 0's; the raw inputs of launch_decode_u16 are [pairs][H][W].
// A non-null `map` ([pairs] arena slots, device) redirects input k to slot map[k].
cudaError_t launch_decode_u16(const uint8_t* img, const uint16_t* depth, unsigned W, unsigned H, PyrLevel out,
                              float fovh, unsigned pairs, size_t pstride, cudaStream_t st,
                              const unsigned* map = nullptr);
// RGB888 [pairs][H][W][3] + millimetre depth [pairs][H][W] (the live application's conversion).
cudaError_t launch_decode_rgb8_mm(const uint8_t* rgb, const uint16_t* depth, unsigned W, unsigned H, PyrLevel out,
                                  float fovh, unsigned pairs, size_t pstride, cudaStream_t st, int rotate180);
cudaError_t launch_pyr_level0(const float* I, const float* Z, unsigned R, unsigned C, PyrLevel out, float fovh,
                              unsigned pairs, size_t pstride, cudaStream_t st, const unsigned* map = nullptr);
cudaError_t launch_pyr_down(PyrLevel prev, unsigned R, unsigned C, PyrLevel out, float fovh, unsigned pairs,
                            size_t pstride, cudaStream_t st, const unsigned* map = nullptr);
// Copies the planes of `src` over `dst` for the mapped slots (frame t becomes t-1).
cudaError_t launch_pyr_copy(PyrLevel src, PyrLevel dst, unsigned n, unsigned pairs, size_t pstride,
                            const unsigned* map, cudaStream_t st);
// `seed` (device, [pairs][3][N]: du, dv, dw in this level's pixels / metres)
// replaces the upsampled coarser solution; the duals then start at zero.
cudaError_t launch_level_init(LevelGeom g, bool first, LevelSol coarse, PyrLevel old_l, PyrLevel new_l,
                              LevelConsts L, State S, cudaStream_t st, const float* seed = nullptr);
// Energy of the level's solution `sol` (total du, dv in pixels, dw in metres),
// for the warp point set by launch_energy_prep + gradients + warping:
// sum over pixels of |dct| + mu |ddt - dw| + lambda_i (|r grad du| + |r grad dv|)
// + lambda_d |r grad dw|; energies[y] for grid index y.
cudaError_t launch_energy_prep(LevelGeom g, LevelSol sol, LevelConsts L, cudaStream_t st);
// part: device scratch of 1024 doubles per pair.
cudaError_t launch_energy(LevelGeom g, LevelSol sol, LevelConsts L, Params p, float* energies, double* part,
                          cudaStream_t st);
cudaError_t launch_im_gradients(LevelGeom g, PyrLevel new_l, LevelConsts L, cudaStream_t st);
// steps: which step-size planes to write (StepPlanes).
cudaError_t launch_warp_steps(LevelGeom g, PyrLevel old_l, PyrLevel new_l, LevelConsts L, Params p,
                              cudaStream_t st, int steps = kStepsRaw);
cudaError_t launch_dual(LevelGeom g, LevelConsts L, State S, Params p, cudaStream_t st);
cudaError_t launch_primal(LevelGeom g, LevelConsts L, State S, Params p, bool last, const float* depth_old,
                          cudaStream_t st);
cudaError_t launch_saturate(LevelGeom g, LevelConsts L, State S, const float* depth_old, cudaStream_t st);
// Copies level g's median output (du, dv, dw) and its motion field (the
// reference's computeMotionField at that level: focal length of the finest
// solved width p.cols, pdflow_cudalib.cu:1150-1167) into keep + slot * stride
// + off: six planes of g.N floats (du, dv, dw, dx, dy, dz).
cudaError_t launch_level_keep(LevelGeom g, LevelSol sol, PyrLevel old_l, Params p, float* keep, size_t stride,
                              size_t off, cudaStream_t st);
// `alt`: the second state buffers, read instead of S by pairs whose map entry
// carries kMapAlt (mixed batches); kMapFinest marks a pair's finest level.
cudaError_t launch_median(LevelGeom g, bool finest, PyrLevel old_l, LevelConsts L, State S, LevelSol out,
                          float* dx, float* dy, float* dz, Params p, int32_t* sel, cudaStream_t st,
                          const State* alt = nullptr, bool ddt_sq = false);   // ddt_sq: L.spd holds powf(ddt, 2)

}  // namespace pdflow
