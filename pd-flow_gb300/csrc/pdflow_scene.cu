// Synthetic RGB-D scene renderer (include/pdflow_scene.h): one thread per
// pixel casts the camera ray against the plane and the objects in double
// precision, textures the closest surface with its value noise, adds the
// sensor noise from a counter-based generator and writes the camera frame
// (and, optionally, the ground-truth scene flow).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "../../include/pdflow_scene.h"
#include "pdflow_internal.h"

namespace {

__device__ double octave(const pdflow_noise_tex& t, double px, double py, double pz, double scale)
{
    const double s = t.cell * scale;
    const double q[3] = {px / s, py / s, pz / s};
    double f[3], w[3];
    long long i[3];
    for (int k = 0; k < 3; ++k) {
        f[k] = floor(q[k]);
        const double tt = q[k] - f[k];
        w[k] = tt * tt * (3.0 - 2.0 * tt);
        i[k] = (long long)f[k];
    }
    double out = 0.0;
    for (int dx = 0; dx < 2; ++dx) {
        const double wx = dx ? w[0] : 1.0 - w[0];
        for (int dy = 0; dy < 2; ++dy) {
            const double wy = dy ? w[1] : 1.0 - w[1];
            for (int dz = 0; dz < 2; ++dz) {
                const double wz = dz ? w[2] : 1.0 - w[2];
                const long long ix = i[0] + dx, iy = i[1] + dy, iz = i[2] + dz;
                const int a = t.perm[ix & 255];
                const int b = t.perm[(a + iy) & 255];
                const int c = t.perm[(b + iz) & 255];
                out = out + wx * wy * wz * t.vals[c];
            }
        }
    }
    return out;
}

__device__ double value_noise(const pdflow_noise_tex& t, double px, double py, double pz)
{
    return (0.65 * octave(t, px, py, pz, 1.0) + 0.35 * octave(t, px + 17.0, py + 17.0, pz + 17.0, 0.5)) / 1.0;
}

__device__ unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ double uniform01(unsigned long long key)
{
    return ((double)(mix64(key) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

__global__ void k_render(const pdflow_scene_frame* __restrict__ frames, uint8_t* __restrict__ inten,
                         uint16_t* __restrict__ depth, float* __restrict__ flow)
{
    const pdflow_scene_frame& F = frames[blockIdx.y];
    const unsigned W = F.width, H = F.height;
    const unsigned pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= W * H) return;
    const unsigned v = pix / W, u = pix % W;   // row-major pixel
    const double xn = ((double)u - F.cx) / F.fx;
    const double yn = ((double)v - F.cy) / F.fy;
    const double d[3] = {xn, yn, 1.0};
    double zbest = F.plane[0] / (1.0 - F.plane[1] * xn - F.plane[2] * yn);
    int hit = -1;
    for (unsigned j = 0; j < F.n_objects; ++j) {
        const pdflow_scene_object& ob = F.objects[j];
        const double* c = ob.center;
        const double* r = ob.rot;
        double t = INFINITY;
        if (ob.kind == 0) {
            const double rad = ob.size[0];
            const double dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const double dc = d[0] * c[0] + d[1] * c[1] + d[2] * c[2];
            const double cc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
            const double disc = dc * dc - dd * (cc - rad * rad);
            if (disc > 0.0) t = (dc - sqrt(disc)) / dd;
        } else {
            double tn = -INFINITY, tf = INFINITY;
            for (int k = 0; k < 3; ++k) {
                // o_l = r^T (-c), d_l = r^T d
                const double ol = -(r[0 * 3 + k] * c[0] + r[1 * 3 + k] * c[1] + r[2 * 3 + k] * c[2]);
                const double dl = r[0 * 3 + k] * d[0] + r[1 * 3 + k] * d[1] + r[2 * 3 + k] * d[2];
                const double inv = 1.0 / dl;
                const double t1 = (-ob.size[k] - ol) * inv, t2 = (ob.size[k] - ol) * inv;
                tn = fmax(tn, fmin(t1, t2));   // fmax/fmin skip NaN as nanmax/nanmin do
                tf = fmin(tf, fmax(t1, t2));
            }
            if (tn <= tf && tf > 0.0) t = tn;
        }
        if (t < zbest) {
            zbest = t;
            hit = (int)j;
        }
    }
    double tex, gt[3] = {0.0, 0.0, 0.0};
    if (hit < 0) {
        tex = 0.15 + 0.8 * value_noise(F.plane_tex, d[0] * zbest, d[1] * zbest, d[2] * zbest);
    } else {
        const pdflow_scene_object& ob = F.objects[hit];
        const double* c = ob.center;
        const double* r = ob.rot;
        const double P[3] = {d[0] * zbest - c[0], d[1] * zbest - c[1], d[2] * zbest - c[2]};
        double L[3];
        for (int k = 0; k < 3; ++k) L[k] = P[0] * r[0 * 3 + k] + P[1] * r[1 * 3 + k] + P[2] * r[2 * 3 + k];
        tex = ob.albedo * (0.1 + 0.9 * value_noise(ob.tex, L[0], L[1], L[2]));
        if (flow) {
            const double* nc = ob.next_center;
            const double* nr = ob.next_rot;
            for (int k = 0; k < 3; ++k) {
                const double pn = nr[k * 3 + 0] * L[0] + nr[k * 3 + 1] * L[1] + nr[k * 3 + 2] * L[2] + nc[k];
                gt[k] = pn - d[k] * zbest;
            }
        }
    }
    double z = zbest;
    bool hole = false;
    if (F.sensor_noise) {
        const unsigned long long key = mix64(F.noise_seed) ^ ((unsigned long long)pix * 0xD1B54A32D192ED03ull);
        const double u1 = uniform01(key), u2 = uniform01(key + 1), u3 = uniform01(key + 2);
        const double g = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
        z = z + g * (1.5e-3 * z * z);
        hole = u3 < 0.02;
    }
    double zq = rint(z * 5000.0);
    zq = zq < 0.0 ? 0.0 : (zq > 65535.0 ? 65535.0 : zq);
    double iq = rint(tex * 255.0);
    iq = iq < 0.0 ? 0.0 : (iq > 255.0 ? 255.0 : iq);
    const size_t o = (size_t)blockIdx.y * W * H + pix;
    inten[o] = (uint8_t)iq;
    depth[o] = hole ? (uint16_t)0 : (uint16_t)zq;
    if (flow) {
        float* fl = flow + (size_t)blockIdx.y * 3 * W * H;
        const size_t cm = (size_t)v + (size_t)u * H;   // column-major, as the solver's output
        fl[cm] = (float)gt[2];                       // depth change
        fl[(size_t)W * H + cm] = (float)gt[0];       // horizontal
        fl[(size_t)2 * W * H + cm] = (float)gt[1];   // vertical
    }
}

}  // namespace

extern "C" int pdflow_render_frames(const pdflow_scene_frame* frames, unsigned n, uint8_t* d_intensity,
                                    uint16_t* d_depth, float* d_flow, void* stream)
{
    if (!frames || !d_intensity || !d_depth || n == 0) {
        pdflow::set_last_error("null argument or no frames");
        return PDFLOW_ERR_ARG;
    }
    for (unsigned k = 0; k < n; ++k)
        if (frames[k].width != frames[0].width || frames[k].height != frames[0].height ||
            frames[k].n_objects > PDFLOW_SCENE_MAX_OBJECTS || frames[k].width == 0 || frames[k].height == 0) {
            pdflow::set_last_error("frames must share one size and have at most 8 objects");
            return PDFLOW_ERR_ARG;
        }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    pdflow_scene_frame* d_frames = nullptr;
    cudaError_t e = cudaMalloc(&d_frames, sizeof(pdflow_scene_frame) * n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_frames, frames, sizeof(pdflow_scene_frame) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const unsigned px = frames[0].width * frames[0].height;
        k_render<<<dim3((px + 127) / 128, n), 128, 0, st>>>(d_frames, d_intensity, d_depth, d_flow);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_frames);
    if (e != cudaSuccess) return pdflow::set_error_code(PDFLOW_ERR_CUDA, "scene render", e);
    return PDFLOW_OK;
}
