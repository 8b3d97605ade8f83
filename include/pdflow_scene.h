/*
 * pdflow_scene.h - GPU renderer of the seeded synthetic RGB-D scenes the
 * solver is tested, trained and benchmarked on (no counterpart in the
 * reference, which reads camera frames or PNG files).
 *
 * A scene is a textured plane plus up to 8 boxes and spheres, each with a
 * two-octave 3D value-noise texture fixed to its surface; a frame is the
 * scene at one time step, ray-cast per pixel in double precision.  The host
 * fills the descriptors (geometry, poses, noise tables) and the kernel writes
 * uint8 intensity and uint16 depth (metres * 5000, the reference's PNG depth
 * scale) row-major, plus, optionally, the ground-truth scene flow to the next
 * time step.
 */
#ifndef PDFLOW_SCENE_H
#define PDFLOW_SCENE_H

#include <stdint.h>

#include "pdflow.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PDFLOW_SCENE_MAX_OBJECTS 8

/* Value noise on an integer lattice: lattice value vals[perm[(perm[(perm[x & 255]
 * + y) & 255] + z) & 255]], smoothstep-weighted trilinear interpolation,
 * octaves 0.65 * n(p / cell) + 0.35 * n((p + 17) / (cell / 2)). */
typedef struct pdflow_noise_tex {
    int32_t perm[256];
    double vals[256];
    double cell;
} pdflow_noise_tex;

typedef struct pdflow_scene_object {
    int32_t kind;           /* 0 = sphere (radius size[0]), 1 = box (half extents size[0..2]) */
    int32_t pad_;
    double center[3];       /* camera frame, metres, at the rendered frame */
    double rot[9];          /* object -> camera rotation, row-major, at the rendered frame */
    double next_center[3];  /* pose at the next frame (ground-truth flow) */
    double next_rot[9];
    double size[3];
    double albedo;
    pdflow_noise_tex tex;
} pdflow_scene_object;

typedef struct pdflow_scene_frame {
    uint32_t width, height;
    double fx, fy, cx, cy;
    double plane[3];                  /* z = plane[0] / (1 - plane[1] x/z - plane[2] y/z): z0 + a x + b y */
    pdflow_noise_tex plane_tex;
    uint32_t n_objects;
    uint32_t sensor_noise;            /* 1: depth noise sigma 1.5e-3 z^2 and 2 % zero holes */
    uint64_t noise_seed;              /* sensor-noise stream of this frame */
    pdflow_scene_object objects[PDFLOW_SCENE_MAX_OBJECTS];
} pdflow_scene_frame;

/* Renders n frames (host descriptors, all of one size) into device buffers
 * d_intensity [n][height][width] (uint8) and d_depth [n][height][width]
 * (uint16).  d_flow (may be NULL) receives [n][3][width*height] floats, the
 * ground-truth motion of each pixel's surface point to the next frame in the
 * solver's output convention and layout: dx = depth change, dy = horizontal,
 * dz = vertical (metres), column-major (idx = v + u * height).  Blocks until
 * done. */
int pdflow_render_frames(const pdflow_scene_frame* frames, unsigned n, uint8_t* d_intensity, uint16_t* d_depth,
                         float* d_flow, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PDFLOW_SCENE_H */
