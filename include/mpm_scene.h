/*
 * mpm_scene.h -- the cellular scenes' particle sets generated on the GPU.
 *
 * The reference builds its scenes on the CPU, voxel by voxel
 * (Canvas2D_CC.cpp:5-262 draws a cross-section, e.g. the ring arrays of
 * PhysicsEngine_initializeWorld_Classic_Cellular_Shim_Square.cpp:197-286, whose
 * active voxels become material points layer by layer).  These entry points
 * do the same for this build's cellular workloads on the device: a
 * square-cell cross-section on a lattice of spacing h/2 (8 particles per grid
 * cell), extruded into layers, with the surface particles (a lattice site with
 * an empty neighbour in the cross-section's plane) flagged.  The lattice
 * arithmetic is code_mpm_gb300/scenes.py's operation for operation (voxel
 * centres (i + 1/2) s, IEEE remainder and floor division, no contraction), so
 * positions, order and flags are that generator's bit for bit.  There is no
 * counterpart entry point in the reference.
 *
 * Outputs: pos, n x 3 row-major doubles, and surface, n bytes (1 = surface),
 * host or device memory (either may be NULL); at most cap particles are
 * written and *n receives the count.  Work runs on `stream` (a cudaStream_t,
 * NULL for the default stream) and the call returns when it is complete.
 * Return values are the MPM_OK / MPM_ERR_* codes of mpm_gb300.h.
 */
#ifndef MPM_SCENE_H
#define MPM_SCENE_H

#include <stdint.h>

#include "mpm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Square honeycomb, cross-section in x-z (scenes.honeycomb): ncell x ncell
 * cells of pitch `pitch` with walls `wall` thick, W = ncell pitch + wall wide;
 * a lattice site at c = (i + 1/2) h/2 on an axis is in a wall when
 * fmod(c, pitch) < wall and c < W, and a site is solid when it is in a wall on
 * x or on z.  Each solid site (x outer, z inner) gives `layers` particles at
 * y = (j + 1/2) h/2; all positions offset by origin. */
typedef struct mpm_honeycomb_desc {
    double wall, pitch, h;
    double origin[3];
    int32_t ncell, layers;
} mpm_honeycomb_desc;
int mpm_scene_honeycomb(const mpm_honeycomb_desc* desc, double* pos, uint8_t* surface, uint64_t cap, uint64_t* n,
                        void* stream);

/* Density-graded square-cell foam, walls extruded along z (scenes.graded_foam):
 * layer k at zc = (k + 1/2) h/2 has wall thickness t = t0 + (t1 - t0) zc /
 * height; on each axis a site c = (i + 1/2) h/2 belongs to cell k_c =
 * min(floor(c / pitch), ncell) and is in that cell's wall when
 * c - k_c pitch < t f[k_c], with f = fx on x and fy on y (ncell + 1 factors
 * each); a site is solid when it is in a wall on x or on y.  Particles layer
 * by layer, each layer x outer and y inner, at (x0 + c_x, y0 + c_y, z0 + zc);
 * `width` sites per axis. */
typedef struct mpm_foam_desc {
    double pitch, t0, t1, h, height;
    double x0, y0, z0;
    int32_t ncell, width, layers, pad;
    const double* fx; /* ncell + 1 factors (host memory) */
    const double* fy;
} mpm_foam_desc;
int mpm_scene_graded_foam(const mpm_foam_desc* desc, double* pos, uint8_t* surface, uint64_t cap, uint64_t* n,
                          void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MPM_SCENE_H */
