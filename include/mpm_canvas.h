/*
 * GPU 2D voxel canvas: scene generation for code_MPM.
 *
 * Replaces Canvas2D_CC (Canvas2D_CC.h:28-76, Canvas2D_CC.cpp:5-262), the
 * serial voxeliser the reference's scenes draw their cross-sections on
 * (e.g. the ring arrays of …Shim_Square.cpp:197-240) before turning the
 * active voxels into material points.  A canvas of floor(width / offset) x
 * floor(height / offset) voxels lives in device memory, voxel (ix, iy) at
 * (ix, iy) * offset + offset / 2, numbered ix + iy * nx.  Drawing calls queue
 * operations; the next read applies all queued operations, in call order, in
 * one pass over the voxels, with the reference's arithmetic (voxel membership
 * and surface flags bit for bit the reference's).  The active voxels come back
 * in voxel order (Canvas2D_CC::getVoxels_Active), to host or device memory.
 *
 * Return values are the MPM_OK / MPM_ERR_* codes of mpm_gb300.h.
 */
#ifndef MPM_CANVAS_H
#define MPM_CANVAS_H

#include <stdint.h>

#include "mpm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpm_canvas mpm_canvas;

/* Voxel flag bits */
#define MPM_VOXEL_ACTIVE 1u  /* Voxel_ST::b_Active */
#define MPM_VOXEL_SURFACE 2u /* Voxel_ST::b_Surface */

/* Canvas2D_CC::Canvas2D_CC(d2Size, dOffset), Canvas2D_CC.cpp:5-30 */
int mpm_canvas_create(double width, double height, double offset, mpm_canvas** out);
int mpm_canvas_destroy(mpm_canvas* canvas);
int mpm_canvas_size(const mpm_canvas* canvas, uint32_t* nx, uint32_t* ny);
const char* mpm_canvas_last_error(const mpm_canvas* canvas);

/* Drawing (queued): Canvas2D_CC::drawCircle (:43-56), drawRing (:58-83),
 * drawRectangle (:85-108, rotation in radians), drawPrism (:110-134),
 * cutCircle (:136-150), cutRectangle (:152-176). */
int mpm_canvas_draw_circle(mpm_canvas* canvas, double cx, double cy, double radius);
int mpm_canvas_draw_ring(mpm_canvas* canvas, double cx, double cy, double radius_outer, double radius_inner);
int mpm_canvas_draw_rectangle(mpm_canvas* canvas, double cx, double cy, double sx, double sy, double rotation);
int mpm_canvas_draw_prism(mpm_canvas* canvas, double cx, double cy, double sx, double sy, double extra,
                          double rotation);
int mpm_canvas_cut_circle(mpm_canvas* canvas, double cx, double cy, double radius);
int mpm_canvas_cut_rectangle(mpm_canvas* canvas, double cx, double cy, double sx, double sy, double rotation);

/* Reads (apply the queued operations first).  Pointers may be host or device
 * memory.  flags: nx * ny bytes.  Active voxels in voxel order: xy n x 2
 * centres, ids (Voxel_ST::u_ID), surface flags; any of the three may be NULL;
 * at most cap are written, *n receives the count (getCount_Active, :199-210). */
int mpm_canvas_flags(mpm_canvas* canvas, uint8_t* flags);
int mpm_canvas_count_active(mpm_canvas* canvas, uint64_t* n);
int mpm_canvas_active_voxels(mpm_canvas* canvas, double* xy, uint32_t* ids, uint8_t* surface, uint64_t cap,
                             uint64_t* n);

#ifdef __cplusplus
}
#endif

#endif /* MPM_CANVAS_H */
