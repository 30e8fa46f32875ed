/*
 * vkvg_gb300.h - entry points of the GB300 library that vkvg does not have.
 *
 * Plain C ABI: pointers, sizes and status codes only.  Each function states
 * which vkvg facility it stands in for, or that it has none.
 */
#ifndef VKVG_GB300_H
#define VKVG_GB300_H

#include "vkvg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Device pointer of the surface's resolved premultiplied RGBA8 image (row
   pitch width*4 bytes).  Replaces vkvg_surface_get_vk_image
   (include/vkvg.h:801) for a headless CUDA surface. */
vkvg_public void *vkvg_surface_get_device_ptr(VkvgSurface surf);
/* MSAA sample count of the surface (1 or 4). */
vkvg_public uint32_t vkvg_surface_get_samples(VkvgSurface surf);

/* ---- recorded frames (command-stream capture and replay) ------------------
 * Stands in for vkvg's recording/replay (src/recording/, vkvg_start_recording /
 * vkvg_replay, include/vkvg.h:1963-1970): the work a context has recorded since
 * its last flush is captured into device-resident command buffers and can be
 * executed any number of times on a surface of the same size. */
typedef struct _vkvg_gb300_frame_t *VkvgFrame;
/* Take the context's pending work (instead of running it at the next flush). */
vkvg_public VkvgFrame     vkvg_gb300_frame_capture(VkvgContext ctx);
/* Run a captured frame on surf (same width, height and sample count as the
   capturing context's surface).  Blocks until the frame has been drawn. */
vkvg_public vkvg_status_t vkvg_gb300_frame_execute(VkvgFrame frame, VkvgSurface surf);
/* Counters of the last execution: out[0] paths (fill/stroke draws), out[1]
   flattened points, out[2] stroke vertices, out[3] stroke indices, out[4] fill
   edges, out[5] bin references, out[6] segments, out[7] draws, out[8] kernel
   launches of the last execution. */
vkvg_public vkvg_status_t vkvg_gb300_frame_stats(VkvgFrame frame, uint64_t out[16]);
/* Average device time per kernel class of the last execution, in ms:
   out[0] flatten, out[1] stroke, out[2] setup+binning, out[3] raster. */
vkvg_public vkvg_status_t vkvg_gb300_frame_timing(VkvgFrame frame, float out[8]);
vkvg_public void          vkvg_gb300_frame_destroy(VkvgFrame frame);

/* ---- parity hooks (no vkvg counterpart) ----------------------------------
 * With debug capture on, a context keeps the device buffers of its last flush
 * so tests can compare them with the CPU restatement. */
vkvg_public void vkvg_gb300_debug_capture(VkvgContext ctx, int enable);
/* out[0] subpaths, out[1] points, out[2] draws, out[3] stroke vertices,
   out[4] stroke indices, out[5] device status word */
vkvg_public vkvg_status_t vkvg_gb300_debug_counts(VkvgContext ctx, uint32_t out[8]);
/* flattened points (x,y pairs) and per-point flags (bit 0: curve segment) */
vkvg_public vkvg_status_t vkvg_gb300_debug_points(VkvgContext ctx, float *xy, uint8_t *flags);
/* per subpath: first point index, point count, flags (bit 0: closed) */
vkvg_public vkvg_status_t vkvg_gb300_debug_subpaths(VkvgContext ctx, uint32_t *first, uint32_t *count,
                                                    uint32_t *flags);
/* draw i: kind (0 EO fill, 1 NZ fill, 2 stroke, 3 paint, 4 clear), first
   subpath, subpath count, stroke vertex count, stroke index count */
vkvg_public vkvg_status_t vkvg_gb300_debug_draw(VkvgContext ctx, uint32_t i, uint32_t info[8]);
/* stroke draw i's vertices (x,y) and draw-relative indices */
vkvg_public vkvg_status_t vkvg_gb300_debug_stroke(VkvgContext ctx, uint32_t i, float *xy, uint32_t *inds);
/* per-sample winding (fills) or covering-triangle count (strokes) of draw i,
   int32 [height][width][samples] */
vkvg_public vkvg_status_t vkvg_gb300_debug_coverage(VkvgContext ctx, uint32_t i, int32_t *out);
/* raw per-sample premultiplied RGBA8 of a surface, [height][width][samples][4] */
vkvg_public vkvg_status_t vkvg_gb300_surface_read_samples(VkvgSurface surf, uint8_t *out);
/* resolved premultiplied RGBA8 of a surface (before unpremultiplication) */
vkvg_public vkvg_status_t vkvg_gb300_surface_read_premult(VkvgSurface surf, uint8_t *out);

/* Portable transcendental functions used by the geometry kernels (fn: 0
   atan2f(a,b), 1 acosf, 2 cosf, 3 sinf, 4 asinf, 5 atanf), evaluated on the
   host (device = 0) or by a kernel (device = 1). */
vkvg_public vkvg_status_t vkvg_gb300_pmath_eval(int fn, const float *a, const float *b, float *out, uint64_t n,
                                                int device);

/* Number of kernels this library launched since the process started. */
vkvg_public uint64_t vkvg_gb300_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
