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
   launches of the last execution, out[9] subpaths, out[10] stroke triangles,
   out[11] device status word, out[12] bytes of the uploaded command buffers. */
vkvg_public vkvg_status_t vkvg_gb300_frame_stats(VkvgFrame frame, uint64_t out[16]);
/* Device time of the last execution on the library's stream, in ms:
   out[0] flatten, out[1] stroke, out[2] setup+binning, out[3] raster,
   out[4] whole frame (first kernel to last, including size read-backs). */
vkvg_public vkvg_status_t vkvg_gb300_frame_timing(VkvgFrame frame, float out[8]);
vkvg_public void          vkvg_gb300_frame_destroy(VkvgFrame frame);

/* ---- command-stream replay ---------------------------------------------------
 * Stands in for vkvg_replay (include/vkvg.h:1965) over a flat wire format:
 * cmds[] holds vkvg's recording command codes (VKVG_CMD_*, the values of
 * src/recording/vkvg_record_internal.h:28-90) and args[] their float
 * arguments in call order (enums as float values, the vkvg_set_source_color
 * word as the bits of one float; VKVG_CMD_SET_DASH takes count, offset, then
 * count dash lengths).
 * Each command calls the matching vkvg_* function on ctx.  Returns the first
 * error: VKVG_STATUS_INVALID_INDEX for an unknown code or short args. */
#define VKVG_CMD_NEW_PATH          0x0101
#define VKVG_CMD_NEW_SUB_PATH      0x0102
#define VKVG_CMD_CLOSE_PATH        0x0103
#define VKVG_CMD_MOVE_TO           0x0104
#define VKVG_CMD_LINE_TO           0x0105
#define VKVG_CMD_RECTANGLE         0x0106
#define VKVG_CMD_ARC               0x0107
#define VKVG_CMD_ARC_NEG           0x0108
#define VKVG_CMD_CURVE_TO          0x010A
#define VKVG_CMD_QUADRATIC_TO      0x010B
#define VKVG_CMD_ELLIPTICAL_ARC_TO 0x010C
#define VKVG_CMD_SET_LINE_WIDTH    0x1101
#define VKVG_CMD_SET_MITER_LIMIT   0x1102
#define VKVG_CMD_SET_LINE_JOIN     0x1103
#define VKVG_CMD_SET_LINE_CAP      0x1104
#define VKVG_CMD_SET_OPERATOR      0x1105
#define VKVG_CMD_SET_FILL_RULE     0x1106
#define VKVG_CMD_SET_DASH          0x1107
#define VKVG_CMD_TRANSLATE         0x2001
#define VKVG_CMD_ROTATE            0x2002
#define VKVG_CMD_SCALE             0x2003
#define VKVG_CMD_IDENTITY_MATRIX   0x2005
#define VKVG_CMD_SET_MATRIX        0x2006
#define VKVG_CMD_REL_MOVE_TO       0x0504
#define VKVG_CMD_REL_LINE_TO       0x0505
#define VKVG_CMD_REL_CURVE_TO      0x050A
#define VKVG_CMD_REL_QUADRATIC_TO  0x050B
#define VKVG_CMD_PAINT             0x0201
#define VKVG_CMD_FILL              0x0202
#define VKVG_CMD_STROKE            0x0203
#define VKVG_CMD_CLEAR             0x0206
#define VKVG_CMD_FILL_PRESERVE     0x0602
#define VKVG_CMD_STROKE_PRESERVE   0x0603
#define VKVG_CMD_SET_SOURCE_RGB    0x0801
#define VKVG_CMD_SET_SOURCE_RGBA   0x0802
#define VKVG_CMD_SET_SOURCE_COLOR  0x0803
#define VKVG_CMD_SAVE              0x0001
#define VKVG_CMD_RESTORE           0x0002
#define VKVG_CMD_CLIP              0x0204
#define VKVG_CMD_RESET_CLIP        0x0205
#define VKVG_CMD_CLIP_PRESERVE     0x0604
vkvg_public vkvg_status_t vkvg_gb300_replay_stream(VkvgContext ctx, const uint32_t *cmds, uint32_t ncmds,
                                                   const float *args, uint64_t nargs);

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
/* The raster form frames use, for the whole process: -1 automatic (the
   default), 0 the register tile of 1024 pixels, 1 of 256 pixels, 2 of 128
   pixels, 3 the row form in half bands (16-bit counters; frames whose
   heaviest cell holds 2^15 records or more run 4 instead), 4 the row form in
   whole bands, 5 the register tile of 64 pixels.  Frames with clipping
   always run the first.  And the form the context's last flush ran (-1
   before any). */
vkvg_public void vkvg_gb300_debug_set_raster_form(int form);
vkvg_public int  vkvg_gb300_debug_raster_form(VkvgContext ctx);
/* Failure injection for the tests, process-wide (no vkvg counterpart; vkvg's
   own failure paths are a fence timeout, src/vkvg_context_internal.c:407-419,
   and allocation failures reported through the status sentinels):
     what 0: the value-th device buffer growth from now fails as an
             allocation failure would (1 the next one, 0 disarms);
     what 1: the row form's staging waits give up after value polls instead
             of 2^20 (0 restores), which sets the device status bit the host
             reports as VKVG_STATUS_DEVICE_ERROR;
     what 2: the subdivision work cap per cubic, in nodes (0 restores 2^22),
             beyond which a curve is cut short and reported the same way. */
vkvg_public void vkvg_gb300_debug_inject(int what, uint32_t value);
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

/* Exclusive prefix sum that allocates nothing.  No counterpart in the
 * reference: vkvg has no device-side scan; this is the scan the library's
 * pipeline uses to turn per-item counts into output offsets, offered to
 * callers that must not allocate device memory - a render loop whose frame
 * budget cannot absorb cudaMalloc's implicit device synchronisation, or a
 * process whose device memory is already held by another allocator.
 *
 * counts (n entries) and offsets (n + 1 entries) are device pointers;
 * offsets[i] = counts[0] + ... + counts[i-1] modulo 2^32 and offsets[n] is
 * the total.  Work is queued on stream (a cudaStream_t, 0 for the default
 * stream) and is finished when that stream is.  The scratch is a fixed array
 * inside the library's device image holding at most
 * VKVG_GB300_SCAN_NOALLOC_MAX items; larger n returns VKVG_STATUS_NO_MEMORY
 * and launches nothing.  Nothing has to be zeroed beforehand.
 *
 * The first call on each device (with that device current) looks the array's
 * address up, which may load the library's device code; make that first call
 * before any stream capture begins.  A device context created anew (after
 * cudaDeviceReset) gets the lookup again on its first call.  All calls on one device share the one
 * array, so calls that overlap in time - on different streams or host
 * threads - race and corrupt each other's results: order them. */
#define VKVG_GB300_SCAN_NOALLOC_MAX (1u << 26)
vkvg_public vkvg_status_t vkvg_gb300_exclusive_scan_noalloc(void *stream, const uint32_t *counts, uint32_t n,
                                                             uint32_t *offsets);

/* ---- batches (no vkvg counterpart): the recorded frames of many contexts
 * (vkvg_gb300_frame_capture), each for its own surface, rendered as one job:
 * one pass of the geometry kernels over all of them and one persistent
 * raster launch over every surface's bands, heaviest first.  The first
 * execution sizes the job, the next twelve time candidate raster settings
 * (tile width, stage threshold, work-list order; kept per class of scene
 * for later batches), later ones replay a CUDA graph of the whole job.
 * Pattern sources (gradients, surface sources) are batched: each surface's
 * source images are filled into a block of their own every execution.
 * Frames with clip, or a surface with an active clip, are not batched
 * (create returns null).  Each surface
 * ends as vkvg_gb300_frame_execute of its frame would leave it.
 * timing out: [0] last execution ms, [1] it was a graph replay, [2] stage
 * threshold, [3] heaviest-first order, [4] work items, [5] surfaces,
 * [6] settings tuned, [7] bin record units, [8] tile width in pixels. */
typedef struct _vkvg_gb300_batch_t *VkvgBatch;
vkvg_public VkvgBatch     vkvg_gb300_batch_create(VkvgFrame *frames, VkvgSurface *targets, uint32_t count);
vkvg_public vkvg_status_t vkvg_gb300_batch_execute(VkvgBatch batch);
vkvg_public vkvg_status_t vkvg_gb300_batch_timing(VkvgBatch batch, float out[9]);
vkvg_public void          vkvg_gb300_batch_destroy(VkvgBatch batch);

/* ---- parsed SVG documents, read back for the parity tests (no vkvg
 * counterpart; the handle is include/vkvg-svg.h's VkvgSvg).  shape: u = fill
 * paint type (0 none, 1 colour, 2 linear gradient, 3 radial gradient), fill
 * colour, stroke paint type, stroke colour (ABGR words, r in the low byte; a
 * gradient gives its first stop's), visible, subpath count; f = opacity,
 * stroke width, box[4] (x0, y0, x1, y1).  path: its cubic points (x, y
 * pairs; 1 + 3n of them), at most cap_points copied, and whether it is
 * closed.  Both return 0, or -1 for an index out of range. */
typedef struct _vkvg_svg_t *VkvgSvgDoc;
vkvg_public uint32_t vkvg_gb300_svg_shape_count(VkvgSvgDoc svg);
vkvg_public int      vkvg_gb300_svg_shape(VkvgSvgDoc svg, uint32_t i, char id[64], uint32_t u[6], float f[6]);
vkvg_public int      vkvg_gb300_svg_path(VkvgSvgDoc svg, uint32_t shape, uint32_t path, float *pts, uint32_t cap_points,
                                         uint32_t *npts, uint32_t *closed);

/* ---- differentiable analytic coverage (no vkvg counterpart) ----
 *
 * A scene of paths, each a list of closed contours of line and cubic
 * segments over one array of control points: a segment of kind k consumes k
 * control points (its start point, then a cubic's two inner control points)
 * and ends at the next segment's start, the last segment of a contour at
 * the contour's first point.  Cubics are flattened by vkvg's
 * _recursive_bezier at vkvg's default tolerance.  Every path draws, in path
 * order, a fill layer (VKVG_GB300_ANALYTIC_FILL: NON_ZERO, coverage
 * min(1, |A|) with A the exact area integral of the winding number over the
 * pixel) and a stroke layer (VKVG_GB300_ANALYTIC_STROKE: one rectangle of
 * half-width w/2 per flattened segment and one bevel triangle on the outer
 * side of every joint, coverage min(1, the sum of their areas in the
 * pixel)), both in the path's premultiplied RGBA colour, composited with
 * source-over onto the background into a W x H fp32 RGBA canvas.
 *
 * Parameters are device pointers (CUDA memory): ctrl [control points][2],
 * colors [paths][4] premultiplied RGBA, widths [paths]; canvas and target
 * [H][W][4].  Calls are queued on the scene's stream (set_stream, default: a
 * stream of its own) and return at once; sync waits and returns the first
 * error of the calls since the last sync.  VKVG_STATUS_NO_MEMORY from sync
 * means a flattening outgrew the point buffer: the results since the last
 * sync are zero, the buffer has been grown, and the calls must be repeated.
 *
 * forward renders the canvas (copied to canvas when it is not null) and,
 * when target is not null, the loss mean((canvas - target)^2) into loss[0].
 * backward returns the gradients of the last forward's parameters: of its
 * loss when d_canvas is null (that forward must have had a target), else of
 * sum(d_canvas * canvas).  d_ctrl, d_colors and d_widths are overwritten.
 * The flattening is walked again in the backward pass, not stored; the
 * parameters must not change between forward and backward.
 * adam applies one Adam step (bias-corrected, step >= 1) to n parameters
 * and clamps them to [lo, hi]. */
#define VKVG_GB300_SEG_LINE        1
#define VKVG_GB300_SEG_CUBIC       3
#define VKVG_GB300_ANALYTIC_FILL   1u
#define VKVG_GB300_ANALYTIC_STROKE 2u
typedef struct _vkvg_gb300_analytic_t *VkvgAnalytic;
vkvg_public VkvgAnalytic  vkvg_gb300_analytic_create(uint32_t width, uint32_t height, const float background[4],
                                                     uint32_t npaths, const uint32_t *path_ncontours,
                                                     const uint32_t *path_flags, uint32_t ncontours,
                                                     const uint32_t *contour_nseg, uint32_t nseg,
                                                     const uint8_t *seg_kind);
/* The same scene evaluated in square tiles of `tile` pixels (16 to 4096):
   after the flattening, each layer's box gives the tiles it reaches (a layer
   is zero outside its box), and every tile runs the coverage and compositing
   of its own layers, its area planes kept resident for the backward (memory:
   the sum over tiles of tile pixels x layers reaching the tile, four bytes
   each, plus a sixteenth of that in checkpoints of sixteen bytes).  For
   canvases whose whole-canvas planes would not fit (a 4096 x 4096 canvas of
   200,000 glyph outlines); results equal the whole-canvas scene's.  A tiled
   forward waits once for the per-tile layer counts. */
vkvg_public VkvgAnalytic  vkvg_gb300_analytic_create_tiled(uint32_t width, uint32_t height, uint32_t tile,
                                                           const float background[4], uint32_t npaths,
                                                           const uint32_t *path_ncontours, const uint32_t *path_flags,
                                                           uint32_t ncontours, const uint32_t *contour_nseg,
                                                           uint32_t nseg, const uint8_t *seg_kind);
vkvg_public void          vkvg_gb300_analytic_destroy(VkvgAnalytic a);
vkvg_public vkvg_status_t vkvg_gb300_analytic_status(VkvgAnalytic a);
vkvg_public uint32_t      vkvg_gb300_analytic_control_point_count(VkvgAnalytic a);
vkvg_public uint32_t      vkvg_gb300_analytic_layer_count(VkvgAnalytic a);
vkvg_public vkvg_status_t vkvg_gb300_analytic_set_stream(VkvgAnalytic a, void *stream);
vkvg_public vkvg_status_t vkvg_gb300_analytic_forward(VkvgAnalytic a, const float *ctrl, const float *colors,
                                                      const float *widths, const float *target, float *canvas,
                                                      float *loss);
vkvg_public vkvg_status_t vkvg_gb300_analytic_backward(VkvgAnalytic a, const float *d_canvas, float *d_ctrl,
                                                       float *d_colors, float *d_widths);
vkvg_public vkvg_status_t vkvg_gb300_analytic_adam(VkvgAnalytic a, float *param, const float *grad, float *m,
                                                   float *v, uint32_t n, float lr, float beta1, float beta2,
                                                   float eps, uint32_t step, float lo, float hi);
vkvg_public vkvg_status_t vkvg_gb300_analytic_sync(VkvgAnalytic a);
/* the last forward's flattened points (host copy, at most cap points; syncs):
   returns their count; seg_offsets, if not null, gets nseg+1 offsets */
vkvg_public uint32_t      vkvg_gb300_analytic_points(VkvgAnalytic a, float *pts, uint32_t cap, uint32_t *seg_offsets);
/* phase times of the last forward and backward, ms (set_timing(a, 1) first;
   syncs): [0] flattening, [1] coverage, [2] compositing and loss, [3]
   compositing adjoint and colour reduction, [4] coverage adjoint, [5]
   flattening adjoint */
vkvg_public vkvg_status_t vkvg_gb300_analytic_set_timing(VkvgAnalytic a, int on);
vkvg_public vkvg_status_t vkvg_gb300_analytic_timing(VkvgAnalytic a, float out[6]);
/* the last backward's gradient with respect to each flattened point (host
   copy of at most cap points, x and y; syncs): returns the point count */
vkvg_public uint32_t      vkvg_gb300_analytic_point_grads(VkvgAnalytic a, float *grads, uint32_t cap);

#ifdef __cplusplus
}
#endif
#endif
