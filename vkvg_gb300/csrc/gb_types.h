/*
 * Record layouts shared by the host recorder and the sm_103a kernels.
 *
 * A flush ships one "frame" of recorded work to the device as structure-of-
 * arrays command buffers:
 *   segments  - one record per path element (point, cubic, arc, elliptic arc)
 *   subpaths  - contiguous runs of segments, with the closed flag
 *   draws     - fill / stroke / paint / clear calls in submission order
 *   pairs     - (draw, subpath) work items of stroke and fill draws
 * and the kernels expand them: flatten -> stroke expansion -> edge setup and
 * band binning -> per-band coverage and compositing.
 */
#ifndef VKVG_GB300_TYPES_H
#define VKVG_GB300_TYPES_H

#include <stdint.h>

/* segment kinds (low 4 bits of seg_info) */
#define GB_SEG_POINT   1u /* one explicit point (move_to, line_to, rectangle corner, arc end point) */
#define GB_SEG_CUBIC   2u /* adaptive Bezier subdivision + end point */
#define GB_SEG_ARC     3u /* fixed-step circular arc, seg_n loop points */
#define GB_SEG_ELLIPSE 4u /* elliptic arc, seg_n points at host-walked angles */
#define GB_SEG_KIND(i) ((i) & 0xFu)
/* segment flags */
#define GB_SEG_CURVED    0x100u /* emitted points lie in a curve segment (curve joins in strokes) */
#define GB_SEG_DROP_LAST 0x200u /* close_path removed this segment's last point */

/* subpath flags */
#define GB_SUB_CLOSED 0x1u

/* draw kinds */
#define GB_DRAW_FILL_EO 0u
#define GB_DRAW_FILL_NZ 1u
#define GB_DRAW_STROKE  2u
#define GB_DRAW_PAINT   3u
#define GB_DRAW_CLEAR   4u
/* clip: vkvg keeps it in the stencil, a clip bit and six save bits per
   sample, plus a full copy of the stencil for every further six saves
   (src/vkvg_context.c:1251-1512).  Here the surface holds it as bit planes,
   one bit per sample: the visibility plane (the inverse of the clip bit), six
   save planes (the save bits) and, per stencil copy, an image of seven planes
   (visibility, then the six save planes).
     CLIP_EO / CLIP_NZ   visibility &= the path's coverage (geometry as a fill)
     CLIP_RESET          visibility = all, save planes = 0 (so does CLEAR)
     CLIP_SAVE    src=p  save plane p = clip bit (= ~visibility)
     CLIP_RESTORE src=p  visibility = ~save plane p
     CLIP_STORE   src=k  image k = visibility and the save planes
     CLIP_LOAD    src=k  visibility and the save planes = image k */
#define GB_DRAW_CLIP_EO      5u
#define GB_DRAW_CLIP_NZ      6u
#define GB_DRAW_CLIP_RESET   7u
#define GB_DRAW_CLIP_SAVE    8u
#define GB_DRAW_CLIP_RESTORE 9u
#define GB_DRAW_CLIP_STORE   10u
#define GB_DRAW_CLIP_LOAD    11u
#define GB_CLIP_SAVE_PLANES  6u
#define GB_CLIP_IMAGE_PLANES 7u

/* operators (vkvg_operator_t) */
#define GB_OP_CLEAR      0u
#define GB_OP_SOURCE     1u
#define GB_OP_OVER       2u
#define GB_OP_DIFFERENCE 3u

/* one recorded draw call */
typedef struct {
    uint32_t kind;
    uint32_t op;
    uint32_t join; /* vkvg_line_join_t */
    uint32_t cap;  /* vkvg_line_cap_t */
    uint32_t src;  /* premultiplied RGBA8 source after opacity, byte 0 = R */
    uint32_t sub_first, sub_count;
    uint32_t dash_first, dash_count;
    float    dash_offset;
    float    hw;       /* line width / 2 */
    float    lh_max;   /* miter limit * line width */
    float    arc_step; /* _get_arc_step(hw) under the draw's CTM */
    float    mat[6];   /* xx yx xy yy x0 y0 */
    uint32_t gsrc;     /* 0: the solid colour src; i + 1: gradient source image i of the frame */
    uint32_t surf;     /* its surface's entry in the frame's surface table (0 but in a batch) */
} gb_draw;

/* One target surface of a frame (one entry for a context's frame; one per
   surface for a batch of frames): its size and sample buffers, its draws
   [draw0, draw0 + ndraws) of the frame, and its bins, cells
   [cell0, cell0 + nbands * ndraws) band-major; init_* describe a first draw
   the raster can apply while loading the tile (a clear or an opaque paint). */
typedef struct {
    uint32_t  W, H, nrows, nbands, wpad;
    uint32_t  draw0, ndraws, draw_first;
    uint32_t  init_mode, init_color;
    uint64_t  cell0;
    uint32_t *samples; /* [nrows][wpad] premultiplied RGBA8 */
    uint32_t *rgba;    /* [H][W] resolved */
    const uint32_t *gsrc; /* the surface's pattern source images [n][H][W] (batches; else null) */
} gb_surf;

/* A pattern source as vkvg's fragment stage sees it (shaders/vkvg_main.frag
   SURFACE, LINEAR and RADIAL cases).  Gradients (data of _update_cur_pattern):
   control points transformed by the pattern's inverse matrix and the CTM at
   vkvg_set_source time, in pixels, in vkvg's layout of two vec4 (linear:
   x0 y0 x1 y1; radial: cx0 cy0 r0 - and cx1 cy1 r1 -); stops; premultiplied
   stop colours.  Surfaces (push constants of the draw): the source surface's
   resolved image, its size, the sampler's extend and filter, the inverse
   matrix and the source offset.  Both: the target size and the draw's
   opacity.  One per distinct source image of a frame. */
#define GB_GRAD_STOPS  16
#define GB_SRC_SURFACE 1u /* vkvg_pattern_type_t values */
#define GB_GRAD_LINEAR 2u
#define GB_GRAD_RADIAL 3u
typedef struct {
    uint32_t type;
    float    cp[8];
    float    w, h;
    uint32_t count;
    float    opacity;
    float    stops[GB_GRAD_STOPS];
    float    colors[GB_GRAD_STOPS * 4];
    /* surface sources */
    uint32_t        sw, sh;         /* source size */
    uint32_t        extend, filter; /* vkvg_extend_t; 1 bilinear, 0 nearest */
    float           m[6];           /* inverse matrix xx yx xy yy x0 y0 */
    float           ox, oy;         /* source offset (push constant source.xy) */
    const uint32_t *texels;         /* [sh][sw] premultiplied RGBA8 */
} gb_grad;
#define GB_MAX_GRAD_SOURCES 8 /* source images per frame; more flush the frame first */

/* stroke event kinds (dashed strokes materialise their events) */
#define GB_EV_JOIN      0u /* _build_vb_step at cp with (iL, iR) */
#define GB_EV_CAP_START 1u
#define GB_EV_CAP_END   2u
#define GB_EV_CLOSE     3u /* closing join of a closed, undashed subpath (+ index patch) */
#define GB_EV_NONE      4u

typedef struct {
    uint32_t kind; /* GB_EV_* | curved << 8 */
    uint32_t cp, iL, iR;
    float    px, py, nx, ny; /* cap position and direction */
} gb_event;

/* bands: 16 sample rows (4 pixel rows at 4x MSAA, 16 at 1x) */
#define GB_BAND_ROWS 16
#define GB_CELL_EVERY 0x80000000u /* a (band, draw) cell count's mark: the draw acts on every band */
#define GB_RASTER_TILE_W 1024 /* pixels of a raster tile (one CTA's columns) */
#define GB_TILE_W    256

/* device status word bits */
#define GB_ERR_CURVE_LIMIT 0x1u /* a cubic exceeded the subdivision work cap */
#define GB_ERR_OVERFLOW    0x2u
#define GB_ERR_RASTER_WAIT 0x4u /* a staged copy in the raster did not arrive within its wait limit */
#define WAIT_LIMIT_POLLS   (1u << 20) /* mbarrier polls before a staged copy counts as lost */

#endif
