/* Internal structures of the vko oracle (test infrastructure). */
#ifndef VKO_INTERNAL_H
#define VKO_INTERNAL_H

#include "vko.h"
#include "vko_pmath.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* path element bits, src/vkvg_internal.h:62-68 of vkvg */
#define VKO_PATH_CLOSED_BIT     0x80000000u
#define VKO_PATH_HAS_CURVES_BIT 0x40000000u
#define VKO_PATH_IS_CONVEX_BIT  0x20000000u
#define VKO_PATH_ELT_MASK       0x1FFFFFFFu

#define VKO_EQUF(a, b) (fabsf((a) - (b)) <= FLT_EPSILON) /* src/vkvg_internal.h:72 */

#define VKO_PIF   3.14159265358979323846f
#define VKO_PIF_2 1.57079632679489661923f
#define VKO_2_PIF 0.63661977236758134308f /* 2/pi: src/vkvg_internal.h:45 */

/* vertex fixed point: 8 sub-pixel bits; clamp for far-away vertices */
#define VKO_SUBPIX      256
#define VKO_FIX_LIMIT   268435456.0f /* 2^28 units = 2^20 px */

typedef struct {
    float x, y;
} v2;

/* a linear gradient as vkvg's fragment stage sees it (shaders/vkvg_main.frag
   LINEAR, data of _update_cur_pattern): control points in pixels after the
   inverse pattern matrix and the CTM of vkvg_set_source time, surface size,
   stops, premultiplied stop colours, the draw's opacity */
#define VKO_GRAD_STOPS 16
typedef struct {
    int      type; /* 2 linear, 3 radial (vkvg_pattern_type_t) */
    float    cp[8];
    float    w, h;
    uint32_t count;
    float    opacity;
    float    stops[VKO_GRAD_STOPS];
    float    colors[VKO_GRAD_STOPS * 4];
    /* surface sources (type 1): the source surface, sampler state, the
       draw's pushed inverse matrix and source offset; texels is its resolved
       image while the draw is rastered */
    const struct vko_surface_t *src;
    int            extend, bilinear;
    vko_matrix     m;
    float          ox, oy;
    const uint8_t *texels;
} vko_grad;

struct vko_pattern_t {
    int        status;
    uint32_t   refs;
    int        type, extend, filter;
    float      cp[8];
    vko_surface *surf; /* surface patterns: referenced */
    uint32_t   count;
    float      stops[VKO_GRAD_STOPS];
    float      colors[VKO_GRAD_STOPS * 4];
    vko_matrix matrix;
    int        has_matrix;
};

/* kinds that carry fill geometry, and the even-odd ones */
#define VKO_FILL_GEOM(k) ((k) == VKO_DRAW_FILL_EO || (k) == VKO_DRAW_FILL_NZ || (k) == VKO_DRAW_CLIP_EO || (k) == VKO_DRAW_CLIP_NZ)
#define VKO_EO(k)        ((k) == VKO_DRAW_FILL_EO || (k) == VKO_DRAW_CLIP_EO)

/* stencil bits, src/vkvg_device_internal.h:28-30 of vkvg; bits 2..7 are the
   save bits of vkvg_save */
#define VKO_STENCIL_FILL 0x1u
#define VKO_STENCIL_CLIP 0x2u
#define VKO_STENCIL_ALL  0x3u

typedef struct {
    int      kind;
    int      param; /* stencil operations: save bit (shift) or image index */
    int      op;
    uint32_t color;
    float    opacity;
    int      grad; /* the source is the gradient g */
    vko_grad g;
    vko_matrix mat;
    /* fills */
    uint32_t npts;
    float   *pts;
    uint32_t nsub;
    uint32_t *sub_counts;
    int      convex;
    float    bounds[4];
    /* strokes */
    uint32_t nverts;
    float   *verts;
    uint32_t ninds;
    uint32_t *inds;
} vko_draw;

struct vko_surface_t {
    int      status;
    uint32_t refs;
    uint32_t width, height, samples;
    uint8_t *data;    /* [y][x][s][4] premultiplied RGBA8 */
    uint8_t *stencil; /* [y][x][s] */
    uint8_t **images; /* stencil copies of vkvg_save beyond six levels */
    uint32_t nimages;
};

/* one vkvg_save level, vkvg_context_save_t (src/vkvg_context_internal.h:101-124) */
typedef struct vko_saved {
    struct vko_saved *next;
    float             line_width, miter_limit, dash_offset, opacity;
    uint32_t          dash_count;
    float            *dashes;
    int               op, line_cap, line_join, fill_rule;
    vko_matrix        mat, mat_inv;
    float             src_x, src_y;
    uint32_t          cur_color;
    vko_pattern      *pattern;
    int               clip_state;
} vko_saved;

/* vkvg_clip_state_t, src/vkvg_context_internal.h:95-99 */
enum { VKO_CLIP_NONE = 0x00, VKO_CLIP_CLEAR = 0x01, VKO_CLIP_CLIP = 0x02, VKO_CLIP_SAVED = 0x06 };

struct vko_context_t {
    int          status;
    vko_surface *surf;

    v2      *points;
    uint32_t point_count, size_points;
    uint32_t *pathes;
    uint32_t path_ptr, segment_ptr, size_pathes;
    uint32_t subpath_count;
    int      simple_convex;

    float    line_width, miter_limit;
    uint32_t dash_count;
    float    dash_offset;
    float   *dashes;
    int      op, line_cap, line_join, fill_rule;
    uint32_t cur_color;
    float    opacity;
    vko_matrix mat;
    vko_pattern *pattern;
    int          grad_on;
    vko_grad     grad_snap;
    float        src_x, src_y; /* push constant source.xy */
    vko_matrix   mat_inv;      /* push constant matInv */
    int          clip_state; /* curClipState */
    uint8_t      sav_bit;    /* curSavBit */
    vko_saved   *saved;      /* pSavedCtxs */

    /* stroke vertex / index emission buffers */
    v2      *verts;
    uint32_t nverts, cap_verts;
    uint32_t *inds;
    uint32_t ninds, cap_inds;

    vko_draw *draws;
    uint32_t  ndraws, cap_draws, nrastered;
    int       keep_draws;
};

/* math dispatch */
extern int vko_math_mode_g;
static inline float VKO_ATAN2F(float y, float x) { return vko_math_mode_g ? atan2f(y, x) : vko_pm_atan2f(y, x); }
static inline float VKO_ACOSF(float x) { return vko_math_mode_g ? acosf(x) : vko_pm_acosf(x); }
static inline float VKO_COSF(float x) { return vko_math_mode_g ? cosf(x) : vko_pm_cosf(x); }
static inline float VKO_SINF(float x) { return vko_math_mode_g ? sinf(x) : vko_pm_sinf(x); }
static inline float VKO_POW2F(float x) { return vko_math_mode_g ? powf(x, 2) : x * x; }

/* vec2 helpers, src/vectors.h:103-167 of vkvg */
static inline v2    v2_add(v2 a, v2 b) { return (v2){a.x + b.x, a.y + b.y}; }
static inline v2    v2_sub(v2 a, v2 b) { return (v2){a.x - b.x, a.y - b.y}; }
static inline v2    v2_mul(v2 a, float m) { return (v2){a.x * m, a.y * m}; }
static inline v2    v2_div(v2 a, float m) { return (v2){a.x / m, a.y / m}; }
static inline float v2_len(v2 v) { return sqrtf(v.x * v.x + v.y * v.y); }
static inline v2    v2_norm(v2 a) {
    float m = sqrtf(a.x * a.x + a.y * a.y);
    return (v2){a.x / m, a.y / m};
}
static inline v2 v2_line_norm(v2 a, v2 b) {
    v2    d  = {b.x - a.x, b.y - a.y};
    float md = sqrtf(d.x * d.x + d.y * d.y);
    d.x /= md;
    d.y /= md;
    return d;
}
static inline v2    v2_perp(v2 a) { return (v2){a.y, -a.x}; }
static inline float v2_dot(v2 a, v2 b) { return (a.x * b.x) + (a.y * b.y); }
static inline int   v2_equ(v2 a, v2 b) { return VKO_EQUF(a.x, b.x) & VKO_EQUF(a.y, b.y); }

/* geometry (vko_geom.c) */
void vko_ctx_init_geom(vko_context *ctx);
void vko_ctx_free_geom(vko_context *ctx);
void vko_draw_free(vko_draw *d);
vko_draw *vko_new_draw(vko_context *ctx, int kind);
int       vko_clip_preserve_geom(vko_context *ctx);
void      vko_clear_path(vko_context *ctx);

/* raster (vko_raster.c) */
void vko_raster_draw(vko_surface *surf, const vko_draw *d);
void vko_draw_coverage_impl(const vko_surface *surf, const vko_draw *d, int mode, int32_t *out);
void vko_snap_point(const vko_matrix *m, uint32_t w, uint32_t h, float x, float y, int32_t *fx, int32_t *fy);
void vko_resolve(const vko_surface *surf, uint8_t *rgba);

/* png (vko_png.c) */
int vko_png_write(const char *path, uint32_t w, uint32_t h, const uint8_t *rgba);

/* _recursive_bezier with a point callback (vko_geom.c); which is one of: */
#define VKO_BEZ_MID 0 /* the sub-curve's midpoint x1234 */
#define VKO_BEZ_C2  1 /* its second control point x2 */
#define VKO_BEZ_C3  2 /* its third control point x3 */
typedef void (*vko_bez_emit)(void *u, float x, float y, int which, double ta, double tb);
void vko_bezier_walk(vko_bez_emit emit, void *u, float distanceTolerance, float x1, float y1, float x2, float y2,
                     float x3, float y3, float x4, float y4, unsigned level, double ta, double tb);

#endif
