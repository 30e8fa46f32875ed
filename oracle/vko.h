/*
 * vko - CPU oracle for the vkvg path hot path (TEST INFRASTRUCTURE ONLY).
 *
 * Parity status: UNPINNED.  vkvg itself cannot be built or run here (its vkh
 * and glutess submodules are empty, and there is no graphics stack), and its
 * tree holds no golden images or numeric fixtures for this path.  The oracle
 * is a function-for-function restatement of vkvg's host geometry (file:line
 * cited at each function in vko_geom.c), plus a software restatement of the
 * fixed-function state vkvg programs into Vulkan (vko_raster.c).  It is
 * cross-checked against vkvg's own behavioural tests (gunit_tests/context.cpp
 * current-point semantics, gunit_tests/matrices.cpp), against an
 * independent pure-Python restatement of the cubic flattening (tests/pyref.py),
 * and against its own committed outputs (tests/golden/).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this library, and only as the checker or the timed CPU baseline.  The
 * product library (vkvg_gb300) never links or calls it.
 *
 * The API mirrors include/vkvg.h of vkvg with a vko_ prefix so that the
 * parity tests drive the oracle and the GPU library with the same call
 * sequence.
 */
#ifndef VKO_H
#define VKO_H

#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VKO_API __attribute__((visibility("default")))

typedef struct vko_surface_t vko_surface;
typedef struct vko_context_t vko_context;
typedef struct vko_pattern_t vko_pattern;

typedef struct {
    float xx, yx, xy, yy, x0, y0;
} vko_matrix;

/* status values are those of vkvg_status_t (include/vkvg.h:125-150 of vkvg) */
enum {
    VKO_STATUS_SUCCESS = 0,
    VKO_STATUS_NO_MEMORY,
    VKO_STATUS_NULL_POINTER,
    VKO_STATUS_INVALID_RESTORE,
    VKO_STATUS_NO_CURRENT_POINT,
    VKO_STATUS_INVALID_MATRIX,
    VKO_STATUS_INVALID_STATUS,
    VKO_STATUS_INVALID_INDEX,
    VKO_STATUS_WRITE_ERROR,
    VKO_STATUS_PATTERN_TYPE_MISMATCH,
    VKO_STATUS_PATTERN_INVALID_GRADIENT,
    VKO_STATUS_INVALID_FORMAT,
    VKO_STATUS_FILE_NOT_FOUND,
    VKO_STATUS_INVALID_DASH,
    VKO_STATUS_INVALID_RECT,
    VKO_STATUS_TIMEOUT,
    VKO_STATUS_DEVICE_ERROR,
    VKO_STATUS_INVALID_DEVICE_CREATE_INFO,
    VKO_STATUS_INVALID_IMAGE,
    VKO_STATUS_INVALID_SURFACE,
    VKO_STATUS_INVALID_FONT,
};

/* draw kinds recorded by the oracle: one per fill/stroke/paint/clear/clip
   call, and the stencil operations of vkvg_reset_clip / vkvg_save /
   vkvg_restore in the order vkvg issues them (src/vkvg_context.c:703-733,
   1251-1512): RESET clears the stencil; SAVE_BIT copies the clip bit into
   save bit `param`; RESTORE_BIT copies bit `param` into the clip bit; STORE
   copies the stencil into stencil image `param`; LOAD copies it back */
enum {
    VKO_DRAW_FILL_EO     = 0,
    VKO_DRAW_FILL_NZ     = 1,
    VKO_DRAW_STROKE      = 2,
    VKO_DRAW_PAINT       = 3,
    VKO_DRAW_CLEAR       = 4,
    VKO_DRAW_CLIP_EO     = 5,
    VKO_DRAW_CLIP_NZ     = 6,
    VKO_DRAW_RESET       = 7,
    VKO_DRAW_SAVE_BIT    = 8,
    VKO_DRAW_RESTORE_BIT = 9,
    VKO_DRAW_STORE       = 10,
    VKO_DRAW_LOAD        = 11
};
/* operators: vkvg_operator_t order (include/vkvg.h) */
enum { VKO_OP_CLEAR = 0, VKO_OP_SOURCE = 1, VKO_OP_OVER = 2, VKO_OP_DIFFERENCE = 3 };

/* global modes */
VKO_API void vko_set_math_mode(int mode);   /* 0 portable (default), 1 host libm */
VKO_API int  vko_get_math_mode(void);
VKO_API void vko_set_raster_mode(int mode); /* 0 scanline crossings (default), 1 literal fan/stencil */
VKO_API void vko_set_threads(int n);        /* raster worker threads (CPU baseline) */

/* portable math, exported for the bit-identity test against the product copy */
VKO_API void vko_pmath_eval(int fn, const float *a, const float *b, float *out, uint64_t n);
/* the interior points of one cubic (x0,y0 .. x3,y3 in p[8]) by the
   subdivision walk at the given squared distance tolerance, in the current
   math mode; returns the count, storing at most cap points in xy */
VKO_API uint32_t vko_flatten_cubic(float distanceTolerance, const float *p, float *xy, uint32_t cap);

/* matrices (src/vkvg_matrix.c of vkvg) */
VKO_API void vko_matrix_init_identity(vko_matrix *m);
VKO_API void vko_matrix_init(vko_matrix *m, float xx, float yx, float xy, float yy, float x0, float y0);
VKO_API void vko_matrix_init_translate(vko_matrix *m, float tx, float ty);
VKO_API void vko_matrix_init_scale(vko_matrix *m, float sx, float sy);
VKO_API void vko_matrix_init_rotate(vko_matrix *m, float radians);
VKO_API void vko_matrix_translate(vko_matrix *m, float tx, float ty);
VKO_API void vko_matrix_scale(vko_matrix *m, float sx, float sy);
VKO_API void vko_matrix_rotate(vko_matrix *m, float radians);
VKO_API void vko_matrix_multiply(vko_matrix *r, const vko_matrix *a, const vko_matrix *b);
VKO_API void vko_matrix_transform_distance(const vko_matrix *m, float *dx, float *dy);
VKO_API void vko_matrix_transform_point(const vko_matrix *m, float *x, float *y);
VKO_API int  vko_matrix_invert(vko_matrix *m);
VKO_API void vko_matrix_get_scale(const vko_matrix *m, float *sx, float *sy);

/* surfaces */
VKO_API vko_surface *vko_surface_create(uint32_t width, uint32_t height, uint32_t samples);
VKO_API void         vko_surface_destroy(vko_surface *surf);
VKO_API int          vko_surface_status(vko_surface *surf);
VKO_API uint32_t     vko_surface_get_width(vko_surface *surf);
VKO_API uint32_t     vko_surface_get_height(vko_surface *surf);
VKO_API void         vko_surface_clear(vko_surface *surf);
/* resolved, unpremultiplied RGBA8 (vkvg_surface_write_to_memory semantics) */
VKO_API int vko_surface_write_to_memory(vko_surface *surf, uint8_t *rgba);
/* resolved premultiplied RGBA8, before the unpremultiply step */
VKO_API int vko_surface_resolve_premult(vko_surface *surf, uint8_t *rgba);
/* raw per-sample premultiplied RGBA8, layout [y][x][sample][channel] */
VKO_API int vko_surface_read_samples(vko_surface *surf, uint8_t *out);
VKO_API int vko_surface_write_to_png(vko_surface *surf, const char *path);

/* contexts */
VKO_API vko_context *vko_create(vko_surface *surf);
VKO_API void         vko_destroy(vko_context *ctx);
VKO_API int          vko_status(vko_context *ctx);
VKO_API void         vko_flush(vko_context *ctx);
VKO_API void         vko_keep_draws(vko_context *ctx, int keep);

/* path construction (src/vkvg_context.c of vkvg) */
VKO_API void vko_new_path(vko_context *ctx);
VKO_API void vko_new_sub_path(vko_context *ctx);
VKO_API void vko_close_path(vko_context *ctx);
VKO_API void vko_move_to(vko_context *ctx, float x, float y);
VKO_API void vko_rel_move_to(vko_context *ctx, float x, float y);
VKO_API void vko_line_to(vko_context *ctx, float x, float y);
VKO_API void vko_rel_line_to(vko_context *ctx, float dx, float dy);
VKO_API void vko_curve_to(vko_context *ctx, float x1, float y1, float x2, float y2, float x3, float y3);
VKO_API void vko_rel_curve_to(vko_context *ctx, float x1, float y1, float x2, float y2, float x3, float y3);
VKO_API void vko_quadratic_to(vko_context *ctx, float x1, float y1, float x2, float y2);
VKO_API void vko_rel_quadratic_to(vko_context *ctx, float x1, float y1, float x2, float y2);
VKO_API void vko_arc(vko_context *ctx, float xc, float yc, float radius, float a1, float a2);
VKO_API void vko_arc_negative(vko_context *ctx, float xc, float yc, float radius, float a1, float a2);
VKO_API void vko_elliptic_arc_to(vko_context *ctx, float x2, float y2, bool large, bool sweep, float rx, float ry,
                                 float phi);
VKO_API void vko_rel_elliptic_arc_to(vko_context *ctx, float x2, float y2, bool large, bool sweep, float rx, float ry,
                                     float phi);
VKO_API void vko_ellipse(vko_context *ctx, float rx, float ry, float x, float y, float rot);
VKO_API int  vko_rectangle(vko_context *ctx, float x, float y, float w, float h);
VKO_API int  vko_rounded_rectangle(vko_context *ctx, float x, float y, float w, float h, float radius);
/* patterns (linear gradients), src/vkvg_pattern.c */
VKO_API vko_pattern *vko_pattern_create_linear(float x0, float y0, float x1, float y1);
VKO_API int          vko_pattern_status(vko_pattern *pat);
VKO_API vko_pattern *vko_pattern_reference(vko_pattern *pat);
VKO_API uint32_t     vko_pattern_get_reference_count(vko_pattern *pat);
VKO_API void         vko_pattern_destroy(vko_pattern *pat);
VKO_API int          vko_pattern_edit_linear(vko_pattern *pat, float x0, float y0, float x1, float y1);
VKO_API vko_pattern *vko_pattern_create_radial(float cx0, float cy0, float r0, float cx1, float cy1, float r1);
VKO_API int vko_pattern_edit_radial(vko_pattern *pat, float cx0, float cy0, float r0, float cx1, float cy1, float r1);
VKO_API int          vko_pattern_add_color_stop(vko_pattern *pat, float offset, float r, float g, float b, float a);
VKO_API int          vko_pattern_get_color_stop_count(vko_pattern *pat, uint32_t *count);
VKO_API void         vko_pattern_set_matrix(vko_pattern *pat, const vko_matrix *m);
VKO_API void         vko_set_source(vko_context *ctx, vko_pattern *pat);
VKO_API vko_pattern *vko_pattern_create_for_surface(vko_surface *surf);
VKO_API void         vko_pattern_set_extend(vko_pattern *pat, int extend);
VKO_API void         vko_pattern_set_filter(vko_pattern *pat, int filter);
VKO_API void         vko_set_source_surface(vko_context *ctx, vko_surface *surf, float x, float y);
VKO_API bool vko_has_current_point(vko_context *ctx);
VKO_API void vko_get_current_point(vko_context *ctx, float *x, float *y);
VKO_API void vko_path_extents(vko_context *ctx, float *x1, float *y1, float *x2, float *y2);

/* drawing */
VKO_API void vko_fill(vko_context *ctx);
VKO_API void vko_fill_preserve(vko_context *ctx);
VKO_API void vko_stroke(vko_context *ctx);
VKO_API void vko_stroke_preserve(vko_context *ctx);
VKO_API void vko_paint(vko_context *ctx);
VKO_API void vko_clear(vko_context *ctx);

/* clip and the state stack */
VKO_API void vko_reset_clip(vko_context *ctx);
VKO_API void vko_clip(vko_context *ctx);
VKO_API void vko_clip_preserve(vko_context *ctx);
VKO_API void vko_save(vko_context *ctx);
VKO_API void vko_restore(vko_context *ctx);

/* state */
VKO_API void     vko_set_source_rgba(vko_context *ctx, float r, float g, float b, float a);
VKO_API void     vko_set_source_rgb(vko_context *ctx, float r, float g, float b);
VKO_API void     vko_set_source_color(vko_context *ctx, uint32_t c);
VKO_API void     vko_set_line_width(vko_context *ctx, float w);
VKO_API void     vko_set_miter_limit(vko_context *ctx, float l);
VKO_API void     vko_set_line_cap(vko_context *ctx, int cap);
VKO_API void     vko_set_line_join(vko_context *ctx, int join);
VKO_API void     vko_set_fill_rule(vko_context *ctx, int fr);
VKO_API void     vko_set_operator(vko_context *ctx, int op);
VKO_API void     vko_set_opacity(vko_context *ctx, float o);
VKO_API void     vko_set_dash(vko_context *ctx, const float *dashes, uint32_t n, float offset);
VKO_API void     vko_set_matrix(vko_context *ctx, const vko_matrix *m);
VKO_API void     vko_get_matrix(vko_context *ctx, vko_matrix *m);
VKO_API float    vko_get_line_width(vko_context *ctx);
VKO_API int      vko_get_line_join(vko_context *ctx);
VKO_API int      vko_get_line_cap(vko_context *ctx);
VKO_API int      vko_get_fill_rule(vko_context *ctx);
VKO_API int      vko_get_operator(vko_context *ctx);
VKO_API void     vko_identity_matrix(vko_context *ctx);
VKO_API void     vko_translate(vko_context *ctx, float dx, float dy);
VKO_API void     vko_scale(vko_context *ctx, float sx, float sy);
VKO_API void     vko_rotate(vko_context *ctx, float r);
VKO_API void     vko_transform(vko_context *ctx, const vko_matrix *m);
VKO_API uint32_t vko_get_color(vko_context *ctx);

/* recorded draws (kept after flush when vko_keep_draws(ctx,1)) */
VKO_API uint32_t vko_draw_count(vko_context *ctx);
/* info[0]=kind info[1]=npts info[2]=nsub info[3]=nverts info[4]=ninds info[5]=color info[6]=convex */
VKO_API int vko_draw_info(vko_context *ctx, uint32_t i, uint32_t *info);
VKO_API int vko_draw_points(vko_context *ctx, uint32_t i, float *xy, uint32_t *sub_counts);
VKO_API int vko_draw_stroke(vko_context *ctx, uint32_t i, float *xy, uint32_t *inds);
/* per-sample winding (fills) or covering-triangle count (strokes) of draw i,
   layout [y][x][sample]; mode = raster mode to use */
VKO_API int vko_draw_coverage(vko_context *ctx, uint32_t i, int mode, int32_t *out);
/* snapped 24.8 fixed-point position of a user-space point under draw i's CTM */
VKO_API void vko_snap(vko_context *ctx, uint32_t i, float x, float y, int32_t *fx, int32_t *fy);

/* coverage of an explicit edge / triangle list (same rules), for unit tests */
VKO_API void vko_coverage_edges(uint32_t w, uint32_t h, uint32_t samples, const int32_t *edges, uint64_t nedges,
                                int32_t *out);

/* ---- analytic-coverage mode, FP64 reference (vko_analytic.c) ---- */
#define VKO_AN_LINE   1 /* segment kinds = control points a segment consumes */
#define VKO_AN_CUBIC  3
#define VKO_AN_FILL   1u
#define VKO_AN_STROKE 2u
typedef struct vko_an_t vko_an;
VKO_API vko_an  *vko_an_create(uint32_t width, uint32_t height, const float *background, uint32_t npaths,
                               const uint32_t *path_ncontours, const uint32_t *path_flags, uint32_t ncontours,
                               const uint32_t *contour_nseg, uint32_t nseg, const uint8_t *seg_kind);
VKO_API void     vko_an_destroy(vko_an *a);
VKO_API void     vko_an_set_points_mode(int f32);
VKO_API uint32_t vko_an_nctrl(const vko_an *a);
VKO_API uint32_t vko_an_nlayers(const vko_an *a);
VKO_API uint32_t vko_an_flatten(const vko_an *a, const double *ctrl, float *pts_f32, double *pts_f64, uint32_t cap,
                                uint32_t *seg_off);
VKO_API double   vko_an_forward(const vko_an *a, const double *ctrl, const double *colors, const double *widths,
                                const double *target, double *canvas, double *area);
VKO_API double   vko_an_backward(const vko_an *a, const double *ctrl, const double *colors, const double *widths,
                                 const double *target, const double *d_canvas, double *d_ctrl, double *d_colors,
                                 double *d_widths, double *d_pts);
VKO_API void     vko_an_fd(const vko_an *a, const double *ctrl, const double *colors, const double *widths,
                           const double *target, uint32_t n, const uint32_t *group, const uint32_t *index, double h,
                           double h2, int full, int threads, double *fd, double *fd2, int32_t *valid);

#ifdef __cplusplus
}
#endif
#endif
