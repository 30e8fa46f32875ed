/*
 * vko_geom.c - oracle restatement of vkvg's host path geometry
 * (TEST INFRASTRUCTURE ONLY; see vko.h for the parity status).
 *
 * Each function follows the vkvg function named in its comment, with the same
 * fp32 expression order, the same path/segment bookkeeping and the same
 * quirks.  Where vkvg's behaviour is undefined (reads out of bounds, unbounded
 * recursion on NaN input) the choice made here is stated at the spot.
 */
#include "vko_internal.h"

#include <stdio.h>

/* ------------------------------------------------------------------ arrays */

static int ensure_points(vko_context *ctx, uint32_t extra) {
    if (ctx->point_count + extra + 8 < ctx->size_points)
        return 0;
    uint32_t ns = ctx->size_points * 2 + extra + 1024;
    v2      *t  = (v2 *)realloc(ctx->points, (size_t)ns * sizeof(v2));
    if (!t) {
        ctx->status = VKO_STATUS_NO_MEMORY;
        return 1;
    }
    ctx->points      = t;
    ctx->size_points = ns;
    return 0;
}
static int ensure_pathes(vko_context *ctx) {
    if (ctx->path_ptr + ctx->segment_ptr + 16 < ctx->size_pathes)
        return 0;
    uint32_t  ns = ctx->size_pathes * 2 + 64;
    uint32_t *t  = (uint32_t *)realloc(ctx->pathes, (size_t)ns * sizeof(uint32_t));
    if (!t) {
        ctx->status = VKO_STATUS_NO_MEMORY;
        return 1;
    }
    memset(t + ctx->size_pathes, 0, (size_t)(ns - ctx->size_pathes) * sizeof(uint32_t));
    ctx->pathes      = t;
    ctx->size_pathes = ns;
    return 0;
}
static void emit_vertex(vko_context *ctx, v2 p) {
    if (ctx->nverts + 1 >= ctx->cap_verts) {
        uint32_t ns = ctx->cap_verts * 2 + 4096;
        v2      *t  = (v2 *)realloc(ctx->verts, (size_t)ns * sizeof(v2));
        if (!t) {
            ctx->status = VKO_STATUS_NO_MEMORY;
            return;
        }
        ctx->verts     = t;
        ctx->cap_verts = ns;
    }
    ctx->verts[ctx->nverts++] = p;
}
static void emit_tri(vko_context *ctx, uint32_t a, uint32_t b, uint32_t c) {
    if (ctx->ninds + 3 >= ctx->cap_inds) {
        uint32_t  ns = ctx->cap_inds * 2 + 12288;
        uint32_t *t  = (uint32_t *)realloc(ctx->inds, (size_t)ns * sizeof(uint32_t));
        if (!t) {
            ctx->status = VKO_STATUS_NO_MEMORY;
            return;
        }
        ctx->inds     = t;
        ctx->cap_inds = ns;
    }
    ctx->inds[ctx->ninds++] = a;
    ctx->inds[ctx->ninds++] = b;
    ctx->inds[ctx->ninds++] = c;
}
/* _add_tri_indices_for_rect, src/vkvg_context_internal.c:340-353 */
static void emit_rect(vko_context *ctx, uint32_t i) {
    emit_tri(ctx, i, i + 2, i + 1);
    emit_tri(ctx, i + 1, i + 2, i + 3);
}

/* ---------------------------------------------------------- path storage */

/* _current_path_is_empty, src/vkvg_context_internal.c:133 */
static int path_empty(const vko_context *ctx) { return ctx->pathes[ctx->path_ptr] == 0; }
/* _get_current_position, :135.  vkvg reads points[-1] on an empty path; the
   oracle returns (0,0) there. */
static v2 cur_pos(const vko_context *ctx) {
    if (ctx->point_count == 0)
        return (v2){0, 0};
    return ctx->points[ctx->point_count - 1];
}
/* _set_curve_start, :137-151 */
static void set_curve_start(vko_context *ctx) {
    uint32_t *pp = ctx->pathes;
    if (ctx->segment_ptr > 0) {
        if ((pp[ctx->path_ptr + ctx->segment_ptr] & VKO_PATH_ELT_MASK) > 0)
            ctx->segment_ptr++;
    } else {
        if (pp[ctx->path_ptr] > 0) {
            pp[ctx->path_ptr + 1] = pp[ctx->path_ptr];
            ctx->segment_ptr      = 2;
        } else
            ctx->segment_ptr = 1;
    }
    if (ensure_pathes(ctx))
        return;
    ctx->pathes[ctx->path_ptr + ctx->segment_ptr] = 0;
}
/* _set_curve_end, :153-160 */
static void set_curve_end(vko_context *ctx) {
    ctx->pathes[ctx->path_ptr + ctx->segment_ptr] |= VKO_PATH_HAS_CURVES_BIT;
    ctx->segment_ptr++;
    if (ensure_pathes(ctx))
        return;
    ctx->pathes[ctx->path_ptr + ctx->segment_ptr] = 0;
}
/* _finish_path, :163-197 */
static void finish_path(vko_context *ctx) {
    uint32_t *pp = ctx->pathes;
    if (pp[ctx->path_ptr] == 0)
        return;
    if ((pp[ctx->path_ptr] & VKO_PATH_ELT_MASK) < 2) {
        ctx->point_count -= pp[ctx->path_ptr];
        pp[ctx->path_ptr] = 0;
        ctx->segment_ptr  = 0;
        return;
    }
    if (ctx->path_ptr == 0 && ctx->simple_convex)
        pp[0] |= VKO_PATH_IS_CONVEX_BIT;
    if (ctx->segment_ptr > 0) {
        pp[ctx->path_ptr] |= VKO_PATH_HAS_CURVES_BIT;
        uint32_t cur = pp[ctx->path_ptr + ctx->segment_ptr];
        if ((cur & VKO_PATH_HAS_CURVES_BIT) == 0 && (cur & VKO_PATH_ELT_MASK) > 0)
            ctx->segment_ptr++;
        ctx->path_ptr += ctx->segment_ptr;
    } else
        ctx->path_ptr++;
    ctx->segment_ptr = 0;
    if (ensure_pathes(ctx))
        return;
    ctx->pathes[ctx->path_ptr] = 0;
    ctx->subpath_count++;
    ctx->simple_convex = 0;
}
/* _clear_path, :199-206 */
static void clear_path(vko_context *ctx) {
    ctx->path_ptr              = 0;
    ctx->pathes[ctx->path_ptr] = 0;
    ctx->point_count           = 0;
    ctx->segment_ptr           = 0;
    ctx->subpath_count         = 0;
    ctx->simple_convex         = 0;
}
/* _remove_last_point, :207-219 */
static void remove_last_point(vko_context *ctx) {
    uint32_t *pp = ctx->pathes;
    pp[ctx->path_ptr]--;
    ctx->point_count--;
    if (ctx->segment_ptr > 0) {
        if (!pp[ctx->path_ptr + ctx->segment_ptr])
            ctx->segment_ptr--;
        pp[ctx->path_ptr + ctx->segment_ptr]--;
        if ((pp[ctx->path_ptr + ctx->segment_ptr] & VKO_PATH_ELT_MASK) == 0)
            pp[ctx->path_ptr + ctx->segment_ptr] = 0;
        else if (pp[ctx->path_ptr + ctx->segment_ptr] & VKO_PATH_HAS_CURVES_BIT)
            ctx->segment_ptr++;
    }
}
/* _add_point, :221-238 (NaN points are dropped) */
static void add_point(vko_context *ctx, float x, float y) {
    if (ensure_points(ctx, 1))
        return;
    if (isnan(x) || isnan(y))
        return;
    ctx->points[ctx->point_count++] = (v2){x, y};
    ctx->pathes[ctx->path_ptr]++;
    if (ctx->segment_ptr > 0)
        ctx->pathes[ctx->path_ptr + ctx->segment_ptr]++;
}
/* _get_arc_step, :245-252 */
static float get_arc_step(const vko_context *ctx, float radius) {
    float sx, sy;
    vko_matrix_get_scale(&ctx->mat, &sx, &sy);
    float r = radius * fabsf(fmaxf(sx, sy));
    if (r < 30.0f)
        return fminf(VKO_PIF / 3.f, VKO_PIF / r);
    return fminf(VKO_PIF / 3.f, VKO_PIF / (r * 0.4f));
}

/* ------------------------------------------------------------ flattening */

#define M_ANGLE_TOLERANCE          0.01
#define M_CUSP_LIMIT               0.01
#define CURVE_RECURSION_LIMIT      100
#define CURVE_COLLINEARITY_EPSILON 1.7

/* _recursive_bezier, :1313-1461 (AGG adaptive subdivision).  The branch
   "M_ANGLE_TOLERANCE < CURVE_ANGLE_TOLERANCE_EPSILON" is constant-false and
   omitted.  "da = M_2_PIF - da" (2/pi, not 2*pi) is kept as in vkvg.
   Every added point is reported to emit() with which sub-curve point it is
   (VKO_BEZ_MID = x1234, VKO_BEZ_C2 = x2, VKO_BEZ_C3 = x3) and the sub-curve's
   parameter interval [ta, tb] on the original cubic. */
void vko_bezier_walk(vko_bez_emit emit, void *u, float distanceTolerance, float x1, float y1, float x2, float y2,
                     float x3, float y3, float x4, float y4, unsigned level, double ta, double tb) {
    if (level > CURVE_RECURSION_LIMIT)
        return;
    float x12   = (x1 + x2) / 2;
    float y12   = (y1 + y2) / 2;
    float x23   = (x2 + x3) / 2;
    float y23   = (y2 + y3) / 2;
    float x34   = (x3 + x4) / 2;
    float y34   = (y3 + y4) / 2;
    float x123  = (x12 + x23) / 2;
    float y123  = (y12 + y23) / 2;
    float x234  = (x23 + x34) / 2;
    float y234  = (y23 + y34) / 2;
    float x1234 = (x123 + x234) / 2;
    float y1234 = (y123 + y234) / 2;

    if (level > 0) {
        float dx = x4 - x1;
        float dy = y4 - y1;
        float d2 = fabsf(((x2 - x4) * dy - (y2 - y4) * dx));
        float d3 = fabsf(((x3 - x4) * dy - (y3 - y4) * dx));
        float da1, da2;
        if (d2 > CURVE_COLLINEARITY_EPSILON && d3 > CURVE_COLLINEARITY_EPSILON) {
            if ((d2 + d3) * (d2 + d3) <= (dx * dx + dy * dy) * distanceTolerance) {
                float a23 = VKO_ATAN2F(y3 - y2, x3 - x2);
                da1       = fabsf(a23 - VKO_ATAN2F(y2 - y1, x2 - x1));
                da2       = fabsf(VKO_ATAN2F(y4 - y3, x4 - x3) - a23);
                if (da1 >= VKO_PIF)
                    da1 = VKO_2_PIF - da1;
                if (da2 >= VKO_PIF)
                    da2 = VKO_2_PIF - da2;
                if (da1 + da2 < (float)M_ANGLE_TOLERANCE) {
                    emit(u, x1234, y1234, VKO_BEZ_MID, ta, tb);
                    return;
                }
                if (da1 > M_CUSP_LIMIT) {
                    emit(u, x2, y2, VKO_BEZ_C2, ta, tb);
                    return;
                }
                if (da2 > M_CUSP_LIMIT) {
                    emit(u, x3, y3, VKO_BEZ_C3, ta, tb);
                    return;
                }
            }
        } else {
            if (d2 > CURVE_COLLINEARITY_EPSILON) {
                if (d2 * d2 <= distanceTolerance * (dx * dx + dy * dy)) {
                    da1 = fabsf(VKO_ATAN2F(y3 - y2, x3 - x2) - VKO_ATAN2F(y2 - y1, x2 - x1));
                    if (da1 >= VKO_PIF)
                        da1 = VKO_2_PIF - da1;
                    if (da1 < M_ANGLE_TOLERANCE) {
                        emit(u, x2, y2, VKO_BEZ_C2, ta, tb);
                        emit(u, x3, y3, VKO_BEZ_C3, ta, tb);
                        return;
                    }
                    if (da1 > M_CUSP_LIMIT) {
                        emit(u, x2, y2, VKO_BEZ_C2, ta, tb);
                        return;
                    }
                }
            } else if (d3 > CURVE_COLLINEARITY_EPSILON) {
                if (d3 * d3 <= distanceTolerance * (dx * dx + dy * dy)) {
                    da1 = fabsf(VKO_ATAN2F(y4 - y3, x4 - x3) - VKO_ATAN2F(y3 - y2, x3 - x2));
                    if (da1 >= VKO_PIF)
                        da1 = VKO_2_PIF - da1;
                    if (da1 < M_ANGLE_TOLERANCE) {
                        emit(u, x2, y2, VKO_BEZ_C2, ta, tb);
                        emit(u, x3, y3, VKO_BEZ_C3, ta, tb);
                        return;
                    }
                    if (da1 > M_CUSP_LIMIT) {
                        emit(u, x3, y3, VKO_BEZ_C3, ta, tb);
                        return;
                    }
                }
            } else {
                dx = x1234 - (x1 + x4) / 2;
                dy = y1234 - (y1 + y4) / 2;
                if (dx * dx + dy * dy <= distanceTolerance) {
                    emit(u, x1234, y1234, VKO_BEZ_MID, ta, tb);
                    return;
                }
            }
        }
    }
    double tm = (ta + tb) * 0.5;
    vko_bezier_walk(emit, u, distanceTolerance, x1, y1, x12, y12, x123, y123, x1234, y1234, level + 1, ta, tm);
    vko_bezier_walk(emit, u, distanceTolerance, x1234, y1234, x234, y234, x34, y34, x4, y4, level + 1, tm, tb);
}

static void ctx_emit(void *u, float x, float y, int which, double ta, double tb) {
    (void)which, (void)ta, (void)tb;
    add_point((vko_context *)u, x, y);
}
static void recursive_bezier(vko_context *ctx, float distanceTolerance, float x1, float y1, float x2, float y2,
                             float x3, float y3, float x4, float y4, unsigned level) {
    vko_bezier_walk(ctx_emit, ctx, distanceTolerance, x1, y1, x2, y2, x3, y3, x4, y4, level, 0.0, 1.0);
}

/* one cubic through the walk alone (the interior points _recursive_bezier
   adds between the start and the end point), for measuring how often the
   math mode changes a subdivision; returns the point count, storing at most
   cap points */
typedef struct {
    float   *xy;
    uint32_t n, cap;
} cubic_sink;
static void cubic_emit(void *u, float x, float y, int which, double ta, double tb) {
    (void)which, (void)ta, (void)tb;
    cubic_sink *s = (cubic_sink *)u;
    if (s->n < s->cap) {
        s->xy[2 * s->n]     = x;
        s->xy[2 * s->n + 1] = y;
    }
    s->n++;
}
uint32_t vko_flatten_cubic(float distanceTolerance, const float *p, float *xy, uint32_t cap) {
    cubic_sink s = {xy, 0, cap};
    vko_bezier_walk(cubic_emit, &s, distanceTolerance, p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], 0, 0.0, 1.0);
    return s.n;
}

static int finite8(float a, float b, float c, float d, float e, float f, float g, float h) {
    return isfinite(a) && isfinite(b) && isfinite(c) && isfinite(d) && isfinite(e) && isfinite(f) && isfinite(g) &&
           isfinite(h);
}

/* _line_to, :1463-1472 */
static void line_to_i(vko_context *ctx, float x, float y) {
    v2 p = {x, y};
    if (!path_empty(ctx)) {
        if (v2_equ(cur_pos(ctx), p))
            return;
    }
    add_point(ctx, x, y);
    ctx->simple_convex = 0;
}

/* _curve_to, src/vkvg_context.c:541-566.  With a non-finite control point
   vkvg's recursion never terminates; the oracle (like the GPU library) then
   skips the subdivision and only adds the end point. */
static void curve_to_i(vko_context *ctx, float x1, float y1, float x2, float y2, float x3, float y3) {
    if (VKO_EQUF(x1, x2) && VKO_EQUF(x2, x3) && VKO_EQUF(y1, y2) && VKO_EQUF(y2, y3)) {
        if (path_empty(ctx) || (VKO_EQUF(cur_pos(ctx).x, x1) && VKO_EQUF(cur_pos(ctx).y, y1)))
            return;
    }
    ctx->simple_convex = 0;
    set_curve_start(ctx);
    if (path_empty(ctx))
        add_point(ctx, x1, y1);
    if (path_empty(ctx)) { /* x1 or y1 NaN: vkvg would read a stale point; stop here */
        set_curve_end(ctx);
        return;
    }
    v2    cp = cur_pos(ctx);
    float sx = 1, sy = 1;
    vko_matrix_get_scale(&ctx->mat, &sx, &sy);
    float distanceTolerance = (float)fabs(0.25f / fmaxf(sx, sy));
    if (finite8(cp.x, cp.y, x1, y1, x2, y2, x3, y3))
        recursive_bezier(ctx, distanceTolerance, cp.x, cp.y, x1, y1, x2, y2, x3, y3, 0);
    add_point(ctx, x3, y3);
    set_curve_end(ctx);
}

/* _quadratic_to, src/vkvg_context.c:567-577: 2/3 is a double constant */
static const double quadraticFact = 2.0 / 3.0;
static void quadratic_to_i(vko_context *ctx, float x1, float y1, float x2, float y2) {
    float x0, y0;
    if (path_empty(ctx)) {
        x0 = x1;
        y0 = y1;
    } else {
        v2 c = cur_pos(ctx);
        x0   = c.x;
        y0   = c.y;
    }
    curve_to_i(ctx, (float)(x0 + (x1 - x0) * quadraticFact), (float)(y0 + (y1 - y0) * quadraticFact),
               (float)(x2 + (x1 - x2) * quadraticFact), (float)(y2 + (y1 - y2) * quadraticFact), x2, y2);
}

/* ------------------------------------------------------------- public path */

void vko_new_path(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    clear_path(ctx);
}
void vko_new_sub_path(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    finish_path(ctx);
}
/* vkvg_close_path, src/vkvg_context.c:350-373 */
void vko_close_path(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    uint32_t *pp = ctx->pathes;
    if (pp[ctx->path_ptr] & VKO_PATH_CLOSED_BIT)
        return;
    if (pp[ctx->path_ptr] < 3)
        return;
    if (v2_equ(ctx->points[ctx->point_count - 1], ctx->points[ctx->point_count - pp[ctx->path_ptr]])) {
        if (pp[ctx->path_ptr] < 4)
            return;
        remove_last_point(ctx);
    }
    ctx->pathes[ctx->path_ptr] |= VKO_PATH_CLOSED_BIT;
    finish_path(ctx);
}
/* vkvg_rel_line_to, :374-385 */
void vko_rel_line_to(vko_context *ctx, float dx, float dy) {
    if (vko_status(ctx))
        return;
    if (path_empty(ctx))
        add_point(ctx, 0, 0);
    v2 cp = cur_pos(ctx);
    line_to_i(ctx, cp.x + dx, cp.y + dy);
}
void vko_line_to(vko_context *ctx, float x, float y) {
    if (vko_status(ctx))
        return;
    line_to_i(ctx, x, y);
}
/* vkvg_arc, :394-449 */
void vko_arc(vko_context *ctx, float xc, float yc, float radius, float a1, float a2) {
    if (vko_status(ctx))
        return;
    while (a2 < a1)
        a2 += 2.f * VKO_PIF;
    if (a2 - a1 > 2.f * VKO_PIF)
        a2 = a1 + 2.f * VKO_PIF;
    v2    v    = {VKO_COSF(a1) * radius + xc, VKO_SINF(a1) * radius + yc};
    float step = get_arc_step(ctx, radius);
    float a    = a1;
    if (path_empty(ctx)) {
        set_curve_start(ctx);
        add_point(ctx, v.x, v.y);
        ctx->simple_convex = !ctx->path_ptr;
    } else {
        line_to_i(ctx, v.x, v.y);
        set_curve_start(ctx);
        ctx->simple_convex = 0;
    }
    a += step;
    if (VKO_EQUF(a2, a1))
        return;
    while (a < a2) {
        v.x = VKO_COSF(a) * radius + xc;
        v.y = VKO_SINF(a) * radius + yc;
        add_point(ctx, v.x, v.y);
        a += step;
    }
    if (VKO_EQUF(a2 - a1, VKO_PIF * 2.f)) {
        set_curve_end(ctx);
        vko_close_path(ctx);
        return;
    }
    a   = a2;
    v.x = VKO_COSF(a) * radius + xc;
    v.y = VKO_SINF(a) * radius + yc;
    add_point(ctx, v.x, v.y);
    set_curve_end(ctx);
}
/* vkvg_arc_negative, :450-503 (the 2*pi limit test is kept as written) */
void vko_arc_negative(vko_context *ctx, float xc, float yc, float radius, float a1, float a2) {
    if (vko_status(ctx))
        return;
    while (a2 > a1)
        a2 -= 2.f * VKO_PIF;
    if (a1 - a2 > a1 + 2.f * VKO_PIF)
        a2 = a1 - 2.f * VKO_PIF;
    v2    v    = {VKO_COSF(a1) * radius + xc, VKO_SINF(a1) * radius + yc};
    float step = get_arc_step(ctx, radius);
    float a    = a1;
    if (path_empty(ctx)) {
        set_curve_start(ctx);
        add_point(ctx, v.x, v.y);
        ctx->simple_convex = !ctx->path_ptr;
    } else {
        line_to_i(ctx, v.x, v.y);
        set_curve_start(ctx);
        ctx->simple_convex = 0;
    }
    a -= step;
    if (VKO_EQUF(a2, a1))
        return;
    while (a > a2) {
        v.x = VKO_COSF(a) * radius + xc;
        v.y = VKO_SINF(a) * radius + yc;
        add_point(ctx, v.x, v.y);
        a -= step;
    }
    if (VKO_EQUF(a1 - a2, VKO_PIF * 2.f)) {
        set_curve_end(ctx);
        vko_close_path(ctx);
        return;
    }
    a   = a2;
    v.x = VKO_COSF(a) * radius + xc;
    v.y = VKO_SINF(a) * radius + yc;
    add_point(ctx, v.x, v.y);
    set_curve_end(ctx);
}
/* vkvg_rel_move_to, :504-514 */
void vko_rel_move_to(vko_context *ctx, float x, float y) {
    if (vko_status(ctx))
        return;
    if (path_empty(ctx))
        add_point(ctx, 0, 0);
    v2 cp = cur_pos(ctx);
    finish_path(ctx);
    add_point(ctx, cp.x + x, cp.y + y);
}
/* vkvg_move_to, :515-522 */
void vko_move_to(vko_context *ctx, float x, float y) {
    if (vko_status(ctx))
        return;
    finish_path(ctx);
    add_point(ctx, x, y);
}
bool vko_has_current_point(vko_context *ctx) {
    if (vko_status(ctx))
        return false;
    return !path_empty(ctx);
}
void vko_get_current_point(vko_context *ctx, float *x, float *y) {
    if (vko_status(ctx) || !x || !y)
        return;
    if (path_empty(ctx)) {
        *x = *y = 0;
        return;
    }
    v2 cp = cur_pos(ctx);
    *x    = cp.x;
    *y    = cp.y;
}
void vko_curve_to(vko_context *ctx, float x1, float y1, float x2, float y2, float x3, float y3) {
    if (vko_status(ctx))
        return;
    curve_to_i(ctx, x1, y1, x2, y2, x3, y3);
}
/* vkvg_rel_curve_to, :600-611 */
void vko_rel_curve_to(vko_context *ctx, float x1, float y1, float x2, float y2, float x3, float y3) {
    if (vko_status(ctx))
        return;
    if (path_empty(ctx)) {
        ctx->status = VKO_STATUS_NO_CURRENT_POINT;
        return;
    }
    v2 cp = cur_pos(ctx);
    curve_to_i(ctx, cp.x + x1, cp.y + y1, cp.x + x2, cp.y + y2, cp.x + x3, cp.y + y3);
}
void vko_quadratic_to(vko_context *ctx, float x1, float y1, float x2, float y2) {
    if (vko_status(ctx))
        return;
    quadratic_to_i(ctx, x1, y1, x2, y2);
}
/* vkvg reads a stale point without a current point; like vkvg_rel_curve_to
   the oracle reports VKO_STATUS_NO_CURRENT_POINT */
void vko_rel_quadratic_to(vko_context *ctx, float x1, float y1, float x2, float y2) {
    if (vko_status(ctx))
        return;
    if (path_empty(ctx)) {
        ctx->status = VKO_STATUS_NO_CURRENT_POINT;
        return;
    }
    v2 cp = cur_pos(ctx);
    quadratic_to_i(ctx, cp.x + x1, cp.y + y1, cp.x + x2, cp.y + y2);
}
/* vkvg_rectangle, :620-639 */
int vko_rectangle(vko_context *ctx, float x, float y, float w, float h) {
    if (vko_status(ctx))
        return ctx ? ctx->status : VKO_STATUS_NULL_POINTER;
    finish_path(ctx);
    if (w <= 0 || h <= 0)
        return VKO_STATUS_INVALID_RECT;
    add_point(ctx, x, y);
    add_point(ctx, x + w, y);
    add_point(ctx, x + w, y + h);
    add_point(ctx, x, y + h);
    if (!path_empty(ctx)) /* vkvg flags an empty subpath here when the corners are NaN */
        ctx->pathes[ctx->path_ptr] |= (VKO_PATH_CLOSED_BIT | VKO_PATH_IS_CONVEX_BIT);
    finish_path(ctx);
    return VKO_STATUS_SUCCESS;
}
/* vkvg_rounded_rectangle, :640-665 */
int vko_rounded_rectangle(vko_context *ctx, float x, float y, float w, float h, float radius) {
    if (vko_status(ctx))
        return ctx ? ctx->status : VKO_STATUS_NULL_POINTER;
    finish_path(ctx);
    if (w <= 0 || h <= 0)
        return VKO_STATUS_INVALID_RECT;
    if ((radius > w / 2.0f) || (radius > h / 2.0f))
        radius = (float)fmin(w / 2.0f, h / 2.0f);
    vko_move_to(ctx, x, y + radius);
    vko_arc(ctx, x + radius, y + radius, radius, VKO_PIF, -VKO_PIF_2);
    vko_line_to(ctx, x + w - radius, y);
    vko_arc(ctx, x + w - radius, y + radius, radius, -VKO_PIF_2, 0);
    vko_line_to(ctx, x + w, y + h - radius);
    vko_arc(ctx, x + w - radius, y + h - radius, radius, 0, VKO_PIF_2);
    vko_line_to(ctx, x + radius, y + h);
    vko_arc(ctx, x + radius, y + h - radius, radius, VKO_PIF_2, VKO_PIF);
    vko_line_to(ctx, x, y + radius);
    vko_close_path(ctx);
    return VKO_STATUS_SUCCESS;
}

typedef struct {
    v2 row0, row1;
} mat2;
static v2 mat2_mul(mat2 m, v2 v) { return (v2){(m.row0.x * v.x) + (m.row0.y * v.y), (m.row1.x * v.x) + (m.row1.y * v.y)}; }

/* _elliptic_arc, src/vkvg_context_internal.c:1473-1580 (double where vkvg
   uses double) */
static void elliptic_arc_i(vko_context *ctx, float x1, float y1, float x2, float y2, bool largeArc,
                           bool counterClockWise, float _rx, float _ry, float phi) {
    if (ctx->status)
        return;
    if (_rx == 0 || _ry == 0) {
        if (path_empty(ctx))
            vko_move_to(ctx, x1, y1);
        vko_line_to(ctx, x2, y2);
        return;
    }
    float rx = fabsf(_rx);
    float ry = fabsf(_ry);

    mat2 m  = {{VKO_COSF(phi), VKO_SINF(phi)}, {-VKO_SINF(phi), VKO_COSF(phi)}};
    v2   p  = {(x1 - x2) / 2, (y1 - y2) / 2};
    v2   p1 = mat2_mul(m, p);

    double lambda = VKO_POW2F(p1.x) / VKO_POW2F(rx) + VKO_POW2F(p1.y) / VKO_POW2F(ry);
    if (lambda > 1) {
        lambda = sqrtf((float)lambda);
        rx     = (float)(rx * lambda);
        ry     = (float)(ry * lambda);
    }
    p     = (v2){rx * p1.y / ry, -ry * p1.x / rx};
    v2 cp = v2_mul(p, sqrtf(fabsf((VKO_POW2F(rx) * VKO_POW2F(ry) - VKO_POW2F(rx) * VKO_POW2F(p1.y) -
                                   VKO_POW2F(ry) * VKO_POW2F(p1.x)) /
                                  (VKO_POW2F(rx) * VKO_POW2F(p1.y) + VKO_POW2F(ry) * VKO_POW2F(p1.x)))));
    if (largeArc == counterClockWise) {
        cp.x = -cp.x;
        cp.y = -cp.y;
    }
    m    = (mat2){{VKO_COSF(phi), -VKO_SINF(phi)}, {VKO_SINF(phi), VKO_COSF(phi)}};
    p    = (v2){(x1 + x2) / 2, (y1 + y2) / 2};
    v2 c = v2_add(mat2_mul(m, cp), p);

    v2     u  = {1.f, 0};
    v2     v  = {(p1.x - cp.x) / rx, (p1.y - cp.y) / ry};
    double sa = VKO_ACOSF(v2_dot(u, v) / (fabsf(v2_len(v)) * fabsf(v2_len(u))));
    if (isnan(sa))
        sa = VKO_PIF;
    if (u.x * v.y - u.y * v.x < 0)
        sa = -sa;
    u                  = v;
    v                  = (v2){(-p1.x - cp.x) / rx, (-p1.y - cp.y) / ry};
    double delta_theta = VKO_ACOSF(v2_dot(u, v) / (fabsf(v2_len(v)) * fabsf(v2_len(u))));
    if (isnan(delta_theta))
        delta_theta = VKO_PIF;
    if (u.x * v.y - u.y * v.x < 0)
        delta_theta = -delta_theta;
    if (counterClockWise) {
        if (delta_theta < 0)
            delta_theta += VKO_PIF * 2.0;
    } else if (delta_theta > 0)
        delta_theta -= VKO_PIF * 2.0;

    m            = (mat2){{VKO_COSF(phi), -VKO_SINF(phi)}, {VKO_SINF(phi), VKO_COSF(phi)}};
    double theta = sa;
    double ea    = sa + delta_theta;
    float  step  = fmaxf(0.001f, fminf(VKO_PIF, get_arc_step(ctx, fminf(rx, ry)) * 0.1f));

    p       = (v2){rx * VKO_COSF((float)theta), ry * VKO_SINF((float)theta)};
    v2 xy   = v2_add(mat2_mul(m, p), c);
    if (path_empty(ctx)) {
        set_curve_start(ctx);
        add_point(ctx, xy.x, xy.y);
        ctx->simple_convex = !ctx->path_ptr;
    } else {
        line_to_i(ctx, xy.x, xy.y);
        set_curve_start(ctx);
        ctx->simple_convex = 0;
    }
    set_curve_start(ctx);
    if (sa < ea) {
        theta += step;
        while (theta < ea) {
            p  = (v2){rx * VKO_COSF((float)theta), ry * VKO_SINF((float)theta)};
            xy = v2_add(mat2_mul(m, p), c);
            add_point(ctx, xy.x, xy.y);
            theta += step;
        }
    } else {
        theta -= step;
        while (theta > ea) {
            p  = (v2){rx * VKO_COSF((float)theta), ry * VKO_SINF((float)theta)};
            xy = v2_add(mat2_mul(m, p), c);
            add_point(ctx, xy.x, xy.y);
            theta -= step;
        }
    }
    p  = (v2){rx * VKO_COSF((float)ea), ry * VKO_SINF((float)ea)};
    xy = v2_add(mat2_mul(m, p), c);
    add_point(ctx, xy.x, xy.y);
    set_curve_end(ctx);
}
/* vkvg_elliptic_arc_to, src/vkvg_context.c:1579-1590 */
void vko_elliptic_arc_to(vko_context *ctx, float x2, float y2, bool large, bool sweep, float rx, float ry, float phi) {
    if (vko_status(ctx))
        return;
    float x1, y1;
    vko_get_current_point(ctx, &x1, &y1);
    elliptic_arc_i(ctx, x1, y1, x2, y2, large, sweep, rx, ry, phi);
}
void vko_rel_elliptic_arc_to(vko_context *ctx, float x2, float y2, bool large, bool sweep, float rx, float ry,
                             float phi) {
    if (vko_status(ctx))
        return;
    float x1, y1;
    vko_get_current_point(ctx, &x1, &y1);
    elliptic_arc_i(ctx, x1, y1, x2 + x1, y2 + y1, large, sweep, rx, ry, phi);
}
/* vkvg_ellipse, src/vkvg_context.c:1605-1639 */
void vko_ellipse(vko_context *ctx, float radiusX, float radiusY, float x, float y, float rotationAngle) {
    if (vko_status(ctx))
        return;
    float width_two_thirds = radiusX * 4 / 3;
    float dx1              = VKO_SINF(rotationAngle) * radiusY;
    float dy1              = VKO_COSF(rotationAngle) * radiusY;
    float dx2              = VKO_COSF(rotationAngle) * width_two_thirds;
    float dy2              = VKO_SINF(rotationAngle) * width_two_thirds;
    float topCenterX       = x - dx1;
    float topCenterY       = y + dy1;
    float topRightX        = topCenterX + dx2;
    float topRightY        = topCenterY + dy2;
    float topLeftX         = topCenterX - dx2;
    float topLeftY         = topCenterY - dy2;
    float bottomCenterX    = x + dx1;
    float bottomCenterY    = y - dy1;
    float bottomRightX     = bottomCenterX + dx2;
    float bottomRightY     = bottomCenterY + dy2;
    float bottomLeftX      = bottomCenterX - dx2;
    float bottomLeftY      = bottomCenterY - dy2;
    finish_path(ctx);
    add_point(ctx, bottomCenterX, bottomCenterY);
    curve_to_i(ctx, bottomRightX, bottomRightY, topRightX, topRightY, topCenterX, topCenterY);
    curve_to_i(ctx, topLeftX, topLeftY, bottomLeftX, bottomLeftY, bottomCenterX, bottomCenterY);
    if (!path_empty(ctx))
        ctx->pathes[ctx->path_ptr] |= VKO_PATH_CLOSED_BIT;
    finish_path(ctx);
}

/* subpath walk used by fills, src/vkvg_context_internal.c:1637-1646 */
static uint32_t next_fill_subpath(const vko_context *ctx, uint32_t ptrPath, uint32_t count) {
    if (ctx->pathes[ptrPath] & VKO_PATH_HAS_CURVES_BIT) {
        ptrPath++;
        uint32_t totPts = 0;
        while (totPts < count && ptrPath < ctx->size_pathes)
            totPts += (ctx->pathes[ptrPath++] & VKO_PATH_ELT_MASK);
        return ptrPath;
    }
    return ptrPath + 1;
}
/* vkvg_path_extents, src/vkvg_context.c:688-699 + _vkvg_path_extents :1878-1917 */
void vko_path_extents(vko_context *ctx, float *x1, float *y1, float *x2, float *y2) {
    if (vko_status(ctx))
        return;
    finish_path(ctx);
    if (!ctx->path_ptr) {
        if (x1 && y1 && x2 && y2)
            *x1 = *x2 = *y1 = *y2 = 0;
        return;
    }
    float    xMin = FLT_MAX, yMin = FLT_MAX, xMax = FLT_MIN, yMax = FLT_MIN;
    uint32_t ptrPath = 0, first = 0;
    while (ptrPath < ctx->path_ptr) {
        uint32_t cnt = ctx->pathes[ptrPath] & VKO_PATH_ELT_MASK;
        for (uint32_t i = first; i < first + cnt; i++) {
            v2 p = ctx->points[i];
            if (p.x < xMin)
                xMin = p.x;
            if (p.x > xMax)
                xMax = p.x;
            if (p.y < yMin)
                yMin = p.y;
            if (p.y > yMax)
                yMax = p.y;
        }
        first += cnt;
        ptrPath = next_fill_subpath(ctx, ptrPath, cnt);
    }
    if (x1 && y1 && x2 && y2) {
        *x1 = xMin;
        *x2 = xMax;
        *y1 = yMin;
        *y2 = yMax;
    }
}

/* ----------------------------------------------------------------- strokes */

/* vkvg's round-join / round-cap loops never end for a zero or negative arc
   step (infinite or negative line width) and its dash walk never ends on an
   infinite segment; the oracle bounds them with the caps the GPU kernels use. */
#define VKO_ARC_LOOP_CAP  65536u
#define VKO_DASH_LOOP_CAP (1u << 22)

typedef struct {
    uint32_t iL, iR, cp;
    uint32_t firstIdx;
    float    hw, lhMax, arcStep;
} stroke_ctx;
typedef struct {
    int      dashOn;
    uint32_t curDash;
    float    curDashOffset;
    float    totDashLength;
    v2       normal;
    uint32_t nev; /* joins and caps emitted by this dashed subpath */
} dash_ctx;

/* _build_vb_step, src/vkvg_context_internal.c:924-1163.  Returns det < 0. */
static int build_vb_step(vko_context *ctx, stroke_ctx *str, int isCurve) {
    v2    p0        = ctx->points[str->cp];
    v2    v0        = v2_sub(p0, ctx->points[str->iL]);
    v2    v1        = v2_sub(ctx->points[str->iR], p0);
    float length_v0 = v2_len(v0);
    float length_v1 = v2_len(v1);
    if (length_v0 < FLT_EPSILON || length_v1 < FLT_EPSILON)
        return 0;
    v2    v0n = v2_div(v0, length_v0);
    v2    v1n = v2_div(v1, length_v1);
    float dot = v2_dot(v0n, v1n);
    float det = v0n.x * v1n.y - v0n.y * v1n.x;
    if (VKO_EQUF(dot, 1.0f))
        return 0;
    if (VKO_EQUF(dot, -1.0f)) {
        v2       vPerp = v2_mul(v2_perp(v0n), str->hw);
        uint32_t idx   = ctx->nverts;
        emit_vertex(ctx, v2_add(p0, vPerp));
        emit_vertex(ctx, v2_sub(p0, vPerp));
        emit_tri(ctx, idx, idx + 1, idx + 2);
        emit_tri(ctx, idx, idx + 2, idx + 3);
        return 1;
    }
    v2    bisec_n = v2_norm(v2_add(v0n, v1n));
    float alpha   = VKO_ACOSF(dot);
    if (det < 0)
        alpha = -alpha;
    float halfAlpha    = alpha / 2.f;
    float cosHalfAlpha = VKO_COSF(halfAlpha);
    float lh           = str->hw / cosHalfAlpha;
    v2    bisec_n_perp = v2_perp(bisec_n);
    float rlh          = lh;
    if (dot < 0.f)
        rlh = fminf(rlh, fminf(length_v0, length_v1));
    v2       bisec = v2_mul(bisec_n_perp, rlh);
    uint32_t idx   = ctx->nverts;
    v2       rlh_inside_pos, rlh_outside_pos;
    if (rlh < lh) {
        v2 vnPerp;
        if (length_v0 < length_v1)
            vnPerp = v2_perp(v1n);
        else
            vnPerp = v2_perp(v0n);
        v2    vHwPerp = v2_mul(vnPerp, str->hw);
        float lbc     = cosHalfAlpha * rlh; /* double in vkvg; the product of two floats rounds the same */
        if (det < 0.f) {
            rlh_inside_pos  = v2_add(v2_add(v2_mul(vnPerp, -lbc), v2_add(p0, bisec)), vHwPerp);
            rlh_outside_pos = v2_sub(p0, v2_mul(bisec_n_perp, lh));
        } else {
            rlh_inside_pos  = v2_sub(v2_add(v2_mul(vnPerp, lbc), v2_sub(p0, bisec)), vHwPerp);
            rlh_outside_pos = v2_add(p0, v2_mul(bisec_n_perp, lh));
        }
    } else {
        if (det < 0.0) {
            rlh_inside_pos  = v2_add(p0, bisec);
            rlh_outside_pos = v2_sub(p0, bisec);
        } else {
            rlh_inside_pos  = v2_sub(p0, bisec);
            rlh_outside_pos = v2_add(p0, bisec);
        }
    }
    int join = ctx->line_join;
    if (isCurve) {
        if (dot < 0.8f)
            join = 1; /* ROUND */
        else
            join = 0; /* MITER */
    }
    if (join == 0) {
        if (lh > str->lhMax) {
            float x         = (lh - str->lhMax) * cosHalfAlpha;
            v2    bisecPerp = v2_mul(bisec_n, x);
            bisec           = v2_mul(bisec_n_perp, str->lhMax);
            if (det < 0) {
                emit_vertex(ctx, rlh_inside_pos);
                v2 p = v2_sub(p0, bisec);
                emit_vertex(ctx, v2_sub(p, bisecPerp));
                emit_vertex(ctx, v2_add(p, bisecPerp));
                emit_tri(ctx, idx, idx + 2, idx + 1);
                emit_tri(ctx, idx + 2, idx + 4, idx);
                emit_tri(ctx, idx, idx + 3, idx + 4);
                return 1;
            } else {
                v2 p = v2_add(p0, bisec);
                emit_vertex(ctx, v2_sub(p, bisecPerp));
                emit_vertex(ctx, rlh_inside_pos);
                emit_vertex(ctx, v2_add(p, bisecPerp));
                emit_tri(ctx, idx, idx + 2, idx + 1);
                emit_tri(ctx, idx + 2, idx + 3, idx + 1);
                emit_tri(ctx, idx + 1, idx + 3, idx + 4);
                return 0;
            }
        } else {
            if (det < 0) {
                emit_vertex(ctx, rlh_inside_pos);
                emit_vertex(ctx, rlh_outside_pos);
            } else {
                emit_vertex(ctx, rlh_outside_pos);
                emit_vertex(ctx, rlh_inside_pos);
            }
            emit_rect(ctx, idx);
            return 0;
        }
    } else {
        v2 vp = v2_perp(v0n);
        v2 pos;
        if (det < 0) {
            if (dot < 0 && rlh < lh)
                pos = rlh_inside_pos;
            else
                pos = v2_add(p0, bisec);
            emit_vertex(ctx, pos);
            pos = v2_sub(p0, v2_mul(vp, str->hw));
        } else {
            emit_vertex(ctx, v2_add(p0, v2_mul(vp, str->hw)));
            if (dot < 0 && rlh < lh)
                pos = rlh_inside_pos;
            else
                pos = v2_sub(p0, bisec);
        }
        emit_vertex(ctx, pos);
        if (join == 2) { /* BEVEL */
            if (det < 0) {
                emit_tri(ctx, idx, idx + 2, idx + 1);
                emit_tri(ctx, idx + 2, idx + 4, idx + 0);
                emit_tri(ctx, idx, idx + 3, idx + 4);
            } else {
                emit_tri(ctx, idx, idx + 2, idx + 1);
                emit_tri(ctx, idx + 2, idx + 3, idx + 1);
                emit_tri(ctx, idx + 1, idx + 3, idx + 4);
            }
        } else if (join == 1) { /* ROUND */
            if (!str->arcStep)
                str->arcStep = get_arc_step(ctx, str->hw);
            float a = VKO_ACOSF(vp.x);
            if (vp.y < 0)
                a = -a;
            if (det < 0) {
                a += VKO_PIF;
                float a1 = a + alpha;
                a -= str->arcStep;
                for (uint32_t it = 0; a > a1 && it < VKO_ARC_LOOP_CAP; it++) {
                    emit_vertex(ctx, (v2){VKO_COSF(a) * str->hw + p0.x, VKO_SINF(a) * str->hw + p0.y});
                    a -= str->arcStep;
                }
            } else {
                float a1 = a + alpha;
                a += str->arcStep;
                for (uint32_t it = 0; a < a1 && it < VKO_ARC_LOOP_CAP; it++) {
                    emit_vertex(ctx, (v2){VKO_COSF(a) * str->hw + p0.x, VKO_SINF(a) * str->hw + p0.y});
                    a += str->arcStep;
                }
            }
            uint32_t p0Idx = ctx->nverts;
            emit_tri(ctx, idx, idx + 2, idx + 1);
            if (det < 0) {
                for (uint32_t p = idx + 2; p < p0Idx; p++)
                    emit_tri(ctx, p, p + 1, idx);
                emit_tri(ctx, p0Idx, p0Idx + 2, idx);
                emit_tri(ctx, idx, p0Idx + 1, p0Idx + 2);
            } else {
                for (uint32_t p = idx + 2; p < p0Idx; p++)
                    emit_tri(ctx, p, p + 1, idx + 1);
                emit_tri(ctx, p0Idx, p0Idx + 1, idx + 1);
                emit_tri(ctx, idx + 1, p0Idx + 1, p0Idx + 2);
            }
        }
        vp = v2_mul(v2_perp(v1n), str->hw);
        if (det < 0)
            emit_vertex(ctx, v2_sub(p0, vp));
        else
            emit_vertex(ctx, v2_add(p0, vp));
    }
    return det < 0;
}

/* _draw_stoke_cap, src/vkvg_context_internal.c:1165-1239 */
static void draw_cap(vko_context *ctx, stroke_ctx *str, v2 p0, v2 n, int isStart) {
    uint32_t firstIdx = ctx->nverts;
    if (isStart) {
        v2 vhw = v2_mul(n, str->hw);
        if (ctx->line_cap == 2) /* SQUARE */
            p0 = v2_sub(p0, vhw);
        vhw = v2_perp(vhw);
        if (ctx->line_cap == 1) { /* ROUND */
            if (!str->arcStep)
                str->arcStep = get_arc_step(ctx, str->hw);
            float a = VKO_ACOSF(n.x) + VKO_PIF_2;
            if (n.y < 0)
                a = VKO_PIF - a;
            float a1 = a + VKO_PIF;
            a += str->arcStep;
            for (uint32_t it = 0; a < a1 && it < VKO_ARC_LOOP_CAP; it++) {
                emit_vertex(ctx, (v2){VKO_COSF(a) * str->hw + p0.x, VKO_SINF(a) * str->hw + p0.y});
                a += str->arcStep;
            }
            uint32_t p0Idx = ctx->nverts;
            for (uint32_t p = firstIdx; p < p0Idx; p++)
                emit_tri(ctx, p0Idx + 1, p, p + 1);
            firstIdx = p0Idx;
        }
        emit_vertex(ctx, v2_add(p0, vhw));
        emit_vertex(ctx, v2_sub(p0, vhw));
        emit_rect(ctx, firstIdx);
    } else {
        v2 vhw = v2_mul(n, str->hw);
        if (ctx->line_cap == 2)
            p0 = v2_add(p0, vhw);
        vhw = v2_perp(vhw);
        emit_vertex(ctx, v2_add(p0, vhw));
        emit_vertex(ctx, v2_sub(p0, vhw));
        firstIdx = ctx->nverts;
        if (ctx->line_cap == 1) {
            if (!str->arcStep)
                str->arcStep = get_arc_step(ctx, str->hw);
            float a = VKO_ACOSF(n.x) + VKO_PIF_2;
            if (n.y < 0)
                a = VKO_PIF - a;
            float a1 = a - VKO_PIF;
            a -= str->arcStep;
            for (uint32_t it = 0; a > a1 && it < VKO_ARC_LOOP_CAP; it++) {
                emit_vertex(ctx, (v2){VKO_COSF(a) * str->hw + p0.x, VKO_SINF(a) * str->hw + p0.y});
                a -= str->arcStep;
            }
            uint32_t p0Idx = ctx->nverts - 1;
            for (uint32_t p = firstIdx - 1; p < p0Idx; p++)
                emit_tri(ctx, p + 1, p, firstIdx - 2);
        }
    }
}
/* _draw_dashed_segment, :1240-1264 */
static void draw_dashed_segment(vko_context *ctx, stroke_ctx *str, dash_ctx *dc, int isCurve) {
    v2 p  = ctx->points[str->cp];
    v2 pR = ctx->points[str->iR];
    if (!dc->dashOn) {
        build_vb_step(ctx, str, isCurve);
        dc->nev++;
    }
    v2 d                = v2_sub(pR, p);
    dc->normal          = v2_norm(d);
    float segmentLength = v2_len(d);
    while (dc->curDashOffset < segmentLength && dc->nev < VKO_DASH_LOOP_CAP) {
        v2 p0 = v2_add(p, v2_mul(dc->normal, dc->curDashOffset));
        draw_cap(ctx, str, p0, dc->normal, dc->dashOn);
        dc->nev++;
        dc->dashOn ^= 1;
        dc->curDashOffset += ctx->dashes[dc->curDash];
        if (++dc->curDash == ctx->dash_count)
            dc->curDash = 0;
    }
    dc->curDashOffset -= segmentLength;
    dc->curDashOffset = fmodf(dc->curDashOffset, dc->totDashLength);
}
/* _draw_segment, :1265-1282 (the 1/3-of-index-range batch split never
   triggers with 32-bit indices and is omitted) */
static void draw_segment(vko_context *ctx, stroke_ctx *str, dash_ctx *dc, int isCurve) {
    str->iR = str->cp + 1;
    if (ctx->dash_count > 0)
        draw_dashed_segment(ctx, str, dc, isCurve);
    else
        build_vb_step(ctx, str, isCurve);
    str->iL = str->cp++;
}

static vko_draw *new_draw(vko_context *ctx, int kind) {
    if (ctx->ndraws == ctx->cap_draws) {
        uint32_t  ns = ctx->cap_draws * 2 + 64;
        vko_draw *t  = (vko_draw *)realloc(ctx->draws, (size_t)ns * sizeof(vko_draw));
        if (!t) {
            ctx->status = VKO_STATUS_NO_MEMORY;
            return NULL;
        }
        ctx->draws     = t;
        ctx->cap_draws = ns;
    }
    vko_draw *d = &ctx->draws[ctx->ndraws++];
    memset(d, 0, sizeof(*d));
    d->kind    = kind;
    d->op      = ctx->op;
    d->color   = ctx->cur_color;
    d->opacity = ctx->opacity;
    d->mat     = ctx->mat;
    if (ctx->grad_on && kind <= VKO_DRAW_PAINT) {
        d->grad      = 1;
        d->g         = ctx->grad_snap;
        d->g.opacity = ctx->opacity;
        if (d->g.type == 1) { /* the push constants of this draw; the draw keeps the source alive */
            d->g.m  = ctx->mat_inv;
            d->g.ox = ctx->src_x;
            d->g.oy = ctx->src_y;
            ((vko_surface *)d->g.src)->refs++;
        }
    }
    return d;
}

/* _stroke_preserve, src/vkvg_context.c:822-948.
   Closed-path index patch (:917-932): vkvg patches the last six indices of
   its whole index cache; the oracle patches the last six of this stroke's
   own indices (identical whenever the stroke emitted six or more). */
static void stroke_preserve(vko_context *ctx) {
    finish_path(ctx);
    if (!ctx->path_ptr)
        return;
    ctx->nverts = ctx->ninds = 0;
    stroke_ctx str           = {0};
    str.hw                   = ctx->line_width * 0.5f;
    str.lhMax                = ctx->miter_limit * ctx->line_width;
    uint32_t  ptrPath        = 0;
    uint32_t *pp             = ctx->pathes;
    while (ptrPath < ctx->path_ptr) {
        uint32_t ptrSegment = 0, lastSegmentPointIdx = 0;
        uint32_t firstPathPointIdx = str.cp;
        uint32_t pathPointCount    = pp[ptrPath] & VKO_PATH_ELT_MASK;
        uint32_t lastPathPointIdx  = str.cp + pathPointCount - 1;
        int      closed            = (pp[ptrPath] & VKO_PATH_CLOSED_BIT) != 0;
        int      curves            = (pp[ptrPath] & VKO_PATH_HAS_CURVES_BIT) != 0;
        dash_ctx dc                = {0};
        if (curves) {
            ptrSegment          = 1;
            lastSegmentPointIdx = str.cp + (pp[ptrPath + ptrSegment] & VKO_PATH_ELT_MASK) - 1;
        }
        str.firstIdx = ctx->nverts;
        if (ctx->dash_count > 0) {
            dc.dashOn        = 1;
            dc.curDash       = 0;
            dc.totDashLength = 0;
            for (uint32_t i = 0; i < ctx->dash_count; i++)
                dc.totDashLength += ctx->dashes[i];
            if (dc.totDashLength == 0) {
                ctx->status = VKO_STATUS_INVALID_DASH;
                return;
            }
            dc.curDashOffset = fmodf(ctx->dash_offset, dc.totDashLength);
            str.iL           = lastPathPointIdx;
        } else if (closed) {
            str.iL = lastPathPointIdx;
        } else {
            draw_cap(ctx, &str, ctx->points[str.cp], v2_line_norm(ctx->points[str.cp], ctx->points[str.cp + 1]), 1);
            str.iL = str.cp++;
        }
        if (curves) {
            uint32_t guard = 0;
            while (str.cp < lastPathPointIdx) {
                int curved = (pp[ptrPath + ptrSegment] & VKO_PATH_HAS_CURVES_BIT) != 0;
                if (lastSegmentPointIdx == lastPathPointIdx)
                    lastSegmentPointIdx--;
                while (str.cp <= lastSegmentPointIdx)
                    draw_segment(ctx, &str, &dc, curved);
                ptrSegment++;
                uint32_t cptSegPts  = pp[ptrPath + ptrSegment] & VKO_PATH_ELT_MASK;
                lastSegmentPointIdx = str.cp + cptSegPts - 1;
                if (lastSegmentPointIdx == lastPathPointIdx && cptSegPts == 1) {
                    ptrSegment++;
                    break;
                }
                if (++guard > pathPointCount + 2) /* malformed segment table: stop */
                    break;
            }
        } else
            while (str.cp < lastPathPointIdx)
                draw_segment(ctx, &str, &dc, 0);

        if (ctx->dash_count > 0) {
            if (closed) {
                str.iR = firstPathPointIdx;
                draw_dashed_segment(ctx, &str, &dc, 0);
                str.iL++;
                str.cp++;
            }
            if (!dc.dashOn) {
                /* vkvg reads dashes[-1] when curDash == 0 (it assigns curDash
                   instead of prevDash); the oracle uses the last dash entry. */
                int32_t prevDash = (int32_t)dc.curDash - 1;
                if (prevDash < 0) {
                    dc.curDash = ctx->dash_count - 1;
                    prevDash   = (int32_t)ctx->dash_count - 1;
                }
                float m = fminf(ctx->dashes[prevDash] - dc.curDashOffset, ctx->dashes[dc.curDash]);
                v2    p = v2_sub(ctx->points[str.iR], v2_mul(dc.normal, m));
                draw_cap(ctx, &str, p, dc.normal, 0);
            }
        } else if (closed) {
            str.iR      = firstPathPointIdx;
            int inverse = build_vb_step(ctx, &str, 0);
            if (ctx->ninds >= 6) {
                uint32_t *inds = &ctx->inds[ctx->ninds - 6];
                uint32_t  ii   = str.firstIdx;
                if (inverse) {
                    inds[1] = ii + 1;
                    inds[4] = ii + 1;
                    inds[5] = ii;
                } else {
                    inds[1] = ii;
                    inds[4] = ii;
                    inds[5] = ii + 1;
                }
            }
            str.cp++;
        } else
            draw_cap(ctx, &str, ctx->points[str.cp], v2_line_norm(ctx->points[str.cp - 1], ctx->points[str.cp]), 0);

        str.cp = firstPathPointIdx + pathPointCount;
        if (ptrSegment > 0)
            ptrPath += ptrSegment;
        else
            ptrPath++;
    }
    vko_draw *d = new_draw(ctx, VKO_DRAW_STROKE);
    if (!d)
        return;
    d->nverts = ctx->nverts;
    d->ninds  = ctx->ninds;
    d->verts  = (float *)malloc((size_t)(ctx->nverts + 1) * 2 * sizeof(float));
    d->inds   = (uint32_t *)malloc((size_t)(ctx->ninds + 1) * sizeof(uint32_t));
    if (!d->verts || !d->inds) {
        ctx->status = VKO_STATUS_NO_MEMORY;
        return;
    }
    memcpy(d->verts, ctx->verts, (size_t)ctx->nverts * sizeof(v2));
    memcpy(d->inds, ctx->inds, (size_t)ctx->ninds * sizeof(uint32_t));
}

/* _fill_preserve, src/vkvg_context.c:796-821, with the EO scissor bounds of
   _poly_fill (src/vkvg_context_internal.c:1583-1655) */
static int fill_geom(vko_context *ctx, int clip) {
    finish_path(ctx);
    if (!ctx->path_ptr)
        return 0;
    int       eo = ctx->fill_rule == 0;
    vko_draw *d  = new_draw(ctx, clip ? (eo ? VKO_DRAW_CLIP_EO : VKO_DRAW_CLIP_NZ)
                                      : (eo ? VKO_DRAW_FILL_EO : VKO_DRAW_FILL_NZ));
    if (!d)
        return 0;
    uint32_t nsub = 0, ptrPath = 0, first = 0;
    while (ptrPath < ctx->path_ptr) {
        uint32_t cnt = ctx->pathes[ptrPath] & VKO_PATH_ELT_MASK;
        nsub++;
        first += cnt;
        ptrPath = next_fill_subpath(ctx, ptrPath, cnt);
    }
    d->npts       = first;
    d->nsub       = nsub;
    d->pts        = (float *)malloc((size_t)(first + 1) * 2 * sizeof(float));
    d->sub_counts = (uint32_t *)malloc((size_t)(nsub + 1) * sizeof(uint32_t));
    if (!d->pts || !d->sub_counts) {
        ctx->status = VKO_STATUS_NO_MEMORY;
        return 0;
    }
    memcpy(d->pts, ctx->points, (size_t)first * sizeof(v2));
    d->bounds[0] = FLT_MAX;
    d->bounds[1] = FLT_MAX;
    d->bounds[2] = FLT_MIN;
    d->bounds[3] = FLT_MIN;
    nsub = 0;
    ptrPath = 0;
    first   = 0;
    while (ptrPath < ctx->path_ptr) {
        uint32_t cnt          = ctx->pathes[ptrPath] & VKO_PATH_ELT_MASK;
        d->sub_counts[nsub++] = cnt;
        if (cnt > 2) {
            for (uint32_t i = 0; i < cnt; i++) {
                v2 p = ctx->points[first + i];
                vko_matrix_transform_point(&ctx->mat, &p.x, &p.y);
                if (p.x < d->bounds[0])
                    d->bounds[0] = p.x;
                if (p.x > d->bounds[2])
                    d->bounds[2] = p.x;
                if (p.y < d->bounds[1])
                    d->bounds[1] = p.y;
                if (p.y > d->bounds[3])
                    d->bounds[3] = p.y;
            }
        }
        first += cnt;
        ptrPath = next_fill_subpath(ctx, ptrPath, cnt);
    }
    d->convex = (ctx->path_ptr == 1 && (ctx->pathes[0] & VKO_PATH_IS_CONVEX_BIT)) ? 1 : 0;
    return 1;
}
static void fill_preserve(vko_context *ctx) { fill_geom(ctx, 0); }
/* the geometry of _clip_preserve (src/vkvg_context.c:754-795): returns
   whether the path had anything to clip with */
int       vko_clip_preserve_geom(vko_context *ctx) { return fill_geom(ctx, 1); }
vko_draw *vko_new_draw(vko_context *ctx, int kind) { return new_draw(ctx, kind); }
void      vko_clear_path(vko_context *ctx) { clear_path(ctx); }

void vko_fill_preserve(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    fill_preserve(ctx);
}
void vko_fill(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    fill_preserve(ctx);
    clear_path(ctx);
}
void vko_stroke_preserve(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    stroke_preserve(ctx);
}
void vko_stroke(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    stroke_preserve(ctx);
    clear_path(ctx);
}
/* vkvg_paint, src/vkvg_context.c:990-1003 */
void vko_paint(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    finish_path(ctx);
    if (ctx->path_ptr) {
        vko_fill(ctx);
        return;
    }
    new_draw(ctx, VKO_DRAW_PAINT);
}
/* vkvg_clear, src/vkvg_context.c:734-753 */
void vko_clear(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    int prev        = ctx->saved ? ctx->saved->clip_state : VKO_CLIP_CLEAR;
    ctx->clip_state = prev == VKO_CLIP_CLEAR ? VKO_CLIP_NONE : VKO_CLIP_CLEAR;
    new_draw(ctx, VKO_DRAW_CLEAR);
}

void vko_ctx_init_geom(vko_context *ctx) {
    ctx->size_points = 1024;
    ctx->points      = (v2 *)malloc(ctx->size_points * sizeof(v2));
    ctx->size_pathes = 64;
    ctx->pathes      = (uint32_t *)calloc(ctx->size_pathes, sizeof(uint32_t));
    if (!ctx->points || !ctx->pathes)
        ctx->status = VKO_STATUS_NO_MEMORY;
    clear_path(ctx);
}
void vko_draw_free(vko_draw *d) {
    if (d->grad && d->g.type == 1 && d->g.src)
        vko_surface_destroy((vko_surface *)d->g.src);
    free(d->pts);
    free(d->sub_counts);
    free(d->verts);
    free(d->inds);
    memset(d, 0, sizeof(*d));
}
void vko_ctx_free_geom(vko_context *ctx) {
    free(ctx->points);
    free(ctx->pathes);
    free(ctx->verts);
    free(ctx->inds);
    for (uint32_t i = 0; i < ctx->ndraws; i++)
        vko_draw_free(&ctx->draws[i]);
    free(ctx->draws);
    free(ctx->dashes);
}
