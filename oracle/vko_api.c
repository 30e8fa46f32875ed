/*
 * vko_api.c - oracle surfaces, contexts, state and matrices
 * (TEST INFRASTRUCTURE ONLY).  Matrix functions restate src/vkvg_matrix.c of
 * vkvg (cairo-derived); state setters restate src/vkvg_context.c:1011-1115.
 */
#include "vko_internal.h"

/* ---------------------------------------------------------------- matrices */

void vko_matrix_init(vko_matrix *m, float xx, float yx, float xy, float yy, float x0, float y0) {
    m->xx = xx;
    m->yx = yx;
    m->xy = xy;
    m->yy = yy;
    m->x0 = x0;
    m->y0 = y0;
}
void vko_matrix_init_identity(vko_matrix *m) { vko_matrix_init(m, 1, 0, 0, 1, 0, 0); }
void vko_matrix_init_translate(vko_matrix *m, float tx, float ty) { vko_matrix_init(m, 1, 0, 0, 1, tx, ty); }
void vko_matrix_init_scale(vko_matrix *m, float sx, float sy) { vko_matrix_init(m, sx, 0, 0, sy, 0, 0); }
void vko_matrix_init_rotate(vko_matrix *m, float radians) {
    float s = VKO_SINF(radians), c = VKO_COSF(radians);
    vko_matrix_init(m, c, s, -s, c, 0, 0);
}
/* vkvg_matrix_multiply, src/vkvg_matrix.c:193-205 */
void vko_matrix_multiply(vko_matrix *result, const vko_matrix *a, const vko_matrix *b) {
    vko_matrix r;
    r.xx    = a->xx * b->xx + a->yx * b->xy;
    r.yx    = a->xx * b->yx + a->yx * b->yy;
    r.xy    = a->xy * b->xx + a->yy * b->xy;
    r.yy    = a->xy * b->yx + a->yy * b->yy;
    r.x0    = a->x0 * b->xx + a->y0 * b->xy + b->x0;
    r.y0    = a->x0 * b->yx + a->y0 * b->yy + b->y0;
    *result = r;
}
void vko_matrix_translate(vko_matrix *m, float tx, float ty) {
    vko_matrix t;
    vko_matrix_init_translate(&t, tx, ty);
    vko_matrix_multiply(m, &t, m);
}
void vko_matrix_scale(vko_matrix *m, float sx, float sy) {
    vko_matrix t;
    vko_matrix_init_scale(&t, sx, sy);
    vko_matrix_multiply(m, &t, m);
}
void vko_matrix_rotate(vko_matrix *m, float radians) {
    vko_matrix t;
    vko_matrix_init_rotate(&t, radians);
    vko_matrix_multiply(m, &t, m);
}
void vko_matrix_transform_distance(const vko_matrix *m, float *dx, float *dy) {
    float nx = (m->xx * *dx + m->xy * *dy);
    float ny = (m->yx * *dx + m->yy * *dy);
    *dx      = nx;
    *dy      = ny;
}
void vko_matrix_transform_point(const vko_matrix *m, float *x, float *y) {
    vko_matrix_transform_distance(m, x, y);
    *x += m->x0;
    *y += m->y0;
}
/* vkvg_matrix_invert, src/vkvg_matrix.c:107-148 */
int vko_matrix_invert(vko_matrix *m) {
    if (m->xy == 0. && m->yx == 0.) {
        m->x0 = -m->x0;
        m->y0 = -m->y0;
        if (m->xx != 1.f) {
            if (m->xx == 0.)
                return VKO_STATUS_INVALID_MATRIX;
            m->xx = 1.f / m->xx;
            m->x0 *= m->xx;
        }
        if (m->yy != 1.f) {
            if (m->yy == 0.)
                return VKO_STATUS_INVALID_MATRIX;
            m->yy = 1.f / m->yy;
            m->y0 *= m->yy;
        }
        return VKO_STATUS_SUCCESS;
    }
    float det = m->xx * m->yy - m->yx * m->xy;
    if (!(det * det >= 0.))
        return VKO_STATUS_INVALID_MATRIX;
    if (det == 0)
        return VKO_STATUS_INVALID_MATRIX;
    float a = m->xx, b = m->yx, c = m->xy, d = m->yy, tx = m->x0, ty = m->y0;
    vko_matrix_init(m, d, -b, -c, a, c * ty - d * tx, b * tx - a * ty);
    float s = 1 / det;
    m->xx *= s;
    m->yx *= s;
    m->xy *= s;
    m->yy *= s;
    m->x0 *= s;
    m->y0 *= s;
    return VKO_STATUS_SUCCESS;
}
/* vkvg_matrix_get_scale, src/vkvg_matrix.c:222-229 (double sqrt) */
void vko_matrix_get_scale(const vko_matrix *m, float *sx, float *sy) {
    *sx = (float)sqrt(m->xx * m->xx + m->xy * m->xy);
    *sy = (float)sqrt(m->yx * m->yx + m->yy * m->yy);
}

/* ---------------------------------------------------------------- surfaces */

vko_surface *vko_surface_create(uint32_t width, uint32_t height, uint32_t samples) {
    vko_surface *s = (vko_surface *)calloc(1, sizeof(vko_surface));
    if (!s)
        return NULL;
    s->width   = width < 1 ? 1 : width;
    s->height  = height < 1 ? 1 : height;
    s->samples = samples == 4 ? 4 : 1;
    s->refs    = 1;
    size_t ns  = (size_t)s->width * s->height * s->samples;
    s->data    = (uint8_t *)calloc(ns, 4);
    s->stencil = (uint8_t *)calloc(ns, 1);
    if (!s->data || !s->stencil)
        s->status = VKO_STATUS_NO_MEMORY;
    return s;
}
static void surface_release(vko_surface *s) {
    if (!s)
        return;
    if (--s->refs > 0)
        return;
    free(s->data);
    free(s->stencil);
    for (uint32_t i = 0; i < s->nimages; i++)
        free(s->images[i]);
    free(s->images);
    free(s);
}
void     vko_surface_destroy(vko_surface *s) { surface_release(s); }
int      vko_surface_status(vko_surface *s) { return s ? s->status : VKO_STATUS_NULL_POINTER; }
uint32_t vko_surface_get_width(vko_surface *s) { return s ? s->width : 0; }
uint32_t vko_surface_get_height(vko_surface *s) { return s ? s->height : 0; }
void     vko_surface_clear(vko_surface *s) {
    if (vko_surface_status(s))
        return;
    size_t ns = (size_t)s->width * s->height * s->samples;
    memset(s->data, 0, ns * 4);
    memset(s->stencil, 0, ns);
}
int vko_surface_read_samples(vko_surface *s, uint8_t *out) {
    if (vko_surface_status(s) || !out)
        return VKO_STATUS_INVALID_STATUS;
    memcpy(out, s->data, (size_t)s->width * s->height * s->samples * 4);
    return 0;
}
int vko_surface_resolve_premult(vko_surface *s, uint8_t *rgba) {
    if (vko_surface_status(s) || !rgba)
        return VKO_STATUS_INVALID_STATUS;
    vko_resolve(s, rgba);
    return 0;
}
/* vkvg_surface_write_to_memory, src/vkvg_surface.c:393-467: resolve, then
   p = (uchar)(p / (a/255.f)) in double, truncating.  Where vkvg's conversion
   is undefined (a == 0, or p > a) the oracle writes 0 / clamps to 255. */
int vko_surface_write_to_memory(vko_surface *s, uint8_t *rgba) {
    if (vko_surface_status(s))
        return VKO_STATUS_INVALID_STATUS;
    if (!rgba)
        return VKO_STATUS_WRITE_ERROR;
    vko_resolve(s, rgba);
    for (size_t p = 0; p < (size_t)s->width * s->height; p++) {
        uint8_t *q     = rgba + p * 4;
        double   alpha = (double)q[3] / 255.f;
        for (int c = 0; c < 3; c++) {
            if (q[3] == 0) {
                q[c] = 0;
                continue;
            }
            double v = (double)q[c] / alpha;
            q[c]     = v >= 255.0 ? 255 : (uint8_t)v;
        }
    }
    return 0;
}
int vko_surface_write_to_png(vko_surface *s, const char *path) {
    if (vko_surface_status(s))
        return VKO_STATUS_INVALID_STATUS;
    if (!path)
        return VKO_STATUS_WRITE_ERROR;
    uint8_t *img = (uint8_t *)malloc((size_t)s->width * s->height * 4);
    if (!img)
        return VKO_STATUS_NO_MEMORY;
    vko_surface_write_to_memory(s, img);
    int r = vko_png_write(path, s->width, s->height, img);
    free(img);
    return r ? VKO_STATUS_WRITE_ERROR : 0;
}

/* ---------------------------------------------------------------- contexts */

/* defaults: _init_ctx, src/vkvg_context.c:24-70 */
vko_context *vko_create(vko_surface *surf) {
    if (vko_surface_status(surf))
        return NULL;
    vko_context *ctx = (vko_context *)calloc(1, sizeof(vko_context));
    if (!ctx)
        return NULL;
    ctx->surf = surf;
    surf->refs++;
    ctx->line_width  = 1.f;
    ctx->miter_limit = 10.f;
    ctx->op          = VKO_OP_OVER;
    ctx->fill_rule   = 1; /* NON_ZERO */
    ctx->cur_color   = 0xff000000u;
    ctx->opacity     = 1.0f;
    vko_matrix_init_identity(&ctx->mat);
    vko_matrix_init_identity(&ctx->mat_inv);
    vko_ctx_init_geom(ctx);
    /* the context's first render pass clears the stencil
       (renderPass_ClearStencil, src/vkvg_context.c:43-49); recorded only when
       a previous context left something in it */
    size_t ns = (size_t)surf->width * surf->height * surf->samples;
    for (size_t i = 0; i < ns; i++)
        if (surf->stencil[i]) {
            vko_new_draw(ctx, VKO_DRAW_RESET);
            break;
        }
    return ctx;
}
int  vko_status(vko_context *ctx) { return ctx ? ctx->status : VKO_STATUS_NULL_POINTER; }
void vko_keep_draws(vko_context *ctx, int keep) {
    if (ctx)
        ctx->keep_draws = keep;
}
/* rasterise pending draws in submission order */
void vko_flush(vko_context *ctx) {
    if (!ctx)
        return;
    for (uint32_t i = ctx->nrastered; i < ctx->ndraws; i++)
        vko_raster_draw(ctx->surf, &ctx->draws[i]);
    ctx->nrastered = ctx->ndraws;
    if (!ctx->keep_draws) {
        for (uint32_t i = 0; i < ctx->ndraws; i++)
            vko_draw_free(&ctx->draws[i]);
        ctx->ndraws = ctx->nrastered = 0;
    }
}
void vko_destroy(vko_context *ctx) {
    if (!ctx)
        return;
    vko_flush(ctx);
    if (ctx->pattern)
        vko_pattern_destroy(ctx->pattern);
    while (ctx->saved) {
        vko_saved *sv = ctx->saved;
        ctx->saved    = sv->next;
        if (sv->pattern)
            vko_pattern_destroy(sv->pattern);
        free(sv->dashes);
        free(sv);
    }
    vko_surface *s = ctx->surf;
    vko_ctx_free_geom(ctx);
    free(ctx);
    surface_release(s);
}

/* ------------------------------------------------------------------- state */

static uint32_t clamp_byte(float v) {
    if (!(v > 0.0f))
        return 0;
    if (v > 255.0f)
        return 255;
    return (uint32_t)v;
}
/* CreateRgbaf, src/vkvg_context_internal.h:59-62 (premultiplied, truncating;
   the oracle clamps products outside [0,255] where vkvg's cast is undefined) */
static uint32_t create_rgbaf(float r, float g, float b, float a) {
    return (clamp_byte(a * 255.0f) << 24) | (clamp_byte(b * a * 255.0f) << 16) | (clamp_byte(g * a * 255.0f) << 8) |
           clamp_byte(r * a * 255.0f);
}
/* ---------------------------------------------------------------- patterns */
/* src/vkvg_pattern.c (linear gradients) */
static vko_pattern s_pattern_no_memory = {VKO_STATUS_NO_MEMORY};
static vko_pattern s_pattern_null      = {VKO_STATUS_NULL_POINTER};
vko_pattern *vko_pattern_create_linear(float x0, float y0, float x1, float y1) {
    vko_pattern *p = (vko_pattern *)calloc(1, sizeof(vko_pattern));
    if (!p)
        return &s_pattern_no_memory;
    p->refs = 1;
    p->type = 2; /* VKVG_PATTERN_TYPE_LINEAR */
    p->cp[0] = x0;
    p->cp[1] = y0;
    p->cp[2] = x1;
    p->cp[3] = y1;
    vko_matrix_init_identity(&p->matrix);
    return p;
}
int vko_pattern_status(vko_pattern *pat) { return pat ? pat->status : VKO_STATUS_NULL_POINTER; }
vko_pattern *vko_pattern_reference(vko_pattern *pat) {
    if (!vko_pattern_status(pat))
        pat->refs++;
    return pat;
}
uint32_t vko_pattern_get_reference_count(vko_pattern *pat) { return vko_pattern_status(pat) ? 0 : pat->refs; }
void     vko_pattern_destroy(vko_pattern *pat) {
    if (vko_pattern_status(pat))
        return;
    if (--pat->refs > 0)
        return;
    if (pat->surf)
        surface_release(pat->surf);
    free(pat);
}
/* vkvg_pattern_create_for_surface, src/vkvg_pattern.c:28-48 */
vko_pattern *vko_pattern_create_for_surface(vko_surface *surf) {
    if (!surf)
        return &s_pattern_null;
    vko_pattern *p = (vko_pattern *)calloc(1, sizeof(vko_pattern));
    if (!p)
        return &s_pattern_null;
    p->refs = 1;
    p->type = 1; /* VKVG_PATTERN_TYPE_SURFACE */
    p->surf = surf;
    surf->refs++;
    vko_matrix_init_identity(&p->matrix);
    if (vko_surface_status(surf))
        p->status = VKO_STATUS_INVALID_SURFACE;
    return p;
}
void vko_pattern_set_extend(vko_pattern *pat, int extend) {
    if (!vko_pattern_status(pat))
        pat->extend = extend;
}
void vko_pattern_set_filter(vko_pattern *pat, int filter) {
    if (!vko_pattern_status(pat))
        pat->filter = filter;
}
/* vkvg_pattern_edit_radial / create_radial, src/vkvg_pattern.c:95-134 */
int vko_pattern_edit_radial(vko_pattern *pat, float cx0, float cy0, float r0, float cx1, float cy1, float r1) {
    if (vko_pattern_status(pat))
        return vko_pattern_status(pat);
    if (pat->type != 3)
        return VKO_STATUS_PATTERN_TYPE_MISMATCH;
    v2 c0 = {cx0, cy0}, c1 = {cx1, cy1};
    if (r0 > r1 - 1.0f)
        r0 = r1 - 1.0f;
    v2    u = v2_sub(c0, c1);
    float l = v2_len(u);
    if (l + r0 + 1.0f >= r1) {
        v2 v = v2_div(u, l);
        c0   = v2_add(c1, v2_mul(v, r1 - r0 - 1.0f));
    }
    float cp[8] = {c0.x, c0.y, r0, 0.0f, c1.x, c1.y, r1, 0.0f};
    memcpy(pat->cp, cp, sizeof(cp));
    return VKO_STATUS_SUCCESS;
}
vko_pattern *vko_pattern_create_radial(float cx0, float cy0, float r0, float cx1, float cy1, float r1) {
    vko_pattern *p = (vko_pattern *)calloc(1, sizeof(vko_pattern));
    if (!p)
        return &s_pattern_no_memory;
    p->refs = 1;
    p->type = 3; /* VKVG_PATTERN_TYPE_RADIAL */
    vko_matrix_init_identity(&p->matrix);
    vko_pattern_edit_radial(p, cx0, cy0, r0, cx1, cy1, r1);
    return p;
}
int vko_pattern_edit_linear(vko_pattern *pat, float x0, float y0, float x1, float y1) {
    if (vko_pattern_status(pat))
        return vko_pattern_status(pat);
    if (pat->type != 2)
        return VKO_STATUS_PATTERN_TYPE_MISMATCH;
    pat->cp[0] = x0;
    pat->cp[1] = y0;
    pat->cp[2] = x1;
    pat->cp[3] = y1;
    return VKO_STATUS_SUCCESS;
}
/* vkvg_pattern_add_color_stop, src/vkvg_pattern.c:149-168: premultiplied
   stop colour; vkvg writes past its 16-entry array, the oracle refuses */
int vko_pattern_add_color_stop(vko_pattern *pat, float offset, float r, float g, float b, float a) {
    if (vko_pattern_status(pat))
        return vko_pattern_status(pat);
    if (pat->count >= VKO_GRAD_STOPS)
        return VKO_STATUS_INVALID_INDEX;
    float *c                 = pat->colors + 4 * pat->count;
    c[0]                     = a * r;
    c[1]                     = a * g;
    c[2]                     = a * b;
    c[3]                     = a;
    pat->stops[pat->count++] = offset;
    return VKO_STATUS_SUCCESS;
}
int vko_pattern_get_color_stop_count(vko_pattern *pat, uint32_t *count) {
    if (vko_pattern_status(pat))
        return vko_pattern_status(pat);
    *count = pat->count;
    return VKO_STATUS_SUCCESS;
}
void vko_pattern_set_matrix(vko_pattern *pat, const vko_matrix *m) {
    if (vko_pattern_status(pat) || !m)
        return;
    pat->matrix     = *m;
    pat->has_matrix = 1;
}
static void set_solid(vko_context *ctx) {
    if (ctx->pattern)
        vko_pattern_destroy(ctx->pattern);
    ctx->pattern = NULL;
    ctx->grad_on = 0;
}
/* vkvg_set_source + _update_cur_pattern (src/vkvg_context.c:1034-1040,
   src/vkvg_context_internal.c:774-826): the gradient as of now, control
   points through the inverse pattern matrix (identity if singular) and the
   CTM, with the target surface's size */
static void snap_gradient(vko_context *ctx, vko_pattern *pat);
void        vko_set_source(vko_context *ctx, vko_pattern *pat) {
    if (vko_status(ctx) || vko_pattern_status(pat))
        return;
    vko_pattern_reference(pat);
    set_solid(ctx);
    ctx->pattern = pat;
    snap_gradient(ctx, pat);
}
/* vkvg_set_source_surface, src/vkvg_context.c:1025-1033 */
void vko_set_source_surface(vko_context *ctx, vko_surface *surf, float x, float y) {
    if (vko_status(ctx) || vko_surface_status(surf))
        return;
    ctx->src_x       = x;
    ctx->src_y       = y;
    vko_pattern *pat = vko_pattern_create_for_surface(surf);
    if (vko_pattern_status(pat)) {
        ctx->status = vko_pattern_status(pat);
        return;
    }
    set_solid(ctx);
    ctx->pattern = pat;
    snap_gradient(ctx, pat);
}
/* _update_cur_pattern, src/vkvg_context_internal.c:682-831 */
static void snap_gradient(vko_context *ctx, vko_pattern *pat) {
    if (pat->type == 1) {
        /* sampled through each draw's push constants; the pattern matrix
           goes into the pushed inverse now */
        vko_grad *g = &ctx->grad_snap;
        memset(g, 0, sizeof(*g));
        g->type     = 1;
        g->w        = (float)ctx->surf->width;
        g->h        = (float)ctx->surf->height;
        g->src      = pat->surf;
        g->extend   = pat->extend;
        g->bilinear = pat->filter == 4 || pat->filter == 2; /* VKVG_FILTER_BILINEAR, _BEST */
        if (pat->has_matrix) {
            vko_matrix r;
            vko_matrix_multiply(&r, &ctx->mat_inv, &pat->matrix);
            ctx->mat_inv = r;
        }
        ctx->grad_on = 1;
        return;
    }
    if (pat->type != 2 && pat->type != 3) {
        ctx->status = VKO_STATUS_PATTERN_TYPE_MISMATCH;
        return;
    }
    /* the push constant source becomes the surface bounds */
    ctx->src_x = (float)ctx->surf->width;
    ctx->src_y = (float)ctx->surf->height;
    if (pat->count < 2) {
        ctx->status = VKO_STATUS_PATTERN_INVALID_GRADIENT;
        return;
    }
    vko_grad *g = &ctx->grad_snap;
    memset(g, 0, sizeof(*g));
    /* grad.cp[0] is g->cp[0..3], grad.cp[1] is g->cp[4..7] */
    memcpy(g->cp, pat->cp, sizeof(g->cp));
    vko_matrix inv;
    vko_matrix_init_identity(&inv);
    if (pat->has_matrix) {
        inv = pat->matrix;
        if (vko_matrix_invert(&inv) != VKO_STATUS_SUCCESS)
            vko_matrix_init_identity(&inv);
        vko_matrix_transform_point(&inv, &g->cp[0], &g->cp[1]);
    }
    vko_matrix_transform_point(&ctx->mat, &g->cp[0], &g->cp[1]);
    if (pat->type == 2) {
        if (pat->has_matrix)
            vko_matrix_transform_point(&inv, &g->cp[2], &g->cp[3]);
        vko_matrix_transform_point(&ctx->mat, &g->cp[2], &g->cp[3]);
    } else {
        if (pat->has_matrix)
            vko_matrix_transform_point(&inv, &g->cp[4], &g->cp[5]);
        vko_matrix_transform_point(&ctx->mat, &g->cp[4], &g->cp[5]);
        /* radii: transform_distance with grad.cp[0].w as y for both
           (src/vkvg_context_internal.c:815-821) */
        if (pat->has_matrix) {
            vko_matrix_transform_distance(&inv, &g->cp[2], &g->cp[3]);
            vko_matrix_transform_distance(&inv, &g->cp[6], &g->cp[3]);
        }
        vko_matrix_transform_distance(&ctx->mat, &g->cp[2], &g->cp[3]);
        vko_matrix_transform_distance(&ctx->mat, &g->cp[6], &g->cp[3]);
    }
    g->type  = pat->type;
    g->w     = (float)ctx->surf->width;
    g->h     = (float)ctx->surf->height;
    g->count = pat->count;
    memcpy(g->stops, pat->stops, sizeof(g->stops));
    memcpy(g->colors, pat->colors, sizeof(g->colors));
    ctx->grad_on = 1;
}
void vko_set_source_rgba(vko_context *ctx, float r, float g, float b, float a) {
    if (vko_status(ctx))
        return;
    set_solid(ctx);
    ctx->cur_color = create_rgbaf(r, g, b, a);
}
void vko_set_source_rgb(vko_context *ctx, float r, float g, float b) {
    if (vko_status(ctx))
        return;
    set_solid(ctx);
    ctx->cur_color = create_rgbaf(r, g, b, 1);
}
void vko_set_source_color(vko_context *ctx, uint32_t c) {
    if (vko_status(ctx))
        return;
    set_solid(ctx);
    ctx->cur_color = c;
}
uint32_t vko_get_color(vko_context *ctx) { return ctx ? ctx->cur_color : 0; }
void     vko_set_line_width(vko_context *ctx, float w) {
    if (!vko_status(ctx))
        ctx->line_width = w;
}
void vko_set_miter_limit(vko_context *ctx, float l) {
    if (!vko_status(ctx))
        ctx->miter_limit = l;
}
void vko_set_line_cap(vko_context *ctx, int cap) {
    if (!vko_status(ctx))
        ctx->line_cap = cap;
}
void vko_set_line_join(vko_context *ctx, int join) {
    if (!vko_status(ctx))
        ctx->line_join = join;
}
void vko_set_fill_rule(vko_context *ctx, int fr) {
    if (!vko_status(ctx))
        ctx->fill_rule = fr;
}
void vko_set_operator(vko_context *ctx, int op) {
    if (!vko_status(ctx))
        ctx->op = op;
}
/* vkvg_set_opacity, src/vkvg_context.c:305-315 */
void vko_set_opacity(vko_context *ctx, float o) {
    if (!vko_status(ctx))
        ctx->opacity = o;
}
/* vkvg_set_dash, src/vkvg_context.c:1103-1115 (the array is copied) */
void vko_set_dash(vko_context *ctx, const float *dashes, uint32_t n, float offset) {
    if (vko_status(ctx))
        return;
    free(ctx->dashes);
    ctx->dashes      = NULL;
    ctx->dash_count  = n;
    ctx->dash_offset = offset;
    if (n == 0)
        return;
    ctx->dashes = (float *)malloc(sizeof(float) * n);
    if (!ctx->dashes) {
        ctx->status = VKO_STATUS_NO_MEMORY;
        return;
    }
    memcpy(ctx->dashes, dashes, sizeof(float) * n);
}
/* _set_mat_inv_and_vkCmdPush, src/vkvg_context_internal.c:672-676: the
   pushed inverse follows every matrix change (a failed inversion keeps
   vkvg_matrix_invert's partial result) */
static void mat_changed(vko_context *ctx) {
    ctx->mat_inv = ctx->mat;
    vko_matrix_invert(&ctx->mat_inv);
}
void vko_set_matrix(vko_context *ctx, const vko_matrix *m) {
    if (vko_status(ctx) || !m)
        return;
    ctx->mat = *m;
    mat_changed(ctx);
}
void vko_get_matrix(vko_context *ctx, vko_matrix *m) {
    if (vko_status(ctx) || !m)
        return;
    *m = ctx->mat;
}
void vko_identity_matrix(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    vko_matrix_init_identity(&ctx->mat);
    mat_changed(ctx);
}
/* vkvg_translate / scale / rotate / transform, src/vkvg_context.c:1513-1559 */
void vko_transform(vko_context *ctx, const vko_matrix *m) {
    if (vko_status(ctx) || !m)
        return;
    vko_matrix r;
    vko_matrix_multiply(&r, &ctx->mat, m);
    ctx->mat = r;
    mat_changed(ctx);
}
void vko_translate(vko_context *ctx, float dx, float dy) {
    if (vko_status(ctx))
        return;
    vko_matrix_translate(&ctx->mat, dx, dy);
    mat_changed(ctx);
}
void vko_scale(vko_context *ctx, float sx, float sy) {
    if (vko_status(ctx))
        return;
    vko_matrix_scale(&ctx->mat, sx, sy);
    mat_changed(ctx);
}
void vko_rotate(vko_context *ctx, float r) {
    if (vko_status(ctx))
        return;
    vko_matrix_rotate(&ctx->mat, r);
    mat_changed(ctx);
}

/* ------------------------------------------------------------- draw access */

uint32_t vko_draw_count(vko_context *ctx) { return ctx ? ctx->ndraws : 0; }
int      vko_draw_info(vko_context *ctx, uint32_t i, uint32_t *info) {
    if (!ctx || i >= ctx->ndraws)
        return -1;
    vko_draw *d = &ctx->draws[i];
    info[0]     = (uint32_t)d->kind;
    info[1]     = d->npts;
    info[2]     = d->nsub;
    info[3]     = d->nverts;
    info[4]     = d->ninds;
    info[5]     = d->color;
    info[6]     = (uint32_t)d->convex;
    return 0;
}
int vko_draw_points(vko_context *ctx, uint32_t i, float *xy, uint32_t *sub_counts) {
    if (!ctx || i >= ctx->ndraws)
        return -1;
    vko_draw *d = &ctx->draws[i];
    if (xy && d->npts)
        memcpy(xy, d->pts, (size_t)d->npts * 2 * sizeof(float));
    if (sub_counts && d->nsub)
        memcpy(sub_counts, d->sub_counts, (size_t)d->nsub * sizeof(uint32_t));
    return 0;
}
int vko_draw_stroke(vko_context *ctx, uint32_t i, float *xy, uint32_t *inds) {
    if (!ctx || i >= ctx->ndraws)
        return -1;
    vko_draw *d = &ctx->draws[i];
    if (xy && d->nverts)
        memcpy(xy, d->verts, (size_t)d->nverts * 2 * sizeof(float));
    if (inds && d->ninds)
        memcpy(inds, d->inds, (size_t)d->ninds * sizeof(uint32_t));
    return 0;
}
int vko_draw_coverage(vko_context *ctx, uint32_t i, int mode, int32_t *out) {
    if (!ctx || i >= ctx->ndraws || !out)
        return -1;
    vko_draw_coverage_impl(ctx->surf, &ctx->draws[i], mode, out);
    return 0;
}
void vko_snap(vko_context *ctx, uint32_t i, float x, float y, int32_t *fx, int32_t *fy) {
    const vko_matrix *m = (ctx && i < ctx->ndraws) ? &ctx->draws[i].mat : &ctx->mat;
    vko_snap_point(m, ctx->surf->width, ctx->surf->height, x, y, fx, fy);
}

/* portable math evaluation: fn 0 atan2f, 1 acosf, 2 cosf, 3 sinf, 4 asinf, 5 atanf */
void vko_pmath_eval(int fn, const float *a, const float *b, float *out, uint64_t n) {
    for (uint64_t i = 0; i < n; i++) {
        switch (fn) {
        case 0:
            out[i] = vko_pm_atan2f(a[i], b[i]);
            break;
        case 1:
            out[i] = vko_pm_acosf(a[i]);
            break;
        case 2:
            out[i] = vko_pm_cosf(a[i]);
            break;
        case 3:
            out[i] = vko_pm_sinf(a[i]);
            break;
        case 4:
            out[i] = vko_pm_asinf(a[i]);
            break;
        default:
            out[i] = vko_pm_atanf(a[i]);
            break;
        }
    }
}

/* ------------------------------------------------- clip and the state stack
   vkvg_reset_clip / vkvg_clip / vkvg_clip_preserve / vkvg_save / vkvg_restore,
   src/vkvg_context.c:698-733, 950-976, 1251-1512.  Each stencil pass vkvg
   issues becomes one draw of the matching VKO_DRAW_* kind, in vkvg's order. */
static int prev_clip_state(vko_context *ctx) {
    /* _get_previous_clip_state, src/vkvg_context.c:698-702 */
    return ctx->saved ? ctx->saved->clip_state : VKO_CLIP_CLEAR;
}
static void stencil_draw(vko_context *ctx, int kind, int param) {
    vko_draw *d = vko_new_draw(ctx, kind);
    if (d)
        d->param = param;
}
void vko_reset_clip(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    if (ctx->clip_state == VKO_CLIP_CLEAR)
        return;
    ctx->clip_state = prev_clip_state(ctx) == VKO_CLIP_CLEAR ? VKO_CLIP_NONE : VKO_CLIP_CLEAR;
    stencil_draw(ctx, VKO_DRAW_RESET, 0);
}
void vko_clip_preserve(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    if (vko_clip_preserve_geom(ctx))
        ctx->clip_state = VKO_CLIP_CLIP;
}
void vko_clip(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    if (vko_clip_preserve_geom(ctx))
        ctx->clip_state = VKO_CLIP_CLIP;
    vko_clear_path(ctx);
}
void vko_save(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    vko_saved *sv = (vko_saved *)calloc(1, sizeof(vko_saved));
    if (!sv) {
        ctx->status = VKO_STATUS_NO_MEMORY;
        return;
    }
    if (ctx->clip_state == VKO_CLIP_CLIP) {
        sv->clip_state = VKO_CLIP_SAVED;
        if (ctx->sav_bit > 0 && ctx->sav_bit % 6 == 0) /* a new stencil image */
            stencil_draw(ctx, VKO_DRAW_STORE, ctx->sav_bit / 6 - 1);
        stencil_draw(ctx, VKO_DRAW_SAVE_BIT, ctx->sav_bit % 6 + 2);
        ctx->sav_bit++;
    } else if (ctx->clip_state == VKO_CLIP_NONE) {
        sv->clip_state = prev_clip_state(ctx) & 0x03;
    } else {
        sv->clip_state = VKO_CLIP_CLEAR;
    }
    sv->dash_offset = ctx->dash_offset;
    sv->dash_count  = ctx->dash_count;
    if (ctx->dash_count > 0) {
        sv->dashes = (float *)malloc(sizeof(float) * ctx->dash_count);
        memcpy(sv->dashes, ctx->dashes, sizeof(float) * ctx->dash_count);
    }
    sv->line_width  = ctx->line_width;
    sv->miter_limit = ctx->miter_limit;
    sv->op          = ctx->op;
    sv->line_cap    = ctx->line_cap;
    sv->fill_rule   = ctx->fill_rule;
    /* lineJoint of vkvg_context_save_t is never written: calloc's 0 */
    sv->mat     = ctx->mat; /* pushConsts */
    sv->mat_inv = ctx->mat_inv;
    sv->src_x   = ctx->src_x;
    sv->src_y   = ctx->src_y;
    sv->opacity = ctx->opacity;
    if (ctx->pattern) {
        sv->pattern = ctx->pattern;
        vko_pattern_reference(ctx->pattern);
    } else {
        sv->cur_color = ctx->cur_color;
    }
    sv->next   = ctx->saved;
    ctx->saved = sv;
}
void vko_restore(vko_context *ctx) {
    if (vko_status(ctx))
        return;
    if (!ctx->saved) {
        ctx->status = VKO_STATUS_INVALID_RESTORE;
        return;
    }
    vko_saved *sv = ctx->saved;
    ctx->saved    = sv->next;
    if (ctx->clip_state) {
        if (ctx->clip_state == VKO_CLIP_CLIP && sv->clip_state == VKO_CLIP_CLEAR)
            stencil_draw(ctx, VKO_DRAW_RESET, 0);
        else /* int arithmetic as in C: with sav_bit 0 this names the clip bit */
            stencil_draw(ctx, VKO_DRAW_RESTORE_BIT, ((int)ctx->sav_bit - 1) % 6 + 2);
    }
    if (sv->clip_state == VKO_CLIP_SAVED) {
        ctx->sav_bit--;
        if (ctx->sav_bit > 0 && ctx->sav_bit % 6 == 0)
            stencil_draw(ctx, VKO_DRAW_LOAD, ctx->sav_bit / 6 - 1);
    }
    ctx->clip_state  = VKO_CLIP_NONE;
    ctx->dash_offset = sv->dash_offset;
    free(ctx->dashes);
    ctx->dashes     = NULL;
    ctx->dash_count = sv->dash_count;
    if (sv->dash_count > 0) {
        ctx->dashes = (float *)malloc(sizeof(float) * sv->dash_count);
        memcpy(ctx->dashes, sv->dashes, sizeof(float) * sv->dash_count);
    }
    ctx->line_width  = sv->line_width;
    ctx->miter_limit = sv->miter_limit;
    ctx->op          = sv->op;
    ctx->line_cap    = sv->line_cap;
    ctx->line_join   = sv->line_join;
    ctx->fill_rule   = sv->fill_rule;
    ctx->mat         = sv->mat;
    ctx->mat_inv     = sv->mat_inv;
    ctx->src_x       = sv->src_x;
    ctx->src_y       = sv->src_y;
    ctx->opacity     = sv->opacity;
    if (sv->pattern) {
        if (sv->pattern != ctx->pattern) {
            /* _update_cur_pattern: the gradient again with the restored CTM;
               the saved reference passes to the context */
            vko_pattern *last = ctx->pattern;
            ctx->pattern      = sv->pattern;
            ctx->grad_on      = 0;
            snap_gradient(ctx, sv->pattern);
            if (last)
                vko_pattern_destroy(last);
        } else {
            vko_pattern_destroy(sv->pattern);
        }
    } else {
        ctx->cur_color = sv->cur_color;
        set_solid(ctx);
    }
    free(sv->dashes);
    free(sv);
}

float vko_get_line_width(vko_context *ctx) { return ctx ? ctx->line_width : 0.f; }
int   vko_get_line_join(vko_context *ctx) { return ctx ? ctx->line_join : 0; }
int   vko_get_line_cap(vko_context *ctx) { return ctx ? ctx->line_cap : 0; }
int   vko_get_fill_rule(vko_context *ctx) { return ctx ? ctx->fill_rule : 0; }
int   vko_get_operator(vko_context *ctx) { return ctx ? ctx->op : 0; }
