/*
 * vko_raster.c - software restatement of the fixed-function state vkvg
 * programs into Vulkan (TEST INFRASTRUCTURE ONLY).
 *
 * Pipeline state restated (src/vkvg_device_internal.c of vkvg):
 *  - vertex stage shaders/vkvg_main.vert:59-81: p' = CTM.p, ndc = p'*2/size-1,
 *    then the viewport transform xf = ndc*(W/2) + W/2;
 *  - rasterisation: vertices snapped to 8 sub-pixel bits (round to nearest
 *    even), standard 4x sample positions (0.375,0.125) (0.875,0.375)
 *    (0.125,0.625) (0.625,0.875) or the pixel centre for 1 sample, top-left
 *    fill rule with y pointing down.  A sample on an edge is covered exactly
 *    when the point moved by (+e, +e^2), e infinitesimal, is inside;
 *  - even-odd fill, :226-232 and :1583-1655: triangle fans from each
 *    subpath's first point INVERT the stencil FILL bit, then a full-screen
 *    triangle limited to the path's scissor blends where FILL is set and
 *    zeroes it (:240-246, _draw_full_screen_quad :1919-1952);
 *  - non-zero fill: vkvg tessellates with glutess (absent from vkvg's tree);
 *    coverage is defined as winding != 0 of the flattened polygon, blended
 *    once;
 *  - strokes and the other pipe_OVER draws: every covering triangle blends
 *    once (stencil test on the CLIP bit only, :240-246);
 *  - clip (src/vkvg_context.c:754-795): the path sets the FILL bit of the
 *    samples it covers that pass the clip test (even-odd: the polyFill fan,
 *    INVERT; non-zero: pipelineClipping, REPLACE), then a full-screen pass of
 *    pipelineClipping (:233-239) sets the CLIP bit where FILL is clear and
 *    zeroes both bits where it is set; vkvg_save / vkvg_restore copy the CLIP
 *    bit to and from save bits 2..7 with the same pipeline and copy the whole
 *    stencil to and from images for deeper levels (src/vkvg_context.c:1251-1512);
 *    stencil clears (vkvg_clear, vkvg_reset_clip) zero every bit;
 *  - blend ONE, ONE_MINUS_SRC_ALPHA on premultiplied UNORM8 (:200-209):
 *    d' = s + round(d*(255-sa)/255) (no ties exist), clamped to 255;
 *    VKVG_OPERATOR_CLEAR writes 0, VKVG_OPERATOR_DIFFERENCE subtracts;
 *  - resolve: per channel (sum of samples + S/2) / S.
 *
 * Two raster modes compute the same per-sample integers:
 *   literal  (1): fan triangles with the stencil / signed-fan winding, and
 *                 one covering test per stroke triangle;
 *   scanline (0): signed crossings of every sample row with the polygon (or
 *                 positively oriented triangle) edges, suffix-summed.
 * The tests check that both modes agree; scanline is the fast one.
 */
#include "vko_internal.h"

#include <pthread.h>
#include <stdio.h>

int        vko_math_mode_g   = 0;
static int vko_raster_mode_g = 0;
static int vko_threads_g     = 1;

void vko_set_math_mode(int mode) { vko_math_mode_g = mode ? 1 : 0; }
int  vko_get_math_mode(void) { return vko_math_mode_g; }
void vko_set_raster_mode(int mode) { vko_raster_mode_g = mode ? 1 : 0; }
void vko_set_threads(int n) { vko_threads_g = n < 1 ? 1 : (n > 256 ? 256 : n); }

/* sample positions in 1/256 px */
static void sample_pos(uint32_t samples, uint32_t s, int32_t *ox, int32_t *oy) {
    static const int32_t p4[4][2] = {{96, 32}, {224, 96}, {32, 160}, {160, 224}};
    if (samples == 4) {
        *ox = p4[s][0];
        *oy = p4[s][1];
    } else {
        *ox = 128;
        *oy = 128;
    }
}

static int32_t to_fixed(float v) {
    float s = v * 256.0f;
    if (s != s)
        return 0;
    if (!(s > -VKO_FIX_LIMIT))
        s = -VKO_FIX_LIMIT;
    if (!(s < VKO_FIX_LIMIT))
        s = VKO_FIX_LIMIT;
    return (int32_t)lrintf(s);
}
/* vertex stage + viewport + snap */
void vko_snap_point(const vko_matrix *m, uint32_t w, uint32_t h, float x, float y, int32_t *fx, int32_t *fy) {
    float px = (m->xx * x + m->xy * y) + m->x0;
    float py = (m->yx * x + m->yy * y) + m->y0;
    float nx = (px * 2.0f) / (float)w - 1.0f;
    float ny = (py * 2.0f) / (float)h - 1.0f;
    float hw = (float)w * 0.5f, hh = (float)h * 0.5f;
    *fx      = to_fixed(nx * hw + hw);
    *fy      = to_fixed(ny * hh + hh);
}
static int device_point_finite(const vko_matrix *m, float x, float y) {
    float px = (m->xx * x + m->xy * y) + m->x0;
    float py = (m->yx * x + m->yy * y) + m->y0;
    return !(px != px || py != py);
}

/* ------------------------------------------------------------ literal mode */

/* edge test with the (+e,+e^2) tie rule, for a positively oriented triangle */
static inline int edge_in(int64_t ax, int64_t ay, int64_t bx, int64_t by, int64_t sx, int64_t sy) {
    int64_t e = (bx - ax) * (sy - ay) - (by - ay) * (sx - ax);
    if (e > 0)
        return 1;
    if (e < 0)
        return 0;
    if (by != ay)
        return by < ay;
    return bx > ax;
}
typedef void (*tri_cb)(void *u, uint32_t px, uint32_t py, uint32_t s);
/* visit samples covered by triangle; returns orientation sign (0 if degenerate) */
static int raster_tri(uint32_t w, uint32_t h, uint32_t samples, const int32_t v[6], tri_cb cb, void *u) {
    int64_t x0 = v[0], y0 = v[1], x1 = v[2], y1 = v[3], x2 = v[4], y2 = v[5];
    int64_t a  = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0);
    if (a == 0)
        return 0;
    int sign = 1;
    if (a < 0) {
        int64_t tx = x1, ty = y1;
        x1 = x2;
        y1 = y2;
        x2 = tx;
        y2 = ty;
        sign = -1;
    }
    int64_t minx = x0 < x1 ? (x0 < x2 ? x0 : x2) : (x1 < x2 ? x1 : x2);
    int64_t maxx = x0 > x1 ? (x0 > x2 ? x0 : x2) : (x1 > x2 ? x1 : x2);
    int64_t miny = y0 < y1 ? (y0 < y2 ? y0 : y2) : (y1 < y2 ? y1 : y2);
    int64_t maxy = y0 > y1 ? (y0 > y2 ? y0 : y2) : (y1 > y2 ? y1 : y2);
    int64_t pxa  = minx >> 8, pxb = maxx >> 8, pya = miny >> 8, pyb = maxy >> 8;
    if (pxa < 0)
        pxa = 0;
    if (pya < 0)
        pya = 0;
    if (pxb >= (int64_t)w)
        pxb = (int64_t)w - 1;
    if (pyb >= (int64_t)h)
        pyb = (int64_t)h - 1;
    for (int64_t py = pya; py <= pyb; py++)
        for (int64_t px = pxa; px <= pxb; px++)
            for (uint32_t s = 0; s < samples; s++) {
                int32_t ox, oy;
                sample_pos(samples, s, &ox, &oy);
                int64_t sx = px * 256 + ox, sy = py * 256 + oy;
                if (edge_in(x0, y0, x1, y1, sx, sy) && edge_in(x1, y1, x2, y2, sx, sy) &&
                    edge_in(x2, y2, x0, y0, sx, sy))
                    cb(u, (uint32_t)px, (uint32_t)py, s);
            }
    return sign;
}
typedef struct {
    uint32_t w, samples;
    int32_t *acc;
    int      add;
    uint8_t *stencil;
} cov_u;
static void cb_add(void *u, uint32_t px, uint32_t py, uint32_t s) {
    cov_u *c = (cov_u *)u;
    c->acc[((size_t)py * c->w + px) * c->samples + s] += c->add;
}
/* one stencil test and update as Vulkan defines them for VK_COMPARE_OP_EQUAL:
   the test passes when (ref & compare mask) == (stencil & compare mask); the
   pass or fail op's value is written through the write mask */
enum { SOP_KEEP, SOP_ZERO, SOP_REPLACE, SOP_INVERT };
static inline uint8_t stencil_apply(uint8_t st, uint8_t ref, uint8_t cmask, uint8_t wmask, int pass_op, int fail_op) {
    int     op = ((ref & cmask) == (st & cmask)) ? pass_op : fail_op;
    uint8_t v  = op == SOP_KEEP ? st : op == SOP_ZERO ? 0 : op == SOP_REPLACE ? ref : (uint8_t)~st;
    return (uint8_t)((st & ~wmask) | (v & wmask));
}
/* pipe_OVER's test with compare mask CLIP and reference 1 (:240-246) */
static inline int visible(uint8_t st) { return (st & VKO_STENCIL_CLIP) == (1u & VKO_STENCIL_CLIP); }
/* polyFill: EQUAL on CLIP with reference 0, INVERT through the FILL mask (:226-232) */
static void cb_invert(void *u, uint32_t px, uint32_t py, uint32_t s) {
    cov_u   *c = (cov_u *)u;
    uint8_t *p = &c->stencil[((size_t)py * c->w + px) * c->samples + s];
    *p         = stencil_apply(*p, 0, VKO_STENCIL_CLIP, VKO_STENCIL_FILL, SOP_INVERT, SOP_KEEP);
}

/* ----------------------------------------------------------- scanline mode */

static inline int64_t floordiv(int64_t a, int64_t b) { /* b > 0 */
    int64_t q = a / b;
    if ((a % b != 0) && (a < 0))
        q--;
    return q;
}
static inline int64_t ceildiv(int64_t a, int64_t b) { /* b > 0 */
    return -floordiv(-a, b);
}
/* accumulate one directed edge into per-row counters; cnt has (w+1) entries
   per sample row; samples to the left of the crossing get the edge's sign */
static void edge_rows(uint32_t w, uint32_t h, uint32_t samples, int64_t x0, int64_t y0, int64_t x1, int64_t y1,
                      int32_t *cnt, int32_t row_lo, int32_t row_hi) {
    if (y0 == y1)
        return;
    int dir = y0 < y1 ? 1 : -1;
    int64_t ylo = y0 < y1 ? y0 : y1, yhi = y0 < y1 ? y1 : y0;
    uint32_t rows_per_px = samples == 4 ? 4 : 1;
    int32_t  nrows       = (int32_t)(h * rows_per_px);
    /* sample rows: row r at y = (r / rpp)*256 + off[r % rpp] */
    int32_t  r0, r1;
    if (samples == 4) {
        /* rows at 32 + 64 k */
        r0 = (int32_t)ceildiv(ylo - 32, 64);
        r1 = (int32_t)ceildiv(yhi - 32, 64) - 1; /* sy < yhi */
    } else {
        r0 = (int32_t)ceildiv(ylo - 128, 256);
        r1 = (int32_t)ceildiv(yhi - 128, 256) - 1;
    }
    if (r0 < row_lo)
        r0 = row_lo;
    if (r1 >= row_hi)
        r1 = row_hi - 1;
    if (r1 >= nrows)
        r1 = nrows - 1;
    int64_t dx = x1 - x0, dy = y1 - y0;
    for (int32_t r = r0; r <= r1; r++) {
        int64_t sy, ox;
        if (samples == 4) {
            static const int32_t offx[4] = {96, 224, 32, 160};
            sy = 32 + 64 * (int64_t)r;
            ox = offx[r & 3];
        } else {
            sy = 128 + 256 * (int64_t)r;
            ox = 128;
        }
        /* samples with sx < x0 + dx*(sy-y0)/dy */
        int64_t num = dx * (sy - y0), den = dy;
        if (den < 0) {
            num = -num;
            den = -den;
        }
        int64_t M = x0 + ceildiv(num, den) - 1; /* largest sx covered */
        int64_t k = floordiv(M - ox, 256) + 1;
        if (k < 0)
            k = 0;
        if (k > (int64_t)w)
            k = w;
        cnt[(size_t)(r - row_lo) * (w + 1) + k] += dir;
    }
}

typedef struct {
    int32_t x0, y0, x1, y1;
} edge_t;

/* build the snapped edge list of a draw (fills: polygon edges incl. closing
   edges of subpaths with > 2 points; strokes: edges of positively oriented
   triangles) */
static edge_t *draw_edges(const vko_surface *surf, const vko_draw *d, uint64_t *n_out) {
    uint32_t w = surf->width, h = surf->height;
    uint64_t n = 0, cap = 0;
    edge_t  *e = NULL;
#define PUSH(a, b, c, dd)                                                                                              \
    do {                                                                                                               \
        if (n == cap) {                                                                                                \
            cap = cap * 2 + 1024;                                                                                      \
            e   = (edge_t *)realloc(e, cap * sizeof(edge_t));                                                          \
        }                                                                                                              \
        e[n++] = (edge_t){a, b, c, dd};                                                                                \
    } while (0)
    if (VKO_FILL_GEOM(d->kind)) {
        uint32_t first = 0;
        for (uint32_t s = 0; s < d->nsub; s++) {
            uint32_t cnt = d->sub_counts[s];
            if (cnt > 2) {
                int32_t fx0, fy0, px, py;
                vko_snap_point(&d->mat, w, h, d->pts[2 * first], d->pts[2 * first + 1], &fx0, &fy0);
                px = fx0;
                py = fy0;
                for (uint32_t i = 1; i < cnt; i++) {
                    int32_t qx, qy;
                    vko_snap_point(&d->mat, w, h, d->pts[2 * (first + i)], d->pts[2 * (first + i) + 1], &qx, &qy);
                    PUSH(px, py, qx, qy);
                    px = qx;
                    py = qy;
                }
                PUSH(px, py, fx0, fy0);
            }
            first += cnt;
        }
    } else if (d->kind == VKO_DRAW_STROKE) {
        for (uint32_t t = 0; t + 2 < d->ninds + 0u && t + 2 < d->ninds; t += 3) {
            int32_t v[6];
            int     ok = 1;
            for (int k = 0; k < 3; k++) {
                uint32_t vi = d->inds[t + k];
                if (vi >= d->nverts) {
                    ok = 0;
                    break;
                }
                if (!device_point_finite(&d->mat, d->verts[2 * vi], d->verts[2 * vi + 1])) {
                    ok = 0;
                    break;
                }
                vko_snap_point(&d->mat, w, h, d->verts[2 * vi], d->verts[2 * vi + 1], &v[2 * k], &v[2 * k + 1]);
            }
            if (!ok)
                continue;
            int64_t a = ((int64_t)v[2] - v[0]) * ((int64_t)v[5] - v[1]) - ((int64_t)v[4] - v[0]) * ((int64_t)v[3] - v[1]);
            if (a == 0)
                continue;
            if (a > 0) {
                PUSH(v[0], v[1], v[2], v[3]);
                PUSH(v[2], v[3], v[4], v[5]);
                PUSH(v[4], v[5], v[0], v[1]);
            } else {
                PUSH(v[0], v[1], v[4], v[5]);
                PUSH(v[4], v[5], v[2], v[3]);
                PUSH(v[2], v[3], v[0], v[1]);
            }
        }
    }
#undef PUSH
    *n_out = n;
    return e;
}

/* per-sample integer (winding or triangle count) for rows [row_lo,row_hi) */
static void coverage_rows_scan(uint32_t w, uint32_t h, uint32_t samples, const edge_t *e, uint64_t n, int32_t row_lo,
                               int32_t row_hi, int32_t *cnt /* (row_hi-row_lo)*(w+1) */, int32_t *out) {
    size_t rows = (size_t)(row_hi - row_lo);
    memset(cnt, 0, rows * (w + 1) * sizeof(int32_t));
    for (uint64_t i = 0; i < n; i++)
        edge_rows(w, h, samples, e[i].x0, e[i].y0, e[i].x1, e[i].y1, cnt, row_lo, row_hi);
    uint32_t rpp = samples == 4 ? 4 : 1;
    for (size_t r = 0; r < rows; r++) {
        int32_t *c   = cnt + r * (w + 1);
        int32_t  acc = c[w];
        uint32_t gr  = (uint32_t)(row_lo + (int32_t)r);
        uint32_t py = gr / rpp, s = gr % rpp;
        for (int32_t px = (int32_t)w - 1; px >= 0; px--) {
            out[((size_t)py * w + (uint32_t)px) * samples + s] = acc;
            acc += c[px];
        }
    }
}

void vko_coverage_edges(uint32_t w, uint32_t h, uint32_t samples, const int32_t *edges, uint64_t nedges,
                        int32_t *out) {
    uint32_t rpp   = samples == 4 ? 4 : 1;
    int32_t  nrows = (int32_t)(h * rpp);
    int32_t *cnt   = (int32_t *)malloc((size_t)nrows * (w + 1) * sizeof(int32_t));
    coverage_rows_scan(w, h, samples, (const edge_t *)edges, nedges, 0, nrows, cnt, out);
    free(cnt);
}

/* full per-sample coverage of a draw in the given mode */
void vko_draw_coverage_impl(const vko_surface *surf, const vko_draw *d, int mode, int32_t *out) {
    uint32_t w = surf->width, h = surf->height, S = surf->samples;
    size_t   ns = (size_t)w * h * S;
    memset(out, 0, ns * sizeof(int32_t));
    if (d->kind == VKO_DRAW_PAINT) {
        for (size_t i = 0; i < ns; i++)
            out[i] = 1;
        return;
    }
    if (d->kind == VKO_DRAW_CLEAR)
        return;
    if (mode == 0) {
        uint64_t n;
        edge_t  *e = draw_edges(surf, d, &n);
        vko_coverage_edges(w, h, S, (const int32_t *)e, n, out);
        free(e);
        return;
    }
    cov_u u = {w, S, out, 1, NULL};
    if (VKO_FILL_GEOM(d->kind)) {
        /* signed fan coverage: sum of orientation signs of the covering fan
           triangles = winding number */
        uint32_t first = 0;
        for (uint32_t s = 0; s < d->nsub; s++) {
            uint32_t cnt = d->sub_counts[s];
            if (cnt > 2) {
                int32_t v[6];
                vko_snap_point(&d->mat, w, h, d->pts[2 * first], d->pts[2 * first + 1], &v[0], &v[1]);
                for (uint32_t i = 1; i + 1 < cnt; i++) {
                    vko_snap_point(&d->mat, w, h, d->pts[2 * (first + i)], d->pts[2 * (first + i) + 1], &v[2], &v[3]);
                    vko_snap_point(&d->mat, w, h, d->pts[2 * (first + i + 1)], d->pts[2 * (first + i + 1) + 1], &v[4],
                                   &v[5]);
                    int64_t a = ((int64_t)v[2] - v[0]) * ((int64_t)v[5] - v[1]) -
                                ((int64_t)v[4] - v[0]) * ((int64_t)v[3] - v[1]);
                    if (a == 0)
                        continue;
                    u.add = a > 0 ? 1 : -1;
                    raster_tri(w, h, S, v, cb_add, &u);
                }
            }
            first += cnt;
        }
    } else if (d->kind == VKO_DRAW_STROKE) {
        for (uint32_t t = 0; t + 2 < d->ninds; t += 3) {
            int32_t v[6];
            int     ok = 1;
            for (int k = 0; k < 3; k++) {
                uint32_t vi = d->inds[t + k];
                if (vi >= d->nverts || !device_point_finite(&d->mat, d->verts[2 * vi], d->verts[2 * vi + 1])) {
                    ok = 0;
                    break;
                }
                vko_snap_point(&d->mat, w, h, d->verts[2 * vi], d->verts[2 * vi + 1], &v[2 * k], &v[2 * k + 1]);
            }
            if (!ok)
                continue;
            u.add = 1;
            raster_tri(w, h, S, v, cb_add, &u);
        }
    }
}

/* ------------------------------------------------------------------ blend */

static void src_color(const vko_draw *d, uint8_t s[4]) {
    for (int c = 0; c < 4; c++) {
        uint32_t b = (d->color >> (8 * c)) & 0xFF;
        float    f = ((float)b / 255.0f) * d->opacity;
        float    v = f * 255.0f;
        if (!(v > 0.0f))
            v = 0.0f;
        if (v > 255.0f)
            v = 255.0f;
        s[c] = (uint8_t)lrintf(v);
    }
}
/* Linear gradient source of pixel (px, py), shaders/vkvg_main.frag:83-108:
   positions normalised by the surface size, signed distance along the
   gradient axis in units of its length, stop colours combined by GLSL's mix
   and smoothstep, times opacity, quantised to UNORM8 by round-to-nearest.
   Plain fp32 operations in the shader's order (no contraction). */
static float g_smoothstep(float e0, float e1, float x) {
    float t = (x - e0) / (e1 - e0);
    t       = fminf(fmaxf(t, 0.0f), 1.0f);
    return (t * t) * (3.0f - 2.0f * t);
}
static float g_mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
/* RADIAL, shaders/vkvg_main.frag:109-144: the ray from centre 0 through p
   is cut by circle 1; the gradient parameter is (|p - c0| - r0) over the
   distance of that point from c0 less r0 (1 if the ray misses).
   normalize(v) is v / length(v). */
static float radial_t(const vko_grad *g, float p_x, float p_y) {
    float c0x = g->cp[0] / g->w, c0y = g->cp[1] / g->h;
    float c1x = g->cp[4] / g->w, c1y = g->cp[5] / g->h;
    float r0 = g->cp[2] / g->w, r1 = g->cp[6] / g->w;
    float gradlen = 1.0f;
    float diffx = c0x - c1x, diffy = c0y - c1y;
    float vx = p_x - c0x, vy = p_y - c0y;
    float vlen = sqrtf(vx * vx + vy * vy);
    float rdx = vx / vlen, rdy = vy / vlen;
    float a    = rdx * rdx + rdy * rdy;
    float b    = 2.0f * (rdx * diffx + rdy * diffy);
    float cc   = (diffx * diffx + diffy * diffy) - r1 * r1;
    float disc = b * b - 4.0f * a * cc;
    if (disc >= 0.0f) {
        float t     = (-b + sqrtf(fabsf(disc))) / (2.0f * a);
        float projx = c0x + rdx * t, projy = c0y + rdy * t;
        float qx = projx - c0x, qy = projy - c0y;
        gradlen = sqrtf(qx * qx + qy * qy) - r0;
    }
    return (vlen - r0) / gradlen;
}
/* LINEAR: signed distance along the axis in units of its length */
static float linear_t(const vko_grad *g, float p_x, float p_y) {
    float dist;
    float p0x = g->cp[0] / g->w, p0y = g->cp[1] / g->h;
    float p1x = g->cp[2] / g->w, p1y = g->cp[3] / g->h;
    float dx = p1x - p0x, dy = p1y - p0y;
    float l  = sqrtf(dx * dx + dy * dy);
    float ux = dx / l, uy = dy / l;
    if (uy == 0.0f) {
        float t = (p_x - p0x) / l;
        dist    = ux < 0.0f ? -t : t;
    } else {
        float m  = -ux / uy;
        float bb = p0y - m * p0x;
        dist     = ((p_y - m * p_x - bb) / sqrtf(1.0f + m * m)) / l;
        if (uy < 0.0f)
            dist = -dist;
    }
    return dist;
}
/* SURFACE, shaders/vkvg_main.frag:72-82, sampled as the Vulkan spec's texel
   filtering defines it for the sampler of src/vkvg_context_internal.c:730-755
   (nearest, or linear with weights quantised to 8 fractional bits; address
   modes by vkvg_extend_t; border transparent black: vkh, which sets the
   border colour, is not in vkvg's tree) */
static int32_t tex_floor(float x) {
    float f = floorf(x);
    if (f != f)
        return 0;
    if (f < -1073741824.0f)
        f = -1073741824.0f;
    if (f > 1073741824.0f)
        f = 1073741824.0f;
    return (int32_t)f;
}
static int32_t tex_wrap(int32_t i, int32_t n, int extend) {
    if (extend == 1) { /* REPEAT */
        int32_t r = i % n;
        return r < 0 ? r + n : r;
    }
    if (extend == 2) { /* REFLECT: mirrored repeat */
        int32_t r = i % (2 * n);
        if (r < 0)
            r += 2 * n;
        r -= n;
        return (n - 1) - (r >= 0 ? r : -(1 + r));
    }
    if (extend == 3) /* PAD: clamp to edge */
        return i < 0 ? 0 : (i >= n ? n - 1 : i);
    return (i < 0 || i >= n) ? -1 : i; /* NONE: clamp to border */
}
static void tex_fetch(const vko_grad *g, int32_t i, int32_t j, float t[4]) {
    int32_t sw = (int32_t)g->src->width, sh = (int32_t)g->src->height;
    i = tex_wrap(i, sw, g->extend);
    j = tex_wrap(j, sh, g->extend);
    for (int k = 0; k < 4; k++)
        t[k] = (i < 0 || j < 0) ? 0.0f : (float)g->texels[((size_t)j * sw + i) * 4 + k] / 255.0f;
}
static void surface_src(const vko_grad *g, uint32_t px, uint32_t py, uint8_t s[4]) {
    float sw = (float)g->src->width, sh = (float)g->src->height;
    float qx = ((float)px + 0.5f) - g->ox, qy = ((float)py + 0.5f) - g->oy;
    float u  = (g->m.xx * qx + g->m.xy * qy + g->m.x0) / sw;
    float v  = (g->m.yx * qx + g->m.yy * qy + g->m.y0) / sh;
    float us = u * sw, vs = v * sh;
    float c[4];
    if (!g->bilinear) {
        tex_fetch(g, tex_floor(us), tex_floor(vs), c);
    } else {
        float   a = us - 0.5f, b = vs - 0.5f;
        float   al = floorf((a - floorf(a)) * 256.0f) * (1.0f / 256.0f);
        float   be = floorf((b - floorf(b)) * 256.0f) * (1.0f / 256.0f);
        int32_t i = tex_floor(a), j = tex_floor(b);
        float   t00[4], t10[4], t01[4], t11[4];
        tex_fetch(g, i, j, t00);
        tex_fetch(g, i + 1, j, t10);
        tex_fetch(g, i, j + 1, t01);
        tex_fetch(g, i + 1, j + 1, t11);
        float w00 = (1.0f - al) * (1.0f - be), w10 = al * (1.0f - be), w01 = (1.0f - al) * be, w11 = al * be;
        for (int k = 0; k < 4; k++)
            c[k] = w00 * t00[k] + w10 * t10[k] + w01 * t01[k] + w11 * t11[k];
    }
    for (int k = 0; k < 4; k++) {
        float x = (c[k] * g->opacity) * 255.0f;
        x       = x > 0.0f ? fminf(x, 255.0f) : 0.0f;
        s[k]    = (uint8_t)lrintf(x);
    }
}
static void grad_src(const vko_grad *g, uint32_t px, uint32_t py, uint8_t s[4]) {
    if (g->type == 1) {
        surface_src(g, px, py, s);
        return;
    }
    float p_x  = ((float)px + 0.5f) / g->w, p_y = ((float)py + 0.5f) / g->h;
    float dist = g->type == 3 ? radial_t(g, p_x, p_y) : linear_t(g, p_x, p_y);
    float c[4];
    float t0 = g_smoothstep(g->stops[0], g->stops[1], dist);
    for (int k = 0; k < 4; k++)
        c[k] = g_mix(g->colors[k], g->colors[4 + k], t0);
    for (uint32_t i = 1; i + 1 < g->count; i++) {
        float t = g_smoothstep(g->stops[i], g->stops[i + 1], dist);
        for (int k = 0; k < 4; k++)
            c[k] = g_mix(c[k], g->colors[4 * (i + 1) + k], t);
    }
    for (int k = 0; k < 4; k++) {
        float v = (c[k] * g->opacity) * 255.0f;
        v       = v > 0.0f ? fminf(v, 255.0f) : 0.0f;
        s[k]    = (uint8_t)lrintf(v);
    }
}
/* the source of a draw at pixel (px, py): its solid colour or its gradient */
static inline void draw_src(const vko_draw *d, const uint8_t solid[4], uint32_t px, uint32_t py, uint8_t s[4]) {
    if (d->grad) {
        grad_src(&d->g, px, py, s);
    } else {
        s[0] = solid[0];
        s[1] = solid[1];
        s[2] = solid[2];
        s[3] = solid[3];
    }
}
static inline void blend(uint8_t *dst, const uint8_t s[4], int op) {
    if (op == VKO_OP_CLEAR) {
        dst[0] = dst[1] = dst[2] = dst[3] = 0;
        return;
    }
    uint32_t inv = 255u - s[3];
    for (int c = 0; c < 4; c++) {
        uint32_t t = ((uint32_t)dst[c] * inv + 127u) / 255u;
        if (op == VKO_OP_DIFFERENCE) {
            int32_t v = (int32_t)s[c] - (int32_t)t;
            dst[c]    = (uint8_t)(v < 0 ? 0 : v);
        } else {
            uint32_t v = s[c] + t;
            dst[c]     = (uint8_t)(v > 255u ? 255u : v);
        }
    }
}

typedef struct {
    const vko_surface *surf;
    const vko_draw    *d;
    const edge_t      *e;
    uint64_t           n;
    int32_t            row_lo, row_hi;
    uint8_t            src[4];
} job_t;
static void apply_rows(const job_t *j) {
    const vko_surface *surf = j->surf;
    uint32_t           w = surf->width, S = surf->samples, rpp = S == 4 ? 4 : 1;
    size_t             rows = (size_t)(j->row_hi - j->row_lo);
    int32_t           *cnt  = (int32_t *)malloc(rows * (w + 1) * sizeof(int32_t));
    memset(cnt, 0, rows * (w + 1) * sizeof(int32_t));
    for (uint64_t i = 0; i < j->n; i++)
        edge_rows(w, surf->height, S, j->e[i].x0, j->e[i].y0, j->e[i].x1, j->e[i].y1, cnt, j->row_lo, j->row_hi);
    int kind = j->d->kind, op = j->d->op;
    for (size_t r = 0; r < rows; r++) {
        int32_t *c   = cnt + r * (w + 1);
        int32_t  acc = c[w];
        uint32_t gr  = (uint32_t)(j->row_lo + (int32_t)r);
        uint32_t py = gr / rpp, s = gr % rpp;
        for (int32_t px = (int32_t)w - 1; px >= 0; px--) {
            int32_t  wv  = acc;
            size_t   si  = ((size_t)py * w + (uint32_t)px) * S + s;
            uint8_t *dst = surf->data + si * 4;
            int      k   = 0;
            if (kind == VKO_DRAW_FILL_EO)
                k = wv & 1;
            else if (kind == VKO_DRAW_FILL_NZ)
                k = wv != 0;
            else
                k = wv;
            if (k > 0 && visible(surf->stencil[si])) {
                uint8_t sc[4];
                draw_src(j->d, j->src, (uint32_t)px, py, sc);
                for (int t = 0; t < k; t++)
                    blend(dst, sc, op);
            }
            acc += c[px];
        }
    }
    free(cnt);
}
static void *job_thread(void *arg) {
    apply_rows((const job_t *)arg);
    return NULL;
}

/* the fan triangles of an even-odd path through polyFill; returns whether
   any subpath had a triangle */
static int eo_fan_invert(vko_surface *surf, const vko_draw *d) {
    uint32_t w = surf->width, h = surf->height, S = surf->samples;
    cov_u    u     = {w, S, NULL, 0, surf->stencil};
    uint32_t first = 0;
    int      any   = 0;
    for (uint32_t s = 0; s < d->nsub; s++) {
        uint32_t cnt = d->sub_counts[s];
        if (cnt > 2) {
            any = 1;
            int32_t v[6];
            vko_snap_point(&d->mat, w, h, d->pts[2 * first], d->pts[2 * first + 1], &v[0], &v[1]);
            for (uint32_t i = 1; i + 1 < cnt; i++) {
                vko_snap_point(&d->mat, w, h, d->pts[2 * (first + i)], d->pts[2 * (first + i) + 1], &v[2], &v[3]);
                vko_snap_point(&d->mat, w, h, d->pts[2 * (first + i + 1)], d->pts[2 * (first + i + 1) + 1], &v[4],
                               &v[5]);
                raster_tri(w, h, S, v, cb_invert, &u);
            }
        }
        first += cnt;
    }
    return any;
}
/* clip draws and the stencil passes of reset / save / restore */
static void stencil_draw(vko_surface *surf, const vko_draw *d) {
    size_t   ns = (size_t)surf->width * surf->height * surf->samples;
    uint8_t *st = surf->stencil;
    switch (d->kind) {
    case VKO_DRAW_CLIP_EO:
    case VKO_DRAW_CLIP_NZ:
        if (vko_raster_mode_g == 1 && d->kind == VKO_DRAW_CLIP_EO) {
            eo_fan_invert(surf, d);
        } else {
            /* non-zero: the covered samples through pipelineClipping with
               reference FILL, compare mask CLIP, write mask FILL; the
               scanline mode sets even-odd's FILL the same way from parity */
            int32_t *cov = (int32_t *)malloc(ns * sizeof(int32_t));
            vko_draw_coverage_impl(surf, d, vko_raster_mode_g == 1 ? 1 : 0, cov);
            for (size_t i = 0; i < ns; i++) {
                int k = d->kind == VKO_DRAW_CLIP_EO ? (cov[i] & 1) : (cov[i] != 0);
                if (k)
                    st[i] = stencil_apply(st[i], VKO_STENCIL_FILL, VKO_STENCIL_CLIP, VKO_STENCIL_FILL, SOP_REPLACE,
                                          SOP_ZERO);
            }
            free(cov);
        }
        /* full-screen pass: reference CLIP, compare mask FILL, write mask ALL */
        for (size_t i = 0; i < ns; i++)
            st[i] = stencil_apply(st[i], VKO_STENCIL_CLIP, VKO_STENCIL_FILL, VKO_STENCIL_ALL, SOP_REPLACE, SOP_ZERO);
        break;
    case VKO_DRAW_RESET: memset(st, 0, ns); break;
    case VKO_DRAW_SAVE_BIT: {
        uint8_t bit = (uint8_t)(1u << d->param);
        for (size_t i = 0; i < ns; i++)
            st[i] = stencil_apply(st[i], VKO_STENCIL_CLIP | bit, VKO_STENCIL_CLIP, bit, SOP_REPLACE, SOP_ZERO);
        break;
    }
    case VKO_DRAW_RESTORE_BIT: {
        uint8_t bit = (uint8_t)(1u << d->param);
        for (size_t i = 0; i < ns; i++)
            st[i] = stencil_apply(st[i], VKO_STENCIL_CLIP | bit, bit, VKO_STENCIL_CLIP, SOP_REPLACE, SOP_ZERO);
        break;
    }
    case VKO_DRAW_STORE: {
        uint32_t k = (uint32_t)d->param;
        if (k >= surf->nimages) {
            uint8_t **t = (uint8_t **)realloc(surf->images, (k + 1) * sizeof(uint8_t *));
            if (!t)
                return;
            for (uint32_t i = surf->nimages; i <= k; i++)
                t[i] = NULL;
            surf->images  = t;
            surf->nimages = k + 1;
        }
        if (!surf->images[k])
            surf->images[k] = (uint8_t *)malloc(ns);
        if (surf->images[k])
            memcpy(surf->images[k], st, ns);
        break;
    }
    case VKO_DRAW_LOAD: {
        uint32_t k = (uint32_t)d->param;
        if (k < surf->nimages && surf->images[k]) {
            memcpy(st, surf->images[k], ns);
            free(surf->images[k]);
            surf->images[k] = NULL;
        }
        break;
    }
    default: break;
    }
}

static void raster_draw(vko_surface *surf, const vko_draw *d);
/* execute one draw against the surface; a surface source is resolved first
   (the image vkvg samples is the source surface's resolved attachment) */
void vko_raster_draw(vko_surface *surf, const vko_draw *d) {
    if (!(d->grad && d->g.type == 1 && d->g.src)) {
        raster_draw(surf, d);
        return;
    }
    const vko_surface *src = d->g.src;
    uint8_t           *tex = (uint8_t *)malloc((size_t)src->width * src->height * 4);
    if (!tex)
        return;
    vko_resolve(src, tex);
    vko_draw dl   = *d;
    dl.g.texels   = tex;
    raster_draw(surf, &dl);
    free(tex);
}
static void raster_draw(vko_surface *surf, const vko_draw *d) {
    uint32_t w = surf->width, h = surf->height, S = surf->samples;
    size_t   ns = (size_t)w * h * S;
    uint8_t  src[4];
    src_color(d, src);
    if (d->kind == VKO_DRAW_CLEAR) {
        memset(surf->data, 0, ns * 4);
        memset(surf->stencil, 0, ns);
        return;
    }
    if (d->kind >= VKO_DRAW_CLIP_EO) {
        stencil_draw(surf, d);
        return;
    }
    if (d->kind == VKO_DRAW_PAINT) {
        for (size_t i = 0; i < ns; i++) {
            if (!visible(surf->stencil[i]))
                continue;
            uint8_t sc[4];
            draw_src(d, src, (uint32_t)((i / S) % w), (uint32_t)(i / S / w), sc);
            blend(surf->data + i * 4, sc, d->op);
        }
        return;
    }
    if (vko_raster_mode_g == 1) {
        /* literal pipeline */
        if (d->kind == VKO_DRAW_FILL_EO) {
            int any = eo_fan_invert(surf, d);
            if (!any)
                return;
            /* cover pass over the scissor of _draw_full_screen_quad */
            const float *b  = d->bounds;
            int64_t      sx = (int64_t)(int32_t)(b[0] > 0 ? b[0] : 0);
            int64_t      sy = (int64_t)(int32_t)(b[1] > 0 ? b[1] : 0);
            float        fw = b[2] - (float)(int32_t)b[0] + 1;
            float        fh = b[3] - (float)(int32_t)b[1] + 1;
            int64_t      ew = (int64_t)(int32_t)(fw > 1 ? fw : 1);
            int64_t      eh = (int64_t)(int32_t)(fh > 1 ? fh : 1);
            for (int64_t py = sy; py < sy + eh && py < (int64_t)h; py++)
                for (int64_t px = sx; px < sx + ew && px < (int64_t)w; px++)
                    for (uint32_t s = 0; s < S; s++) {
                        size_t i = ((size_t)py * w + (size_t)px) * S + s;
                        if (surf->stencil[i] & 1) {
                            uint8_t sc[4];
                            draw_src(d, src, (uint32_t)px, (uint32_t)py, sc);
                            blend(surf->data + i * 4, sc, d->op);
                            surf->stencil[i] &= (uint8_t)~1u;
                        }
                    }
            return;
        }
        int32_t *cov = (int32_t *)malloc(ns * sizeof(int32_t));
        vko_draw_coverage_impl(surf, d, 1, cov);
        for (size_t i = 0; i < ns; i++) {
            int k = d->kind == VKO_DRAW_FILL_NZ ? (cov[i] != 0) : cov[i];
            if (k > 0 && visible(surf->stencil[i])) {
                uint8_t sc[4];
                draw_src(d, src, (uint32_t)((i / S) % w), (uint32_t)(i / S / w), sc);
                for (int t = 0; t < k; t++)
                    blend(surf->data + i * 4, sc, d->op);
            }
        }
        free(cov);
        return;
    }
    /* scanline mode, rows split over worker threads */
    uint64_t n;
    edge_t  *e     = draw_edges(surf, d, &n);
    int32_t  nrows = (int32_t)(h * (S == 4 ? 4 : 1));
    int      nt    = vko_threads_g;
    if (nt > nrows)
        nt = nrows;
    if (nt <= 1) {
        job_t j = {surf, d, e, n, 0, nrows, {src[0], src[1], src[2], src[3]}};
        apply_rows(&j);
    } else {
        job_t     jobs[256];
        pthread_t th[256];
        for (int t = 0; t < nt; t++) {
            jobs[t] = (job_t){surf, d, e, n, (int32_t)((int64_t)nrows * t / nt), (int32_t)((int64_t)nrows * (t + 1) / nt),
                              {src[0], src[1], src[2], src[3]}};
            pthread_create(&th[t], NULL, job_thread, &jobs[t]);
        }
        for (int t = 0; t < nt; t++)
            pthread_join(th[t], NULL);
    }
    free(e);
}

void vko_resolve(const vko_surface *surf, uint8_t *rgba) {
    uint32_t w = surf->width, h = surf->height, S = surf->samples;
    for (size_t p = 0; p < (size_t)w * h; p++)
        for (int c = 0; c < 4; c++) {
            uint32_t sum = 0;
            for (uint32_t s = 0; s < S; s++)
                sum += surf->data[(p * S + s) * 4 + c];
            rgba[p * 4 + c] = (uint8_t)((sum + S / 2) / S);
        }
}
