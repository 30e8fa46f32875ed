/*
 * vko_analytic.c - FP64 CPU reference of the analytic-coverage mode
 * (TEST INFRASTRUCTURE ONLY: tests/, smoke() and bench.py's CPU-baseline leg
 * use it, as the checker or as the timed CPU baseline).
 *
 * The analytic mode has no vkvg counterpart.  The function restated here is
 * the one the GPU library computes (vkvg_gb300/csrc/analytic*.cu):
 *  - geometry: each path is a list of closed contours of line and cubic
 *    segments over one control-point array (a segment starts at its first
 *    control point and ends at the next segment's start, the last one at the
 *    contour's first).  Cubics are flattened by vkvg's _recursive_bezier
 *    (src/vkvg_context_internal.c:1313-1461) at vkvg's default tolerance
 *    (0.25 squared px, src/vkvg_context.c:558): the subdivision decisions are
 *    taken in fp32 exactly as vkvg takes them (vko_bezier_walk), and every
 *    point is evaluated here in double as the blossom of its sub-curve
 *    interval, so it is an exact linear function of the control points.
 *  - layers: a path draws a fill layer, then a stroke layer, both in the
 *    path's premultiplied RGBA colour.
 *  - fill: coverage = min(1, |A|), A = the integral over the pixel of the
 *    winding number of the flattened contours (exact signed area).
 *  - stroke: one rectangle per flattened segment (half-width w/2 on both
 *    sides) and one bevel triangle on the outer side of every joint, all
 *    positively oriented; coverage = min(1, sum of their areas in the pixel).
 *  - compositing: premultiplied source-over onto the background, in order.
 *  - loss: mean over pixels and RGBA channels of (canvas - target)^2.
 * vko_an_backward is the adjoint of that forward derived by hand, in double;
 * vko_an_fd gives central finite differences of the same double forward.
 */
#include "vko.h"
#include "vko_internal.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define AN_TOL 0.25f

/* diagnostics: 1 = evaluate the geometry at vkvg's fp32 points instead of the
   double blossom points (the derivatives keep the blossom weights) */
static int g_points_f32 = 0;
VKO_API void vko_an_set_points_mode(int f32) { g_points_f32 = f32; }

struct vko_an_t {
    uint32_t  W, H, npaths, ncontours, nseg, ncp, nlayers;
    double    bg[4];
    uint32_t *path_c0;      /* npaths+1: first contour of each path */
    uint32_t *path_flags;   /* VKO_AN_FILL | VKO_AN_STROKE */
    uint32_t *cont_s0;      /* ncontours+1: first segment of each contour */
    uint32_t *cont_path;    /* ncontours */
    uint8_t  *seg_kind;     /* VKO_AN_LINE or VKO_AN_CUBIC */
    uint32_t *seg_cp;       /* nseg+1: first control point of each segment */
    uint32_t *seg_end;      /* nseg: the control point the segment ends at */
    uint32_t *layer_path;   /* nlayers */
    uint8_t  *layer_stroke; /* nlayers */
};

/* one flattened point: where it is, and how it was made */
typedef struct {
    double   x, y;   /* double evaluation (the reference) */
    float    fx, fy; /* vkvg's fp32 evaluation */
    int      which;  /* -1: the segment's start point, else VKO_BEZ_* */
    double   ta, tb; /* sub-curve interval of a cubic point */
    uint32_t seg;
} an_pt;

typedef struct {
    an_pt    *p;
    uint32_t  n, cap;
    uint32_t *cont_p0; /* ncontours+1 */
    uint32_t *seg_p0;  /* nseg+1 */
} an_flat;

typedef struct {
    double x, y;
} d2;

static d2     d2v(double x, double y) { return (d2){x, y}; }
static d2     add(d2 a, d2 b) { return d2v(a.x + b.x, a.y + b.y); }
static d2     sub(d2 a, d2 b) { return d2v(a.x - b.x, a.y - b.y); }
static d2     scl(d2 a, double s) { return d2v(a.x * s, a.y * s); }
static double dot(d2 a, d2 b) { return a.x * b.x + a.y * b.y; }
static double crs(d2 a, d2 b) { return a.x * b.y - a.y * b.x; }
static d2     perp(d2 a) { return d2v(-a.y, a.x); } /* R a, R = rotation by +90 degrees */
static d2     perpT(d2 a) { return d2v(a.y, -a.x); } /* R^T a */

/* ------------------------------------------------------------------ scene */

VKO_API vko_an *vko_an_create(uint32_t width, uint32_t height, const float *background, uint32_t npaths,
                              const uint32_t *path_ncontours, const uint32_t *path_flags, uint32_t ncontours,
                              const uint32_t *contour_nseg, uint32_t nseg, const uint8_t *seg_kind) {
    if (!width || !height || !npaths || !path_ncontours || !path_flags || !contour_nseg || !seg_kind)
        return NULL;
    vko_an *a = calloc(1, sizeof *a);
    a->W = width, a->H = height, a->npaths = npaths, a->ncontours = ncontours, a->nseg = nseg;
    for (int c = 0; c < 4; c++)
        a->bg[c] = background ? background[c] : 1.0;
    a->path_c0    = calloc(npaths + 1, 4);
    a->path_flags = calloc(npaths, 4);
    a->cont_s0    = calloc(ncontours + 1, 4);
    a->cont_path  = calloc(ncontours + 1, 4);
    a->seg_kind   = calloc(nseg + 1, 1);
    a->seg_cp     = calloc(nseg + 1, 4);
    a->seg_end    = calloc(nseg + 1, 4);
    a->layer_path   = calloc(2 * npaths, 4);
    a->layer_stroke = calloc(2 * npaths, 1);
    uint32_t c = 0, s = 0, cp = 0;
    for (uint32_t p = 0; p < npaths; p++) {
        a->path_c0[p]    = c;
        a->path_flags[p] = path_flags[p];
        for (uint32_t k = 0; k < path_ncontours[p]; k++, c++) {
            if (c >= ncontours)
                goto bad;
            a->cont_s0[c]   = s;
            a->cont_path[c] = p;
            uint32_t s0 = s, cp0 = cp;
            for (uint32_t q = 0; q < contour_nseg[c]; q++, s++) {
                if (s >= nseg || (seg_kind[s] != VKO_AN_LINE && seg_kind[s] != VKO_AN_CUBIC))
                    goto bad;
                a->seg_kind[s] = seg_kind[s];
                a->seg_cp[s]   = cp;
                cp += seg_kind[s];
            }
            for (uint32_t q = s0; q < s; q++)
                a->seg_end[q] = q + 1 < s ? a->seg_cp[q + 1] : cp0;
        }
        if (path_flags[p] & VKO_AN_FILL)
            a->layer_path[a->nlayers] = p, a->layer_stroke[a->nlayers++] = 0;
        if (path_flags[p] & VKO_AN_STROKE)
            a->layer_path[a->nlayers] = p, a->layer_stroke[a->nlayers++] = 1;
    }
    if (c != ncontours || s != nseg)
        goto bad;
    a->path_c0[npaths] = c;
    a->cont_s0[c]      = s;
    a->seg_cp[s]       = cp;
    a->ncp             = cp;
    return a;
bad:
    vko_an_destroy(a);
    return NULL;
}

VKO_API void vko_an_destroy(vko_an *a) {
    if (!a)
        return;
    free(a->path_c0), free(a->path_flags), free(a->cont_s0), free(a->cont_path), free(a->seg_kind);
    free(a->seg_cp), free(a->seg_end), free(a->layer_path), free(a->layer_stroke);
    free(a);
}

VKO_API uint32_t vko_an_nctrl(const vko_an *a) { return a ? a->ncp : 0; }
VKO_API uint32_t vko_an_nlayers(const vko_an *a) { return a ? a->nlayers : 0; }

/* --------------------------------------------------------------- flatten */

static void blossom(int which, double ta, double tb, double w[4]) {
    double u, v, s;
    if (which == VKO_BEZ_MID)
        u = v = s = 0.5 * (ta + tb);
    else if (which == VKO_BEZ_C2)
        u = ta, v = ta, s = tb;
    else
        u = ta, v = tb, s = tb;
    double iu = 1 - u, iv = 1 - v, is = 1 - s;
    w[0] = iu * iv * is;
    w[1] = u * iv * is + iu * v * is + iu * iv * s;
    w[2] = u * v * is + u * iv * s + iu * v * s;
    w[3] = u * v * s;
}

static void push_pt(an_flat *f, an_pt p) {
    if (f->n == f->cap) {
        f->cap = f->cap ? 2 * f->cap : 1024;
        f->p   = realloc(f->p, f->cap * sizeof *f->p);
    }
    f->p[f->n++] = p;
}

typedef struct {
    an_flat     *f;
    const double *P;
    uint32_t     seg, cp[4];
} emit_u;

static void an_emit(void *u, float x, float y, int which, double ta, double tb) {
    emit_u *e = u;
    if (x != x || y != y) /* _add_point drops NaN points */
        return;
    double w[4];
    blossom(which, ta, tb, w);
    an_pt p = {0};
    p.fx = x, p.fy = y, p.which = which, p.ta = ta, p.tb = tb, p.seg = e->seg;
    for (int k = 0; k < 4; k++) {
        p.x += w[k] * e->P[2 * e->cp[k]];
        p.y += w[k] * e->P[2 * e->cp[k] + 1];
    }
    if (g_points_f32)
        p.x = x, p.y = y;
    push_pt(e->f, p);
}

static void an_flatten(const vko_an *a, const double *ctrl, an_flat *f) {
    f->n = 0;
    if (!f->cont_p0) {
        f->cont_p0 = calloc(a->ncontours + 1, 4);
        f->seg_p0  = calloc(a->nseg + 1, 4);
    }
    for (uint32_t c = 0; c < a->ncontours; c++) {
        f->cont_p0[c] = f->n;
        for (uint32_t s = a->cont_s0[c]; s < a->cont_s0[c + 1]; s++) {
            f->seg_p0[s] = f->n;
            uint32_t c0  = a->seg_cp[s];
            float    fx = (float)ctrl[2 * c0], fy = (float)ctrl[2 * c0 + 1];
            if (!(fx != fx || fy != fy)) {
                an_pt p = {0};
                p.x = ctrl[2 * c0], p.y = ctrl[2 * c0 + 1], p.fx = fx, p.fy = fy, p.which = -1, p.seg = s;
                push_pt(f, p);
            }
            if (a->seg_kind[s] == VKO_AN_CUBIC) {
                emit_u e = {f, ctrl, s, {c0, c0 + 1, c0 + 2, a->seg_end[s]}};
                float  v[8];
                int    fin = 1;
                for (int k = 0; k < 4; k++) {
                    v[2 * k]     = (float)ctrl[2 * e.cp[k]];
                    v[2 * k + 1] = (float)ctrl[2 * e.cp[k] + 1];
                }
                for (int k = 0; k < 8; k++)
                    fin &= isfinite(v[k]) != 0;
                if (fin)
                    vko_bezier_walk(an_emit, &e, AN_TOL, v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], 0, 0.0, 1.0);
            }
        }
    }
    f->cont_p0[a->ncontours] = f->n;
    f->seg_p0[a->nseg]       = f->n;
}

static void flat_free(an_flat *f) { free(f->p), free(f->cont_p0), free(f->seg_p0); }

/* fp32 points, double points and per-segment offsets of the flattening */
VKO_API uint32_t vko_an_flatten(const vko_an *a, const double *ctrl, float *pts_f32, double *pts_f64, uint32_t cap,
                                uint32_t *seg_off) {
    an_flat f = {0};
    an_flatten(a, ctrl, &f);
    for (uint32_t i = 0; i < f.n && i < cap; i++) {
        if (pts_f32)
            pts_f32[2 * i] = f.p[i].fx, pts_f32[2 * i + 1] = f.p[i].fy;
        if (pts_f64)
            pts_f64[2 * i] = f.p[i].x, pts_f64[2 * i + 1] = f.p[i].y;
    }
    if (seg_off)
        memcpy(seg_off, f.seg_p0, (a->nseg + 1) * 4);
    uint32_t n = f.n;
    flat_free(&f);
    return n;
}

/* ------------------------------------------------------------ cell walk */

typedef void (*an_cell_fn)(void *u, int i, int j, double ta, double tb);

/* Liang-Barsky: restrict [t0, t1] to p * t <= q */
static int lb_clip(double p, double q, double *t0, double *t1) {
    if (p == 0)
        return q >= 0;
    double r = q / p;
    if (p < 0) {
        if (r > *t1)
            return 0;
        if (r > *t0)
            *t0 = r;
    } else {
        if (r < *t0)
            return 0;
        if (r < *t1)
            *t1 = r;
    }
    return 1;
}

/* Visit, in order of t, the pieces [ta, tb] of the edge (x0,y0)-(x1,y1)
   inside the box [bx0,bx1] x [by0,by1] that lie in one pixel cell (i, j);
   with xlines == 0 only the pixel rows split the edge and i is -1. */
static void an_walk(double x0, double y0, double x1, double y1, double bx0, double bx1, double by0, double by1,
                    int xlines, an_cell_fn fn, void *u) {
    double dx = x1 - x0, dy = y1 - y0, t0 = 0, t1 = 1;
    if (!lb_clip(-dx, x0 - bx0, &t0, &t1) || !lb_clip(dx, bx1 - x0, &t0, &t1) ||
        !lb_clip(-dy, y0 - by0, &t0, &t1) || !lb_clip(dy, by1 - y0, &t0, &t1) || !(t0 < t1))
        return;
    double tx = INFINITY, ty = INFINITY, kx = 0, ky = 0, sx = 0, sy = 0;
    if (xlines && dx != 0) {
        double xa = x0 + dx * t0;
        sx = dx > 0 ? 1 : -1;
        kx = dx > 0 ? floor(xa) + 1 : ceil(xa) - 1;
        tx = (kx - x0) / dx;
    }
    if (dy != 0) {
        double ya = y0 + dy * t0;
        sy = dy > 0 ? 1 : -1;
        ky = dy > 0 ? floor(ya) + 1 : ceil(ya) - 1;
        ty = (ky - y0) / dy;
    }
    double ta = t0;
    for (;;) {
        double tn = tx < ty ? tx : ty;
        double tb = tn < t1 ? tn : t1;
        if (tb > ta) {
            double tm = 0.5 * (ta + tb);
            int    i  = -1;
            if (xlines) {
                i = (int)floor(x0 + dx * tm);
                i = i < (int)bx0 ? (int)bx0 : i >= (int)bx1 ? (int)bx1 - 1 : i;
            }
            int j = (int)floor(y0 + dy * tm);
            j     = j < (int)by0 ? (int)by0 : j >= (int)by1 ? (int)by1 - 1 : j;
            fn(u, i, j, ta, tb);
            ta = tb;
        }
        if (tn >= t1)
            break;
        if (tx <= ty)
            kx += sx, tx = (kx - x0) / dx;
        else
            ky += sy, ty = (ky - y0) / dy;
    }
}

/* forward: deposit the edge's signed area into acc (H rows of W+1 cells) so
   that the row prefix sums are the pixels' winding-area integrals */
typedef struct {
    double  *acc;
    uint32_t W;
    double   x0, y0, dx, dy;
} acc_u;

static void acc_cell(void *uu, int i, int j, double ta, double tb) {
    acc_u  *u   = uu;
    double  dys = u->dy * (tb - ta);
    double *row = u->acc + (size_t)j * (u->W + 1);
    if (i < 0) { /* left of the canvas: covers the whole row */
        row[0] += dys;
        return;
    }
    double f = 0.5 * (u->x0 + u->dx * ta + u->x0 + u->dx * tb) - i;
    f        = f < 0 ? 0 : f > 1 ? 1 : f;
    row[i] += dys * (1 - f);
    row[i + 1] += dys * f;
}

static void edge_acc(double *acc, uint32_t W, uint32_t H, d2 p0, d2 p1) {
    if (p0.y == p1.y)
        return;
    acc_u u = {acc, W, p0.x, p0.y, p1.x - p0.x, p1.y - p0.y};
    an_walk(p0.x, p0.y, p1.x, p1.y, 0, W, 0, H, 1, acc_cell, &u);
    if (!(p1.x == p0.x && p0.x >= 0)) /* the part left of x = 0 */
        an_walk(p0.x, p0.y, p1.x, p1.y, -INFINITY, 0, 0, H, 0, acc_cell, &u);
}

/* backward: the pixel gradients gA integrated along the edge against the two
   endpoint hat functions: dL/dp0 = N*w0, dL/dp1 = N*w1, N = perp(p1 - p0) */
typedef struct {
    const double *gA;
    uint32_t      W;
    double        w0, w1;
} grad_u;

static void grad_cell(void *uu, int i, int j, double ta, double tb) {
    grad_u *u  = uu;
    double  g  = u->gA[(size_t)j * u->W + i];
    double  tm = 0.5 * (ta + tb);
    u->w0 += g * (tb - ta) * (1 - tm);
    u->w1 += g * (tb - ta) * tm;
}

static void edge_grad(const double *gA, uint32_t W, uint32_t H, d2 p0, d2 p1, d2 *g0, d2 *g1) {
    grad_u u = {gA, W, 0, 0};
    an_walk(p0.x, p0.y, p1.x, p1.y, 0, W, 0, H, 1, grad_cell, &u);
    d2 N = perp(sub(p1, p0));
    *g0  = add(*g0, scl(N, u.w0));
    *g1  = add(*g1, scl(N, u.w1));
}

/* ------------------------------------------------------- stroke pieces */

/* rectangle around segment a->b, half-width h */
static int quad_verts(d2 a, d2 b, double h, d2 q[4]) {
    d2     d = sub(b, a);
    double L = sqrt(dot(d, d));
    if (L == 0)
        return 0;
    d2 n = scl(perp(d), 1 / L);
    q[0] = add(a, scl(n, h)), q[1] = add(b, scl(n, h)), q[2] = sub(b, scl(n, h)), q[3] = sub(a, scl(n, h));
    return 1;
}

/* bevel triangle on the outer side of the joint pa->p->pb */
static int bevel_verts(d2 pa, d2 p, d2 pb, double h, d2 v[3], int *side) {
    d2     da = sub(p, pa), db = sub(pb, p);
    double La = sqrt(dot(da, da)), Lb = sqrt(dot(db, db));
    if (La == 0 || Lb == 0)
        return 0;
    double c = crs(da, db);
    if (c == 0)
        return 0;
    d2 na = scl(perp(da), 1 / La), nb = scl(perp(db), 1 / Lb);
    v[0] = p;
    if (c > 0)
        v[1] = sub(p, scl(nb, h)), v[2] = sub(p, scl(na, h)), *side = 1;
    else
        v[1] = add(p, scl(na, h)), v[2] = add(p, scl(nb, h)), *side = -1;
    return 1;
}

/* adjoint of n = perp(d)/|d|: dL/dd from dL/dn */
static d2 dnormal(d2 d, d2 gn) {
    double L = sqrt(dot(d, d));
    d2     u = scl(d, 1 / L), m = perpT(gn);
    return scl(sub(m, scl(u, dot(u, m))), 1 / L);
}

static void quad_adjoint(d2 a, d2 b, double h, const d2 gq[4], d2 *ga, d2 *gb, double *gh) {
    d2     d = sub(b, a);
    double L = sqrt(dot(d, d));
    d2     n = scl(perp(d), 1 / L);
    d2     S = sub(add(gq[0], gq[1]), add(gq[2], gq[3]));
    *gh += dot(n, S);
    d2 dd = dnormal(d, scl(S, h));
    *ga   = add(*ga, sub(add(gq[0], gq[3]), dd));
    *gb   = add(*gb, add(add(gq[1], gq[2]), dd));
}

static void bevel_adjoint(d2 pa, d2 p, d2 pb, double h, int side, const d2 gv[3], d2 *gpa, d2 *gp, d2 *gpb,
                          double *gh) {
    d2 da = sub(p, pa), db = sub(pb, p);
    d2 na = scl(perp(da), 1 / sqrt(dot(da, da))), nb = scl(perp(db), 1 / sqrt(dot(db, db)));
    d2 gna, gnb;
    if (side > 0) { /* v1 = p - h nb, v2 = p - h na */
        gnb = scl(gv[1], -h), gna = scl(gv[2], -h);
        *gh -= dot(nb, gv[1]) + dot(na, gv[2]);
    } else { /* v1 = p + h na, v2 = p + h nb */
        gna = scl(gv[1], h), gnb = scl(gv[2], h);
        *gh += dot(na, gv[1]) + dot(nb, gv[2]);
    }
    d2 gda = dnormal(da, gna), gdb = dnormal(db, gnb);
    *gp    = add(*gp, add(add(gv[0], add(gv[1], gv[2])), sub(gda, gdb)));
    *gpa   = sub(*gpa, gda);
    *gpb   = add(*gpb, gdb);
}

/* ----------------------------------------------------------- layers */

static d2 ptd(const an_flat *f, uint32_t k) { return d2v(f->p[k].x, f->p[k].y); }

/* the signed area of layer l per pixel (A, W*H); acc is H*(W+1) scratch */
static void layer_area(const vko_an *a, const an_flat *f, uint32_t l, const double *widths, double *acc,
                       double *A) {
    uint32_t W = a->W, H = a->H, p = a->layer_path[l];
    double   h = 0.5 * widths[p];
    memset(acc, 0, sizeof(double) * H * (W + 1));
    for (uint32_t c = a->path_c0[p]; c < a->path_c0[p + 1]; c++) {
        uint32_t p0 = f->cont_p0[c], n = f->cont_p0[c + 1] - p0;
        for (uint32_t k = 0; k < n; k++) {
            d2 P = ptd(f, p0 + k), Pn = ptd(f, p0 + (k + 1) % n), Pp = ptd(f, p0 + (k + n - 1) % n);
            if (!a->layer_stroke[l]) {
                edge_acc(acc, W, H, P, Pn);
                continue;
            }
            d2  q[4], v[3];
            int side;
            if (quad_verts(P, Pn, h, q))
                for (int e = 0; e < 4; e++)
                    edge_acc(acc, W, H, q[e], q[(e + 1) & 3]);
            if (bevel_verts(Pp, P, Pn, h, v, &side))
                for (int e = 0; e < 3; e++)
                    edge_acc(acc, W, H, v[e], v[(e + 1) % 3]);
        }
    }
    for (uint32_t j = 0; j < H; j++) {
        double s = 0;
        for (uint32_t i = 0; i < W; i++) {
            s += acc[(size_t)j * (W + 1) + i];
            A[(size_t)j * W + i] = s;
        }
    }
}

/* adjoint of layer_area: gA (W*H) -> point gradients gp and gh[path] */
static void layer_grad(const vko_an *a, const an_flat *f, uint32_t l, const double *widths, const double *gA, d2 *gp,
                       double *gh) {
    uint32_t W = a->W, H = a->H, p = a->layer_path[l];
    double   h = 0.5 * widths[p];
    for (uint32_t c = a->path_c0[p]; c < a->path_c0[p + 1]; c++) {
        uint32_t p0 = f->cont_p0[c], n = f->cont_p0[c + 1] - p0;
        for (uint32_t k = 0; k < n; k++) {
            uint32_t ik = p0 + k, in = p0 + (k + 1) % n, ip = p0 + (k + n - 1) % n;
            d2       P = ptd(f, ik), Pn = ptd(f, in), Pp = ptd(f, ip);
            if (!a->layer_stroke[l]) {
                if (n > 1)
                    edge_grad(gA, W, H, P, Pn, &gp[ik], &gp[in]);
                continue;
            }
            d2  q[4], v[3];
            int side;
            if (quad_verts(P, Pn, h, q)) {
                d2 gq[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
                for (int e = 0; e < 4; e++)
                    edge_grad(gA, W, H, q[e], q[(e + 1) & 3], &gq[e], &gq[(e + 1) & 3]);
                quad_adjoint(P, Pn, h, gq, &gp[ik], &gp[in], &gh[p]);
            }
            if (bevel_verts(Pp, P, Pn, h, v, &side)) {
                d2 gv[3] = {{0, 0}, {0, 0}, {0, 0}};
                for (int e = 0; e < 3; e++)
                    edge_grad(gA, W, H, v[e], v[(e + 1) % 3], &gv[e], &gv[(e + 1) % 3]);
                bevel_adjoint(Pp, P, Pn, h, side, gv, &gp[ip], &gp[ik], &gp[in], &gh[p]);
            }
        }
    }
}

static double cover(double A) {
    double m = fabs(A);
    return m < 1 ? m : 1;
}

/* ----------------------------------------------------------- forward */

VKO_API double vko_an_forward(const vko_an *a, const double *ctrl, const double *colors, const double *widths,
                              const double *target, double *canvas, double *area) {
    size_t  np = (size_t)a->W * a->H;
    an_flat f  = {0};
    an_flatten(a, ctrl, &f);
    double *C   = canvas ? canvas : malloc(np * 4 * sizeof(double));
    double *acc = malloc(sizeof(double) * a->H * (a->W + 1));
    double *Al  = malloc(sizeof(double) * np);
    for (size_t px = 0; px < np; px++)
        for (int ch = 0; ch < 4; ch++)
            C[px * 4 + ch] = a->bg[ch];
    for (uint32_t l = 0; l < a->nlayers; l++) {
        layer_area(a, &f, l, widths, acc, Al);
        if (area)
            memcpy(area + l * np, Al, np * sizeof(double));
        const double *col = colors + 4 * a->layer_path[l];
        for (size_t px = 0; px < np; px++) {
            double al = cover(Al[px]), keep = 1 - al * col[3];
            for (int ch = 0; ch < 4; ch++)
                C[px * 4 + ch] = al * col[ch] + keep * C[px * 4 + ch];
        }
    }
    double loss = 0;
    if (target) {
        for (size_t k = 0; k < np * 4; k++)
            loss += (C[k] - target[k]) * (C[k] - target[k]);
        loss /= (double)(np * 4);
    }
    if (!canvas)
        free(C);
    free(acc), free(Al);
    flat_free(&f);
    return loss;
}

/* ---------------------------------------------------------- backward */

/* dL/dcontrol points from dL/dpoints through the flattening: every point is
   a fixed combination of its segment's control points */
static void flatten_grad(const vko_an *a, const an_flat *f, const d2 *gp, double *d_ctrl) {
    for (uint32_t k = 0; k < f->n; k++) {
        const an_pt *p  = &f->p[k];
        uint32_t     s  = p->seg, c0 = a->seg_cp[s];
        if (p->which < 0) {
            d_ctrl[2 * c0] += gp[k].x, d_ctrl[2 * c0 + 1] += gp[k].y;
            continue;
        }
        uint32_t cp[4] = {c0, c0 + 1, c0 + 2, a->seg_end[s]};
        double   w[4];
        blossom(p->which, p->ta, p->tb, w);
        for (int q = 0; q < 4; q++)
            d_ctrl[2 * cp[q]] += w[q] * gp[k].x, d_ctrl[2 * cp[q] + 1] += w[q] * gp[k].y;
    }
}

VKO_API double vko_an_backward(const vko_an *a, const double *ctrl, const double *colors, const double *widths,
                               const double *target, const double *d_canvas, double *d_ctrl, double *d_colors,
                               double *d_widths, double *d_pts) {
    size_t   np = (size_t)a->W * a->H;
    uint32_t nl = a->nlayers;
    double  *A  = malloc(sizeof(double) * np * (nl ? nl : 1));
    double  *C  = malloc(sizeof(double) * np * 4);
    double   loss = vko_an_forward(a, ctrl, colors, widths, target, C, A);
    an_flat  f    = {0};
    an_flatten(a, ctrl, &f);
    memset(d_ctrl, 0, sizeof(double) * 2 * a->ncp);
    memset(d_colors, 0, sizeof(double) * 4 * a->npaths);
    memset(d_widths, 0, sizeof(double) * a->npaths);
    double *B = malloc(sizeof(double) * 4 * (nl + 1)), *al = malloc(sizeof(double) * (nl + 1));
    for (size_t px = 0; px < np; px++) {
        double g[4], c[4];
        for (int ch = 0; ch < 4; ch++) {
            g[ch] = d_canvas ? d_canvas[px * 4 + ch] : 2 * (C[px * 4 + ch] - target[px * 4 + ch]) / (double)(np * 4);
            c[ch] = a->bg[ch];
        }
        for (uint32_t l = 0; l < nl; l++) { /* the colour under every layer */
            const double *col = colors + 4 * a->layer_path[l];
            al[l]             = cover(A[l * np + px]);
            double keep       = 1 - al[l] * col[3];
            for (int ch = 0; ch < 4; ch++) {
                B[4 * l + ch] = c[ch];
                c[ch]         = al[l] * col[ch] + keep * c[ch];
            }
        }
        double T = 1; /* transmittance of the layers above */
        for (uint32_t l = nl; l-- > 0;) {
            const double *col = colors + 4 * a->layer_path[l];
            double       *dc  = d_colors + 4 * a->layer_path[l];
            double        gB = 0, gc = 0;
            for (int ch = 0; ch < 4; ch++)
                gB += g[ch] * B[4 * l + ch], gc += g[ch] * col[ch];
            double dal = T * (gc - col[3] * gB);
            double Av  = A[l * np + px];
            A[l * np + px] = fabs(Av) < 1 ? (Av > 0 ? dal : Av < 0 ? -dal : 0) : 0;
            for (int ch = 0; ch < 4; ch++)
                dc[ch] += T * al[l] * g[ch];
            dc[3] -= T * al[l] * gB;
            T *= 1 - al[l] * col[3];
        }
    }
    d2     *gp = calloc(f.n + 1, sizeof(d2));
    double *gh = calloc(a->npaths, sizeof(double));
    for (uint32_t l = 0; l < nl; l++)
        layer_grad(a, &f, l, widths, A + l * np, gp, gh);
    flatten_grad(a, &f, gp, d_ctrl);
    if (d_pts)
        memcpy(d_pts, gp, sizeof(d2) * f.n);
    for (uint32_t p = 0; p < a->npaths; p++)
        d_widths[p] = 0.5 * gh[p];
    free(gp), free(gh), free(B), free(al), free(A), free(C);
    flat_free(&f);
    return loss;
}

/* ------------------------------------------------ finite differences */

static uint32_t cp_path(const vko_an *a, uint32_t cp) {
    uint32_t lo = 0, hi = a->nseg; /* last segment with seg_cp <= cp */
    while (hi - lo > 1) {
        uint32_t m = (lo + hi) / 2;
        if (a->seg_cp[m] <= cp)
            lo = m;
        else
            hi = m;
    }
    uint32_t c = 0, ch = a->ncontours;
    while (ch - c > 1) {
        uint32_t m = (c + ch) / 2;
        if (a->cont_s0[m] <= lo)
            c = m;
        else
            ch = m;
    }
    return a->cont_path[c];
}

/* same subdivision of path p in both flattenings */
static int same_topology(const vko_an *a, const an_flat *x, const an_flat *y, uint32_t p) {
    uint32_t c0 = a->path_c0[p], c1 = a->path_c0[p + 1];
    if (x->cont_p0[c1] - x->cont_p0[c0] != y->cont_p0[c1] - y->cont_p0[c0])
        return 0;
    for (uint32_t c = c0; c < c1; c++)
        if (x->cont_p0[c] - x->cont_p0[c0] != y->cont_p0[c] - y->cont_p0[c0])
            return 0;
    for (uint32_t k = 0; k < x->cont_p0[c1] - x->cont_p0[c0]; k++) {
        const an_pt *u = &x->p[x->cont_p0[c0] + k], *v = &y->p[y->cont_p0[c0] + k];
        if (u->which != v->which || u->seg != v->seg || u->ta != v->ta || u->tb != v->tb)
            return 0;
    }
    return 1;
}

/* one FD worker: the parameters of a set of paths */
typedef struct {
    const vko_an  *a;
    const double  *ctrl, *colors, *widths, *target, *A, *C;
    const an_flat *base;
    const uint32_t *group, *index, *order, *path_of, *first, *last;
    uint32_t        o0, o1; /* its range of order[] */
    double          hs[2];
    int             nh;
    double         *fd[2];
    int32_t        *valid;
} fd_job;

static void *fd_worker(void *arg) {
    fd_job        *J = arg;
    const vko_an  *a = J->a;
    size_t         np = (size_t)a->W * a->H;
    uint32_t       nl = a->nlayers;
    double        *ct = malloc(sizeof(double) * 2 * a->ncp), *co = malloc(sizeof(double) * 4 * a->npaths);
    double        *wd = malloc(sizeof(double) * a->npaths);
    double        *Bb = malloc(sizeof(double) * np * 4), *Ta = malloc(sizeof(double) * np);
    double        *Xb = malloc(sizeof(double) * np * 4), *X = malloc(sizeof(double) * np * 4);
    double        *acc = malloc(sizeof(double) * a->H * (a->W + 1)), *Al = malloc(sizeof(double) * np);
    an_flat        pert = {0};
    memcpy(ct, J->ctrl, sizeof(double) * 2 * a->ncp);
    memcpy(co, J->colors, sizeof(double) * 4 * a->npaths);
    memcpy(wd, J->widths, sizeof(double) * a->npaths);
    uint32_t cur = UINT32_MAX;
    for (uint32_t oi = J->o0; oi < J->o1; oi++) {
        uint32_t i = J->order[oi], p = J->path_of[i];
        if (J->first[p] == UINT32_MAX) { /* a path with no layer */
            for (int e = 0; e < J->nh; e++)
                J->fd[e][i] = 0;
            J->valid[i] = 1;
            continue;
        }
        uint32_t l0 = J->first[p], l1 = J->last[p];
        if (p != cur) { /* colour under the path, transmittance above it, its base composite */
            cur = p;
            for (size_t px = 0; px < np; px++) {
                double c[4] = {a->bg[0], a->bg[1], a->bg[2], a->bg[3]};
                for (uint32_t l = 0; l < l0; l++) {
                    const double *col = J->colors + 4 * a->layer_path[l];
                    double        al = cover(J->A[l * np + px]), keep = 1 - al * col[3];
                    for (int ch = 0; ch < 4; ch++)
                        c[ch] = al * col[ch] + keep * c[ch];
                }
                memcpy(Bb + 4 * px, c, sizeof c);
                for (uint32_t l = l0; l <= l1; l++) {
                    const double *col = J->colors + 4 * p;
                    double        al = cover(J->A[l * np + px]), keep = 1 - al * col[3];
                    for (int ch = 0; ch < 4; ch++)
                        c[ch] = al * col[ch] + keep * c[ch];
                }
                memcpy(Xb + 4 * px, c, sizeof c);
                double T = 1;
                for (uint32_t l = l1 + 1; l < nl; l++)
                    T *= 1 - cover(J->A[l * np + px]) * J->colors[4 * a->layer_path[l] + 3];
                Ta[px] = T;
            }
        }
        double *par = J->group[i] == 0 ? &ct[J->index[i]] : J->group[i] == 1 ? &co[J->index[i]] : &wd[J->index[i]];
        double  v0  = *par;
        int     ok  = 1;
        for (int e = 0; e < J->nh; e++) {
            double Ls = 0; /* (L(+h) - L(-h)) * 4 np, from the two canvases */
            double *Xp = X;
            double *Xm = malloc(sizeof(double) * np * 4);
            for (int sgn = 0; sgn < 2; sgn++) {
                double *Xs = sgn ? Xm : Xp;
                *par       = sgn ? v0 - J->hs[e] : v0 + J->hs[e];
                const an_flat *fl = J->base;
                if (J->group[i] == 0) {
                    an_flatten(a, ct, &pert);
                    ok &= same_topology(a, J->base, &pert, p);
                    fl = &pert;
                }
                const double *col = co + 4 * p;
                memcpy(Xs, Bb, sizeof(double) * np * 4);
                for (uint32_t l = l0; l <= l1; l++) {
                    layer_area(a, fl, l, wd, acc, Al);
                    for (size_t px = 0; px < np; px++) {
                        double al = cover(Al[px]), keep = 1 - al * col[3];
                        for (int ch = 0; ch < 4; ch++)
                            Xs[px * 4 + ch] = al * col[ch] + keep * Xs[px * 4 + ch];
                    }
                }
            }
            *par = v0;
            /* C(theta') = Ta X(theta') + R with R = C - Ta Xb;
               L+ - L- = sum (C+ - C-)(C+ + C- - 2 target) / (4 np) */
            for (size_t k = 0; k < np * 4; k++) {
                double t  = Ta[k / 4];
                double R  = J->C[k] - t * Xb[k];
                double cp = t * Xp[k] + R, cm = t * Xm[k] + R;
                Ls += (cp - cm) * (cp + cm - 2 * J->target[k]);
            }
            free(Xm);
            J->fd[e][i] = Ls / (double)(np * 4) / (2 * J->hs[e]);
        }
        J->valid[i] = ok;
    }
    free(ct), free(co), free(wd), free(Bb), free(Ta), free(Xb), free(X), free(acc), free(Al);
    flat_free(&pert);
    return NULL;
}

/* Central differences (L(theta+h) - L(theta-h)) / 2h of the MSE loss for n
   parameters: group 0 = control-point coordinate index (x = 2*cp, y = 2*cp+1),
   1 = colour component (4*path + channel), 2 = width (path); also at h2
   into fd2 when h2 > 0.  A change of one path's parameters changes only that
   path's layers, so the perturbed canvas is rebuilt from that path's layers,
   the colour under them and the transmittance and colour of the layers above
   (all in double); full != 0 runs the whole forward for every evaluation
   instead.  valid[i] = 0 where the subdivision of the path differs at a
   perturbed value from theta (the loss is not smooth there).  threads > 1
   shares the paths among that many threads. */
VKO_API void vko_an_fd(const vko_an *a, const double *ctrl, const double *colors, const double *widths,
                       const double *target, uint32_t n, const uint32_t *group, const uint32_t *index, double h,
                       double h2, int full, int threads, double *fd, double *fd2, int32_t *valid) {
    size_t   np = (size_t)a->W * a->H;
    uint32_t nl = a->nlayers;
    an_flat  base = {0};
    an_flatten(a, ctrl, &base);
    uint32_t *path_of = malloc(sizeof(uint32_t) * (n + 1));
    for (uint32_t i = 0; i < n; i++)
        path_of[i] = group[i] == 0 ? cp_path(a, index[i] / 2) : group[i] == 1 ? index[i] / 4 : index[i];
    if (full) {
        double *ct = malloc(sizeof(double) * 2 * a->ncp), *co = malloc(sizeof(double) * 4 * a->npaths);
        double *wd = malloc(sizeof(double) * a->npaths);
        memcpy(ct, ctrl, sizeof(double) * 2 * a->ncp);
        memcpy(co, colors, sizeof(double) * 4 * a->npaths);
        memcpy(wd, widths, sizeof(double) * a->npaths);
        an_flat pert = {0};
        for (uint32_t i = 0; i < n; i++) {
            double *par = group[i] == 0 ? &ct[index[i]] : group[i] == 1 ? &co[index[i]] : &wd[index[i]];
            double  v0  = *par, hh[2] = {h, h2};
            int     ok  = 1;
            for (int e = 0; e < (h2 > 0 ? 2 : 1); e++) {
                double L[2];
                for (int sgn = 0; sgn < 2; sgn++) {
                    *par   = sgn ? v0 - hh[e] : v0 + hh[e];
                    L[sgn] = vko_an_forward(a, ct, co, wd, target, NULL, NULL);
                    an_flatten(a, ct, &pert);
                    ok &= same_topology(a, &base, &pert, path_of[i]);
                }
                *par = v0;
                (e ? fd2 : fd)[i] = (L[0] - L[1]) / (2 * hh[e]);
            }
            valid[i] = ok;
        }
        free(ct), free(co), free(wd);
        flat_free(&pert);
    } else {
        double   *A = malloc(sizeof(double) * np * (nl ? nl : 1)), *C = malloc(sizeof(double) * np * 4);
        uint32_t *first = malloc(4 * a->npaths), *last = malloc(4 * a->npaths);
        uint32_t *order = malloc(sizeof(uint32_t) * (n + 1));
        vko_an_forward(a, ctrl, colors, widths, target, C, A);
        for (uint32_t p = 0; p < a->npaths; p++)
            first[p] = UINT32_MAX, last[p] = 0;
        for (uint32_t l = 0; l < nl; l++) {
            uint32_t p = a->layer_path[l];
            if (first[p] == UINT32_MAX)
                first[p] = l;
            last[p] = l;
        }
        for (uint32_t i = 0; i < n; i++)
            order[i] = i;
        for (uint32_t i = 1; i < n; i++) { /* insertion sort by path, stable */
            uint32_t v = order[i], j = i;
            while (j > 0 && path_of[order[j - 1]] > path_of[v])
                order[j] = order[j - 1], j--;
            order[j] = v;
        }
        if (threads < 1)
            threads = 1;
        if (threads > 64)
            threads = 64;
        fd_job    jobs[64];
        pthread_t th[64];
        uint32_t  o = 0;
        for (int t = 0; t < threads; t++) {
            fd_job *J = &jobs[t];
            *J = (fd_job){a, ctrl, colors, widths, target, A, C, &base, group, index, order, path_of, first, last,
                          0, 0, {h, h2}, h2 > 0 ? 2 : 1, {fd, fd2}, valid};
            /* an even share of the parameters, split between paths */
            uint32_t end = (uint32_t)((uint64_t)n * (t + 1) / threads);
            while (end < n && end > 0 && path_of[order[end]] == path_of[order[end - 1]])
                end++;
            if (end < o)
                end = o;
            J->o0 = o, J->o1 = end, o = end;
        }
        for (int t = 0; t < threads; t++)
            pthread_create(&th[t], NULL, fd_worker, &jobs[t]);
        for (int t = 0; t < threads; t++)
            pthread_join(th[t], NULL);
        free(A), free(C), free(first), free(last), free(order);
    }
    free(path_of);
    flat_free(&base);
}
