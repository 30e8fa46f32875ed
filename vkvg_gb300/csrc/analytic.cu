/*
 * K7/K8 - analytic area coverage, compositing and their adjoints, sm_103a.
 *
 * Forward (K7):
 *   ak_cover      grid (layers) x (bands of 16 or 32 rows).  Every thread takes
 *                 flattened points of the layer's path and builds the
 *                 polygons of that point - the fill edge to the next point,
 *                 or the stroke's rectangle of the segment to the next point
 *                 and the bevel triangle on the outer side of its joint - and
 *                 walks each polygon edge through the pixel cells of the band
 *                 (ak_walk).  Each piece of edge in a cell deposits its signed
 *                 area into two shared-memory cells of the row (the cell, and
 *                 the one right of it for the rest of the row); a row prefix
 *                 sum then gives every pixel's exact winding-area integral A,
 *                 written to area[layer][y][x].  Edges left of the canvas
 *                 cover the whole row (deposit in column 0).
 *   ak_composite  one thread per pixel: coverage min(1, |A|) per layer,
 *                 premultiplied source-over in layer order onto the
 *                 background, the colour under every AK_CHUNK-th layer kept
 *                 as a checkpoint, canvas and per-block loss partials (in a
 *                 tiled scene, every AK_CHUNK-th of the layers reaching the
 *                 block).
 * Backward (K8):
 *   ak_composite_bwd  one thread per pixel, chunks of AK_CHUNK layers from the
 *                 top: the chunk's under-colours are recomputed from its
 *                 checkpoint, then the layers are walked downwards with the
 *                 transmittance of the layers above; writes dL/dA in place of
 *                 A and per-block colour-gradient partials.
 *   ak_cover_bwd  the same grid and polygons as ak_cover; every edge
 *                 integrates the pixel gradients along itself against its two
 *                 endpoint hat functions (the derivative of a polygon's area
 *                 in a pixel is the integral of the normal motion of its
 *                 boundary inside the pixel), which gives dL/dvertex, then
 *                 chains through the rectangle and bevel construction to the
 *                 points and the stroke width.
 * The flattening and its adjoint are in analytic_flat.cu.
 */
#include "analytic.h"

#include <cuda_runtime.h>
#include <math_constants.h>

#define AK_THREADS 256
#define AK_CB_THREADS 128 /* pixels per compositing-adjoint block (and tiled compositing block) */

__device__ __forceinline__ float2 v2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return v2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return v2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 operator*(float2 a, float s) { return v2(a.x * s, a.y * s); }
__device__ __forceinline__ float  dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ float  crs2(float2 a, float2 b) { return a.x * b.y - a.y * b.x; }
__device__ __forceinline__ float2 perp(float2 a) { return v2(-a.y, a.x); }
__device__ __forceinline__ float2 perpT(float2 a) { return v2(a.y, -a.x); }
__device__ __forceinline__ bool   fin2(float2 a) {
    return ((__float_as_uint(a.x) & 0x7f800000u) != 0x7f800000u) &&
           ((__float_as_uint(a.y) & 0x7f800000u) != 0x7f800000u);
}

/* ------------------------------------------------------------ cell walk */

/* Liang-Barsky: restrict [t0, t1] to p t <= q; id names the boundary that
   set t0 (in id0) or t1 (in id1) */
__device__ __forceinline__ bool lb_clip(float p, float q, float &t0, float &t1, int id, int &id0, int &id1) {
    if (p == 0.f)
        return q >= 0.f;
    float r = q / p;
    if (p < 0.f) {
        if (r > t1)
            return false;
        if (r > t0)
            t0 = r, id0 = id;
    } else {
        if (r < t0)
            return false;
        if (r < t1)
            t1 = r, id1 = id;
    }
    return true;
}

/* Visit, in order of t, the pieces [ta, tb] of edge a->b inside the box
   [bx0,bx1] x [by0,by1] that lie in one pixel cell (i, j), with the piece's
   end points (pa, pb); without xlines only rows split the edge and i = -1.
   Coordinates are those of a local frame whose origin is an integer pixel
   corner (box and cells included), so positions near the origin keep their
   full fp32 precision.  A piece ends where the next one starts, at the same
   float values, and a point on a grid line or box side has that line's exact
   coordinate: sums over consecutive pieces telescope.  At most lim steps;
   false if the bound was hit (it cannot be for a finite edge: lim covers
   every crossing of the box). */
template <class V>
__device__ __forceinline__ bool ak_walk(float2 a, float2 b, float bx0, float bx1, float by0, float by1, bool xlines,
                                        int lim, V &v) {
    float dx = b.x - a.x, dy = b.y - a.y, t0 = 0.f, t1 = 1.f;
    int   id0 = -1, id1 = -1;
    if (!lb_clip(-dx, a.x - bx0, t0, t1, 0, id0, id1) || !lb_clip(dx, bx1 - a.x, t0, t1, 1, id0, id1) ||
        !lb_clip(-dy, a.y - by0, t0, t1, 2, id0, id1) || !lb_clip(dy, by1 - a.y, t0, t1, 3, id0, id1) || !(t0 < t1))
        return true;
    const float bnd[4] = {bx0, bx1, by0, by1};
    float2      pa = a, pend = b;
    if (id0 >= 0)
        pa = id0 < 2 ? v2(bnd[id0], a.y + dy * t0) : v2(a.x + dx * t0, bnd[id0]);
    if (id1 >= 0)
        pend = id1 < 2 ? v2(bnd[id1], a.y + dy * t1) : v2(a.x + dx * t1, bnd[id1]);
    float tx = CUDART_INF_F, ty = CUDART_INF_F, kx = 0.f, ky = 0.f, sx = 0.f, sy = 0.f;
    if (xlines && dx != 0.f) {
        sx = dx > 0.f ? 1.f : -1.f;
        kx = dx > 0.f ? floorf(pa.x) + 1.f : ceilf(pa.x) - 1.f;
        tx = (kx - a.x) / dx;
    }
    if (dy != 0.f) {
        sy = dy > 0.f ? 1.f : -1.f;
        ky = dy > 0.f ? floorf(pa.y) + 1.f : ceilf(pa.y) - 1.f;
        ty = (ky - a.y) / dy;
    }
    float ta  = t0;
    int   ix0 = xlines ? (int)bx0 : 0, ix1 = xlines ? (int)bx1 - 1 : 0;
    int   jy0 = (int)by0, jy1 = (int)by1 - 1;
    for (int it = 0; it < lim; it++) {
        bool   xs = tx <= ty;
        float  tn = xs ? tx : ty;
        bool   last = tn >= t1;
        float  tb   = last ? t1 : tn;
        float2 pb   = last ? pend : xs ? v2(kx, a.y + dy * tn) : v2(a.x + dx * tn, ky);
        if (tb > ta) {
            float tm = 0.5f * (ta + tb);
            int   i  = -1;
            if (xlines) {
                i = (int)floorf(a.x + dx * tm);
                i = i < ix0 ? ix0 : i > ix1 ? ix1 : i;
            }
            int j = (int)floorf(a.y + dy * tm);
            j     = j < jy0 ? jy0 : j > jy1 ? jy1 : j;
            v(i, j, ta, tb, pa, pb);
            ta = tb;
        }
        pa = pb;
        if (last)
            return true;
        if (xs)
            kx += sx, tx = (kx - a.x) / dx;
        else
            ky += sy, ty = (ky - a.y) / dy;
    }
    return false;
}

/* Areas accumulate in fixed point (AK_FIX units per px^2) with integer
   shared-memory atomics: the sums are exact and order-independent.  A piece
   deposits the fixed-point difference of its end points' y, so the deposits
   of consecutive pieces, of consecutive edges and of the two walks of an
   edge telescope: past a closed polygon a row holds its exact integer
   winding, and rounding stays in the pixels the edges cross. */
#define AK_FIX     1048576.f /* 2^20 */
#define AK_FIX_INV (1.f / 1048576.f)

/* the visitors get cells of the local frame whose origin is (ox, oy) */
struct ak_acc_v {
    int *acc;
    int  ox, oy, y0, W1, sgn;
    __device__ void operator()(int i, int j, float ta, float tb, float2 pa, float2 pb) {
        int dys = (int)(__float2ll_rn(pb.y * AK_FIX) - __float2ll_rn(pa.y * AK_FIX)) * sgn;
        int *row = acc + (j + oy - y0) * W1;
        if (i < 0 && ox == 0) { /* left of the canvas: covers the whole row */
            atomicAdd(row, dys);
            return;
        }
        /* mean x of the piece relative to its cell's left side */
        float f  = fminf(fmaxf(0.5f * ((pa.x - (float)i) + (pb.x - (float)i)), 0.f), 1.f);
        int   d1 = __float2int_rn((float)dys * f);
        atomicAdd(row + i + ox, dys - d1);
        atomicAdd(row + i + ox + 1, d1);
    }
};

struct ak_grad_v {
    const float *g;
    int          ox, oy, y0, W;
    float        w0, w1;
    __device__ void operator()(int i, int j, float ta, float tb, float2, float2) {
        float gv = g[(j + oy - y0) * W + i + ox];
        float d  = (tb - ta) * gv;
        float tm = 0.5f * (ta + tb);
        w0 += d * (1.f - tm);
        w1 += d * tm;
    }
};

struct ak_band {
    int       y0, y1, W;
    uint32_t *status;
};

/* An edge a->b of a polygon given in the local frame with integer origin o. */
__device__ __forceinline__ bool edge_in_band(const ak_band &bd, float2 a, float2 b, float2 o) {
    return fmaxf(a.y, b.y) + o.y >= (float)bd.y0 && fminf(a.y, b.y) + o.y <= (float)bd.y1 && fin2(a) && fin2(b);
}

/* Positions along an edge are evaluated from the endpoint nearer the band:
   from the far one, a + t (b - a) would lose the fp32 bits of the far
   coordinate's magnitude exactly where the edge crosses the canvas. */
__device__ __forceinline__ bool far_first(const ak_band &bd, float2 a, float2 b, float2 o) {
    float cx = 0.5f * (float)bd.W - o.x, cy = 0.5f * (float)(bd.y0 + bd.y1) - o.y;
    return fmaxf(fabsf(a.x - cx), fabsf(a.y - cy)) > fmaxf(fabsf(b.x - cx), fabsf(b.y - cy));
}

__device__ __forceinline__ void edge_fwd(int *acc, const ak_band &bd, float2 a, float2 b, float2 o) {
    if (a.y == b.y || !edge_in_band(bd, a, b, o))
        return;
    int sgn = 1;
    if (far_first(bd, a, b, o)) { /* walk b->a: the deposits change sign */
        float2 t = a;
        a = b, b = t, sgn = -1;
    }
    ak_acc_v v{acc, (int)o.x, (int)o.y, bd.y0, bd.W + 1, sgn};
    float    bx1 = (float)bd.W - o.x, by0 = (float)bd.y0 - o.y, by1 = (float)bd.y1 - o.y;
    int      lim = bd.W + (bd.y1 - bd.y0) + 8;
    bool     ok  = ak_walk(a, b, -o.x, bx1, by0, by1, true, lim, v);
    if (!(b.x == a.x && a.x + o.x >= 0.f) && fminf(a.x, b.x) + o.x < 0.f) { /* the part left of x = 0 */
        v.ox = 0;
        ok   = ak_walk(a, b, -CUDART_INF_F, -o.x, by0, by1, false, lim, v) && ok;
    }
    if (!ok)
        atomicOr(bd.status, AK_ERR_WALK);
}

/* dL/da += N*w0, dL/db += N*w1 for edge a->b, N = perp(b - a); walked from
   the nearer endpoint, whose hat function is then the walk's first */
__device__ __forceinline__ void edge_bwd(const float *g, const ak_band &bd, float2 a, float2 b, float2 o,
                                         float2 &ga, float2 &gb) {
    if (!edge_in_band(bd, a, b, o))
        return;
    bool      rev = far_first(bd, a, b, o);
    ak_grad_v v{g, (int)o.x, (int)o.y, bd.y0, bd.W, 0.f, 0.f};
    if (!ak_walk(rev ? b : a, rev ? a : b, -o.x, (float)bd.W - o.x, (float)bd.y0 - o.y, (float)bd.y1 - o.y, true,
                 bd.W + (bd.y1 - bd.y0) + 8, v))
        atomicOr(bd.status, AK_ERR_WALK);
    float2 N = perp(b - a);
    ga       = ga + N * (rev ? v.w1 : v.w0);
    gb       = gb + N * (rev ? v.w0 : v.w1);
}

/* ------------------------------------------------------- stroke pieces */

__device__ __forceinline__ bool quad_verts(float2 a, float2 b, float h, float2 q[4]) {
    float2 d  = b - a;
    float  L2 = dot2(d, d);
    if (L2 == 0.f)
        return false;
    float2 n = perp(d) * (h / sqrtf(L2));
    q[0] = a + n, q[1] = b + n, q[2] = b - n, q[3] = a - n;
    return true;
}

__device__ __forceinline__ int bevel_verts(float2 pa, float2 p, float2 pb, float h, float2 v[3]) {
    float2 da = p - pa, db = pb - p;
    float  La = dot2(da, da), Lb = dot2(db, db);
    if (La == 0.f || Lb == 0.f)
        return 0;
    float c = crs2(da, db);
    if (c == 0.f)
        return 0;
    float2 na = perp(da) * (h / sqrtf(La)), nb = perp(db) * (h / sqrtf(Lb));
    v[0] = p;
    if (c > 0.f) {
        v[1] = p - nb, v[2] = p - na;
        return 1;
    }
    v[1] = p + na, v[2] = p + nb;
    return -1;
}

__device__ __forceinline__ float2 dnormal(float2 d, float2 gn) {
    float  iL = rsqrtf(dot2(d, d));
    float2 u = d * iL, m = perpT(gn);
    return (m - u * dot2(u, m)) * iL;
}

__device__ __forceinline__ bool pieces_in_band(const ak_band &bd, float2 pp, float2 p, float2 pn, float h) {
    float lo = fminf(fminf(pp.y, p.y), pn.y) - h, hi = fmaxf(fmaxf(pp.y, p.y), pn.y) + h;
    return hi >= (float)bd.y0 && lo <= (float)bd.y1;
}

/* the point's neighbours in its contour */
__device__ __forceinline__ void neighbours(const ak_scene &, const ak_bufs &B, uint32_t k, uint32_t &kp,
                                           uint32_t &kn) {
    const uint2 nb = B.pt_nb[k];
    kp = nb.x, kn = nb.y;
}

/* ---------------------------------------------------------- windows */

/* the part of the canvas a block covers: the canvas, or one tile (its
   origin, size, layers and checkpoint offset) */
struct ak_win {
    uint32_t x0, y0, W, H, nl, first;
    size_t   ckpt;
};
__device__ __forceinline__ ak_win ak_window(const ak_scene &S, uint32_t t) {
    ak_win w;
    if (!S.tiles) {
        w.x0 = w.y0 = 0, w.W = S.W, w.H = S.H, w.nl = S.nlayers, w.first = 0, w.ckpt = 0;
        return w;
    }
    const ak_tile_info ti = S.tinfo[t];
    w.x0    = (t % S.ntx) * S.tiles;
    w.y0    = (t / S.ntx) * S.tiles;
    w.W     = min(S.tiles, S.CW - w.x0);
    w.H     = min(S.tiles, S.CH - w.y0);
    w.nl    = ti.count;
    w.first = ti.first;
    w.ckpt  = (size_t)ti.ckpt;
    return w;
}
/* a (tile, layer) pair's box inside its tile: x0, y0, w, h */
__device__ __forceinline__ uint4 ak_pair_box(const ak_scene &S, uint32_t j) {
    const uint2 b = S.pair_box[j];
    return make_uint4(b.x & 0xFFFFu, b.x >> 16, b.y & 0xFFFFu, b.y >> 16);
}
/* blocks of n pixels per window (the canvas, or a tile) */
__host__ __device__ __forceinline__ uint32_t window_blocks(const ak_scene &S, uint32_t n) {
    return (uint32_t)(((size_t)S.W * S.H + n - 1) / n);
}
/* a coverage block's window, its scene layer and its area plane:
   blockIdx.x is the layer (the window is the canvas), or the (tile, layer)
   pair of a tiled scene (the window is the layer's box inside the tile) */
__device__ __forceinline__ ak_win ak_cover_window(const ak_scene &S, const ak_bufs &B, uint32_t &lg, float *&plane) {
    const uint32_t j = blockIdx.x;
    if (!S.tiles) {
        lg    = j;
        plane = B.area + (size_t)j * S.W * S.H;
        return ak_window(S, 0);
    }
    const uint32_t t  = S.pair_tile[j];
    const uint4    bx = ak_pair_box(S, j);
    ak_win         w;
    w.x0  = (t % S.ntx) * S.tiles + bx.x;
    w.y0  = (t / S.ntx) * S.tiles + bx.y;
    w.W   = bx.z;
    w.H   = bx.w;
    w.nl  = 1;
    w.first = j;
    w.ckpt  = 0;
    lg    = S.layer_map[j];
    plane = B.area + S.pair_off[j];
    return w;
}

/* ------------------------------------------------- band work compaction */

/* one flattened point whose polygons reach the band: its neighbours and the
   vertices of its polygons - the fill edge (v0, v1), or the stroke's
   rectangle (v0..v3) and bevel triangle (v4..v6) - relative to the integer
   pixel corner o at or below the point (exact, and small near the point) */
struct ak_slot {
    uint32_t k, kp, kn, flags; /* flags: 1 rectangle, 2 bevel, 4 bevel on the -n side */
    float2   o;
    float2   v[7];
};
#define AK_SLOT_RECT  1u
#define AK_SLOT_BEVEL 2u
#define AK_SLOT_NEG   4u

/* Phase 1 of a round: threads test the points [base, base + AK_THREADS) of
   the layer and append those reaching the band to the slot list. */
__device__ __forceinline__ void gather_slots(const ak_scene &S, const ak_bufs &B, const ak_band &bd, float2 org,
                                             bool stroke, bool fwd, float h, uint32_t k, uint32_t p1, ak_slot *slots,
                                             int *nslot) {
    if (k >= p1)
        return;
    uint32_t kp, kn;
    neighbours(S, B, k, kp, kn);
    /* org: the window's origin, an integer (exact in the subtraction) */
    float2 P = B.pts[k] - org, Pn = B.pts[kn] - org;
    float2 O = v2(floorf(P.x), floorf(P.y));
    if (!fin2(O))
        O = v2(0.f, 0.f);
    if (!stroke) {
        /* a horizontal edge adds no area but moves it: the backward keeps it */
        if ((fwd && P.y == Pn.y) || !edge_in_band(bd, P, Pn, v2(0.f, 0.f)))
            return;
        int      n = atomicAdd(nslot, 1);
        ak_slot &o = slots[n];
        o.k = k, o.kp = kp, o.kn = kn, o.flags = 0, o.o = O, o.v[0] = P - O, o.v[1] = Pn - O;
        return;
    }
    float2 Pp = B.pts[kp] - org;
    if (!pieces_in_band(bd, Pp, P, Pn, h))
        return;
    float2   q[4], v[3];
    uint32_t fl   = quad_verts(P - O, Pn - O, h, q) ? AK_SLOT_RECT : 0u;
    int      side = bevel_verts(Pp - O, P - O, Pn - O, h, v);
    fl |= side ? AK_SLOT_BEVEL : 0u;
    fl |= side > 0 ? AK_SLOT_NEG : 0u;
    if (!fl)
        return;
    int      n = atomicAdd(nslot, 1);
    ak_slot &o = slots[n];
    o.k = k, o.kp = kp, o.kn = kn, o.flags = fl, o.o = O;
#pragma unroll
    for (int e = 0; e < 4; e++)
        o.v[e] = q[e];
#pragma unroll
    for (int e = 0; e < 3; e++)
        o.v[4 + e] = v[e];
}

/* edge e of a slot: (a, b); false if that polygon is absent */
__device__ __forceinline__ bool slot_edge(const ak_slot &o, bool stroke, int e, float2 &a, float2 &b) {
    if (!stroke) {
        a = o.v[0], b = o.v[1];
        return true;
    }
    if (e < 4) {
        a = o.v[e], b = o.v[(e + 1) & 3];
        return (o.flags & AK_SLOT_RECT) != 0;
    }
    a = o.v[e], b = o.v[e == 6 ? 4 : e + 1];
    return (o.flags & AK_SLOT_BEVEL) != 0;
}

/* ------------------------------------------------------------- forward */

/* NT threads: 256 for layers by bands, 128 for the small (tile, layer) pairs
   (more of them in flight per SM) */
template <int NT>
__global__ void __launch_bounds__(NT) ak_cover(ak_scene S, ak_bufs B, const float *__restrict__ widths) {
    extern __shared__ __align__(16) unsigned char ak_smem[];
    ak_slot *slots = reinterpret_cast<ak_slot *>(ak_smem);
    int     *acc   = reinterpret_cast<int *>(slots + NT);
    __shared__ int nslot;
    /* grid: layers by bands (one window), or one block per (tile, layer)
       pair, which takes its box in bands as tall as the accumulator holds at
       the box's width (most glyph boxes in one) */
    uint32_t       lg;
    float         *plane;
    const ak_win   w    = ak_cover_window(S, B, lg, plane);
    const uint32_t bh   = S.tiles ? (S.band * (S.W + 1)) / (w.W + 1) : S.band;
    const uint32_t nb   = S.tiles ? (w.H + bh - 1) / bh : 1u;
    const int      W1   = w.W + 1;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float2   org  = v2((float)w.x0, (float)w.y0);
    for (uint32_t bi = 0; bi < nb; bi++) {
        const uint32_t band = S.tiles ? bi : blockIdx.y;
        ak_band        bd{(int)(band * bh), 0, (int)w.W, B.status};
        bd.y1    = min((int)w.H, bd.y0 + (int)bh);
        int rows = bd.y1 - bd.y0;
        __syncthreads(); /* the previous band's prefix sums have read the accumulator */
        for (int i = threadIdx.x; i < rows * W1; i += NT)
            acc[i] = 0;
        if (B.off[S.nseg] <= B.cap) {
            uint32_t p = S.layer_path[lg];
            bool     stroke = S.layer_stroke[lg] != 0;
            int      E      = stroke ? 7 : 1;
            float    h      = 0.5f * widths[p];
            uint32_t p1     = B.off[S.path_s0[p + 1]];
            for (uint32_t base = B.off[S.path_s0[p]]; base < p1; base += NT) {
                if (threadIdx.x == 0)
                    nslot = 0;
                __syncthreads();
                gather_slots(S, B, bd, org, stroke, true, h, base + threadIdx.x, p1, slots, &nslot);
                __syncthreads();
                int ne = nslot * E;
                for (int t = threadIdx.x; t < ne; t += NT) {
                    float2 a, b;
                    const ak_slot &sl = slots[t / E];
                    if (slot_edge(sl, stroke, t % E, a, b))
                        edge_fwd(acc, bd, a, b, sl.o);
                }
                __syncthreads();
            }
        }
        __syncthreads();
        /* row prefix sums, one warp per row, 32 cells per step */
        float *out = plane + (size_t)bd.y0 * w.W;
        for (int r = warp; r < rows; r += NT / 32) {
            int carry = 0;
            for (uint32_t c = 0; c < w.W; c += 32) {
                uint32_t i = c + lane;
                int      x = i < w.W ? acc[r * W1 + i] : 0;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int t = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= (uint32_t)o)
                        x += t;
                }
                if (i < w.W)
                    out[(size_t)r * w.W + i] = (float)(carry + x) * AK_FIX_INV;
                carry += __shfl_sync(0xffffffffu, x, 31);
            }
        }
    }
}

__device__ __forceinline__ float4 blend(float al, float4 c, float4 d) {
    float keep = 1.f - al * c.w;
    return make_float4(fmaf(al, c.x, keep * d.x), fmaf(al, c.y, keep * d.y), fmaf(al, c.z, keep * d.z),
                       fmaf(al, c.w, keep * d.w));
}
__device__ __forceinline__ float cover(float A) { return fminf(fabsf(A), 1.f); }

template <int N>
__device__ __forceinline__ float block_sum(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    float s = 0.f;
    if (threadIdx.x == 0)
        for (int w = 0; w < N / 32; w++)
            s += red[w];
    return s;
}

/* Tiled compositing walks, per block, only the layers whose planes reach the
   block's window rows, packed AK_CHUNK to a chunk.  ak_block_lists lists
   them first (one warp per compositing block, 32 layers of its tile a
   step, compacted with a ballot); chunk c of a block holds its listed
   layers [16 c, 16 c + 16) in the forward and in the adjoint alike (their
   blocks cover the same pixels), so the forward's checkpoint c is the
   colour under the adjoint's chunk c. */
__device__ __forceinline__ size_t ak_blist_base(const ak_win &w, uint32_t bpw, uint32_t b) {
    return (size_t)w.first * bpw + (size_t)b * w.nl;
}
__global__ void __launch_bounds__(128) ak_block_lists(ak_scene S, ak_bufs B, uint32_t nblocks) {
    const uint32_t gb = blockIdx.x * 4u + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
    if (gb >= nblocks)
        return;
    const uint32_t bpw = window_blocks(S, AK_CB_THREADS), b = gb % bpw;
    const ak_win   w   = ak_window(S, gb / bpw);
    const uint32_t ry0 = (uint32_t)((size_t)b * AK_CB_THREADS / w.W);
    const uint32_t ry1 = (uint32_t)(((size_t)b * AK_CB_THREADS + AK_CB_THREADS - 1) / w.W);
    uint32_t      *out = B.blist + ak_blist_base(w, bpw, b);
    uint32_t       n   = 0;
    for (uint32_t l0 = 0; l0 < w.nl; l0 += 32) {
        const uint32_t l  = l0 + lane;
        bool           on = false;
        if (l < w.nl) {
            const uint4 bx = ak_pair_box(S, w.first + l);
            on             = bx.y <= ry1 && bx.y + bx.w > ry0;
        }
        const uint32_t m = __ballot_sync(0xffffffffu, on);
        if (on)
            out[n + __popc(m & ((1u << lane) - 1u))] = l;
        n += __popc(m);
    }
    if (lane == 0)
        B.blk_na[gb] = n;
}
/* A listed layer as the compositing kernels keep it in shared memory: its
   pair's plane offset and box inside the tile (x0 | y0 << 16, w | h << 16),
   its tile-local index and colour.  A block loads AK_WIN entries of its list
   at a time (one thread each), so the dependent loads behind an entry
   (list, pair, path, colour) are paid once per AK_WIN / AK_CHUNK chunks. */
#define AK_WIN 64
struct ak_tplane {
    uint32_t base, xy, wh;
};
__device__ __forceinline__ long long ak_tplane_at(const ak_tplane &P, uint32_t x, uint32_t y) {
    const uint32_t dx = x - (P.xy & 0xFFFFu), dy = y - (P.xy >> 16), pw = P.wh & 0xFFFFu;
    return dx < pw && dy < (P.wh >> 16) ? (long long)P.base + (long long)dy * pw + dx : -1ll;
}
/* threads [0, n) of a block: list entries [e0, e0 + n) into (col, pl, cl) */
__device__ __forceinline__ void ak_load_window(const ak_scene &S, const ak_win &w, const float4 *__restrict__ colors,
                                               const uint32_t *__restrict__ list, uint32_t e0, uint32_t n,
                                               float4 *col, ak_tplane *pl, uint32_t *cl) {
    const uint32_t i = threadIdx.x;
    if (i < n) {
        const uint32_t l = list[e0 + i], j = w.first + l;
        const uint2    bx = S.pair_box[j];
        cl[i]             = l;
        pl[i]             = ak_tplane{S.pair_off[j], bx.x, bx.y};
        col[i]            = colors[S.layer_path[S.layer_map[j]]];
    }
}

/* TILED: the tiles of a tiled scene (layers read through their planes'
   boxes, packed chunks of the layers reaching the block); else the one
   window, every layer's plane the whole canvas */
template <bool TILED>
__global__ void __launch_bounds__(TILED ? AK_CB_THREADS : AK_THREADS)
    ak_composite(ak_scene S, ak_bufs B, const float4 *__restrict__ colors, const float4 *__restrict__ target,
                 float *__restrict__ loss_part) {
    constexpr int        NT = TILED ? AK_CB_THREADS : AK_THREADS;
    __shared__ float4    col[TILED ? AK_WIN : AK_CHUNK];
    __shared__ ak_tplane pl[TILED ? AK_WIN : 1];
    __shared__ uint32_t  cl[TILED ? AK_WIN : 1];
    __shared__ float     red[NT / 32];
    /* grid: the window's pixel blocks, window after window */
    const uint32_t bpw = window_blocks(S, NT), b = blockIdx.x % bpw;
    const ak_win   w   = ak_window(S, blockIdx.x / bpw);
    size_t         np = (size_t)w.W * w.H, px = (size_t)b * NT + threadIdx.x;
    bool           valid = px < np;
    const uint32_t x = valid ? (uint32_t)(px % w.W) : 0u, y = valid ? (uint32_t)(px / w.W) : 0u;
    float4         C     = S.bg;
    float4        *ckpt  = B.ckpt + w.ckpt;
    if (TILED) {
        const uint32_t  ntot = B.blk_na[blockIdx.x];
        const uint32_t *list = B.blist + ak_blist_base(w, bpw, b);
        for (uint32_t c = 0; c * AK_CHUNK < ntot; c++) {
            const uint32_t e0 = c * AK_CHUNK, wb = e0 % AK_WIN;
            const int      na = (int)min((uint32_t)AK_CHUNK, ntot - e0);
            if (wb == 0) {
                __syncthreads();
                ak_load_window(S, w, colors, list, e0, min((uint32_t)AK_WIN, ntot - e0), col, pl, cl);
                __syncthreads();
            }
            if (!valid)
                continue;
            ckpt[(size_t)c * np + px] = C;
            float A[AK_CHUNK];
#pragma unroll
            for (int i = 0; i < AK_CHUNK; i++) {
                const long long k = i < na ? ak_tplane_at(pl[wb + i], x, y) : -1ll;
                A[i]              = k >= 0 ? B.area[k] : 0.f;
            }
#pragma unroll
            for (int i = 0; i < AK_CHUNK; i++)
                if (i < na)
                    C = blend(cover(A[i]), col[wb + i], C);
        }
    } else {
        for (uint32_t lb = 0; lb < w.nl; lb += AK_CHUNK) {
            uint32_t n = min((uint32_t)AK_CHUNK, w.nl - lb);
            __syncthreads();
            if (threadIdx.x < n)
                col[threadIdx.x] = colors[S.layer_path[lb + threadIdx.x]];
            __syncthreads();
            if (!valid)
                continue;
            ckpt[(size_t)(lb / AK_CHUNK) * np + px] = C;
            float A[AK_CHUNK];
#pragma unroll
            for (int i = 0; i < AK_CHUNK; i++)
                A[i] = i < (int)n ? B.area[(size_t)(lb + i) * np + px] : 0.f;
#pragma unroll
            for (int i = 0; i < AK_CHUNK; i++)
                if (i < (int)n)
                    C = blend(cover(A[i]), col[i], C);
        }
    }
    float        s  = 0.f;
    const size_t cp = valid ? ((size_t)w.y0 + px / w.W) * S.CW + w.x0 + px % w.W : 0; /* on the canvas */
    if (valid) {
        B.canvas[cp] = C;
        if (target) {
            float4 t = target[cp];
            float  a = C.x - t.x, b = C.y - t.y, c = C.z - t.z, d = C.w - t.w;
            s        = a * a + b * b + c * c + d * d;
        }
    }
    if (target) {
        s = block_sum<NT>(s, red);
        if (threadIdx.x == 0)
            loss_part[blockIdx.x] = s;
    }
}

/* ------------------------------------------------------------ backward */

__device__ __forceinline__ float4 warp_sum4(float4 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
        v.w += __shfl_xor_sync(0xffffffffu, v.w, o);
    }
    return v;
}

/* Sum of v[0..31] over the warp, scattered: lane l returns the warp's sum of
   v[l] (recursive halving, 31 shuffles for 32 sums). */
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32]) {
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        bool up = (lane & (unsigned)o) != 0;
#pragma unroll
        for (int k = 0; k < o; k++) {
            float send = up ? v[k] : v[k + o];
            float keep = up ? v[k + o] : v[k];
            v[k]       = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0];
}

template <bool TILED>
__global__ void __launch_bounds__(AK_CB_THREADS)
    ak_composite_bwd(ak_scene S, ak_bufs B, const float4 *__restrict__ colors, const float4 *__restrict__ target,
                     const float4 *__restrict__ d_canvas, float *__restrict__ color_part) {
    __shared__ float4    col[TILED ? AK_WIN : AK_CHUNK];
    __shared__ ak_tplane pl[TILED ? AK_WIN : 1];
    __shared__ uint32_t  cl[TILED ? AK_WIN : 1];
    __shared__ float4 sB[AK_CHUNK][AK_CB_THREADS]; /* colour under each layer of the chunk */
    __shared__ float  sA[AK_CHUNK][AK_CB_THREADS]; /* the chunk's areas */
    __shared__ float  red[AK_CB_THREADS / 32][AK_CHUNK * 4];
    /* grid: the window's pixel blocks, window after window */
    const uint32_t bpw = window_blocks(S, AK_CB_THREADS), b = blockIdx.x % bpw;
    const ak_win   w   = ak_window(S, blockIdx.x / bpw);
    size_t         np = (size_t)w.W * w.H, px = (size_t)b * AK_CB_THREADS + threadIdx.x;
    bool           valid = px < np;
    float4         g     = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4  *ckpt  = B.ckpt + w.ckpt;
    const uint32_t x = valid ? (uint32_t)(px % w.W) : 0u, y = valid ? (uint32_t)(px / w.W) : 0u;
    if (valid) {
        const size_t cp = ((size_t)w.y0 + px / w.W) * S.CW + w.x0 + px % w.W; /* on the canvas */
        if (d_canvas) {
            g = d_canvas[cp];
        } else {
            float  s = 2.f / (float)((size_t)S.CW * S.CH * 4);
            float4 c = B.canvas[cp], t = target[cp];
            g        = make_float4((c.x - t.x) * s, (c.y - t.y) * s, (c.z - t.z) * s, (c.w - t.w) * s);
        }
    }
    float    T    = 1.f; /* transmittance of the layers above */
    uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    /* chunks from the top: tiled, the block's listed layers (the layers
       whose planes reach its rows: a layer outside them has no coverage, no
       gradient and no colour partial here, and the reduction reads a
       layer's partials only from the blocks its plane reaches) in chunks of
       AK_CHUNK, the top one holding the remainder; else chunks of AK_CHUNK
       layers */
    const uint32_t  ntot = TILED ? B.blk_na[blockIdx.x] : w.nl;
    const uint32_t *list = TILED ? B.blist + ak_blist_base(w, bpw, b) : nullptr;
    uint32_t        nch  = (ntot + AK_CHUNK - 1) / AK_CHUNK;
    uint32_t        held = 0xFFFFFFFFu; /* the list window in shared memory */
    for (uint32_t ch = nch; ch-- > 0;) {
        const uint32_t lb = ch * AK_CHUNK, n = min((uint32_t)AK_CHUNK, ntot - lb);
        const uint32_t wb = TILED ? lb % AK_WIN : 0u; /* the chunk's first entry in the window */
        __syncthreads();
        if (TILED) {
            const uint32_t w0 = lb - wb;
            if (w0 != held) {
                ak_load_window(S, w, colors, list, w0, min((uint32_t)AK_WIN, ntot - w0), col, pl, cl);
                held = w0;
            }
        } else if (threadIdx.x < n) {
            col[threadIdx.x] = colors[S.layer_path[lb + threadIdx.x]];
        }
        __syncthreads();
        const int na = (int)n; /* the chunk's layers [0, na), in order */
        float4 Bc = valid ? ckpt[(size_t)ch * np + px] : make_float4(0.f, 0.f, 0.f, 0.f);
        {
            float A[AK_CHUNK];
#pragma unroll
            for (int i = 0; i < AK_CHUNK; i++) {
                if (TILED) {
                    const long long k = (valid && i < na) ? ak_tplane_at(pl[wb + i], x, y) : -1ll;
                    A[i]              = k >= 0 ? B.area[k] : 0.f;
                } else {
                    A[i] = (valid && i < na) ? B.area[(size_t)(lb + i) * np + px] : 0.f;
                }
            }
#pragma unroll
            for (int i = 0; i < AK_CHUNK; i++) {
                if (i < na) {
                    sB[i][threadIdx.x] = Bc;
                    sA[i][threadIdx.x] = A[i];
                    Bc                 = blend(cover(A[i]), col[wb + i], Bc);
                }
            }
        }
        /* the chunk's layers in groups of 8, top group first; colour partials per group */
#pragma unroll
        for (int hf = 1; hf >= 0; hf--) {
            if (hf * 8 >= na)
                continue;
            float dc[32];
#pragma unroll
            for (int q8 = 7; q8 >= 0; q8--) {
                const int i = hf * 8 + q8;
                dc[4 * q8] = dc[4 * q8 + 1] = dc[4 * q8 + 2] = dc[4 * q8 + 3] = 0.f;
                if (i >= na)
                    continue;
                float4 c = col[wb + i], Bq = sB[i][threadIdx.x];
                float  Aq = sA[i][threadIdx.x];
                float  al = cover(Aq);
                float  gB = g.x * Bq.x + g.y * Bq.y + g.z * Bq.z + g.w * Bq.w;
                float  gc = g.x * c.x + g.y * c.y + g.z * c.z + g.w * c.w;
                float  da = T * (gc - c.w * gB);
                float  gA = fabsf(Aq) < 1.f ? (Aq > 0.f ? da : Aq < 0.f ? -da : 0.f) : 0.f;
                if (valid) {
                    const long long k = TILED ? ak_tplane_at(pl[wb + i], x, y) : (long long)((size_t)(lb + i) * np + px);
                    if (k >= 0)
                        B.area[k] = gA;
                }
                float ta = T * al;
                dc[4 * q8] = ta * g.x, dc[4 * q8 + 1] = ta * g.y, dc[4 * q8 + 2] = ta * g.z;
                dc[4 * q8 + 3] = ta * (g.w - gB);
                T *= 1.f - al * c.w;
            }
            red[warp][hf * 32 + lane] = warp_reduce_scatter32(dc);
        }
        __syncthreads();
        if ((int)threadIdx.x < na * 4) {
            float s = 0.f;
            for (int k = 0; k < AK_CB_THREADS / 32; k++)
                s += red[k][threadIdx.x];
            /* one window: [block][layer][channel]; tiled: [pair][block of the tile][channel] */
            const uint32_t q = threadIdx.x >> 2, c = threadIdx.x & 3;
            const size_t   i = S.tiles ? ((size_t)(w.first + cl[wb + q]) * bpw + b) * 4 + c
                                       : ((size_t)b * S.nlayers + lb + q) * 4 + c;
            color_part[i] = s;
        }
    }
}

__device__ __forceinline__ void add_grad(float2 *g, float2 v) {
    if (v.x != 0.f || v.y != 0.f) {
        atomicAdd(&g->x, v.x);
        atomicAdd(&g->y, v.y);
    }
}

template <int NT>
__global__ void __launch_bounds__(NT)
    ak_cover_bwd(ak_scene S, ak_bufs B, const float *__restrict__ widths, float2 *__restrict__ gpts,
                 float *__restrict__ gwidth) {
    extern __shared__ __align__(16) unsigned char ak_smem[];
    ak_slot *slots = reinterpret_cast<ak_slot *>(ak_smem);
    float4  *eg    = reinterpret_cast<float4 *>(slots + NT); /* per slot edge: dL/da, dL/db */
    float   *gs    = reinterpret_cast<float *>(eg + NT * 7);
    __shared__ float red[NT / 32];
    __shared__ int   nslot;
    /* the grid of ak_cover: a pair's block takes its box in bands as tall as
       the gradient buffer holds at the box's width */
    uint32_t       lg;
    float         *plane;
    const ak_win   w  = ak_cover_window(S, B, lg, plane);
    const uint32_t bh = S.tiles ? (S.band * S.W) / w.W : S.band;
    const uint32_t nb = S.tiles ? (w.H + bh - 1) / bh : 1u;
    if (B.off[S.nseg] > B.cap)
        return;
    const float2 org    = v2((float)w.x0, (float)w.y0);
    uint32_t     p      = S.layer_path[lg];
    bool         stroke = S.layer_stroke[lg] != 0;
    int          E      = stroke ? 7 : 1;
    float        h      = 0.5f * widths[p], gh = 0.f;
    uint32_t     p1     = B.off[S.path_s0[p + 1]];
    for (uint32_t bi = 0; bi < nb; bi++) {
    const uint32_t band = S.tiles ? bi : blockIdx.y;
    ak_band        bd{(int)(band * bh), 0, (int)w.W, B.status};
    bd.y1             = min((int)w.H, bd.y0 + (int)bh);
    int          rows = bd.y1 - bd.y0;
    const float *src  = plane + (size_t)bd.y0 * w.W;
    __syncthreads(); /* the previous band's edges have read the buffer */
    for (int i = threadIdx.x; i < rows * (int)w.W; i += NT)
        gs[i] = src[i];
    for (uint32_t base = B.off[S.path_s0[p]]; base < p1; base += NT) {
        if (threadIdx.x == 0)
            nslot = 0;
        __syncthreads();
        gather_slots(S, B, bd, org, stroke, false, h, base + threadIdx.x, p1, slots, &nslot);
        __syncthreads();
        int ns = nslot, ne = ns * E;
        for (int t = threadIdx.x; t < ne; t += NT) {
            float2 a, b, ga = v2(0.f, 0.f), gb = v2(0.f, 0.f);
            const ak_slot &sl = slots[t / E];
            if (slot_edge(sl, stroke, t % E, a, b))
                edge_bwd(gs, bd, a, b, sl.o, ga, gb);
            eg[t] = make_float4(ga.x, ga.y, gb.x, gb.y);
        }
        __syncthreads();
        if ((int)threadIdx.x < ns) {
            const ak_slot &o = slots[threadIdx.x];
            const float4  *g = eg + threadIdx.x * E;
            if (!stroke) {
                add_grad(&gpts[o.k], v2(g[0].x, g[0].y));
                add_grad(&gpts[o.kn], v2(g[0].z, g[0].w));
            } else {
                float2 P = B.pts[o.k], Pn = B.pts[o.kn], Pp = B.pts[o.kp];
                float2 gP = v2(0.f, 0.f), gPn = v2(0.f, 0.f), gPp = v2(0.f, 0.f);
                if (o.flags & AK_SLOT_RECT) {
                    float2 gq[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) /* vertex e starts edge e and ends edge e-1 */
                        gq[e] = v2(g[e].x + g[(e + 3) & 3].z, g[e].y + g[(e + 3) & 3].w);
                    float2 d  = Pn - P;
                    float2 n  = perp(d) * rsqrtf(dot2(d, d));
                    float2 Sg = (gq[0] + gq[1]) - (gq[2] + gq[3]);
                    gh += dot2(n, Sg);
                    float2 dd = dnormal(d, Sg * h);
                    gP        = gP + (gq[0] + gq[3]) - dd;
                    gPn       = gPn + (gq[1] + gq[2]) + dd;
                }
                if (o.flags & AK_SLOT_BEVEL) {
                    float2 gv[3];
#pragma unroll
                    for (int e = 0; e < 3; e++)
                        gv[e] = v2(g[4 + e].x + g[4 + (e + 2) % 3].z, g[4 + e].y + g[4 + (e + 2) % 3].w);
                    float2 da = P - Pp, db = Pn - P;
                    float2 na = perp(da) * rsqrtf(dot2(da, da)), nb = perp(db) * rsqrtf(dot2(db, db));
                    float2 gna, gnb;
                    if (o.flags & AK_SLOT_NEG) { /* v1 = p - h nb, v2 = p - h na */
                        gnb = gv[1] * -h, gna = gv[2] * -h;
                        gh -= dot2(nb, gv[1]) + dot2(na, gv[2]);
                    } else { /* v1 = p + h na, v2 = p + h nb */
                        gna = gv[1] * h, gnb = gv[2] * h;
                        gh += dot2(na, gv[1]) + dot2(nb, gv[2]);
                    }
                    float2 gda = dnormal(da, gna), gdb = dnormal(db, gnb);
                    gP         = gP + (gv[0] + gv[1] + gv[2]) + (gda - gdb);
                    gPp        = gPp - gda;
                    gPn        = gPn + gdb;
                }
                add_grad(&gpts[o.kp], gPp);
                add_grad(&gpts[o.k], gP);
                add_grad(&gpts[o.kn], gPn);
            }
        }
        __syncthreads();
    }
    } /* bands */
    if (stroke) {
        float s = block_sum<NT>(gh, red);
        if (threadIdx.x == 0 && s != 0.f)
            atomicAdd(&gwidth[p], 0.5f * s);
    }
}

/* dL/dcolour of every path: sum of its layers' per-block partials */
__global__ void ak_reduce_colors(ak_scene S, uint32_t nblocks, const float *__restrict__ part,
                                 float *__restrict__ d_colors) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.nlayers * 4)
        return;
    float s = 0.f;
    if (S.tiles) { /* t: (pair, channel); the blocks of rows the pair's plane reaches wrote partials */
        const uint32_t j = t >> 2, tl = S.pair_tile[j];
        const uint32_t W  = min(S.tiles, S.CW - (tl % S.ntx) * S.tiles);
        const uint2    bx = S.pair_box[j];
        const uint32_t y0 = bx.x >> 16, h = bx.y >> 16;
        const uint32_t b0 = (uint32_t)((size_t)y0 * W / AK_CB_THREADS);
        const uint32_t b1 = (uint32_t)(((size_t)(y0 + h) * W - 1) / AK_CB_THREADS);
        for (uint32_t b = b0; b <= b1 && b < nblocks; b++)
            s += part[((size_t)j * nblocks + b) * 4 + (t & 3)];
    } else
        for (uint32_t b = 0; b < nblocks; b++)
            s += part[(size_t)b * S.nlayers * 4 + t];
    const uint32_t l = t >> 2;
    atomicAdd(&d_colors[S.layer_path[S.layer_map ? S.layer_map[l] : l] * 4 + (t & 3)], s);
}

__global__ void ak_reduce_loss(uint32_t nblocks, float scale, const float *__restrict__ part, float *__restrict__ loss) {
    __shared__ float red[AK_THREADS / 32];
    float            s = 0.f;
    for (uint32_t b = threadIdx.x; b < nblocks; b += AK_THREADS)
        s += part[b];
    s = block_sum<AK_THREADS>(s, red);
    if (threadIdx.x == 0)
        *loss = s * scale;
}

/* ------------------------------------------------------------- tiling */

/* one warp per scene layer: the box of its path's flattened points in
   pixels (x0, y0, x1, y1 inclusive, clipped to the canvas; x0 > x1 when
   empty), a stroke's widened by half its width and one pixel (its
   rectangles and bevels reach at most half the width from a point), a
   fill's by one pixel (the winding of a closed contour, and with it every
   area the coverage deposits, is exactly zero outside its points' box);
   the boxes' pixel total is added to *total */
__global__ void ak_layer_boxes(ak_scene S, ak_bufs B, const float *__restrict__ widths, int4 *__restrict__ box,
                               unsigned long long *__restrict__ total) {
    const uint32_t l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (l >= S.nlayers)
        return;
    const uint32_t p  = S.layer_path[l];
    const uint32_t q0 = B.off[S.path_s0[p]], q1 = B.off[S.path_s0[p + 1]];
    float          x0 = CUDART_INF_F, y0 = CUDART_INF_F, x1 = -CUDART_INF_F, y1 = -CUDART_INF_F;
    if (B.off[S.nseg] <= B.cap)
        for (uint32_t k = q0 + lane; k < q1; k += 32) {
            const float2 P = B.pts[k];
            if (!fin2(P))
                continue;
            x0 = fminf(x0, P.x), y0 = fminf(y0, P.y), x1 = fmaxf(x1, P.x), y1 = fmaxf(y1, P.y);
        }
    for (int o = 16; o > 0; o >>= 1) {
        x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    }
    if (lane)
        return;
    const bool  stroke = S.layer_stroke[l] != 0;
    const float pad    = stroke ? 0.5f * fabsf(widths[p]) + 1.f : 1.f;
    int4        b      = make_int4(1, 1, 0, 0); /* empty */
    if (x0 <= x1 && isfinite(pad)) {
        /* clamped in float first: the box may reach far beyond the canvas */
        const float W = (float)S.CW, H = (float)S.CH;
        const float fx0 = fminf(fmaxf(floorf(x0 - pad), 0.f), W), fx1 = fminf(fmaxf(floorf(x1 + pad), -1.f), W - 1.f);
        const float fy0 = fminf(fmaxf(floorf(y0 - pad), 0.f), H), fy1 = fminf(fmaxf(floorf(y1 + pad), -1.f), H - 1.f);
        if (fx0 <= fx1 && fy0 <= fy1)
            b = make_int4((int)fx0, (int)fy0, (int)fx1, (int)fy1);
    }
    box[l] = b;
    if (b.x <= b.z)
        atomicAdd(total, (unsigned long long)(b.z - b.x + 1) * (unsigned long long)(b.w - b.y + 1));
}

/* flags[t * nlayers + l] = 1 when layer l's box meets tile t */
/* (tile, layer) entries: a block takes AK_TP_TILES consecutive tiles and
   AK_TP_LAYERS consecutive layers (one run per tile), a warp 512 of the
   layers as 16 rows of 32 (coalesced box loads); each box is loaded once
   and tested against the block's tiles */
#define AK_TP_THREADS 512
#define AK_TP_TILES   8
#define AK_TP_ROWS    (AK_TP_LAYERS / AK_TP_THREADS)
__device__ __forceinline__ bool ak_tp_hit(const int4 &b, uint32_t t, uint32_t ntx, uint32_t tile) {
    const int tx0 = (int)((t % ntx) * tile), ty0 = (int)((t / ntx) * tile);
    return b.x <= tx0 + (int)tile - 1 && b.z >= tx0 && b.y <= ty0 + (int)tile - 1 && b.w >= ty0;
}
/* hits[tt] bit k: this lane's layer of row k meets tile t0 + tt; the warp's
   pairs per tile into s_w[warp][tt] */
__device__ __forceinline__ void ak_tp_sweep(uint32_t nt, uint32_t nl, uint32_t ntx, uint32_t tile,
                                            const int4 *__restrict__ box, uint32_t t0, uint32_t l0,
                                            uint32_t (&hits)[AK_TP_TILES], uint32_t (*s_w)[AK_TP_TILES]) {
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t       cnt[AK_TP_TILES];
#pragma unroll
    for (int tt = 0; tt < AK_TP_TILES; tt++)
        hits[tt] = 0u, cnt[tt] = 0u;
    for (int k = 0; k < AK_TP_ROWS; k++) {
        const uint32_t l  = l0 + w * (32u * AK_TP_ROWS) + 32u * (uint32_t)k + lane;
        const bool     lv = l < nl;
        const int4     b  = lv ? box[l] : make_int4(1, 1, 0, 0);
#pragma unroll
        for (int tt = 0; tt < AK_TP_TILES; tt++) {
            const bool hit = lv && t0 + tt < nt && ak_tp_hit(b, t0 + tt, ntx, tile);
            hits[tt] |= (hit ? 1u : 0u) << k;
            cnt[tt] += __popc(__ballot_sync(0xffffffffu, hit));
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int tt = 0; tt < AK_TP_TILES; tt++)
            s_w[w][tt] = cnt[tt];
    }
    __syncthreads();
}
__global__ void __launch_bounds__(AK_TP_THREADS)
    ak_tile_count(uint32_t nt, uint32_t nl, uint32_t ntx, uint32_t tile, const int4 *__restrict__ box,
                  uint32_t *__restrict__ bsum, uint32_t *__restrict__ tcount) {
    __shared__ uint32_t s_w[AK_TP_THREADS / 32][AK_TP_TILES];
    const uint32_t      c = blockIdx.x, t0 = blockIdx.y * AK_TP_TILES, nch = gridDim.x;
    uint32_t            hits[AK_TP_TILES];
    ak_tp_sweep(nt, nl, ntx, tile, box, t0, c * AK_TP_LAYERS, hits, s_w);
    if (threadIdx.x < AK_TP_TILES && t0 + threadIdx.x < nt) {
        uint32_t v = 0;
        for (int q = 0; q < AK_TP_THREADS / 32; q++)
            v += s_w[q][threadIdx.x];
        bsum[(size_t)(t0 + threadIdx.x) * nch + c] = v;
        if (v)
            atomicAdd(&tcount[t0 + threadIdx.x], v);
    }
}
__global__ void __launch_bounds__(AK_TP_THREADS)
    ak_tile_lists(uint32_t nt, uint32_t nl, uint32_t ntx, uint32_t tile, const int4 *__restrict__ box,
                  const uint32_t *__restrict__ bpos, uint32_t *__restrict__ list, uint32_t *__restrict__ ptile,
                  uint2 *__restrict__ pbox, uint32_t *__restrict__ psize) {
    __shared__ uint32_t s_w[AK_TP_THREADS / 32][AK_TP_TILES];
    const uint32_t      c = blockIdx.x, t0 = blockIdx.y * AK_TP_TILES, nch = gridDim.x;
    const uint32_t      lane = threadIdx.x & 31u, w = threadIdx.x >> 5, lt = (1u << lane) - 1u;
    const uint32_t      l0   = c * AK_TP_LAYERS;
    uint32_t            hits[AK_TP_TILES];
    ak_tp_sweep(nt, nl, ntx, tile, box, t0, l0, hits, s_w);
    uint32_t j[AK_TP_TILES]; /* this warp's next pair of each tile */
#pragma unroll
    for (int tt = 0; tt < AK_TP_TILES; tt++) {
        j[tt] = t0 + tt < nt ? bpos[(size_t)(t0 + tt) * nch + c] : 0u;
        for (uint32_t q = 0; q < w; q++)
            j[tt] += s_w[q][tt];
    }
    for (int k = 0; k < AK_TP_ROWS; k++) {
        const uint32_t l = l0 + w * (32u * AK_TP_ROWS) + 32u * (uint32_t)k + lane;
        int4           b = make_int4(0, 0, 0, 0);
        bool           any = false;
#pragma unroll
        for (int tt = 0; tt < AK_TP_TILES; tt++)
            any |= ((hits[tt] >> k) & 1u) != 0u;
        if (any)
            b = box[l];
#pragma unroll
        for (int tt = 0; tt < AK_TP_TILES; tt++) {
            const bool     hit = (hits[tt] >> k) & 1u;
            const uint32_t m   = __ballot_sync(0xffffffffu, hit);
            if (hit) {
                const uint32_t t = t0 + tt, p = j[tt] + __popc(m & lt);
                const int      tx0 = (int)((t % ntx) * tile), ty0 = (int)((t / ntx) * tile);
                const int      x0 = max(b.x, tx0) - tx0, x1 = min(b.z, tx0 + (int)tile - 1) - tx0;
                const int      y0 = max(b.y, ty0) - ty0, y1 = min(b.w, ty0 + (int)tile - 1) - ty0;
                list[p]  = l;
                ptile[p] = t;
                pbox[p]  = make_uint2((uint32_t)x0 | (uint32_t)y0 << 16,
                                      (uint32_t)(x1 - x0 + 1) | (uint32_t)(y1 - y0 + 1) << 16);
                psize[p] = (uint32_t)((x1 - x0 + 1) * (y1 - y0 + 1));
            }
            j[tt] += __popc(m);
        }
    }
}

__global__ void ak_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                        float *__restrict__ v, uint32_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                        float lo, float hi) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi, v[i] = vi;
    float x = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i]    = fminf(fmaxf(x, lo), hi);
}

/* ------------------------------------------------------------ launchers */

/* compositing blocks per window: 256 pixels, or 128 in a tiled scene (its
   forward and adjoint blocks cover the same pixels) */
uint32_t ak_pixel_blocks(const ak_scene &S) {
    const uint32_t nt = S.tiles ? AK_CB_THREADS : AK_THREADS;
    return (uint32_t)(((size_t)S.W * S.H + nt - 1) / nt);
}
uint32_t ak_band_rows(uint32_t W) { return W <= AK_BAND_WIDE_MAX ? 32u : 16u; }
static size_t cover_fwd_smem(uint32_t W, uint32_t band, uint32_t nt) {
    return sizeof(ak_slot) * nt + sizeof(int) * band * (W + 1);
}
static size_t cover_bwd_smem(uint32_t W, uint32_t band, uint32_t nt) {
    return sizeof(ak_slot) * nt + sizeof(float4) * nt * 7 + sizeof(float) * band * W;
}
size_t ak_cover_smem(uint32_t W) {
    uint32_t band = ak_band_rows(W);
    size_t   fwd = cover_fwd_smem(W, band, AK_THREADS), bwd = cover_bwd_smem(W, band, AK_THREADS);
    return fwd > bwd ? fwd : bwd;
}
/* tiled scenes take the small blocks */
#define AK_PAIR_THREADS 64
static uint32_t cover_threads(const ak_scene &S) { return S.tiles ? AK_PAIR_THREADS : AK_THREADS; }

template <int NT> static cudaError_t launch_cover(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float *widths) {
    const size_t smem = cover_fwd_smem(S.W, S.band, NT);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(ak_cover<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    /* tiled: one block per pair, which walks its box's bands */
    ak_cover<NT><<<dim3(S.nlayers, S.tiles ? 1u : S.nbands), NT, smem, st>>>(S, B, widths);
    return cudaGetLastError();
}
cudaError_t ak_launch_cover(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float *widths) {
    if (!S.nlayers)
        return cudaSuccess;
    return cover_threads(S) == AK_PAIR_THREADS ? launch_cover<AK_PAIR_THREADS>(st, S, B, widths)
                                             : launch_cover<AK_THREADS>(st, S, B, widths);
}
static uint32_t windows(const ak_scene &S) { return S.tiles ? S.ntiles : 1u; }
uint32_t ak_pixel_blocks_all(const ak_scene &S) { return ak_pixel_blocks(S) * windows(S); }
cudaError_t ak_launch_composite(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float4 *colors,
                                const float4 *target, float *loss_part) {
    if (S.tiles) {
        const uint32_t nb = ak_pixel_blocks_all(S);
        ak_block_lists<<<(nb + 3) / 4, 128, 0, st>>>(S, B, nb);
        ak_composite<true><<<nb, AK_CB_THREADS, 0, st>>>(S, B, colors, target, loss_part);
    }
    else
        ak_composite<false><<<ak_pixel_blocks_all(S), AK_THREADS, 0, st>>>(S, B, colors, target, loss_part);
    return cudaGetLastError();
}
uint32_t ak_composite_bwd_blocks(const ak_scene &S) {
    return (uint32_t)(((size_t)S.W * S.H + AK_CB_THREADS - 1) / AK_CB_THREADS);
}
size_t ak_color_partials(const ak_scene &S) { return (size_t)ak_composite_bwd_blocks(S) * S.nlayers; }
cudaError_t ak_launch_composite_bwd(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float4 *colors,
                                    const float4 *target, const float4 *d_canvas, float4 *color_part) {
    if (S.tiles)
        ak_composite_bwd<true><<<ak_composite_bwd_blocks(S) * windows(S), AK_CB_THREADS, 0, st>>>(
            S, B, colors, target, d_canvas, reinterpret_cast<float *>(color_part));
    else
        ak_composite_bwd<false><<<ak_composite_bwd_blocks(S), AK_CB_THREADS, 0, st>>>(
            S, B, colors, target, d_canvas, reinterpret_cast<float *>(color_part));
    return cudaGetLastError();
}
template <int NT>
static cudaError_t launch_cover_bwd(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float *widths,
                                    float2 *gpts, float *gwidth) {
    const size_t smem = cover_bwd_smem(S.W, S.band, NT);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(ak_cover_bwd<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    ak_cover_bwd<NT><<<dim3(S.nlayers, S.tiles ? 1u : S.nbands), NT, smem, st>>>(S, B, widths, gpts, gwidth);
    return cudaGetLastError();
}
cudaError_t ak_launch_cover_bwd(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float *widths,
                                float2 *gpts, float *gwidth) {
    if (!S.nlayers)
        return cudaSuccess;
    return cover_threads(S) == AK_PAIR_THREADS ? launch_cover_bwd<AK_PAIR_THREADS>(st, S, B, widths, gpts, gwidth)
                                             : launch_cover_bwd<AK_THREADS>(st, S, B, widths, gpts, gwidth);
}
cudaError_t ak_launch_reduce(cudaStream_t st, const ak_scene &S, uint32_t nblocks, const float4 *color_part,
                             float4 *d_colors, const float *loss_part, float *loss) {
    if (color_part && S.nlayers)
        ak_reduce_colors<<<(S.nlayers * 4 + 255) / 256, 256, 0, st>>>(
            S, nblocks, reinterpret_cast<const float *>(color_part), reinterpret_cast<float *>(d_colors));
    if (loss_part)
        ak_reduce_loss<<<1, AK_THREADS, 0, st>>>(nblocks, 1.f / (float)((size_t)S.CW * S.CH * 4), loss_part, loss);
    return cudaGetLastError();
}
cudaError_t ak_launch_layer_boxes(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float *widths, int4 *box,
                                  unsigned long long *total) {
    if (S.nlayers)
        ak_layer_boxes<<<(S.nlayers * 32 + 255) / 256, 256, 0, st>>>(S, B, widths, box, total);
    return cudaGetLastError();
}
static uint32_t tile_chunks(uint32_t nl) { return (nl + AK_TP_LAYERS - 1) / AK_TP_LAYERS; }
uint32_t ak_tile_runs(uint32_t ntiles, uint32_t nlayers) { return ntiles * tile_chunks(nlayers); }
cudaError_t ak_launch_tile_count(cudaStream_t st, uint32_t ntiles, uint32_t nlayers, uint32_t ntx, uint32_t tile,
                                 const int4 *box, uint32_t *bsum, uint32_t *tcount) {
    if (ntiles && nlayers)
        ak_tile_count<<<dim3(tile_chunks(nlayers), (ntiles + AK_TP_TILES - 1) / AK_TP_TILES), AK_TP_THREADS, 0, st>>>(
            ntiles, nlayers, ntx, tile, box, bsum, tcount);
    return cudaGetLastError();
}
cudaError_t ak_launch_tile_lists(cudaStream_t st, uint32_t ntiles, uint32_t nlayers, uint32_t ntx, uint32_t tile,
                                 const int4 *box, const uint32_t *bpos, uint32_t *list, uint32_t *ptile, uint2 *pbox,
                                 uint32_t *psize) {
    if (ntiles && nlayers)
        ak_tile_lists<<<dim3(tile_chunks(nlayers), (ntiles + AK_TP_TILES - 1) / AK_TP_TILES), AK_TP_THREADS, 0, st>>>(
            ntiles, nlayers, ntx, tile, box, bpos, list, ptile, pbox, psize);
    return cudaGetLastError();
}
cudaError_t ak_launch_adam(cudaStream_t st, float *param, const float *grad, float *m, float *v, uint32_t n, float lr,
                           float beta1, float beta2, float eps, uint32_t step, float lo, float hi) {
    float c1 = 1.f / (1.f - powf(beta1, (float)step)), c2 = 1.f / (1.f - powf(beta2, (float)step));
    if (n)
        ak_adam<<<(n + 255) / 256, 256, 0, st>>>(param, grad, m, v, n, lr, beta1, beta2, eps, c1, c2, lo, hi);
    return cudaGetLastError();
}
