/*
 * K3 - primitive setup and band binning on sm_103a.
 *
 * Fill draws become directed polygon edges (each subpath with more than two
 * points, closed by its implicit last edge, as vkvg's triangle fan and
 * glutess contour are); stroke draws become positively oriented triangles
 * from vkvg's own vertex/index buffers.  Every vertex goes through vkvg's
 * vertex stage (shaders/vkvg_main.vert:74-79: p' = CTM p, ndc = p'*2/size - 1)
 * and the viewport transform, then is snapped to 8 sub-pixel bits (round to
 * nearest even).  This unit is built with -fmad=false so the float steps match
 * the CPU restatement exactly.
 *
 * Binning: the surface is cut into bands of 16 sample rows.  Each primitive is
 * counted into (band, draw) cells, an exclusive scan in band-major order gives
 * every band a contiguous, draw-ordered list, and a scatter pass writes the
 * primitives' records (not indices) into it.
 */
#include "gb_types.h"

#include <cuda_runtime.h>

#include <algorithm>

#define GB_FIX_LIMIT 268435456.0f /* 2^28 units = 2^20 px */

__device__ __forceinline__ int32_t gb_to_fixed(float v) {
    float s = v * 256.0f;
    if (s != s)
        return 0;
    if (!(s > -GB_FIX_LIMIT))
        s = -GB_FIX_LIMIT;
    if (!(s < GB_FIX_LIMIT))
        s = GB_FIX_LIMIT;
    return __float2int_rn(s);
}
struct gb_vp {
    float xx, yx, xy, yy, x0, y0, w, h, hw, hh;
};
__device__ __forceinline__ gb_vp make_vp(const gb_draw &d, uint32_t W, uint32_t H) {
    gb_vp v;
    v.xx = d.mat[0];
    v.yx = d.mat[1];
    v.xy = d.mat[2];
    v.yy = d.mat[3];
    v.x0 = d.mat[4];
    v.y0 = d.mat[5];
    v.w  = (float)W;
    v.h  = (float)H;
    v.hw = (float)W * 0.5f;
    v.hh = (float)H * 0.5f;
    return v;
}
__device__ __forceinline__ int2 gb_snap(const gb_vp &m, float2 p, bool *finite) {
    float px = (m.xx * p.x + m.xy * p.y) + m.x0;
    float py = (m.yx * p.x + m.yy * p.y) + m.y0;
    if (finite)
        *finite = !(px != px || py != py);
    float nx = (px * 2.0f) / m.w - 1.0f;
    float ny = (py * 2.0f) / m.h - 1.0f;
    return make_int2(gb_to_fixed(nx * m.hw + m.hw), gb_to_fixed(ny * m.hh + m.hh));
}

/* the largest i in [lo, hi) with off[i] <= e (off non-decreasing, off[lo] <= e),
   by the whole warp: 32 probes a step, so a few dependent loads */
__device__ __forceinline__ uint32_t gb_warp_find(const uint32_t *__restrict__ off, uint32_t lo, uint32_t hi,
                                                 uint32_t e) {
    const uint32_t lane = threadIdx.x & 31u;
    while (hi - lo > 1) {
        const uint32_t step = (hi - lo + 31u) / 32u;
        const uint32_t i    = lo + lane * step;
        const uint32_t m    = __ballot_sync(0xFFFFFFFFu, i < hi && off[i] <= e) | 1u;
        lo += (31u - (uint32_t)__clz(m)) * step;
        hi = min(hi, lo + step);
    }
    return lo;
}
/* the block's items [i0, i1] lie in ranges [p0, p1] of off (n ranges):
   warp 0 finds both ends */
__device__ __forceinline__ void gb_block_range(const uint32_t *__restrict__ off, uint32_t n, uint32_t i0,
                                               uint32_t i1, uint32_t *s_p) {
    if (threadIdx.x < 32) {
        const uint32_t p0 = gb_warp_find(off, 0, n, i0);
        const uint32_t p1 = gb_warp_find(off, p0, n, i1);
        if (threadIdx.x == 0)
            s_p[0] = p0, s_p[1] = p1;
    }
    __syncthreads();
}
__device__ __forceinline__ uint32_t gb_find(const uint32_t *__restrict__ off, uint32_t n, uint32_t e,
                                            uint32_t lo = 0) {
    uint32_t hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= e)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

/* edges per fill (draw, subpath) pair */
__global__ void gb_fill_pair_edges(uint32_t npairs, const uint32_t *__restrict__ pair_sub,
                                   const uint32_t *__restrict__ sub_npts, uint32_t *__restrict__ counts) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs)
        return;
    uint32_t n = sub_npts[pair_sub[p]];
    counts[p]  = n > 2 ? n : 0;
}
/* snapped directed edges; edge j of a subpath joins point j to point j+1 (mod n) */
__global__ void gb_fill_edges(uint32_t nedges, uint32_t npairs, const uint32_t *__restrict__ e_off,
                              const uint32_t *__restrict__ pair_draw, const uint32_t *__restrict__ pair_sub,
                              const gb_draw *__restrict__ draws, const uint32_t *__restrict__ sub_pt0,
                              const uint32_t *__restrict__ sub_npts, const float2 *__restrict__ pts,
                              const gb_surf *__restrict__ surfs, int4 *__restrict__ edges,
                              uint32_t *__restrict__ edge_draw) {
    /* the block's edges lie in pairs [p0, p1]: two searches over all pairs,
       then each thread's search within them */
    __shared__ uint32_t s_p[2];
    const uint32_t      e0 = blockIdx.x * blockDim.x, e = e0 + threadIdx.x;
    gb_block_range(e_off, npairs, e0, min(e0 + blockDim.x, nedges) - 1u, s_p);
    if (e >= nedges)
        return;
    uint32_t p = gb_find(e_off, s_p[1] + 1u, e, s_p[0]);
    uint32_t s = pair_sub[p], d = pair_draw[p];
    uint32_t j = e - e_off[p], n = sub_npts[s], first = sub_pt0[s];
    const gb_surf &sf = surfs[draws[d].surf];
    gb_vp          m  = make_vp(draws[d], sf.W, sf.H);
    int2     a = gb_snap(m, pts[first + j], nullptr);
    int2     b = gb_snap(m, pts[first + (j + 1 == n ? 0 : j + 1)], nullptr);
    edges[e]     = make_int4(a.x, a.y, b.x, b.y);
    edge_draw[e] = d;
}
/* snapped, positively oriented stroke triangles; degenerate or non-finite
   triangles are marked with w = 0 */
__global__ void gb_stroke_tris(uint32_t ntris, uint32_t ndraw_s, const uint32_t *__restrict__ draw_tri0,
                               const uint32_t *__restrict__ sdraw_id, const uint32_t *__restrict__ draw_vbase,
                               const gb_draw *__restrict__ draws, const float2 *__restrict__ verts,
                               const uint32_t *__restrict__ inds, const gb_surf *__restrict__ surfs,
                               int4 *__restrict__ tri_a,
                               int4 *__restrict__ tri_b, uint32_t *__restrict__ tri_draw,
                               uint4 *__restrict__ tri_idx) {
    __shared__ uint32_t s_p[2];
    const uint32_t      t0 = blockIdx.x * blockDim.x, t = t0 + threadIdx.x;
    gb_block_range(draw_tri0, ndraw_s, t0, min(t0 + blockDim.x, ntris) - 1u, s_p);
    if (t >= ntris)
        return;
    uint32_t k  = gb_find(draw_tri0, s_p[1] + 1u, t, s_p[0]);
    uint32_t d  = sdraw_id[k];
    const gb_surf &sf = surfs[draws[d].surf];
    gb_vp          m  = make_vp(draws[d], sf.W, sf.H);
    uint32_t vb = draw_vbase[k], nv = draw_vbase[k + 1] - vb;
    uint32_t i0 = inds[3 * t], i1 = inds[3 * t + 1], i2 = inds[3 * t + 2];
    bool     inb = i0 < nv && i1 < nv && i2 < nv;
    if (!inb)
        i0 = i1 = i2 = 0;
    bool     f0, f1, f2;
    int2     a  = gb_snap(m, verts[vb + i0], &f0);
    int2     b  = gb_snap(m, verts[vb + i1], &f1);
    int2     c  = gb_snap(m, verts[vb + i2], &f2);
    long long area = (long long)(b.x - a.x) * (long long)(c.y - a.y) - (long long)(c.x - a.x) * (long long)(b.y - a.y);
    int valid = (inb && f0 && f1 && f2 && area != 0) ? 1 : 0;
    if (area < 0) {
        int2 tmp = b;
        b        = c;
        c        = tmp;
        uint32_t ti = i1;
        i1          = i2;
        i2          = ti;
    }
    tri_a[t]    = make_int4(a.x, a.y, b.x, b.y);
    tri_b[t]    = make_int4(c.x, c.y, valid, 0);
    tri_draw[t] = d;
    tri_idx[t]  = make_uint4(i0, i1, i2, valid ? d + 1 : 0u); /* oriented vertex indices, draw + 1 if valid */
}

/* Stroke triangles as directed edges for the coverage count.  A positively
   oriented triangle's coverage is the winding of its three edges, so a
   stroke's covering-triangle count is the winding of all its triangles'
   edges.  Two opposite occurrences of one edge (the same two vertices of one
   draw, reversed) add exactly opposite crossings at every sample and are
   dropped: the quad diagonals and the rungs between consecutive quads that
   vkvg's vertex buffer shares between neighbouring triangles.  An edge is
   paired only with the reversed edge of the next or previous triangle, and
   only when the triangles two steps away cannot claim either occurrence, so
   every occurrence has at most one partner.  Dropped and degenerate slots are
   written as empty (horizontal) edges, which binning skips. */
__device__ __forceinline__ bool tri_has(const uint4 &T, uint32_t a, uint32_t b) {
    return (T.x == a && T.y == b) || (T.y == a && T.z == b) || (T.z == a && T.x == b);
}
__global__ void gb_stroke_edges(uint32_t ntris, const int4 *__restrict__ tri_a, const int4 *__restrict__ tri_b,
                                const uint4 *__restrict__ tri_idx, const uint32_t *__restrict__ tri_draw,
                                int4 *__restrict__ edges, uint32_t *__restrict__ edge_draw) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntris)
        return;
    const uint4    me = tri_idx[t];
    const uint32_t d  = tri_draw[t];
    if (!me.w) {
        for (int k = 0; k < 3; k++) {
            edges[3 * t + k]     = make_int4(0, 0, 0, 0);
            edge_draw[3 * t + k] = d;
        }
        return;
    }
    const uint4 none = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0);
    uint4       nb[4]; /* t-2, t-1, t+1, t+2, valid triangles of the same draw only */
    for (int k = 0; k < 4; k++) {
        const int64_t u = (int64_t)t + (k < 2 ? k - 2 : k - 1);
        nb[k]           = none;
        if (u >= 0 && u < (int64_t)ntris) {
            const uint4 T = tri_idx[u];
            if (T.w == me.w)
                nb[k] = T;
        }
    }
    const int4 ta = tri_a[t], tb = tri_b[t];
    const int2 v[3] = {make_int2(ta.x, ta.y), make_int2(ta.z, ta.w), make_int2(tb.x, tb.y)};
    const uint32_t ix[3] = {me.x, me.y, me.z};
    for (int k = 0; k < 3; k++) {
        const uint32_t a = ix[k], b = ix[(k + 1) % 3];
        const bool     fwd = tri_has(nb[2], b, a) && !tri_has(nb[1], b, a) && !tri_has(nb[3], a, b);
        const bool     bwd = tri_has(nb[1], b, a) && !tri_has(nb[2], b, a) && !tri_has(nb[0], a, b);
        const int2     p = v[k], q = v[(k + 1) % 3];
        edges[3 * t + k]     = (fwd || bwd) ? make_int4(0, 0, 0, 0) : make_int4(p.x, p.y, q.x, q.y);
        edge_draw[3 * t + k] = d;
    }
}

/* sample-row range [r0, r1] crossed by the half-open y interval [ylo, yhi) */
__device__ __forceinline__ void gb_row_range(int32_t ylo, int32_t yhi, uint32_t samples, int32_t *r0, int32_t *r1) {
    long long off  = samples == 4 ? 32 : 128;
    long long step = samples == 4 ? 64 : 256;
    long long a = (long long)ylo - off, b = (long long)yhi - off;
    /* ceil(a / step) */
    long long ca = a >= 0 ? (a + step - 1) / step : -((-a) / step);
    long long cb = b >= 0 ? (b + step - 1) / step : -((-b) / step);
    *r0          = (int32_t)(ca < -2147483647LL ? -2147483647LL : ca);
    *r1          = (int32_t)((cb - 1) > 2147483647LL ? 2147483647LL : cb - 1);
}

/* band range of a primitive, or false if it can touch no sample */
__device__ __forceinline__ bool gb_prim_bands(int32_t ylo, int32_t yhi, int32_t xmax, uint32_t samples,
                                              uint32_t nrows, uint32_t *b0, uint32_t *b1) {
    if (yhi <= ylo)
        return false;
    int32_t r0, r1;
    gb_row_range(ylo, yhi, samples, &r0, &r1);
    if (r0 < 0)
        r0 = 0;
    if (r1 > (int32_t)nrows - 1)
        r1 = (int32_t)nrows - 1;
    if (r0 > r1)
        return false;
    /* a crossing left of every sample adds nothing (an edge right of every
       sample still adds to whole rows) */
    if (xmax < 32)
        return false;
    *b0 = (uint32_t)r0 / GB_BAND_ROWS;
    *b1 = (uint32_t)r1 / GB_BAND_ROWS;
    return true;
}

/* Binning: count (SCATTER false) or write (SCATTER true) each edge's record
   (x0, y0, x1, y1) into every (band, draw) cell of its surface it touches,
   so that a cell is one contiguous block of 16-byte records the raster can
   stage with a single bulk copy.  The counting pass also folds every edge's
   x extent into its draw's box (min x, -max x), one set of atomics per draw
   of a warp (per block where the block's edges belong to one draw).  Every
   edge that is not horizontal
   counts, binned or not: a draw is passed over in a tile only when all of
   the edges that can cross a row lie right of the tile (a net zero on every
   row) or all left of it. */
template <bool SCATTER>
__global__ void gb_bin_edges(uint32_t nedges, const int4 *__restrict__ edges, const uint32_t *__restrict__ edge_draw,
                             const gb_draw *__restrict__ draws, const gb_surf *__restrict__ surfs, uint32_t samples,
                             uint32_t *__restrict__ cell, int4 *__restrict__ recs, uint32_t nunits,
                             int2 *__restrict__ dbox, uint32_t *__restrict__ dcnt,
                             unsigned long long *__restrict__ total) {
    const uint32_t e     = blockIdx.x * blockDim.x + threadIdx.x;
    const bool     valid = e < nedges;
    bool           ok    = valid;
    int4           ed    = make_int4(0, 0, 0, 0);
    uint32_t       d = 0xFFFFFFFFu, b0 = 0, b1 = 0;
    const gb_surf *sf = nullptr;
    if (ok) {
        ed = edges[e];
        d  = edge_draw[e];
        sf = &surfs[draws[d].surf];
        ok = gb_prim_bands(min(ed.y, ed.w), max(ed.y, ed.w), max(ed.x, ed.z), samples, sf->nrows, &b0, &b1);
    }
    if (!SCATTER && dbox) { /* every thread of the (full) block reaches the votes */
        __shared__ uint32_t s_d[8], s_n[8];
        __shared__ int32_t  s_mn[8], s_nmx[8];
        const bool          xb = valid && ed.y != ed.w;
        const int32_t       mn = xb ? min(ed.x, ed.z) : 0x7FFFFFFF, nmx = xb ? -max(ed.x, ed.z) : 0x7FFFFFFF;
        const uint32_t      dk = xb ? d : 0xFFFFFFFFu;
        const uint32_t      d0 = __reduce_min_sync(0xFFFFFFFFu, dk);
        const bool          wu = __all_sync(0xFFFFFFFFu, dk == d0 || dk == 0xFFFFFFFFu);
        const int32_t wmn = __reduce_min_sync(0xFFFFFFFFu, mn), wnmx = __reduce_min_sync(0xFFFFFFFFu, nmx);
        const uint32_t wn = __reduce_add_sync(0xFFFFFFFFu, xb ? 1u : 0u);
        const uint32_t w  = threadIdx.x >> 5;
        if ((threadIdx.x & 31u) == 0) { /* a warp of one draw hands its box to the block */
            s_d[w]   = wu ? d0 : 0xFFFFFFFEu;
            s_mn[w]  = wmn;
            s_nmx[w] = wnmx;
            s_n[w]   = wn;
        }
        if (!wu) { /* a warp of several draws: one set of atomics per draw (they come in runs) */
            bool left = xb;
            while (__any_sync(0xFFFFFFFFu, left)) {
                const uint32_t lead = __ffs(__ballot_sync(0xFFFFFFFFu, left)) - 1u;
                const uint32_t dl   = __shfl_sync(0xFFFFFFFFu, dk, lead);
                const bool     mine = left && dk == dl;
                const int32_t  rmn  = __reduce_min_sync(0xFFFFFFFFu, mine ? mn : 0x7FFFFFFF);
                const int32_t  rnmx = __reduce_min_sync(0xFFFFFFFFu, mine ? nmx : 0x7FFFFFFF);
                const uint32_t rn   = __popc(__ballot_sync(0xFFFFFFFFu, mine));
                if ((threadIdx.x & 31u) == lead) {
                    atomicMin(&dbox[dl].x, rmn);
                    atomicMin(&dbox[dl].y, rnmx);
                    atomicAdd(&dcnt[dl], rn);
                }
                left = left && !mine;
            }
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            const uint32_t nw  = blockDim.x >> 5, l = threadIdx.x;
            const uint32_t bd  = l < nw ? s_d[l] : 0xFFFFFFFFu;
            const int32_t  bmn = l < nw ? s_mn[l] : 0x7FFFFFFF, bnmx = l < nw ? s_nmx[l] : 0x7FFFFFFF;
            const uint32_t bn  = l < nw && bd < 0xFFFFFFFEu ? s_n[l] : 0u;
            const uint32_t b0d = __reduce_min_sync(0xFFFFFFFFu, bd);
            if (__all_sync(0xFFFFFFFFu, bd == b0d || bd == 0xFFFFFFFFu)) { /* the block's edges: one draw */
                const int32_t  m = __reduce_min_sync(0xFFFFFFFFu, bmn), n = __reduce_min_sync(0xFFFFFFFFu, bnmx);
                const uint32_t c = __reduce_add_sync(0xFFFFFFFFu, bn);
                if (l == 0 && b0d < 0xFFFFFFFEu) {
                    atomicMin(&dbox[b0d].x, m);
                    atomicMin(&dbox[b0d].y, n);
                    atomicAdd(&dcnt[b0d], c);
                }
            } else if (bd < 0xFFFFFFFEu) {
                atomicMin(&dbox[bd].x, bmn);
                atomicMin(&dbox[bd].y, bnmx);
                atomicAdd(&dcnt[bd], bn);
            }
        }
    }
    if (!SCATTER && total) {
        /* the record total in 64 bits (the cells' scan wraps at 2^32): the
           block's sum into one of 32 counters (every thread of the block
           reaches the barriers) */
        __shared__ unsigned long long s_tot;
        if (threadIdx.x == 0)
            s_tot = 0;
        __syncthreads();
        const uint32_t wn = __reduce_add_sync(0xFFFFFFFFu, ok ? b1 - b0 + 1u : 0u);
        if ((threadIdx.x & 31u) == 0 && wn)
            atomicAdd(&s_tot, (unsigned long long)wn);
        __syncthreads();
        if (threadIdx.x == 0 && s_tot)
            atomicAdd(&total[blockIdx.x & 31u], s_tot);
    }
    if (!ok)
        return;
    uint32_t *c = cell + sf->cell0 + (d - sf->draw0);
    for (uint32_t b = b0; b <= b1; b++) {
        uint32_t slot = atomicAdd(&c[(size_t)b * sf->ndraws], 1u);
        if (SCATTER && slot < nunits)
            recs[slot] = ed;
    }
}

/* The mean width of a frame's fill and stroke draws, clipped to the surface
   (W pixels), weighted by their edges (the draws that carry the raster's
   work decide): stats[0] += width x edges, stats[1] += edges.  It picks the
   raster's tile form. */
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}
__global__ void gb_draw_width_stats(uint32_t ndraws, const gb_draw *__restrict__ draws, const int2 *__restrict__ dbox,
                                    const uint32_t *__restrict__ dcnt, int32_t W,
                                    unsigned long long *__restrict__ stats) {
    const uint32_t     d = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long w = 0, n = 0;
    if (d < ndraws && draws[d].kind <= GB_DRAW_STROKE) {
        const int2    b  = dbox[d];
        const int32_t lo = max(0, min(W, b.x >> 8)), hi = max(0, min(W, ((-b.y) >> 8) + 1));
        if (b.x <= -b.y) {
            n = dcnt[d];
            w = (unsigned long long)max(0, hi - lo) * n;
        }
    }
    w = warp_sum_u64(w);
    n = warp_sum_u64(n);
    if ((threadIdx.x & 31u) == 0 && n) {
        atomicAdd(&stats[0], w);
        atomicAdd(&stats[1], n);
    }
}

/* *mx = max(*mx, the largest cell count): the heaviest (band, draw) cell,
   which one raster CTA works through on its own */
/* The draws that act on every band (paint, clear, the clip kinds) are
   active in every band of their surface: their cells' counts get
   GB_CELL_EVERY (bit 31; record counts stay below it, the frame's record
   total being limited to 2^31 - 1). */
__global__ void gb_cell_flags_every_band(uint32_t ndraws, const gb_draw *__restrict__ draws,
                                         const gb_surf *__restrict__ surfs, uint32_t *__restrict__ counts) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= ndraws || draws[d].kind <= GB_DRAW_STROKE)
        return;
    const gb_surf &sf = surfs[draws[d].surf];
    for (uint32_t b = 0; b < sf.nbands; b++)
        atomicOr(&counts[sf.cell0 + (uint64_t)b * sf.ndraws + (d - sf.draw0)], GB_CELL_EVERY); /* no read back */
}

/* The cells' record offsets and the raster's per-band draw lists, in two
   sweeps over the cell counts (band-major, draw-minor; bit 31 marks an
   every-band draw's cell): a cell's records start at the exclusive sum of
   the record counts before it (off), an active cell (one with records or
   with the mark) takes the next entry of alist, in cell order, so every
   band's entries are its active draws in draw order, and apos gets, at
   each band's first cell of every surface, the band's first alist entry
   (the raster reads apos only there and at the surface's end).  A tile of
   8192 cells per block: a warp takes 512 consecutive cells as 16 rows of 32
   (coalesced loads), summing counts with a warp scan and ranking active
   cells with a ballot per row. */
#define CELL_THREADS 512
#define CELL_ITEMS   16
#define CELL_TILE    (CELL_THREADS * CELL_ITEMS)

__global__ void __launch_bounds__(CELL_THREADS) gb_cells_reduce(uint64_t n, const uint32_t *__restrict__ cnt,
                                                                uint2 *__restrict__ bsum, uint32_t *__restrict__ mx) {
    __shared__ uint32_t s_s[CELL_THREADS / 32], s_a[CELL_THREADS / 32], s_m[CELL_THREADS / 32];
    const uint32_t      lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint64_t      base = (uint64_t)blockIdx.x * CELL_TILE + (uint64_t)w * (32u * CELL_ITEMS) + lane;
    uint32_t            s = 0, a = 0, m = 0;
#pragma unroll
    for (int k = 0; k < CELL_ITEMS; k++) {
        const uint64_t c = base + 32u * (uint32_t)k;
        const uint32_t v = c < n ? cnt[c] : 0u;
        s += v & ~GB_CELL_EVERY;
        a += v != 0u ? 1u : 0u;
        m = max(m, v & ~GB_CELL_EVERY);
    }
    s = __reduce_add_sync(0xFFFFFFFFu, s);
    a = __reduce_add_sync(0xFFFFFFFFu, a);
    m = __reduce_max_sync(0xFFFFFFFFu, m);
    if (lane == 0) {
        s_s[w] = s;
        s_a[w] = a;
        s_m[w] = m;
    }
    __syncthreads();
    if (w == 0) {
        s = lane < CELL_THREADS / 32 ? s_s[lane] : 0u;
        a = lane < CELL_THREADS / 32 ? s_a[lane] : 0u;
        m = lane < CELL_THREADS / 32 ? s_m[lane] : 0u;
        s = __reduce_add_sync(0xFFFFFFFFu, s);
        a = __reduce_add_sync(0xFFFFFFFFu, a);
        m = __reduce_max_sync(0xFFFFFFFFu, m);
        if (lane == 0) {
            bsum[blockIdx.x] = make_uint2(s, a);
            if (mx && m)
                atomicMax(mx, m);
        }
    }
}

/* one block: exclusive scan of the nb tiles' (records, active cells) in
   place, the totals at bsum[nb]; each thread sums a run of consecutive tiles */
__global__ void __launch_bounds__(1024) gb_cells_prefix(uint32_t nb, uint2 *__restrict__ bsum) {
    __shared__ uint32_t s_s[32], s_a[32];
    const uint32_t      per = (nb + 1023u) / 1024u, i0 = min(threadIdx.x * per, nb), i1 = min(i0 + per, nb);
    const uint32_t      lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t            s = 0, a = 0;
    for (uint32_t i = i0; i < i1; i++) {
        const uint2 v = bsum[i];
        s += v.x;
        a += v.y;
    }
    /* inclusive warp scans, then the warps' totals */
    uint32_t is = s, ia = a;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ts = __shfl_up_sync(0xFFFFFFFFu, is, o), ta = __shfl_up_sync(0xFFFFFFFFu, ia, o);
        if (lane >= (uint32_t)o) {
            is += ts;
            ia += ta;
        }
    }
    if (lane == 31) {
        s_s[w] = is;
        s_a[w] = ia;
    }
    __syncthreads();
    if (w == 0) {
        uint32_t vs = s_s[lane], va = s_a[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t ts = __shfl_up_sync(0xFFFFFFFFu, vs, o), ta = __shfl_up_sync(0xFFFFFFFFu, va, o);
            if (lane >= (uint32_t)o) {
                vs += ts;
                va += ta;
            }
        }
        s_s[lane] = vs;
        s_a[lane] = va;
    }
    __syncthreads();
    uint32_t rs = (w ? s_s[w - 1] : 0u) + is - s, ra = (w ? s_a[w - 1] : 0u) + ia - a;
    for (uint32_t i = i0; i < i1; i++) {
        const uint2 v = bsum[i];
        bsum[i]       = make_uint2(rs, ra);
        rs += v.x;
        ra += v.y;
    }
    if (threadIdx.x == 1023u)
        bsum[nb] = make_uint2(rs, ra);
}

__global__ void __launch_bounds__(CELL_THREADS)
    gb_cells_apply(uint64_t n, const uint32_t *__restrict__ cnt, const uint2 *__restrict__ bsum,
                   uint32_t *__restrict__ off, uint32_t *__restrict__ alist, uint32_t *__restrict__ apos,
                   const gb_surf *__restrict__ surfs, uint32_t nsurf) {
    __shared__ uint32_t s_pos[CELL_TILE]; /* per cell: active cells before it in the tile */
    __shared__ uint32_t s_s[CELL_THREADS / 32], s_a[CELL_THREADS / 32];
    const uint32_t      lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint64_t      c0   = (uint64_t)blockIdx.x * CELL_TILE;
    const uint64_t      base = c0 + (uint64_t)w * (32u * CELL_ITEMS) + lane;
    uint32_t            v[CELL_ITEMS], s = 0, a = 0;
#pragma unroll
    for (int k = 0; k < CELL_ITEMS; k++) {
        const uint64_t c = base + 32u * (uint32_t)k;
        v[k]             = c < n ? cnt[c] : 0u;
        s += v[k] & ~GB_CELL_EVERY;
        a += v[k] != 0u ? 1u : 0u;
    }
    s = __reduce_add_sync(0xFFFFFFFFu, s);
    a = __reduce_add_sync(0xFFFFFFFFu, a);
    if (lane == 0) {
        s_s[w] = s;
        s_a[w] = a;
    }
    __syncthreads();
    const uint2 bp = bsum[blockIdx.x];
    uint32_t    rs = bp.x, ra = 0;
    for (uint32_t j = 0; j < w; j++) {
        rs += s_s[j];
        ra += s_a[j];
    }
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < CELL_ITEMS; k++) {
        const uint32_t cn  = v[k] & ~GB_CELL_EVERY;
        uint32_t       inc = cn;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
            if (lane >= (uint32_t)o)
                inc += t;
        }
        const uint32_t am = __ballot_sync(0xFFFFFFFFu, v[k] != 0u);
        const uint32_t ea = ra + (uint32_t)__popc(am & lt);
        const uint64_t c  = base + 32u * (uint32_t)k;
        if (c < n) {
            off[c]            = rs + inc - cn;
            s_pos[c - c0]     = ea;
            if (v[k])
                alist[bp.y + ea] = (uint32_t)c;
        }
        rs += __shfl_sync(0xFFFFFFFFu, inc, 31);
        ra += (uint32_t)__popc(am);
    }
    __syncthreads();
    /* the band starts inside this tile, surface by surface (the surfaces'
       cells are consecutive ranges in table order) */
    const uint64_t c1 = min(c0 + (uint64_t)CELL_TILE, n);
    uint32_t       lo = 0, hi = nsurf;
    while (lo < hi) { /* the first surface whose cells end after c0 */
        const uint32_t mid = (lo + hi) >> 1;
        const gb_surf &S   = surfs[mid];
        if (S.cell0 + (uint64_t)S.nbands * S.ndraws <= c0)
            lo = mid + 1;
        else
            hi = mid;
    }
    for (uint32_t si = lo; si < nsurf; si++) {
        const gb_surf &S = surfs[si];
        if (S.cell0 >= c1)
            break;
        const uint64_t nd = S.ndraws;
        if (!nd)
            continue;
        const uint64_t kf = S.cell0 >= c0 ? 0u : (c0 - S.cell0 + nd - 1u) / nd;
        for (uint64_t k = kf + threadIdx.x; k <= S.nbands; k += CELL_THREADS) {
            const uint64_t c = S.cell0 + k * nd;
            if (c >= c1)
                break;
            apos[c] = bp.y + s_pos[c - c0];
        }
    }
    if (blockIdx.x == gridDim.x - 1u && threadIdx.x == 0) {
        const uint2 t = bsum[gridDim.x];
        off[n]        = t.x;
        apos[n]       = t.y;
    }
}
/* out[i] = src[idx[i]] */
__global__ void gb_gather_u32(uint32_t n, const uint64_t *__restrict__ idx, const uint32_t *__restrict__ src,
                              uint32_t *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = src[idx[i]];
}
extern "C" {
cudaError_t gb_launch_gather_u32(cudaStream_t st, uint32_t n, const uint64_t *idx, const uint32_t *src,
                                 uint32_t *out) {
    if (!n)
        return cudaSuccess;
    gb_gather_u32<<<(n + 255) / 256, 256, 0, st>>>(n, idx, src, out);
    return cudaGetLastError();
}
cudaError_t gb_launch_fill_pair_edges(cudaStream_t st, uint32_t npairs, const uint32_t *pair_sub,
                                      const uint32_t *sub_npts, uint32_t *counts) {
    if (!npairs)
        return cudaSuccess;
    gb_fill_pair_edges<<<(npairs + 255) / 256, 256, 0, st>>>(npairs, pair_sub, sub_npts, counts);
    return cudaGetLastError();
}
cudaError_t gb_launch_fill_edges(cudaStream_t st, uint32_t nedges, uint32_t npairs, const uint32_t *e_off,
                                 const uint32_t *pair_draw, const uint32_t *pair_sub, const gb_draw *draws,
                                 const uint32_t *sub_pt0, const uint32_t *sub_npts, const float2 *pts,
                                 const gb_surf *surfs, int4 *edges, uint32_t *edge_draw) {
    if (!nedges)
        return cudaSuccess;
    gb_fill_edges<<<(nedges + 255) / 256, 256, 0, st>>>(nedges, npairs, e_off, pair_draw, pair_sub, draws, sub_pt0,
                                                         sub_npts, pts, surfs, edges, edge_draw);
    return cudaGetLastError();
}
cudaError_t gb_launch_stroke_tris(cudaStream_t st, uint32_t ntris, uint32_t ndraw_s, const uint32_t *draw_tri0,
                                  const uint32_t *sdraw_id, const uint32_t *draw_vbase, const gb_draw *draws,
                                  const float2 *verts, const uint32_t *inds, const gb_surf *surfs, int4 *tri_a,
                                  int4 *tri_b, uint32_t *tri_draw, uint4 *tri_idx, int4 *edges, uint32_t *edge_draw) {
    if (!ntris)
        return cudaSuccess;
    gb_stroke_tris<<<(ntris + 255) / 256, 256, 0, st>>>(ntris, ndraw_s, draw_tri0, sdraw_id, draw_vbase, draws, verts,
                                                         inds, surfs, tri_a, tri_b, tri_draw, tri_idx);
    gb_stroke_edges<<<(ntris + 255) / 256, 256, 0, st>>>(ntris, tri_a, tri_b, tri_idx, tri_draw, edges, edge_draw);
    return cudaGetLastError();
}
cudaError_t gb_launch_bin(cudaStream_t st, int scatter, uint32_t nedges, const int4 *edges, const uint32_t *edge_draw,
                          const gb_draw *draws, const gb_surf *surfs, uint32_t samples, uint32_t *cell, int4 *recs,
                          uint32_t nunits, int2 *dbox, uint32_t *dcnt, unsigned long long *total) {
    if (nedges) {
        if (scatter)
            gb_bin_edges<true><<<(nedges + 255) / 256, 256, 0, st>>>(nedges, edges, edge_draw, draws, surfs, samples,
                                                                      cell, recs, nunits, nullptr, nullptr, nullptr);
        else
            gb_bin_edges<false><<<(nedges + 255) / 256, 256, 0, st>>>(nedges, edges, edge_draw, draws, surfs,
                                                                       samples, cell, nullptr, 0u, dbox, dcnt, total);
    }
    return cudaGetLastError();
}
cudaError_t gb_launch_cell_flags(cudaStream_t st, uint32_t ndraws, const gb_draw *draws, const gb_surf *surfs,
                                 uint32_t *counts) {
    if (ndraws)
        gb_cell_flags_every_band<<<(ndraws + 255) / 256, 256, 0, st>>>(ndraws, draws, surfs, counts);
    return cudaGetLastError();
}
cudaError_t gb_launch_draw_width_stats(cudaStream_t st, uint32_t ndraws, const gb_draw *draws, const int2 *dbox,
                                       const uint32_t *dcnt, uint32_t W, unsigned long long *stats) {
    if (ndraws)
        gb_draw_width_stats<<<(ndraws + 255) / 256, 256, 0, st>>>(ndraws, draws, dbox, dcnt, (int32_t)W, stats);
    return cudaGetLastError();
}
size_t gb_cells_scratch_words(uint64_t ncells) { return 2 * ((ncells + CELL_TILE - 1) / CELL_TILE + 1); }
cudaError_t gb_launch_cells_reduce(cudaStream_t st, uint64_t ncells, const uint32_t *counts, uint32_t *scratch,
                                   uint32_t *mx) {
    if (ncells)
        gb_cells_reduce<<<(uint32_t)((ncells + CELL_TILE - 1) / CELL_TILE), CELL_THREADS, 0, st>>>(
            ncells, counts, (uint2 *)scratch, mx);
    return cudaGetLastError();
}
cudaError_t gb_launch_cells_lists(cudaStream_t st, uint64_t ncells, const uint32_t *counts, uint32_t *scratch,
                                  uint32_t *off, uint32_t *alist, uint32_t *apos, const gb_surf *surfs, uint32_t nsurf) {
    if (!ncells) {
        cudaError_t e = cudaMemsetAsync(off, 0, 4, st);
        return e != cudaSuccess ? e : cudaMemsetAsync(apos, 0, 4, st);
    }
    const uint32_t nb = (uint32_t)((ncells + CELL_TILE - 1) / CELL_TILE);
    uint2         *bs = (uint2 *)scratch;
    gb_cells_prefix<<<1, 1024, 0, st>>>(nb, bs);
    gb_cells_apply<<<nb, CELL_THREADS, 0, st>>>(ncells, counts, bs, off, alist, apos, surfs, nsurf);
    return cudaGetLastError();
}
}
