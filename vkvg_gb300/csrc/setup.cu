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
 * Crossings: the surface is cut into bands of 16 sample rows.  Every edge's
 * exact crossing of every sample row is computed once per frame and stored as
 * a 32-bit record in its (band, draw) cell: a count pass sizes the cells, an
 * exclusive scan in band-major order gives every band a contiguous,
 * draw-ordered list, and an emit pass writes the records.
 */
#include "gb_types.h"
#include "xdiv.cuh"

#include <cuda_runtime.h>

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

__device__ __forceinline__ uint32_t gb_find(const uint32_t *__restrict__ off, uint32_t n, uint32_t e) {
    uint32_t lo = 0, hi = n;
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
                              const uint32_t *__restrict__ sub_npts, const float2 *__restrict__ pts, uint32_t W,
                              uint32_t H, int4 *__restrict__ edges, uint32_t *__restrict__ edge_draw) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedges)
        return;
    uint32_t p = gb_find(e_off, npairs, e);
    uint32_t s = pair_sub[p], d = pair_draw[p];
    uint32_t j = e - e_off[p], n = sub_npts[s], first = sub_pt0[s];
    gb_vp    m = make_vp(draws[d], W, H);
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
                               const uint32_t *__restrict__ inds, uint32_t W, uint32_t H, int4 *__restrict__ tri_a,
                               int4 *__restrict__ tri_b, uint32_t *__restrict__ tri_draw) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntris)
        return;
    uint32_t k  = gb_find(draw_tri0, ndraw_s, t);
    uint32_t d  = sdraw_id[k];
    gb_vp    m  = make_vp(draws[d], W, H);
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
    }
    tri_a[t]    = make_int4(a.x, a.y, b.x, b.y);
    tri_b[t]    = make_int4(c.x, c.y, valid, 0);
    tri_draw[t] = d;
}

/* sample rows R (0 <= R < nrows) with ylo <= off + R*step < yhi */
__device__ __forceinline__ bool gb_rows(int32_t ylo, int32_t yhi, uint32_t S, uint32_t nrows, int32_t *ra,
                                        int32_t *rb) {
    const int32_t off = S == 4 ? 32 : 128;
    const int32_t sh  = S == 4 ? 6 : 8;
    long long     a   = ((long long)ylo - off + (1 << sh) - 1) >> sh; /* ceil((ylo - off) / step) */
    long long     b   = (((long long)yhi - off + (1 << sh) - 1) >> sh) - 1;
    if (a < 0)
        a = 0;
    if (b > (long long)nrows - 1)
        b = (long long)nrows - 1;
    *ra = (int32_t)a;
    *rb = (int32_t)b;
    return a <= b;
}

/* One directed edge's crossings of the surface's sample rows.
   Count pass: add the number of crossings per band to its (band, draw) cell.
   Emit pass: reserve the slots with one atomic per band and write one 32-bit
   record per row: (k << 5) | (dir > 0) << 4 | (row within band), where k is
   the number of samples of that row left of the crossing (clamped to
   [0, W]); the exact crossing comes from one division at the first row and a
   quotient/remainder walk down the rows. */
template <bool EMIT>
__device__ __forceinline__ void gb_edge_xings(int32_t x0, int32_t y0, int32_t x1, int32_t y1, uint32_t d, uint32_t nd,
                                              uint32_t W, uint32_t S, uint32_t nrows, uint32_t *__restrict__ cell,
                                              uint32_t *__restrict__ recs, uint32_t nrecs) {
    if (y0 == y1)
        return;
    if (max(x0, x1) < 32)
        return; /* left of every sample: adds to none */
    int32_t ra, rb;
    if (!gb_rows(min(y0, y1), max(y0, y1), S, nrows, &ra, &rb))
        return;
    const uint32_t b0 = (uint32_t)ra / GB_BAND_ROWS, b1 = (uint32_t)rb / GB_BAND_ROWS;
    if (!EMIT) {
        for (uint32_t b = b0; b <= b1; b++) {
            int32_t lo = max(ra, (int32_t)(b * GB_BAND_ROWS)), hi = min(rb, (int32_t)(b * GB_BAND_ROWS + GB_BAND_ROWS - 1));
            atomicAdd(&cell[(size_t)b * nd + d], (uint32_t)(hi - lo + 1));
        }
        return;
    }
    const uint32_t  dbit = y0 < y1 ? 16u : 0u;
    const int32_t   off  = S == 4 ? 32 : 128;
    const int32_t   sh   = S == 4 ? 6 : 8;
    const int32_t   dy   = y1 - y0;
    const int32_t   den  = dy < 0 ? -dy : dy;
    const int32_t   dxn  = dy < 0 ? x0 - x1 : x1 - x0;
    const long long num  = (long long)dxn * ((long long)off + ((long long)ra << sh) - y0);
    long long       c    = gb_ceil_div(num, den); /* crossing - x0 at row ra, rounded up */
    long long       rem  = c * den - num;         /* in [0, den) */
    const long long dl   = (long long)dxn << sh;
    const long long qd   = gb_floor_div(dl, den);
    const long long rd   = dl - qd * den; /* in [0, den) */
    int32_t         R    = ra;
    for (uint32_t b = b0; b <= b1; b++) {
        int32_t  hi   = min(rb, (int32_t)(b * GB_BAND_ROWS + GB_BAND_ROWS - 1));
        uint32_t slot = atomicAdd(&cell[(size_t)b * nd + d], (uint32_t)(hi - R + 1));
        for (; R <= hi; R++) {
            const int32_t ox = S == 4 ? ((R & 3) == 0 ? 96 : (R & 3) == 1 ? 224 : (R & 3) == 2 ? 32 : 160) : 128;
            long long     k  = (((long long)x0 + c - 1 - ox) >> 8) + 1; /* samples px*256+ox <= crossing */
            if (k < 0)
                k = 0;
            if (k > (long long)W)
                k = W;
            if (slot < nrecs)
                recs[slot] = ((uint32_t)k << 5) | dbit | (uint32_t)(R & (GB_BAND_ROWS - 1));
            slot++;
            rem -= rd;
            c += qd;
            if (rem < 0) {
                rem += den;
                c += 1;
            }
        }
    }
}

template <bool EMIT>
__global__ void gb_xing_edges(uint32_t nedges, const int4 *__restrict__ edges, const uint32_t *__restrict__ edge_draw,
                              uint32_t nd, uint32_t W, uint32_t S, uint32_t nrows, uint32_t *__restrict__ cell,
                              uint32_t *__restrict__ recs, uint32_t nrecs) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nedges)
        return;
    int4 ed = edges[e];
    gb_edge_xings<EMIT>(ed.x, ed.y, ed.z, ed.w, edge_draw[e], nd, W, S, nrows, cell, recs, nrecs);
}
template <bool EMIT>
__global__ void gb_xing_tris(uint32_t ntris, const int4 *__restrict__ tri_a, const int4 *__restrict__ tri_b,
                             const uint32_t *__restrict__ tri_draw, uint32_t nd, uint32_t W, uint32_t S, uint32_t nrows,
                             uint32_t *__restrict__ cell, uint32_t *__restrict__ recs, uint32_t nrecs) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntris)
        return;
    int4 a = tri_a[t], b = tri_b[t];
    if (!b.z)
        return;
    /* a closed triangle right of every sample adds +1 and -1 per row: nothing */
    if (min(min(a.x, a.z), b.x) > (int32_t)((W - 1) * 256 + 224))
        return;
    uint32_t d = tri_draw[t];
    gb_edge_xings<EMIT>(a.x, a.y, a.z, a.w, d, nd, W, S, nrows, cell, recs, nrecs);
    gb_edge_xings<EMIT>(a.z, a.w, b.x, b.y, d, nd, W, S, nrows, cell, recs, nrecs);
    gb_edge_xings<EMIT>(b.x, b.y, a.x, a.y, d, nd, W, S, nrows, cell, recs, nrecs);
}

extern "C" {
cudaError_t gb_launch_fill_pair_edges(cudaStream_t st, uint32_t npairs, const uint32_t *pair_sub,
                                      const uint32_t *sub_npts, uint32_t *counts) {
    if (!npairs)
        return cudaSuccess;
    gb_fill_pair_edges<<<(npairs + 255) / 256, 256, 0, st>>>(npairs, pair_sub, sub_npts, counts);
    return cudaGetLastError();
}
cudaError_t gb_launch_fill_edges(cudaStream_t st, uint32_t nedges, uint32_t npairs, const uint32_t *e_off,
                                 const uint32_t *pair_draw, const uint32_t *pair_sub, const gb_draw *draws,
                                 const uint32_t *sub_pt0, const uint32_t *sub_npts, const float2 *pts, uint32_t W,
                                 uint32_t H, int4 *edges, uint32_t *edge_draw) {
    if (!nedges)
        return cudaSuccess;
    gb_fill_edges<<<(nedges + 255) / 256, 256, 0, st>>>(nedges, npairs, e_off, pair_draw, pair_sub, draws, sub_pt0,
                                                         sub_npts, pts, W, H, edges, edge_draw);
    return cudaGetLastError();
}
cudaError_t gb_launch_stroke_tris(cudaStream_t st, uint32_t ntris, uint32_t ndraw_s, const uint32_t *draw_tri0,
                                  const uint32_t *sdraw_id, const uint32_t *draw_vbase, const gb_draw *draws,
                                  const float2 *verts, const uint32_t *inds, uint32_t W, uint32_t H, int4 *tri_a,
                                  int4 *tri_b, uint32_t *tri_draw) {
    if (!ntris)
        return cudaSuccess;
    gb_stroke_tris<<<(ntris + 255) / 256, 256, 0, st>>>(ntris, ndraw_s, draw_tri0, sdraw_id, draw_vbase, draws, verts,
                                                         inds, W, H, tri_a, tri_b, tri_draw);
    return cudaGetLastError();
}
cudaError_t gb_launch_xings(cudaStream_t st, int emit, uint32_t nedges, const int4 *edges, const uint32_t *edge_draw,
                            uint32_t ntris, const int4 *tri_a, const int4 *tri_b, const uint32_t *tri_draw,
                            uint32_t ndraws, uint32_t W, uint32_t S, uint32_t nrows, uint32_t *cell, uint32_t *recs,
                            uint32_t nrecs) {
    if (nedges) {
        if (emit)
            gb_xing_edges<true><<<(nedges + 255) / 256, 256, 0, st>>>(nedges, edges, edge_draw, ndraws, W, S, nrows,
                                                                       cell, recs, nrecs);
        else
            gb_xing_edges<false><<<(nedges + 255) / 256, 256, 0, st>>>(nedges, edges, edge_draw, ndraws, W, S, nrows,
                                                                        cell, nullptr, 0u);
    }
    if (ntris) {
        if (emit)
            gb_xing_tris<true><<<(ntris + 255) / 256, 256, 0, st>>>(ntris, tri_a, tri_b, tri_draw, ndraws, W, S, nrows,
                                                                     cell, recs, nrecs);
        else
            gb_xing_tris<false><<<(ntris + 255) / 256, 256, 0, st>>>(ntris, tri_a, tri_b, tri_draw, ndraws, W, S,
                                                                      nrows, cell, nullptr, 0u);
    }
    return cudaGetLastError();
}
}
